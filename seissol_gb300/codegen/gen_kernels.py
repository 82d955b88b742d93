"""Generator of the FP32 CUDA-core kernels of the ADER-DG element update.

For each convergence order it writes one header with two kernels:

* ``sei_local_o{N}``    Cauchy-Kovalevskaya predictor (codegen/kernels/aderdg.py:463-537),
                        volume integral (:337-351) and local flux (:373-386);
* ``sei_neighbor_o{N}`` neighbour flux rDivM_i fP_h rT_j I_nb AminusT_i (:414-428);

plus ``sei_taylor_o{N}`` (derivativeTaylorExpansion, :531-536) for derivative
evaluation.  The global matrices enter the code as literals: every non-zero becomes
one FFMA with an immediate operand, zero entries produce no instruction, so each
kernel executes exactly the non-zero flops of the reference's sparse kernels.

Thread mapping: a CTA holds 32 cells and 9 warps; warp q owns quantity column q of
those 32 cells (lane = cell).  Products with a global matrix act on one column and
are thread-local; the per-cell 9x9 operators (star, A+, A-) mix columns and exchange
data through shared memory laid out [q][row][lane] (conflict-free).
"""
from __future__ import annotations

import os

import numpy as np

from .basis import global_matrices, nb2, nb3

NQ = 9
CPB = 32  # cells per block

# Non-zero pattern of the elastic star matrix (codegen/matrices/star.xml): for output
# column p, the source rows q.  The 24 non-zeros are stored per cell in this order
# (column-major over (q, p)).
STAR_NZ = [(6, 0), (7, 0), (8, 0), (6, 1), (7, 1), (8, 1), (6, 2), (7, 2), (8, 2), (6, 3), (7, 3), (7, 4), (8, 4),
           (6, 5), (8, 5), (0, 6), (3, 6), (5, 6), (1, 7), (3, 7), (4, 7), (2, 8), (4, 8), (5, 8)]


def star_sources():
    src, idx = [], []
    for p in range(NQ):
        ent = [(q, i) for i, (q, pp) in enumerate(STAR_NZ) if pp == p]
        while len(ent) < 3:
            ent.append((ent[0][0], -1))
        src.append([e[0] for e in ent])
        idx.append([e[1] for e in ent])
    return src, idx


def flit(v: float) -> str:
    """Exact float32 literal (hexadecimal)."""
    return float(np.float32(v)).hex() + "f"


def padded(b: int) -> int:
    """Column stride of DOF tensors: basis count rounded up to 4 floats (16 bytes)."""
    return (b + 3) // 4 * 4


def _cols(mat, rows=None, cols=None):
    """Non-zeros grouped by column: {l: [(k, val), ...]}, float32-rounded, zero-skipped."""
    r = mat.shape[0] if rows is None else rows
    c = mat.shape[1] if cols is None else cols
    out = {}
    for l in range(c):
        ent = [(k, float(mat[k, l])) for k in range(r) if mat[k, l] != 0.0 and np.float32(mat[k, l]) != 0]
        if ent:
            out[l] = ent
    return out


def _matvec(lines, ind, mat, src, dst, rows, cols, init_zero):
    """dst[k] (+)= sum_l mat[k, l] * src[l] (thread-local, column form)."""
    bycol = _cols(mat, rows, cols)
    touched = set()
    if init_zero:
        for k in range(rows):
            lines.append(f"{ind}{dst}[{k}] = 0.f;")
    for l in sorted(bycol):
        for k, v in bycol[l]:
            lines.append(f"{ind}{dst}[{k}] = fmaf({flit(v)}, {src}[{l}], {dst}[{k}]);")
            touched.add(k)
    return touched


def gen_order(order: int) -> str:
    B, F = nb3(order), nb2(order)
    G = global_matrices(order)
    src, idx = star_sources()
    L = []
    a = L.append
    a(f"// Generated by seissol_gb300/codegen/gen_kernels.py for convergence order {order} (B={B}, F={F}).")
    a("// Do not edit.")
    a("#pragma once")
    a(f"namespace sei_o{order} {{")
    a(f"constexpr int kOrder = {order}, kB = {B}, kBp = {padded(B)}, kF = {F}, kFP = {padded(F)}, kQ = 9, kCPB = {CPB};")
    a(f"constexpr int kDerivSize = {sum(nb3(order - i) for i in range(order)) * NQ};")
    a("// Cell stride (floats) of a DOF block staged in shared memory: 16 bytes of padding per cell.")
    a("constexpr int kSt = 9 * kBp + 4;")
    a("// Cell stride (floats) of the staged face traces of the volume-and-traces kernel.")
    a("constexpr int kTs = 9 * kFP + 4;")
    fl = nnz_flops(order)
    a(f"// Non-zero flops per cell of the ADER, local-integral and neighbour kernels (literal FFMAs and premixes).")
    a(f"constexpr double kFlopAder = {fl['ader']:.1f}, kFlopLocal = {fl['local']:.1f}, kFlopNeighbor = {fl['neighbor']:.1f};")
    a("__constant__ int c_src[9][3] = {" + ",".join("{" + ",".join(map(str, s)) + "}" for s in src) + "};")
    a("__constant__ int c_nzi[9][3] = {" + ",".join("{" + ",".join(map(str, s)) + "}" for s in idx) + "};")

    # ---------------- ADER + local kernels ----------------
    prologue = f"""
  extern __shared__ float sm[];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kCPB + lane;
  const bool valid = cell < n;
  const int cl = valid ? cell : n - 1;
  float* X = sm;  // [9][kB][32]
  const int s0 = c_src[q][0], s1 = c_src[q][1], s2 = c_src[q][2];
  const float* Xs0 = X + s0 * kB * 32 + lane;
  const float* Xs1 = X + s1 * kB * 32 + lane;
  const float* Xs2 = X + s2 * kB * 32 + lane;
  float* Xq = X + q * kB * 32 + lane;
  float st[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e)
#pragma unroll
    for (int s = 0; s < 3; ++s) {{
      const int i = c_nzi[q][s];
      st[e][s] = i >= 0 ? __ldg(star_nz + (size_t)cl * 72 + e * 24 + i) : 0.f;
    }}
  const float* qcol = Q + ((size_t)cl * 9 + q) * kBp;"""

    def emit_ck(staged=False):
        if staged:
            # the block's DOFs arrive by one bulk copy per cell into X (cell stride kSt floats,
            # 16 bytes of padding per cell spread the column reads over the banks); each thread
            # then reads its column from there instead of 14 strided float4 loads from HBM
            a("""  __shared__ uint64_t sei_mbar;
  const int cell0 = blockIdx.x * kCPB;
  const int cnt = n - cell0 < kCPB ? n - cell0 : kCPB;
  if (threadIdx.x == 0) sei_tc::mbarInit(&sei_mbar, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    if (lane == 0) sei_tc::mbarExpectTx(&sei_mbar, (unsigned)(cnt * 9 * kBp * 4));
    __syncwarp();
    if (lane < cnt) sei_tc::bulkCopyG2S(X + lane * kSt, Q + (size_t)(cell0 + lane) * 9 * kBp, 9 * kBp * 4, &sei_mbar);
  }
  if (!sei_tc::mbarWait(&sei_mbar, 0, 1u << 26)) {
    if (threadIdx.x == 0 && status) atomicExch(status, 1);
    (void)sei_tc::mbarWait(&sei_mbar, 0, 1u << 26);  // the copies in flight land before X is reused
  }
  float z[kBp];
  {
    const float4* src = reinterpret_cast<const float4*>(X + lane * kSt + q * kBp);
#pragma unroll
    for (int k4 = 0; k4 < kBp / 4; ++k4) {
      const float4 t = src[k4];
      z[4 * k4] = t.x;
      z[4 * k4 + 1] = t.y;
      z[4 * k4 + 2] = t.z;
      z[4 * k4 + 3] = t.w;
    }
  }
  __syncthreads();""")
        else:
            a("""  float z[kBp];
  sei_load_col<kBp>(qcol, z);""")
        a("""  float I[kBp];
#pragma unroll
  for (int k = 0; k < kBp; ++k) I[k] = coeffs.c[0] * z[k];
  const int dsl = derivs ? (dslot ? __ldg(dslot + cl) : cl) : -1;
  float* dbase = (dsl >= 0 && valid) ? derivs + (size_t)dsl * kDerivSize : nullptr;
  if (dbase) sei_store_col_scalar<kB>(dbase + q * kB, z);""")
        off = B * NQ
        for i in range(1, order):
            bp, bc = nb3(order - i + 1), nb3(order - i)
            a(f"  // ---- CK stage {i}: rows {bc} from {bp}")
            a("  {")
            a(f"#pragma unroll\n    for (int k = 0; k < {bp}; ++k) Xq[k * 32] = z[k];")
            a("    __syncthreads();")
            a(f"    float zn[{bc}];")
            a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) zn[k] = 0.f;")
            cols = [_cols(G["kDivMT"][e], bc, bp) for e in range(3)]
            for l in range(bp):
                if not any(l in c for c in cols):
                    continue
                a(f"    {{ const float x0 = Xs0[{l * 32}], x1 = Xs1[{l * 32}], x2 = Xs2[{l * 32}];")
                for e in range(3):
                    if l in cols[e]:
                        a(f"      const float y{e} = st[{e}][0] * x0 + st[{e}][1] * x1 + st[{e}][2] * x2;")
                for e in range(3):
                    for k, v in cols[e].get(l, []):
                        a(f"      zn[{k}] = fmaf({flit(v)}, y{e}, zn[{k}]);")
                a("    }")
            a("    __syncthreads();")
            a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) {{ I[k] = fmaf(coeffs.c[{i}], zn[k], I[k]); z[k] = zn[k]; }}")
            a(f"    if (dbase) sei_store_col_scalar<{bc}>(dbase + {off} + q * {bc}, zn);")
            off += bc * NQ
            a("  }")

    def emit_ck_lowreg():
        """CK predictor with I parked in the exchange area as its rows become final.

        The exchange keeps q-slabs of kB rows ([q][k][lane]).  Stage i reads rows [0, bp) and
        leaves rows [bc, bp) untouched, so after it the rows [bc, bp) of I (no later stage adds
        to them) are written there, each thread into its own column; only the rows still
        accumulating stay in registers.  dQ(0) is not kept in registers at all: after stage 1,
        c0 dQ(0) is read back from the exchange.  At the end the slabs hold all of I."""
        a("""  __shared__ uint64_t sei_mbar;
  const int cell0 = blockIdx.x * kCPB;
  const int cnt = n - cell0 < kCPB ? n - cell0 : kCPB;
  if (threadIdx.x == 0) sei_tc::mbarInit(&sei_mbar, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    if (lane == 0) sei_tc::mbarExpectTx(&sei_mbar, (unsigned)(cnt * 9 * kBp * 4));
    __syncwarp();
    if (lane < cnt) sei_tc::bulkCopyG2S(X + lane * kSt, Q + (size_t)(cell0 + lane) * 9 * kBp, 9 * kBp * 4, &sei_mbar);
  }
  if (!sei_tc::mbarWait(&sei_mbar, 0, 1u << 26)) {
    if (threadIdx.x == 0 && status) atomicExch(status, 1);
    (void)sei_tc::mbarWait(&sei_mbar, 0, 1u << 26);  // the copies in flight land before X is reused
  }
  const int dsl = derivs ? (dslot ? __ldg(dslot + cl) : cl) : -1;
  float* dbase = (dsl >= 0 && valid) ? derivs + (size_t)dsl * kDerivSize : nullptr;
  {
    float z[kBp];
    const float4* src = reinterpret_cast<const float4*>(X + lane * kSt + q * kBp);
#pragma unroll
    for (int k4 = 0; k4 < kBp / 4; ++k4) {
      const float4 t = src[k4];
      z[4 * k4] = t.x;
      z[4 * k4 + 1] = t.y;
      z[4 * k4 + 2] = t.z;
      z[4 * k4 + 3] = t.w;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kB; ++k) Xq[k * 32] = z[k];
    if (dbase) sei_store_col_scalar<kB>(dbase + q * kB, z);
  }
  __syncthreads();""")
        off = B * NQ
        ireg = 0  # rows of I held in registers (0 before stage 1)
        for i in range(1, order):
            bp, bc = nb3(order - i + 1), nb3(order - i)
            a(f"  // ---- CK stage {i}: rows {bc} from {bp}")
            a("  {")
            a(f"    float zn[{bc}];")
            a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) zn[k] = 0.f;")
            cols = [_cols(G["kDivMT"][e], bc, bp) for e in range(3)]
            for l in range(bp):
                if not any(l in c for c in cols):
                    continue
                a(f"    {{ const float x0 = Xs0[{l * 32}], x1 = Xs1[{l * 32}], x2 = Xs2[{l * 32}];")
                for e in range(3):
                    if l in cols[e]:
                        a(f"      const float y{e} = st[{e}][0] * x0 + st[{e}][1] * x1 + st[{e}][2] * x2;")
                for e in range(3):
                    for k, v in cols[e].get(l, []):
                        a(f"      zn[{k}] = fmaf({flit(v)}, y{e}, zn[{k}]);")
                a("    }")
            a("    __syncthreads();")
            if i == 1:
                # I = c0 dQ(0) + c1 dQ(1) on rows < bc; rows [bc, bp) of I are c0 dQ(0), final
                a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) I[k] = fmaf(coeffs.c[1], zn[k], coeffs.c[0] * Xq[k * 32]);")
                a(f"#pragma unroll\n    for (int k = {bc}; k < {bp}; ++k) Xq[k * 32] = coeffs.c[0] * Xq[k * 32];")
            else:
                a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) I[k] = fmaf(coeffs.c[{i}], zn[k], I[k]);")
                a(f"#pragma unroll\n    for (int k = {bc}; k < {bp}; ++k) Xq[k * 32] = I[k];")
            if i < order - 1:
                a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) Xq[k * 32] = zn[k];")
            else:
                a(f"#pragma unroll\n    for (int k = 0; k < {bc}; ++k) Xq[k * 32] = I[k];")
            a(f"    if (dbase) sei_store_col_scalar<{bc}>(dbase + {off} + q * {bc}, zn);")
            off += bc * NQ
            a("  }")
            a("  __syncthreads();")

    def emit_volume_flux(with_trace=False):
        emit_volume_part()
        emit_flux_part(with_trace)

    def emit_volume_part(acc_zero=False):
        a("  // ---- volume: Q += sum_e kDivM_e (I star_e)")
        a(f"#pragma unroll\n  for (int k = 0; k < kB; ++k) Xq[k * 32] = I[k];")
        a("  __syncthreads();")
        a("  float acc[kBp];")
        if acc_zero:
            a("#pragma unroll\n  for (int k = 0; k < kBp; ++k) acc[k] = 0.f;")
        else:
            a("  sei_load_col<kBp>(qcol, acc);")
        cols = [_cols(G["kDivM"][e]) for e in range(3)]
        for l in range(B):
            if not any(l in c for c in cols):
                continue
            a(f"  {{ const float x0 = Xs0[{l * 32}], x1 = Xs1[{l * 32}], x2 = Xs2[{l * 32}];")
            for e in range(3):
                if l in cols[e]:
                    a(f"    const float y{e} = st[{e}][0] * x0 + st[{e}][1] * x1 + st[{e}][2] * x2;")
            for e in range(3):
                for k, v in cols[e].get(l, []):
                    a(f"    acc[{k}] = fmaf({flit(v)}, y{e}, acc[{k}]);")
            a("  }")
        a("  __syncthreads();")

    def emit_flux_part(with_trace):
        for f in range(4):
            a(f"  // ---- local flux, face {f}: Q += rDivM_{f} ((fMrT_{f} I) AplusT_{f})")
            a("  {")
            a("    float T[kF];")
            _matvec(L, "    ", G["fMrT"][f], "I", "T", F, B, True)
            if with_trace:
                a("    sei_stage_trace<kF, kF, kFP>(sm, lane, q, T);")
            a(f"#pragma unroll\n    for (int m = 0; m < kF; ++m) X[(q * kF + m) * 32 + lane] = T[m];")
            a("    __syncthreads();")
            if with_trace:
                a(f"    sei_store_traces<kF, kF, kFP, kCPB>(n, sm, trace, {f}, tplane);")
            a(f"    const bool on = valid && ftype[(size_t)cl * 4 + {f}] != 1;")
            a(f"    const float* ap = aplus + ((size_t)cl * 4 + {f}) * 81 + 9 * q;")
            a("    float av[9];")
            a("#pragma unroll\n    for (int s = 0; s < 9; ++s) av[s] = on ? __ldg(ap + s) : 0.f;")
            bycol = _cols(G["rDivM"][f])
            for m in range(F):
                if m not in bycol:
                    continue
                a(f"    {{ float g = 0.f;")
                a(f"#pragma unroll\n      for (int s = 0; s < 9; ++s) g = fmaf(X[(s * kF + {m}) * 32 + lane], av[s], g);")
                for k, v in bycol[m]:
                    a(f"      acc[{k}] = fmaf({flit(v)}, g, acc[{k}]);")
                a("    }")
            a("    __syncthreads();")
            a("  }")

    def emit_traces_volume_reduce():
        """From I in registers: the four face traces through the shared area (as many faces at a
        time as the area holds, one bulk copy per cell and face out), then the volume integral,
        added to Q by bulk reduce-adds."""
        kst, kts = 9 * padded(B) + 4, 9 * padded(F) + 4
        slots = max(1, min(4, max(9 * B * 32, 32 * kst) // (32 * kts)))
        a(f"  // ---- face traces fMrT_f I, {slots} face(s) at a time through the shared area")
        for g0 in range(0, 4, slots):
            group = list(range(g0, min(4, g0 + slots)))
            if g0 > 0:
                a("  if (threadIdx.x < 32) sei_tc::bulkWaitRead();  // the previous faces' copies have read the area")
                a("  __syncthreads();")
            for f in group:
                a("  {")
                a("    float T[kF];")
                _matvec(L, "    ", G["fMrT"][f], "I", "T", F, B, True)
                a(f"    float4* stg = reinterpret_cast<float4*>(X + ({f - g0} * 32 + lane) * kTs + q * kFP);")
                a("#pragma unroll\n    for (int m4 = 0; m4 < kFP / 4; ++m4)")
                a("      stg[m4] = make_float4(4 * m4 < kF ? T[4 * m4 < kF ? 4 * m4 : 0] : 0.f, 4 * m4 + 1 < kF ? T[4 * m4 + 1 < kF ? 4 * m4 + 1 : 0] : 0.f,")
                a("                            4 * m4 + 2 < kF ? T[4 * m4 + 2 < kF ? 4 * m4 + 2 : 0] : 0.f, 4 * m4 + 3 < kF ? T[4 * m4 + 3 < kF ? 4 * m4 + 3 : 0] : 0.f);")
                a("  }")
            a("  sei_tc::fenceProxyAsync();")
            a("  __syncthreads();")
            a("  if (threadIdx.x < 32 && lane < cnt) {")
            for f in group:
                a(f"    sei_tc::bulkCopyS2G(trace + ((size_t){f} * tplane + cell0 + lane) * 9 * kFP, X + ({f - g0} * 32 + lane) * kTs, 9 * kFP * 4);")
            a("    sei_tc::bulkCommit();")
            a("  }")
        a("  if (threadIdx.x < 32) sei_tc::bulkWaitRead();")
        a("  __syncthreads();")
        emit_volume_part(acc_zero=True)
        a("""  // ---- Q += volume: staged, then one bulk reduce-add per cell
  {
    float4* dst = reinterpret_cast<float4*>(X + lane * kSt + q * kBp);
#pragma unroll
    for (int k4 = 0; k4 < kBp / 4; ++k4) dst[k4] = make_float4(acc[4 * k4], acc[4 * k4 + 1], acc[4 * k4 + 2], acc[4 * k4 + 3]);
  }
  sei_tc::fenceProxyAsync();
  __syncthreads();
  if (threadIdx.x < 32 && lane < cnt) {
    sei_tc::bulkReduceAddS2G(Q + (size_t)(cell0 + lane) * 9 * kBp, X + lane * kSt, 9 * kBp * 4);
    sei_tc::bulkCommit();
    sei_tc::bulkWaitRead();
  }""")

    # fused ADER + local integral
    a(f"""
// ADER + local integral in one launch.
// Q[n][9][Bp] in/out (in place), I[n][9][Bp] out, star_nz[n][3][24], aplus[n][4][81] (column-major 9x9),
// ftype[n][4] (1 = dynamic rupture: no local flux), coeffs Taylor integration coefficients,
// derivs: optional packed derivative output [slots][kDerivSize] (nullptr to skip); the slot of a
// cell is dslot[cell] (-1: not stored), or the cell itself when dslot is nullptr.
extern "C" __global__ void __launch_bounds__(288, 1)
sei_local_o{order}(int n, float* __restrict__ Q, float* __restrict__ Iout, const float* __restrict__ star_nz,
                   const float* __restrict__ aplus, const unsigned char* __restrict__ ftype,
                   SeiCoeffs coeffs, float* __restrict__ derivs, const int* __restrict__ dslot) {{""" + prologue)
    emit_ck()
    emit_volume_flux()
    a("  if (valid) {")
    a("    sei_store_col<kBp>(Q + ((size_t)cell * 9 + q) * kBp, acc);")
    a("    sei_store_col<kBp>(Iout + ((size_t)cell * 9 + q) * kBp, I);")
    a("  }")
    a("}")

    # ADER alone (Spacetime::computeAder)
    ader_ctas = int(os.environ.get("SEI_GEN_ADER_CTAS", "3"))
    lintv_ctas = int(os.environ.get("SEI_GEN_LINTV_CTAS", "2"))
    a(f"""
// Cauchy-Kovalevskaya predictor alone: I = sum_i coeffs[i] dQ(i) (Q unchanged), optional derivatives.
// {ader_ctas} CTAs per SM (rows of I that are final wait in shared memory, which keeps the registers
// low).  The block's 32 cells of Q arrive in shared memory by bulk copies and I leaves the same
// way (one 16-byte-aligned copy per cell each way), so HBM sees whole contiguous rows instead of
// every thread's strided column loads; status is set when a copy wait gives up.
extern "C" __global__ void __launch_bounds__(288, {ader_ctas})
sei_ader_o{order}(int n, const float* __restrict__ Q, float* __restrict__ Iout, const float* __restrict__ star_nz,
                  SeiCoeffs coeffs, float* __restrict__ derivs, const int* __restrict__ dslot, int* __restrict__ status) {{""" + prologue)
    a(f"  float I[{nb3(order - 1)}];")
    emit_ck_lowreg()
    a("""  // I of the block, complete in the exchange slabs, to the staging layout, then out by bulk copies
  {
    float Io[kBp];
#pragma unroll
    for (int k = 0; k < kB; ++k) Io[k] = Xq[k * 32];
#pragma unroll
    for (int k = kB; k < kBp; ++k) Io[k] = 0.f;
    __syncthreads();
    float4* dst = reinterpret_cast<float4*>(X + lane * kSt + q * kBp);
#pragma unroll
    for (int k4 = 0; k4 < kBp / 4; ++k4) dst[k4] = make_float4(Io[4 * k4], Io[4 * k4 + 1], Io[4 * k4 + 2], Io[4 * k4 + 3]);
  }
  sei_tc::fenceProxyAsync();
  __syncthreads();
  if (threadIdx.x < 32 && lane < cnt) {
    sei_tc::bulkCopyS2G(Iout + (size_t)(cell0 + lane) * 9 * kBp, X + lane * kSt, 9 * kBp * 4);
    sei_tc::bulkCommit();
    sei_tc::bulkWaitRead();
  }""")
    a("}")

    # local integral alone (Local::computeIntegral)
    a(f"""
// Volume + local flux from the time-integrated DOFs: Q += ... (in place).
extern "C" __global__ void __launch_bounds__(288, 1)
sei_lint_o{order}(int n, float* __restrict__ Q, const float* __restrict__ Iin, const float* __restrict__ star_nz,
                  const float* __restrict__ aplus, const unsigned char* __restrict__ ftype) {{""" + prologue)
    a("  float I[kBp];")
    a("  sei_load_col<kBp>(Iin + ((size_t)cl * 9 + q) * kBp, I);")
    emit_volume_flux()
    a("  if (valid) sei_store_col<kBp>(Q + ((size_t)cell * 9 + q) * kBp, acc);")
    a("}")
    a(f"""
// The same local integral, which also stores the face traces fMrT_f I of every cell,
// trace[4][tplane][9][kFP] (tplane cells per face plane; trace points at the first cell of this
// launch), for the neighbour kernel of the tensor-core path.
extern "C" __global__ void __launch_bounds__(288, 1)
sei_lint_trace_o{order}(int n, float* __restrict__ Q, const float* __restrict__ Iin, const float* __restrict__ star_nz,
                        const float* __restrict__ aplus, const unsigned char* __restrict__ ftype,
                        float* __restrict__ trace, int tplane) {{""" + prologue)
    a("  float I[kBp];")
    a("  sei_load_col<kBp>(Iin + ((size_t)cl * 9 + q) * kBp, I);")
    emit_volume_flux(with_trace=True)
    a("  if (valid) sei_store_col<kBp>(Q + ((size_t)cell * 9 + q) * kBp, acc);")
    a("}")
    a(f"""
// Volume integral alone (no local flux) plus the face traces fMrT_f I of every cell and face,
// trace[4][tplane][9][kFP]: the local integral of the path whose tensor-core neighbour kernel also
// applies the local flux (from these traces).  Shared memory is one area of max(exchange, DOF
// staging) floats: the block's I rows arrive in it by one bulk copy per cell (cell stride kSt);
// the traces go first, from I in registers, one face at a time staged in it ([cell][q][kFP],
// cell stride kTs) and out by one bulk copy per cell; then the volume integral uses it as its
// exchange, and its contribution, staged there ([cell][q][kBp]), is added to Q in L2 by one
// bulk f32 reduce-add per cell, so the kernel never reads Q.  The traces before the volume keep
// either I or the volume accumulator live, not both: {lintv_ctas} CTAs per SM.  status is set when
// the copy wait gives up.
extern "C" __global__ void __launch_bounds__(288, {lintv_ctas})
sei_lintv_o{order}(int n, float* __restrict__ Q, const float* __restrict__ Iin, const float* __restrict__ star_nz,
                   float* __restrict__ trace, int tplane, int* __restrict__ status) {{""" + prologue)
    a("""  __shared__ uint64_t sei_mbar;
  const int cell0 = blockIdx.x * kCPB;
  const int cnt = n - cell0 < kCPB ? n - cell0 : kCPB;
  if (threadIdx.x == 0) sei_tc::mbarInit(&sei_mbar, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    if (lane == 0) sei_tc::mbarExpectTx(&sei_mbar, (unsigned)(cnt * 9 * kBp * 4));
    __syncwarp();
    if (lane < cnt) sei_tc::bulkCopyG2S(X + lane * kSt, Iin + (size_t)(cell0 + lane) * 9 * kBp, 9 * kBp * 4, &sei_mbar);
  }
  if (!sei_tc::mbarWait(&sei_mbar, 0, 1u << 26)) {
    if (threadIdx.x == 0 && status) atomicExch(status, 1);
    (void)sei_tc::mbarWait(&sei_mbar, 0, 1u << 26);  // the copies in flight land before X is reused
  }
  float I[kBp];
  {
    const float4* src = reinterpret_cast<const float4*>(X + lane * kSt + q * kBp);
#pragma unroll
    for (int k4 = 0; k4 < kBp / 4; ++k4) {
      const float4 t = src[k4];
      I[4 * k4] = t.x;
      I[4 * k4 + 1] = t.y;
      I[4 * k4 + 2] = t.z;
      I[4 * k4 + 3] = t.w;
    }
  }
  __syncthreads();""")
    emit_traces_volume_reduce()
    a("}")

    # ADER + volume + traces (the predictor of the fused-flux path); at order 6 the 96 registers of
    # two CTAs per SM spill, one CTA keeps everything in registers
    lv_ctas = 1 if order >= 6 else 2
    a(f"""
// ADER, volume integral and face traces in one launch: the cell-local part of the step whose
// tensor-core neighbour kernel applies both the local and the neighbour flux (from these traces).
// I never leaves the chip.  Shared memory is one area of max(exchange, DOF staging) floats:
// the block's Q rows arrive in it by bulk copies; the CK stages use it as their exchange; the
// traces of one face at a time are staged in it ([cell][q][kFP], cell stride kTs) and leave by
// one bulk copy per cell; the volume integral uses it as its exchange; finally the volume
// contribution is staged in it ([cell][q][kBp], cell stride kSt) and added to Q in L2 by one
// bulk f32 reduce-add per cell, so Q is read from HBM once and written once.  {lv_ctas} CTA(s) per SM.
// derivs / dslot: optional packed derivative output as in sei_local.  status is set when the
// DOF copy wait gives up.
extern "C" __global__ void __launch_bounds__(288, {lv_ctas})
sei_localv_o{order}(int n, float* __restrict__ Q, const float* __restrict__ star_nz, SeiCoeffs coeffs,
                    float* __restrict__ derivs, const int* __restrict__ dslot, float* __restrict__ trace, int tplane,
                    int* __restrict__ status) {{""" + prologue)
    emit_ck(staged=True)
    emit_traces_volume_reduce()
    a("}")

    # ---------------- neighbour kernel ----------------
    a(f"""
// Q[n][9][B] updated in place with the neighbour flux of all regular faces.
// I[n][9][B] time-integrated DOFs of all cells, aminus[n][4][81], nbr[n][4], rel[n][4] = side | orient << 2,
// ftype[n][4] (0 = regular face).  Two CTAs per SM: at order 6 the register cap this implies
// (96) spills ~0.5 KB per thread to L1 but doubles the warps that hide the neighbour loads
// (measured 1.91 -> 1.72 ms per launch on 400k cells).
extern "C" __global__ void __launch_bounds__(288, 2)
sei_neighbor_o{order}(int n, float* __restrict__ Q, const float* __restrict__ I, const float* __restrict__ aminus,
                      const int* __restrict__ nbr, const unsigned char* __restrict__ rel,
                      const unsigned char* __restrict__ ftype) {{
  extern __shared__ float sm[];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kCPB + lane;
  const bool valid = cell < n;
  const int cl = valid ? cell : n - 1;
  float* X = sm;  // [9][kF][32]
  float* Xq = X + q * kF * 32 + lane;
  float acc[kBp];
  sei_load_col<kBp>(Q + ((size_t)cl * 9 + q) * kBp, acc);
#pragma unroll 1
  for (int f = 0; f < 4; ++f) {{
    const int nb = __ldg(nbr + (size_t)cl * 4 + f);
    const int r = rel[(size_t)cl * 4 + f];
    const bool on = valid && nb >= 0 && ftype[(size_t)cl * 4 + f] == 0;
    float x[kBp];
    sei_load_col<kBp>(I + ((size_t)(on ? nb : cl) * 9 + q) * kBp, x);
    float R[kF];
    switch (r & 3) {{""")
    for j in range(4):
        a(f"      case {j}: {{")
        _matvec(L, "        ", G["rT"][j], "x", "R", F, B, True)
        a("        break; }")
    a("    }")
    a("    float S[kF];")
    a("    switch (r >> 2) {")
    for h in range(3):
        a(f"      {'default' if h == 2 else 'case ' + str(h)}: {{")
        _matvec(L, "        ", G["fP"][h], "R", "S", F, F, True)
        a("        break; }")
    a("    }")
    a(f"#pragma unroll\n    for (int m = 0; m < kF; ++m) Xq[m * 32] = S[m];")
    a("    __syncthreads();")
    a("    const float* am = aminus + ((size_t)cl * 4 + f) * 81 + 9 * q;")
    a("    float av[9];")
    a("#pragma unroll\n    for (int s = 0; s < 9; ++s) av[s] = on ? __ldg(am + s) : 0.f;")
    a("    switch (f) {")
    for f in range(4):
        a(f"      case {f}: {{")
        bycol = _cols(G["rDivM"][f])
        for m in range(F):
            if m not in bycol:
                continue
            a(f"        {{ float g = 0.f;")
            a(f"#pragma unroll\n          for (int s = 0; s < 9; ++s) g = fmaf(X[(s * kF + {m}) * 32 + lane], av[s], g);")
            for k, v in bycol[m]:
                a(f"          acc[{k}] = fmaf({flit(v)}, g, acc[{k}]);")
            a("        }")
        a("        break; }")
    a("    }")
    a("    __syncthreads();")
    a("  }")
    a("  if (valid) sei_store_col<kBp>(Q + ((size_t)cell * 9 + q) * kBp, acc);")
    a("}")

    # ---------------- face traces of listed pool blocks (local time stepping) ----------------
    a(f"""
// Face traces fMrT_f I of the pool blocks blk[e], e < m, into trace[4][tplane][9][kFP] (zero padded):
// under local time stepping the half-step integrals a finer neighbour reads (their faces' traces
// feed the tensor-core neighbour kernel).  One thread per (entry, quantity).
extern "C" __global__ void __launch_bounds__(256)
sei_trace_blocks_o{order}(int m, const int* __restrict__ blk, const float* __restrict__ pool, float* __restrict__ trace,
                          int tplane) {{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)m * 9) return;
  const long e = t / 9;
  const int q = (int)(t % 9);
  const int b = __ldg(blk + e);
  float I[kBp];
  sei_load_col<kBp>(pool + ((size_t)b * 9 + q) * kBp, I);""")
    for f in range(4):
        a("  {")
        a("    float T[kF];")
        _matvec(L, "    ", G["fMrT"][f], "I", "T", F, B, True)
        a(f"    float4* o = reinterpret_cast<float4*>(trace + (((size_t){f} * tplane + b) * 9 + q) * kFP);")
        a("#pragma unroll\n    for (int m4 = 0; m4 < kFP / 4; ++m4)")
        a("      o[m4] = make_float4(4 * m4 < kF ? T[4 * m4 < kF ? 4 * m4 : 0] : 0.f, 4 * m4 + 1 < kF ? T[4 * m4 + 1 < kF ? 4 * m4 + 1 : 0] : 0.f,")
        a("                          4 * m4 + 2 < kF ? T[4 * m4 + 2 < kF ? 4 * m4 + 2 : 0] : 0.f, 4 * m4 + 3 < kF ? T[4 * m4 + 3 < kF ? 4 * m4 + 3 : 0] : 0.f);")
        a("  }")
    a("}")

    # ---------------- Taylor evaluation ----------------
    a(f"""
// out[n][9][B] = sum_i coeffs[i] dQ(i) from packed derivatives [n][kDerivSize]; one thread per (cell, q).
extern "C" __global__ void sei_taylor_o{order}(int n, const float* __restrict__ derivs, SeiCoeffs coeffs,
                                               float* __restrict__ out) {{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * 9) return;
  const long cell = t / 9;
  const int q = (int)(t % 9);
  const float* d = derivs + cell * kDerivSize;
  float o[kBp];
#pragma unroll
  for (int k = 0; k < kBp; ++k) o[k] = 0.f;""")
    off = 0
    for i in range(order):
        bi = nb3(order - i)
        a(f"  {{ const float* s = d + {off} + q * {bi};")
        a(f"#pragma unroll\n    for (int k = 0; k < {bi}; ++k) o[k] = fmaf(coeffs.c[{i}], s[k], o[k]); }}")
        off += bi * NQ
    a("  sei_store_col<kBp>(out + ((size_t)cell * 9 + q) * kBp, o);")
    a("}")

    # Taylor evaluation gathered into a block pool (local time stepping: a coarser neighbour's
    # derivatives integrated over the sub-interval of the finer cell; TimeCommon.cpp:40-87)
    a(f"""
// pool[dst[e]][9][Bp] = sum_i coeffs[i] dQ(i) of derivative slot src[e], e < m; one thread per (e, q).
extern "C" __global__ void sei_taylor_gather_o{order}(int m, const int* __restrict__ src, const int* __restrict__ dst,
                                                      const float* __restrict__ derivs, SeiCoeffs coeffs,
                                                      float* __restrict__ pool) {{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)m * 9) return;
  const long e = t / 9;
  const int q = (int)(t % 9);
  const float* d = derivs + (size_t)__ldg(src + e) * kDerivSize;
  float o[kBp];
#pragma unroll
  for (int k = 0; k < kBp; ++k) o[k] = 0.f;""")
    off = 0
    for i in range(order):
        bi = nb3(order - i)
        a(f"  {{ const float* s = d + {off} + q * {bi};")
        a(f"#pragma unroll\n    for (int k = 0; k < {bi}; ++k) o[k] = fmaf(coeffs.c[{i}], s[k], o[k]); }}")
        off += bi * NQ
    a("  sei_store_col<kBp>(pool + ((size_t)__ldg(dst + e) * 9 + q) * kBp, o);")
    a("}")
    a(f"}}  // namespace sei_o{order}")
    return "\n".join(L) + "\n"


def nnz_flops(order: int) -> dict:
    """Non-zero flop counts per cell of the generated kernels (ADER, local, neighbour)."""
    B, F = nb3(order), nb2(order)
    G = global_matrices(order)
    nz = lambda m, r=None, c=None: sum(len(v) for v in _cols(m, r, c).values())
    ader = 0
    for i in range(1, order):
        bp, bc = nb3(order - i + 1), nb3(order - i)
        ader += NQ * 2 * sum(nz(G["kDivMT"][e], bc, bp) for e in range(3)) + 3 * 2 * 24 * bc // NQ * NQ
        ader += 2 * bc * NQ
    ader += B * NQ
    vol = NQ * 2 * sum(nz(G["kDivM"][e]) for e in range(3)) + 3 * 2 * 24 * B
    lflux = sum(NQ * 2 * (nz(G["fMrT"][f]) + nz(G["rDivM"][f])) + 2 * 81 * F for f in range(4))
    rt = sum(nz(G["rT"][j]) for j in range(4)) / 4.0
    fp = sum(nz(G["fP"][h]) for h in range(3)) / 3.0
    nflux = sum(NQ * 2 * (rt + fp + nz(G["rDivM"][f])) + 2 * 81 * F for f in range(4))
    return {"ader": ader, "local": vol + lflux, "neighbor": nflux}


def write_all(outdir: str, orders=(4, 5, 6)) -> list:
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for o in orders:
        p = os.path.join(outdir, f"kernels_o{o}.cuh")
        src = gen_order(o)
        if not os.path.exists(p) or open(p).read() != src:
            with open(p, "w") as fh:
                fh.write(src)
        paths.append(p)
    return paths


def gen_dr_tables(order: int) -> str:
    """Device tables of the dynamic-rupture face matrices for one order."""
    from .basis import dr_matrices, gauss_legendre01
    D = dr_matrices(order)
    B = nb3(order)
    npts = D["points"].shape[0]
    glx, glw = gauss_legendre01(order)
    L = [f"// Generated by seissol_gb300/codegen/gen_kernels.py: dynamic-rupture tables, order {order}.",
         "#pragma once", f"namespace sei_dr_o{order} {{",
         f"constexpr int kOrder = {order}, kB = {B}, kNP = {npts};"]

    def arr(name, ty, vals, fmt):
        L.append(f"__device__ const {ty} {name}[{len(vals)}] = {{" + ",".join(fmt(v) for v in vals) + "};")

    f32 = lambda v: flit(v)
    f64 = lambda v: float(v).hex()
    # V3mTo2n[rel combo][k][l] row-major (point k, basis l)
    arr("kV3m", "float", np.concatenate([m.ravel() for m in D["V3mTo2n"]]), f32)
    # V3mTo2nTWDivM[rel combo][l][k] row-major (basis l, point k)
    arr("kTW", "float", np.concatenate([m.ravel() for m in D["V3mTo2nTWDivM"]]), f32)
    arr("kResample", "double", D["resample"].ravel(), f64)
    arr("kGLx", "double", glx, f64)
    arr("kGLw", "double", glw, f64)
    L.append(f"}}  // namespace sei_dr_o{order}")
    return "\n".join(L) + "\n"


def write_dr_tables(outdir: str, orders=(4,)) -> list:
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for o in orders:
        p = os.path.join(outdir, f"dr_tables_o{o}.cuh")
        src = gen_dr_tables(o)
        if not os.path.exists(p) or open(p).read() != src:
            with open(p, "w") as fh:
                fh.write(src)
        paths.append(p)
    return paths


# ---------------------------------------------------------------------------
# Tensor-core tables: stacked global matrices as the B operand (N x K, K-major) of
# tcgen05 kind::f16 MMAs, split into FP16 hi/lo after scaling every row n by 2^-f_n
# (max |row| in [0.5, 1)); stored in the core-matrix layout (8 rows x 16 bytes blocks,
# block (g, j) at (g * KC + j) * 128 bytes, KC = Kpad / 8).
# ---------------------------------------------------------------------------
def _pad(x, m):
    return (x + m - 1) // m * m


def _f16_split_rows(Mx):
    """Returns (hi, lo, exps): float16 parts of Mx * 2^-exps[n] per row n."""
    import math as _m
    exps = np.zeros(Mx.shape[0], dtype=np.int64)
    for n in range(Mx.shape[0]):
        mx = np.abs(Mx[n]).max()
        exps[n] = _m.frexp(mx)[1] if mx > 0 else 0
    S = Mx * np.ldexp(1.0, -exps)[:, None]
    hi = S.astype(np.float16)
    lo = (S - hi.astype(np.float64)).astype(np.float16)
    return hi, lo, exps


def _core_layout(A16, kpad):
    """N x Kpad float16 -> flat uint16 array in the K-major core-matrix layout."""
    n = A16.shape[0]
    kc = kpad // 8
    out = np.zeros(n * kpad, dtype=np.uint16)
    bits = A16.view(np.uint16)
    for r in range(n):
        for k in range(kpad):
            off = (((r >> 3) * kc + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2) // 2
            out[off] = bits[r, k]
    return out


def tc_operands(order):
    """Stacked B operands of the tensor-core kernels for one order (dense float64, padded)."""
    B, F = nb3(order), nb2(order)
    G = global_matrices(order)
    ops = {}
    # CK stages: rows e * bc + k, columns l < bp: kDivMT_e[k, l]
    for i in range(1, order):
        bp, bc = nb3(order - i + 1), nb3(order - i)
        N, K = _pad(3 * bc, 16), _pad(bp, 16)
        M = np.zeros((N, K))
        for e in range(3):
            M[e * bc:(e + 1) * bc, :bp] = G["kDivMT"][e][:bc, :bp]
        ops[f"ck{i}"] = M
    # volume and local-flux traces: rows e * B + k (kDivM_e), 3 B + f F + m (fMrT_f)
    N1, KB = _pad(3 * B + 4 * F, 16), _pad(B, 16)
    M = np.zeros((N1, KB))
    for e in range(3):
        M[e * B:(e + 1) * B, :B] = G["kDivM"][e]
    for f in range(4):
        M[3 * B + f * F:3 * B + (f + 1) * F, :B] = G["fMrT"][f]
    ops["vol"] = M
    # face projections back to the volume: rows k < B, columns f F + m: rDivM_f[k, m]
    M = np.zeros((_pad(B, 16), _pad(4 * F, 16)))
    for f in range(4):
        M[:B, f * F:(f + 1) * F] = G["rDivM"][f]
    ops["rdivm"] = M
    # neighbour traces of all four sides: rows j F + m: rT_j[m, l]
    M = np.zeros((_pad(4 * F, 16), KB))
    for j in range(4):
        M[j * F:(j + 1) * F, :B] = G["rT"][j]
    ops["rt"] = M
    # lift of the face-space flux back to the volume, as the A operand (M = 64 rows k) of the
    # transposed neighbour kernel: K = (face i, face basis m) with every face padded to KF = F
    # rounded up to 4 and then to 8 (whole core-matrix chunks per face)
    KF = _pad(_pad(F, 4), 8)
    M = np.zeros((64, 4 * KF))
    for f in range(4):
        M[:B, f * KF:f * KF + F] = G["rDivM"][f]
    ops["nbt"] = M
    # transposed local integral: volume stiffness blocks kDivM_d (rows 64 d + k, K = basis l, 64
    # wide) and the face-trace stack rT (rows KF i + m, 128 rows, K = basis l, 64 wide; read
    # K-major for the traces and MN-major, as rT^T, for the lift rDivM_i = diag(1/M) rT_i^T)
    M = np.zeros((192, 64))
    for e in range(3):
        M[64 * e:64 * e + B, :B] = G["kDivM"][e]
    ops["volt"] = M
    M = np.zeros((128, 64))
    for f in range(4):
        M[f * KF:f * KF + F, :B] = G["rT"][f]
    ops["rtt"] = M
    return ops


def gen_tc_tables(order: int) -> str:
    ops = tc_operands(order)
    L = [f"// Generated by seissol_gb300/codegen/gen_kernels.py: tensor-core operand tables, order {order}.",
         "#pragma once", "#include <cstdint>", f"namespace sei_tc_o{order} {{"]
    for name, M in ops.items():
        hi, lo, ex = _f16_split_rows(M)
        N, K = M.shape
        both = np.concatenate([_core_layout(hi, K), _core_layout(lo, K)])
        L.append(f"constexpr int k{name}_N = {N}, k{name}_K = {K};")
        L.append(f"__device__ __align__(16) const uint16_t k{name}_op[{both.size}] = {{" + ",".join(str(int(v)) for v in both) + "};")
        L.append(f"__device__ const float k{name}_scale[{N}] = {{" + ",".join(flit(np.ldexp(1.0, int(e))) for e in ex) + "};")
    # constants of the transposed local integral: fM_m of every trace row (times the row's
    # power-of-two scale) and 1/M_k of every basis function
    B, F = nb3(order), nb2(order)
    G = global_matrices(order)
    KF = _pad(_pad(F, 4), 8)
    _, _, ex = _f16_split_rows(ops["rtt"])
    fm = np.asarray(G["fM"], dtype=float)
    tsc = np.zeros(128)
    for f in range(4):
        for m in range(F):
            tsc[f * KF + m] = np.ldexp(1.0, int(ex[f * KF + m])) * fm[m]
    mass = np.asarray(G["M"], dtype=float)
    invm = np.zeros(64)
    invm[:B] = 1.0 / mass
    L.append("__device__ const float krtt_tsc[128] = {" + ",".join(flit(v) for v in tsc) + "};")
    L.append("__device__ const float kinvm[64] = {" + ",".join(flit(v) for v in invm) + "};")
    L.append(f"}}  // namespace sei_tc_o{order}")
    return "\n".join(L) + "\n"


def gen_tc_nb(order: int) -> str:
    """Face-trace map of the tensor-core neighbour kernel: S = fP_h diag(fM)^-1 T.

    The local integral stores the traces T_j = fMrT_j I = diag(fM) rT_j I of every face
    (fM, the face mass matrix, is diagonal), so the neighbour chain fP_h rT_j I_nb
    (codegen/kernels/aderdg.py:414-428) becomes fP_h diag(fM)^-1 T_j(nb).
    """
    F = nb2(order)
    G = global_matrices(order)
    fm = np.asarray(G["fM"], dtype=float)
    L = [f"// Generated by seissol_gb300/codegen/gen_kernels.py: neighbour face-trace map, order {order}.",
         "// Do not edit.", "#pragma once", f"namespace sei_tcnb_o{order} {{",
         f"constexpr int kF = {F}, kFP = {padded(F)};",
         "// s = fP_h diag(fM)^-1 t (orientation h; t: one quantity row of a stored face trace).",
         "__device__ __forceinline__ void applyFp(int h, const float (&t)[kFP], float (&s)[kF]) {",
         "  switch (h) {"]
    for h in range(3):
        M = np.asarray(G["fP"][h], dtype=float) / fm[None, :]
        L.append(f"    {'default' if h == 2 else 'case ' + str(h)}: {{")
        _matvec(L, "      ", M, "t", "s", F, F, True)
        L.append("      break;")
        L.append("    }")
    L.append("  }")
    L.append("}")
    L.append(f"}}  // namespace sei_tcnb_o{order}")
    return "\n".join(L) + "\n"


def write_tc_tables(outdir: str, orders=(4, 5, 6)) -> list:
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for o in orders:
        for name, gen in (("tc_tables", gen_tc_tables), ("tc_nb", gen_tc_nb)):
            p = os.path.join(outdir, f"{name}_o{o}.cuh")
            src = gen(o)
            if not os.path.exists(p) or open(p).read() != src:
                with open(p, "w") as fh:
                    fh.write(src)
            paths.append(p)
    return paths
