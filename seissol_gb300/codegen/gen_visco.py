"""Generator of the FP32 CUDA-core kernels of the viscoelastic element update (3 mechanisms,
27 quantities: 9 elastic + 6 memory variables per mechanism).

The 27 x 27 operators of the reference (codegen/kernels/equations/viscoelastic.py,
src/Equations/viscoelastic/Model/ViscoelasticSetup.h) have a structure these kernels use:

* the star matrices couple only velocities into memory variables, and mechanism l's coupling is
  -omega_l S_e with one strain-rate operator S_e (from the reference gradients) shared by all l;
* the source matrix E^T adds theta-weighted memory variables to the stresses and -omega_l to the
  diagonal of mechanism l's block;
* the flux into the memory variables of mechanism l is omega_l W with one 9 x 6 block W per face.

So a CTA holds 16 cells and 15 column tasks of 16 threads (half a warp each, one thread per cell):
tasks 0..8 run the elastic column q exactly like the elastic kernels (premix with the star
non-zeros, global matrices as FFMA literals), tasks 9..14 run the strain column j = q - 9 through
the same code with the strain sources (velocities) and coefficients, and then update the three
memory variables j of their cell elementwise.  Two CTAs share an SM (128 registers a thread), so
one CTA's loads and barriers overlap the other's arithmetic:

  ADER    dQ_i(mem l j) = -omega_l (E_i(j) + dQ_{i-1}(mem l j)),  E_i = sum_e kDivMT_e (dQ_{i-1} S_e)
  volume  Q(mem l j) += -omega_l (V(j) + I(mem l j)),             V   = sum_e kDivM_e (I S_e)
  flux    Q(mem l j) +=  omega_l sum_f R_f (I W_f)(j)

With the source term the derivatives keep all B basis rows at every stage (aderdg.py:463-537).
"""
from __future__ import annotations

import os

from .basis import global_matrices, nb2, nb3
from .gen_kernels import _cols, _matvec, flit, padded, star_sources

NQ = 27
NW = 15  # warps per CTA: 9 elastic + 6 strain columns
CPB = 32

# strain column j: velocity sources q, gradient component x and factor of S_e(q, j) = fac * grad_e(x),
# where star_e(q, mem l j) = -omega_l S_e(q, j) (A_x^T coupling entries -omega_l C_x with
# x = 0: C(6,0) = 1, C(7,3) = C(8,5) = 1/2; x = 1: C(7,1) = 1, C(6,3) = C(8,4) = 1/2;
# x = 2: C(8,2) = 1, C(7,4) = C(6,5) = 1/2)
STRAIN = [
    [(6, 0, 1.0)],
    [(7, 1, 1.0)],
    [(8, 2, 1.0)],
    [(7, 0, 0.5), (6, 1, 0.5)],
    [(8, 1, 0.5), (7, 2, 0.5)],
    [(8, 0, 0.5), (6, 2, 0.5)],
]


def _tables(lines):
    src, idx = star_sources()
    vsrc, vx, vfac = [], [], []
    for ent in STRAIN:
        e = ent + [(ent[0][0], 0, 0.0)] * (3 - len(ent))
        vsrc.append([t[0] for t in e])
        vx.append([t[1] for t in e])
        vfac.append([t[2] for t in e])
    allsrc = src + vsrc
    lines.append("__constant__ int c_src[15][3] = {" + ",".join("{" + ",".join(map(str, s)) + "}" for s in allsrc) + "};")
    lines.append("__constant__ int c_nzi[9][3] = {" + ",".join("{" + ",".join(map(str, s)) + "}" for s in idx) + "};")
    lines.append("__constant__ int c_vx[6][3] = {" + ",".join("{" + ",".join(map(str, s)) + "}" for s in vx) + "};")
    lines.append("__constant__ float c_vfac[6][3] = {" + ",".join("{" + ",".join(f"{v}f" for v in s) + "}"
                                                            for s in vfac) + "};")


PROLOGUE = """
  extern __shared__ float sm[];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kCPB + lane;
  const bool valid = cell < n;
  const int cl = valid ? cell : n - 1;
  const bool el = q < 9;
  const int jv = el ? 0 : q - 9;
  float* X = sm;  // [9][kB][32]: elastic columns exchanged for the premix
  const int s0 = c_src[q][0], s1 = c_src[q][1], s2 = c_src[q][2];
  const float* Xs0 = X + s0 * kB * 32 + lane;
  const float* Xs1 = X + s1 * kB * 32 + lane;
  const float* Xs2 = X + s2 * kB * 32 + lane;
  float* Xq = X + (el ? q : 0) * kB * 32 + lane;
  float st[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e)
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      if (el) {
        const int i = c_nzi[q][s];
        st[e][s] = i >= 0 ? __ldg(star_nz + (size_t)cl * 72 + e * 24 + i) : 0.f;
      } else {
        st[e][s] = c_vfac[jv][s] * __ldg(grad + (size_t)cl * 9 + e * 3 + c_vx[jv][s]);
      }
    }"""


# The ADER kernel: CPB_ADER cells per CTA, thread (column task q < 15, cell lane < CPB_ADER); at 16
# cells (240 threads) its exchange X [9][B][16] and memory variables M, IM [18][B][16] take 100.8 KB
# at order 5 and two CTAs share an SM (their stage barriers and compute overlap).
CPBA = 16
CPB_ADER = 16  # cells per CTA of the ADER kernel (column tasks of CPB_ADER threads; 8 measured 3 % slower)
ADER_CTAS = 2  # its CTAs per SM


def _prologue(w, const):
    """PROLOGUE for w cells per CTA (column tasks of w threads); const names w in the kernel."""
    return PROLOGUE.replace("const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;",
                            f"const int q = threadIdx.x / {const}, lane = threadIdx.x % {const};") \
                   .replace("const int cell = blockIdx.x * kCPB + lane;", f"const int cell = blockIdx.x * {const} + lane;") \
                   .replace("[9][kB][32]", f"[9][kB][{w}]").replace("kB * 32 + lane", f"kB * {const} + lane")


PROLOGUE_ADER = _prologue(16, "kCPBA")


def _premix_matvec(a, mats, dst, rows, cols, ind, w=32):
    """dst[k] += sum_e mats[e][k, l] (st_e . (Xs0, Xs1, Xs2)[l]) over the non-zero columns l
    (w cells per row of the exchange)."""
    cl = [_cols(m, rows, cols) for m in mats]
    for l in range(cols):
        if not any(l in c for c in cl):
            continue
        a(f"{ind}{{ const float x0 = Xs0[{l * w}], x1 = Xs1[{l * w}], x2 = Xs2[{l * w}];")
        for e in range(3):
            if l in cl[e]:
                a(f"{ind}  const float y{e} = st[{e}][0] * x0 + st[{e}][1] * x1 + st[{e}][2] * x2;")
        for e in range(3):
            for k, v in cl[e].get(l, []):
                a(f"{ind}  {dst}[{k}] = fmaf({flit(v)}, y{e}, {dst}[{k}]);")
        a(f"{ind}}}")


def _theta_from_smem(a, base, ind, w=32):
    """Stress column q < 6 of zn += sum_l theta coupling of the memory variables in shared memory
    (w cells per row)."""
    a(f"""{ind}if (el && q < 6) {{
{ind}#pragma unroll 1
{ind}  for (int m = 0; m < 3; ++m) {{
{ind}    const float* th = theta + (size_t)cl * 9 + m * 3;
{ind}    const int lo = q < 3 ? 0 : q, hi = q < 3 ? 3 : q + 1;
{ind}#pragma unroll 1
{ind}    for (int jj = lo; jj < hi; ++jj) {{
{ind}      const float c = q < 3 ? __ldg(th + (jj == q ? 0 : 1)) : __ldg(th + 2);
{ind}      const float* src = {base} + (m * 6 + jj) * kB * {w} + lane;
{ind}#pragma unroll
{ind}      for (int k = 0; k < kB; ++k) zn[k] = fmaf(c, src[k * {w}], zn[k]);
{ind}    }}
{ind}  }}
{ind}}}""")


def gen_visco(order: int) -> str:
    B, F = nb3(order), nb2(order)
    G = global_matrices(order)
    L = []
    a = L.append
    a(f"// Generated by seissol_gb300/codegen/gen_visco.py for convergence order {order} (B={B}, F={F}).")
    a("// Do not edit.")
    a("#pragma once")
    a(f"namespace sei_v{order} {{")
    a(f"constexpr int kOrder = {order}, kB = {B}, kBp = {padded(B)}, kF = {F}, kNQ = {NQ}, kCPB = {CPB}, kCPBA = {CPBA}, "
      f"kWA = {CPB_ADER};")
    a("// Stored derivatives of one cell: [stage][27][kB] (the source term keeps all basis rows).")
    a(f"constexpr int kDerivSize = {order} * {NQ} * {B};")
    _tables(L)

    # ---------------- ADER ----------------
    a(f"""
// Cauchy-Kovalevskaya predictor with the viscoelastic source term: I = sum_i coeffs[i] dQ(i).
// Q, I [n][27][Bp]; star_nz [n][3][24] (elastic, unrelaxed moduli); grad [n][3][3]; theta [n][3][3];
// omega: relaxation frequencies.  kWA cells per CTA, 15 kWA threads (column task q = tid / kWA:
// 0..8 elastic, 9..14 strain; cell lane = tid % kWA); shared memory: X [9][B][kWA], M and IM
// [18][B][kWA] (100.8 KB at order 5 and 16 cells: two CTAs per SM).
// derivs (nullable): derivative output [slots][kDerivSize]; the slot of a cell is dslot[cell]
// (-1: not stored), or the cell itself when dslot is nullptr.
extern "C" __global__ void __launch_bounds__({15 * CPB_ADER}, {ADER_CTAS})
sei_vader_o{order}(int n, const float* __restrict__ Q, float* __restrict__ Iout, const float* __restrict__ star_nz,
                   const float* __restrict__ grad, const float* __restrict__ theta, SeiOmega omega,
                   SeiCoeffs coeffs, float* __restrict__ derivs, const int* __restrict__ dslot) {{""" + _prologue(CPB_ADER, "kWA"))
    a("""  float* M = X + 9 * kB * kWA;    // memory variables of the current stage [l * 6 + j][kB][kWA]
  float* IM = M + 18 * kB * kWA;   // their time integral
  float z[kBp];
  float I[kBp];
  const int dsl = derivs ? (dslot ? __ldg(dslot + cl) : cl) : -1;
  float* dbase = (dsl >= 0 && valid) ? derivs + (size_t)dsl * kDerivSize : nullptr;
  if (el) {
    sei_load_col<kBp>(Q + ((size_t)cl * kNQ + q) * kBp, z);
#pragma unroll
    for (int k = 0; k < kBp; ++k) I[k] = coeffs.c[0] * z[k];
#pragma unroll
    for (int k = 0; k < kB; ++k) Xq[k * kWA] = z[k];
    if (dbase) sei_store_col_scalar<kB>(dbase + q * kB, z);
  } else {
#pragma unroll 1
    for (int m = 0; m < 3; ++m) {
      sei_load_col<kBp>(Q + ((size_t)cl * kNQ + 9 + 6 * m + jv) * kBp, z);
      float* Mm = M + (m * 6 + jv) * kB * kWA + lane;
      float* IMm = IM + (m * 6 + jv) * kB * kWA + lane;
#pragma unroll
      for (int k = 0; k < kB; ++k) {
        Mm[k * kWA] = z[k];
        IMm[k * kWA] = coeffs.c[0] * z[k];
      }
      if (dbase) sei_store_col_scalar<kB>(dbase + (9 + 6 * m + jv) * kB, z);
    }
  }""")
    for i in range(1, order):
        a(f"  // ---- stage {i}")
        a("  {")
        a("    __syncthreads();")
        a("    float zn[kB];")
        a("#pragma unroll\n    for (int k = 0; k < kB; ++k) zn[k] = 0.f;")
        _premix_matvec(a, G["kDivMT"], "zn", B, B, "    ", w=CPB_ADER)
        _theta_from_smem(a, "M", "    ", w=CPB_ADER)
        a("    __syncthreads();")
        a("    if (el) {")
        a(f"#pragma unroll\n      for (int k = 0; k < kB; ++k) I[k] = fmaf(coeffs.c[{i}], zn[k], I[k]);")
        if i < order - 1:  # the next stage's exchange (every thread has read X: the barrier above)
            a("#pragma unroll\n      for (int k = 0; k < kB; ++k) Xq[k * kWA] = zn[k];")
        a(f"      if (dbase) sei_store_col_scalar<kB>(dbase + {i} * kNQ * kB + q * kB, zn);")
        a("    } else {")
        a("#pragma unroll 1")
        a("      for (int m = 0; m < 3; ++m) {")
        a("        const float w = -omega.w[m];")
        a("        float* Mm = M + (m * 6 + jv) * kB * kWA + lane;")
        a("        float* IMm = IM + (m * 6 + jv) * kB * kWA + lane;")
        a("#pragma unroll")
        a("        for (int k = 0; k < kB; ++k) {")
        a("          const float nw = w * (zn[k] + Mm[k * kWA]);")
        a("          Mm[k * kWA] = nw;")
        a(f"          IMm[k * kWA] = fmaf(coeffs.c[{i}], nw, IMm[k * kWA]);")
        a(f"          if (dbase) dbase[{i} * kNQ * kB + (9 + 6 * m + jv) * kB + k] = nw;")
        a("        }")
        a("      }")
        a("    }")
        a("  }")
    a("""  if (valid) {
    if (el) {
      sei_store_col<kBp>(Iout + ((size_t)cell * kNQ + q) * kBp, I);
    } else {
#pragma unroll 1
      for (int m = 0; m < 3; ++m) {
        const float* IMm = IM + (m * 6 + jv) * kB * kWA + lane;
#pragma unroll
        for (int k = 0; k < kB; ++k) z[k] = IMm[k * kWA];
#pragma unroll
        for (int k = kB; k < kBp; ++k) z[k] = 0.f;
        sei_store_col<kBp>(Iout + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, z);
      }
    }
  }
}""")

    # ---------------- volume + local flux ----------------
    a(f"""
// Volume + local flux from the time-integrated DOFs (in place on Q).  aplus [n][4][81] (elastic
// block), wplus [n][4][54] (memory block per unit omega), ftype [n][4].
extern "C" __global__ void __launch_bounds__(240, 2)
sei_vlint_o{order}(int n, float* __restrict__ Q, const float* __restrict__ Iin, const float* __restrict__ star_nz,
                   const float* __restrict__ grad, const float* __restrict__ theta, SeiOmega omega,
                   const float* __restrict__ aplus, const float* __restrict__ wplus,
                   const unsigned char* __restrict__ ftype) {{""" + PROLOGUE_ADER)
    a("""  float I[kBp];
  // TH [9][kB][16]: theta-weighted sums of the time-integrated memory variables, formed by the
  // strain tasks from the columns they own: slot j < 3 A_j = sum_l theta_l0 I(l, j), slot j in
  // 3..5 C_j = sum_l theta_l2 I(l, j), slot 6 + j (j < 3) B_j = sum_l theta_l1 I(l, j)
  float* TH = X + 9 * kB * 16;
  if (el) {
    sei_load_col<kBp>(Iin + ((size_t)cl * kNQ + q) * kBp, I);
#pragma unroll
    for (int k = 0; k < kB; ++k) Xq[k * 16] = I[k];
  } else {
    float* ta = TH + jv * kB * 16 + lane;
    float* tb = TH + (6 + (jv < 3 ? jv : 0)) * kB * 16 + lane;
#pragma unroll 1
    for (int m = 0; m < 3; ++m) {
      const float* th = theta + (size_t)cl * 9 + m * 3;
      const float ca = __ldg(th + (jv < 3 ? 0 : 2)), cb = __ldg(th + 1);
      sei_load_col<kBp>(Iin + ((size_t)cl * kNQ + 9 + 6 * m + jv) * kBp, I);
#pragma unroll
      for (int k = 0; k < kB; ++k) {
        ta[k * 16] = m ? fmaf(ca, I[k], ta[k * 16]) : ca * I[k];
        if (jv < 3) tb[k * 16] = m ? fmaf(cb, I[k], tb[k * 16]) : cb * I[k];
      }
    }
  }
  __syncthreads();
  float acc[kBp];
  if (el) {
    sei_load_col<kBp>(Q + ((size_t)cl * kNQ + q) * kBp, acc);
  } else {
#pragma unroll
    for (int k = 0; k < kBp; ++k) acc[k] = 0.f;
  }
  // ---- volume: elastic columns Q += sum_e kDivM_e (I star_e); strain columns V = sum_e kDivM_e (I S_e)""")
    _premix_matvec(a, G["kDivM"], "acc", B, B, "  ", w=16)
    a("""  if (!el) {  // strain columns accumulate D = flux - V
#pragma unroll
    for (int k = 0; k < kBp; ++k) acc[k] = -acc[k];
  }
  // ---- source term of the stresses: normal stress q < 3 adds A_q + B_j + B_j' (j, j' != q),
  // shear stress q in 3..5 adds C_q
  if (el && q < 3) {
    const float* a0 = TH + q * kB * 16 + lane;
    const float* b1 = TH + (6 + (q + 1) % 3) * kB * 16 + lane;
    const float* b2 = TH + (6 + (q + 2) % 3) * kB * 16 + lane;
#pragma unroll
    for (int k = 0; k < kB; ++k) acc[k] += a0[k * 16] + b1[k * 16] + b2[k * 16];
  } else if (el && q < 6) {
    const float* c0 = TH + q * kB * 16 + lane;
#pragma unroll
    for (int k = 0; k < kB; ++k) acc[k] += c0[k * 16];
  }
  __syncthreads();""")
    for f in range(4):
        a(f"  // ---- local flux, face {f}: elastic Q += rDivM_{f} ((fMrT_{f} I) A+), strain D += rDivM_{f} ((fMrT_{f} I) W+)")
        a("  {")
        a("    if (el) {")
        a("      float T[kF];")
        _matvec(L, "      ", G["fMrT"][f], "I", "T", F, B, True)
        a("#pragma unroll\n      for (int m = 0; m < kF; ++m) Xq[m * 16] = T[m];")
        a("    }")
        a("    __syncthreads();")
        a(f"    const bool on = valid && ftype[(size_t)cl * 4 + {f}] != 1;")
        a(f"    const float* ap = el ? aplus + ((size_t)cl * 4 + {f}) * 81 + 9 * q : wplus + ((size_t)cl * 4 + {f}) * 54 + 9 * jv;")
        a("    float av[9];")
        a("#pragma unroll\n    for (int s = 0; s < 9; ++s) av[s] = on ? __ldg(ap + s) : 0.f;")
        bycol = _cols(G["rDivM"][f])
        for m in range(F):
            if m not in bycol:
                continue
            a("    { float g = 0.f;")
            a(f"#pragma unroll\n      for (int s = 0; s < 9; ++s) g = fmaf(X[(s * kB + {m}) * 16 + lane], av[s], g);")
            for k, v in bycol[m]:
                a(f"      acc[{k}] = fmaf({flit(v)}, g, acc[{k}]);")
            a("    }")
        a("    __syncthreads();")
        a("  }")
    a("""  if (valid) {
    if (el) {
      sei_store_col<kBp>(Q + ((size_t)cell * kNQ + q) * kBp, acc);
    } else {
      // memory variable j of mechanism l: Q += omega_l (D - I)
#pragma unroll 1
      for (int m = 0; m < 3; ++m) {
        float qm[kBp], im[kBp];
        sei_load_col<kBp>(Q + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, qm);
        sei_load_col<kBp>(Iin + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, im);
#pragma unroll
        for (int k = 0; k < kB; ++k) qm[k] = fmaf(omega.w[m], acc[k] - im[k], qm[k]);
        sei_store_col<kBp>(Q + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, qm);
      }
    }
  }
}""")

    # ---------------- neighbour flux ----------------
    a(f"""
// Neighbour flux of the regular faces (in place on Q): elastic columns as in the elastic kernel
// with A- (elastic block); the memory variables j of mechanism l receive omega_l rDivM_f ((traces) W-).
extern "C" __global__ void __launch_bounds__(240, 2)
sei_vneighbor_o{order}(int n, float* __restrict__ Q, const float* __restrict__ I, const float* __restrict__ aminus,
                       const float* __restrict__ wminus, const int* __restrict__ nbr,
                       const unsigned char* __restrict__ rel, const unsigned char* __restrict__ ftype,
                       SeiOmega omega) {{
  extern __shared__ float sm[];
  const int q = threadIdx.x >> 4, lane = threadIdx.x & 15;
  const int cell = blockIdx.x * kCPBA + lane;
  const bool valid = cell < n;
  const int cl = valid ? cell : n - 1;
  const bool el = q < 9;
  const int jv = el ? 0 : q - 9;
  float* X = sm;  // [9][kF][16]
  float* Xq = X + (el ? q : 0) * kF * 16 + lane;
  float acc[kBp];
  if (el) {{
    sei_load_col<kBp>(Q + ((size_t)cl * kNQ + q) * kBp, acc);
  }} else {{
#pragma unroll
    for (int k = 0; k < kBp; ++k) acc[k] = 0.f;
  }}
#pragma unroll 1
  for (int f = 0; f < 4; ++f) {{
    const int nb = __ldg(nbr + (size_t)cl * 4 + f);
    const int r = rel[(size_t)cl * 4 + f];
    const bool on = valid && nb >= 0 && ftype[(size_t)cl * 4 + f] == 0;
    if (el) {{
      float x[kBp];
      sei_load_col<kBp>(I + ((size_t)(on ? nb : cl) * kNQ + q) * kBp, x);
      float R[kF];
      switch (r & 3) {{""")
    for j in range(4):
        a(f"        case {j}: {{")
        _matvec(L, "          ", G["rT"][j], "x", "R", F, B, True)
        a("          break; }")
    a("      }")
    a("      float S[kF];")
    a("      switch (r >> 2) {")
    for h in range(3):
        a(f"        {'default' if h == 2 else 'case ' + str(h)}: {{")
        _matvec(L, "          ", G["fP"][h], "R", "S", F, F, True)
        a("          break; }")
    a("      }")
    a("#pragma unroll\n      for (int m = 0; m < kF; ++m) Xq[m * 16] = S[m];")
    a("    }")
    a("    const float* am = el ? aminus + ((size_t)cl * 4 + f) * 81 + 9 * q : wminus + ((size_t)cl * 4 + f) * 54 + 9 * jv;")
    a("    float av[9];")
    a("#pragma unroll\n    for (int s = 0; s < 9; ++s) av[s] = on ? __ldg(am + s) : 0.f;")
    a("    __syncthreads();")
    a("    switch (f) {")
    for f in range(4):
        a(f"      case {f}: {{")
        bycol = _cols(G["rDivM"][f])
        for m in range(F):
            if m not in bycol:
                continue
            a("        { float g = 0.f;")
            a(f"#pragma unroll\n          for (int s = 0; s < 9; ++s) g = fmaf(X[(s * kF + {m}) * 16 + lane], av[s], g);")
            for k, v in bycol[m]:
                a(f"          acc[{k}] = fmaf({flit(v)}, g, acc[{k}]);")
            a("        }")
        a("        break; }")
    a("    }")
    a("    __syncthreads();")
    a("  }")
    a("""  if (valid) {
    if (el) {
      sei_store_col<kBp>(Q + ((size_t)cell * kNQ + q) * kBp, acc);
    } else {
#pragma unroll 1
      for (int m = 0; m < 3; ++m) {
        float qm[kBp];
        sei_load_col<kBp>(Q + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, qm);
#pragma unroll
        for (int k = 0; k < kB; ++k) qm[k] = fmaf(omega.w[m], acc[k], qm[k]);
        sei_store_col<kBp>(Q + ((size_t)cell * kNQ + 9 + 6 * m + jv) * kBp, qm);
      }
    }
  }
}""")
    a(f"}}  // namespace sei_v{order}")
    return "\n".join(L) + "\n"


VISCO_ORDERS = (4, 5)


def write_all(outdir: str, orders=VISCO_ORDERS) -> list:
    os.makedirs(outdir, exist_ok=True)
    paths = []
    for o in orders:
        p = os.path.join(outdir, f"kernels_visco_o{o}.cuh")
        src = gen_visco(o)
        if not os.path.exists(p) or open(p).read() != src:
            with open(p, "w") as fh:
                fh.write(src)
        paths.append(p)
    return paths
