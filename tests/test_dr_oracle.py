"""Dynamic-rupture oracle pins and host set-up checks (CPU only).

* face quadrature and matrices vs codegen/matrices/dr_stroud_matrices_{4,5,6}.json (fixture);
* precompute / postcompute of tests/DynamicRupture/FrictionLaws/FrictionSolverCommon.t.h,
  restated with its analytic inputs (qP = o + q + p, qM = 2 (o + q + p), impedances 10/20/15/25,
  time weights 1, 2, ...; tolerance 1e6 eps);
* the product's C++ fault set-up (face list, TinvT, flux solvers, impedances) vs the oracle;
* the oracle's Newton root of the rate-and-state residual vs a bracketing bisection.
"""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

from oracle import dg_setup, oracle_py

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("order", [4, 5, 6])
def test_dr_matrices_pinned(order):
    pin = json.load(open(os.path.join(HERE, "golden", "dr_matrices_pin.json")))[str(order)]
    m = dg_setup.dr_matrices(order)
    P = np.zeros(pin["quadpoints"]["shape"])
    for r, c, v in pin["quadpoints"]["entries"]:
        P[r, c] = v
    W = np.zeros(pin["quadweights"]["shape"][0])
    for r, c, v in pin["quadweights"]["entries"]:
        W[r] = v
    assert np.abs(m["points"] - P).max() < 1e-14
    assert np.abs(m["weights"] - W).max() < 1e-15
    for side in range(4):
        for rel in range(4):
            for name, mat in (("V3mTo2n", m["V3mTo2n"][side * 4 + rel]), ("V3mTo2nTWDivM", m["V3mTo2nTWDivM"][side * 4 + rel])):
                spec = pin[f"{name}({side},{rel})"]
                assert list(mat.shape) == spec["shape"]
                assert math.isclose(np.linalg.norm(mat), spec["fro"], rel_tol=1e-12)
                for r, c, v in spec["sample"]:
                    assert abs(mat[r, c] - v) <= 1e-12 * max(1.0, abs(v))
    spec = pin["resample"]
    for r, c, v in spec["sample"]:
        assert abs(m["resample"][r, c] - v) <= 1e-12


def _kat_inputs(npts, nts):
    qp = np.zeros((nts, 9, npts))
    qm = np.zeros((nts, 9, npts))
    for o in range(nts):
        for q in range(9):
            for p in range(npts):
                qp[o, q, p] = o + q + p
                qm[o, q, p] = 2 * (o + q + p)
    zp, zs, zpn, zsn = 10.0, 20.0, 15.0, 25.0
    imp = np.array([zp, zs, zpn, zsn, zp * zpn / (zp + zpn), zs * zsn / (zs + zsn), 1 / zs + 1 / zsn])
    return qp, qm, imp


def test_friction_common_known_answer():
    L = oracle_py.lib(np.float64)
    npts, nts = 32, 4
    qp, qm, imp = _kat_inputs(npts, nts)
    out = np.zeros((3, nts, npts))
    L.oracle_dr_precompute.restype = None
    L.oracle_dr_precompute(npts, nts, imp.ctypes.data_as(C.c_void_p), qp.ctypes.data_as(C.c_void_p),
                           qm.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    eps = 1e6 * np.finfo(np.float64).eps
    etap, etas = imp[4], imp[5]
    for o in range(nts):
        for p in range(npts):
            qP = lambda q: o + q + p
            qM = lambda q: 2 * (o + q + p)
            exp_n = etap * (qM(6) - qP(6) + qP(0) / 10 + qM(0) / 15)
            exp_1 = etas * (qM(7) - qP(7) + qP(3) / 20 + qM(3) / 25)
            exp_2 = etas * (qM(8) - qP(8) + qP(5) / 20 + qM(5) / 25)
            assert out[0, o, p] == pytest.approx(exp_n, abs=eps, rel=eps)
            assert out[1, o, p] == pytest.approx(exp_1, abs=eps, rel=eps)
            assert out[2, o, p] == pytest.approx(exp_2, abs=eps, rel=eps)
    # postcompute with tractions t1 = o + p, t2 = 2 (o + p) and weights 1, 2, 3, 4
    t1 = np.array([[o + p for p in range(npts)] for o in range(nts)], float)
    t2 = 2 * t1
    w = np.arange(1, nts + 1, dtype=float)
    isp = np.zeros((9, npts))
    ism = np.zeros((9, npts))
    L.oracle_dr_postcompute.restype = None
    L.oracle_dr_postcompute(npts, nts, imp.ctypes.data_as(C.c_void_p), qp.ctypes.data_as(C.c_void_p),
                            qm.ctypes.data_as(C.c_void_p), np.ascontiguousarray(out[0]).ctypes.data_as(C.c_void_p),
                            t1.ctypes.data_as(C.c_void_p), t2.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                            isp.ctypes.data_as(C.c_void_p), ism.ctypes.data_as(C.c_void_p))
    for p in range(npts):
        e = np.zeros((2, 6))
        for o in range(nts):
            sn = out[0, o, p]
            qP = lambda q: o + q + p
            qM = lambda q: 2 * (o + q + p)
            e[0] += w[o] * np.array([sn, t1[o, p], t2[o, p], qM(6) - (sn - qM(0)) / 15, qM(7) - (t1[o, p] - qM(3)) / 25,
                                     qM(8) - (t2[o, p] - qM(5)) / 25])
            e[1] += w[o] * np.array([sn, t1[o, p], t2[o, p], qP(6) + (sn - qP(0)) / 10, qP(7) + (t1[o, p] - qP(3)) / 20,
                                     qP(8) + (t2[o, p] - qP(5)) / 20])
        for j, q in enumerate((0, 3, 5, 6, 7, 8)):
            assert ism[q, p] == pytest.approx(e[0, j], rel=eps, abs=eps)
            assert isp[q, p] == pytest.approx(e[1, j], rel=eps, abs=eps)


def _rs():
    return oracle_py.RSParamsC(0.6, 0.014, 1e-6, 0.02, 0.1, 0.1, 1e-8, 1e-8, 60, 10)


def test_newton_matches_bisection():
    L = oracle_py.lib(np.float64)
    L.oracle_dr_newton_point.restype = C.c_int
    L.oracle_dr_mu.restype = C.c_double
    L.oracle_dr_mu.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    P = _rs()
    rng = np.random.default_rng(1)
    zs = 2700 * 3464.0
    inv_etas = 2 / zs
    for _ in range(200):
        a = rng.uniform(0.008, 0.02)
        sn = -rng.uniform(40e6, 120e6)
        tau = rng.uniform(20e6, 75e6)
        psi = rng.uniform(0.3, 0.9)
        v = C.c_double()
        conv = C.c_int()
        L.oracle_dr_newton_point(C.c_double(a), C.c_double(psi), C.c_double(sn), C.c_double(tau), C.c_double(inv_etas),
                                 C.c_double(1e-10), C.byref(P), C.byref(v), C.byref(conv))
        g = lambda x: -inv_etas * (abs(sn) * L.oracle_dr_mu(C.byref(P), a, psi, x) - tau) - x
        lo, hi = 0.0, tau * inv_etas  # g(0) >= 0 > g(tau / eta_s)
        if g(1e-300) < 0:
            continue
        for _ in range(400):
            mid = 0.5 * (lo + hi)
            if g(mid) > 0:
                lo = mid
            else:
                hi = mid
        if conv.value:
            assert abs(v.value - 0.5 * (lo + hi)) <= 1e-12 * max(1.0, abs(v.value)) + 1e-8


def test_fault_setup_matches_oracle(built_lib):
    from seissol_gb300 import Context
    with Context(4, device=-1) as ctx:
        ctx.build_periodic_cube(8, 4, 4, perturb=0.1, seed=9, fault_plane=4)
        coords, material, topo = ctx.get_geometry()
        cells = ctx.get_cells()
        faces = ctx.dr_faces()
    nf = faces["cells"].shape[0]
    assert nf == 2 * 4 * 4  # 4 x 4 cube faces on the plane, two triangles each
    pc, mc = faces["cells"][:, 0], faces["cells"][:, 1]
    ps, ms, rel = faces["sides"][:, 0], faces["sides"][:, 1], faces["sides"][:, 2]
    # plus cells lie at x < x_f, minus cells at x > x_f; relations consistent with the mesh
    xf = 400.0
    assert (coords[pc][:, :, 0].mean(axis=1) < xf).all() and (coords[mc][:, :, 0].mean(axis=1) > xf).all()
    assert np.array_equal(cells["neighbor"][pc, ps], mc) and np.array_equal(cells["side"][pc, ps], ms)
    assert np.array_equal(cells["orient"][pc, ps] + 1, rel)
    assert (cells["face_type"][pc, ps] == 1).all() and (cells["face_type"][mc, ms] == 1).all()
    assert (cells["face_type"] == 1).sum() == 2 * nf
    assert np.abs(cells["AplusT"][pc, ps]).max() == 0.0  # no local flux on fault faces
    ref = dg_setup.fault_face_data(coords, material, np.stack([pc, ps, mc, ms], axis=1))
    for k in ("TinvT", "fluxSolverPlus", "fluxSolverMinus"):
        scale = np.abs(ref[k]).max(axis=(1, 2), keepdims=True)
        assert np.abs(faces[k] - ref[k]).max() <= 1e-6 * scale.max(), k
    assert np.allclose(faces["imp"][:, :7], ref["imp"], rtol=1e-12)
    # fault normal along +x: the first row of Tinv holds the normal for velocities
    assert np.allclose(faces["TinvT"][:, 6:, 6], [[1, 0, 0]] * nf, atol=1e-6)
