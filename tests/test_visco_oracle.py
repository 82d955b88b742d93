"""Viscoelastic oracle (CPU only).

* attenuation fit vs the known answers of the reference's tests/Model/Attenuation.t.h (3 mechanisms,
  one Northridge cell; relative 1e-12);
* structure of the 27 x 27 operators that the GPU kernels exploit: star coupling of mechanism m =
  -omega_m x one strain-rate operator shared by all mechanisms, flux into memory variables = omega_m x
  one 9 x 6 block, E^T = theta coupling + -omega_m diagonal;
* with the memory coupling switched off (theta = 0, omega = 0) the elastic quantities follow the
  elastic oracle exactly (1e-12), so the viscoelastic restatement inherits its pins.
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py, visco
from tests.helpers import seeded_dofs

# tests/Model/Attenuation.t.h:22-53
ATT_IN = dict(rho=2787.216864690955845, mu=30969716301.94932938, lam=30969716301.94934082, qp=58.40512125971850566,
              qs=29.20256062985925283, fc=0.3, ratio=100.0)
ATT_OUT = dict(mu=33628014790.452877, lam=29578827039.733589,
               omega=[0.18849555921538758, 1.8849555921538763, 18.849555921538762],
               theta=[[-2662632131.4096899, 777200013.84026122, -3439832145.2499514],
                      [-2233089891.3828750, 739358274.28576028, -2972448165.6686354],
                      [-2833117392.9633269, 1061064406.7129726, -3894181799.6762996]])


def test_attenuation_known_answer():
    a = ATT_IN
    mu, lam, omega, theta = visco.fit_attenuation(a["rho"], a["mu"], a["lam"], a["qp"], a["qs"], a["fc"], a["ratio"])
    assert mu == pytest.approx(ATT_OUT["mu"], rel=1e-12)
    assert lam == pytest.approx(ATT_OUT["lam"], rel=1e-12)
    assert np.allclose(omega, ATT_OUT["omega"], rtol=1e-12)
    assert np.allclose(theta, ATT_OUT["theta"], rtol=1e-11)


def _mesh(order=4):
    from seissol_gb300 import Context
    with Context(order, device=-1) as ctx:
        n = ctx.build_periodic_cube(4, 4, 4, perturb=0.05, seed=6)
        cells = ctx.get_cells()
        coords, material, _ = ctx.get_geometry()
    return n, cells, coords, material


def _visco_material(material, qp=100.0, qs=50.0, fc=0.5, ratio=100.0):
    mats, thetas = [], []
    for rho, mu, lam in material:
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, qp, qs, fc, ratio)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    return np.array(mats), omega, np.array(thetas)


def test_operator_structure(built_lib):
    n, cells, coords, material = _mesh()
    mats, omega, thetas = _visco_material(material[:20])
    ops = visco.cell_operators(coords[:20], mats, omega, thetas, np.where(cells["neighbor"][:20] < 20,
                                                                            cells["neighbor"][:20], -1))
    star, ap, am, et = ops["star"], ops["AplusT"], ops["AminusT"], ops["ET"]
    mem = lambda m: slice(9 + 6 * m, 15 + 6 * m)
    # memory variables take no part as star sources; only velocities couple into them
    assert np.abs(star[:, :, 9:, :]).max() == 0.0
    assert np.abs(star[:, :, :6, 9:]).max() == 0.0
    s0 = star[:, :, :, mem(0)] / -omega[0]
    for m in range(1, 3):
        assert np.allclose(star[:, :, :, mem(m)] / -omega[m], s0, rtol=1e-12, atol=1e-9 * np.abs(s0).max())
        for a in (ap, am):
            w0 = a[:, :, :, mem(0)] / omega[0]
            assert np.allclose(a[:, :, :, mem(m)] / omega[m], w0, rtol=1e-10, atol=1e-10 * np.abs(w0).max())
    for a in (ap, am):
        assert np.abs(a[:, :, 9:, :]).max() == 0.0
    for m in range(3):
        blk = et[:, mem(m), mem(m)]
        assert np.allclose(blk, -omega[m] * np.eye(6)[None], rtol=0, atol=0)


def test_without_coupling_elastic_part_is_elastic_oracle(built_lib):
    order = 4
    n, cells, coords, material = _mesh(order)
    omega = np.zeros(3)
    thetas = np.zeros((n, 3, 3))
    ops = visco.cell_operators(coords, material, omega, thetas, cells["neighbor"])
    q9 = seeded_dofs(n, order, 4).astype(np.float64)[:, :, :dg_setup.nbasis3(order)]
    q27 = np.zeros((n, visco.NQ, q9.shape[2]))
    q27[:, :9] = q9
    dt = dg_setup.cfl_timestep(coords, np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0]), order).min()
    out = visco.Visco(order).steps(q27, ops, cells["neighbor"], cells["side"], cells["orient"], cells["face_type"],
                                   dt, 2)
    el = dg_setup.cell_operators(coords, material, cells["neighbor"])
    ref = oracle_py.Oracle(order).steps(q9, el["star"], el["AplusT"], el["AminusT"], cells["neighbor"], cells["side"],
                                        cells["orient"], dt, 2, cells["face_type"])
    assert np.abs(out[:, :9] - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(out[:, 9:]).max() == 0.0


def test_library_attenuation_fit_known_answer(built_lib):
    from seissol_gb300 import fit_attenuation
    a = ATT_IN
    mu, lam, omega, theta = fit_attenuation(a["mu"], a["lam"], a["qp"], a["qs"], a["fc"], a["ratio"])
    assert mu == pytest.approx(ATT_OUT["mu"], rel=1e-12)
    assert lam == pytest.approx(ATT_OUT["lam"], rel=1e-12)
    assert np.allclose(omega, ATT_OUT["omega"], rtol=1e-12)
    assert np.allclose(theta, ATT_OUT["theta"], rtol=1e-11)


def test_library_visco_operators_match_oracle(built_lib):
    """The product's host set-up (host-only context) against the dense oracle operators: the
    unrelaxed elastic blocks, the memory-variable flux blocks W (= oracle flux column / omega),
    the gradients and theta; float32 storage, relative 1e-6."""
    from seissol_gb300 import Context
    with Context(4, device=-1) as ctx:
        ctx.build_periodic_cube(4, 4, 4, perturb=0.1, seed=7)
        coords, material, _ = ctx.get_geometry()
        ctx.visco_setup(100.0, 50.0, 0.5, 100.0)
        cells = ctx.get_cells()
        grad, theta, wp, wm, omega = ctx.visco_operators()
    mats, om, thetas = _visco_material(material)
    assert np.allclose(omega, om, rtol=1e-7)  # stored as float (kernel argument)
    assert np.allclose(theta, thetas, rtol=1e-6)
    ops = visco.cell_operators(coords, mats, om, thetas, cells["neighbor"])
    close = lambda a, b: np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    assert close(cells["star"], ops["star"][:, :, :9, :9])
    assert close(cells["AplusT"], ops["AplusT"][:, :, :9, :9])
    assert close(cells["AminusT"], ops["AminusT"][:, :, :9, :9])
    assert close(wp, ops["AplusT"][:, :, :9, 9:15] / om[0])
    assert close(wm, ops["AminusT"][:, :, :9, 9:15] / om[0])
    ref_grad = np.stack([np.array(dg_setup.reference_jacobian(*coords[c].T)) for c in range(coords.shape[0])])
    assert close(grad, ref_grad)
