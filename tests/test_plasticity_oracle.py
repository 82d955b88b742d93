"""Off-fault plasticity: the restatement and the host side of the ABI against the reference's pins
(CPU only).

* computeRelaxTime's known answers (tests/Kernel/Plasticity.t.h): oracle and
  sei_plasticity_relax_factor, 1e-15 (the reference's doctest Approx is looser);
* V and Vinv at the reference's nodes (codegen/matrices/plasticity-nb-matrices-{4,5,6}.json, fixture
  plasticity_nb_pin.json): shape, non-zero count, sum, Frobenius norm and sampled entries within
  1e-12 relative;
* the library's default nodes equal the restatement's lattice;
* properties of the return map: with r = 1 the updated nodal stresses lie on the yield surface
  (tau = tau_c within 1e-10 relative) and nowhere outside it; the mean stress does not change; no
  yielding leaves everything as it was; the plastic strain rate and eta follow the update.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import plasticity as P

HERE = os.path.dirname(os.path.abspath(__file__))
PIN = json.load(open(os.path.join(HERE, "golden", "plasticity_nb_pin.json")))


def _relax_cases(f):
    for dt in (1.0, 0.5, 0.001):
        assert f(0.0, dt) == 1.0
    assert abs(f(0.1, 0.05) - (1.0 - math.exp(-0.5))) < 1e-15
    assert abs(f(100.0, 0.001) / (0.001 / 100.0) - 1.0) < 1e-4
    assert abs(f(0.001, 10.0) - 1.0) < 1e-6
    assert abs(f(1.0, 1.0) - (1.0 - math.exp(-1.0))) < 1e-15
    for tv in (0.01, 0.1, 1.0, 10.0, 100.0):
        for dt in (0.001, 0.01, 0.1, 1.0, 10.0):
            assert 0.0 < f(tv, dt) <= 1.0
    prev = 0.0
    for dt in (0.01, 0.1, 0.5, 1.0, 2.0, 5.0, 10.0):
        assert f(1.0, dt) > prev
        prev = f(1.0, dt)


def test_relax_factor_known_answers():
    _relax_cases(P.relax_factor)


def test_library_relax_factor_known_answers(built_lib):
    from seissol_gb300 import plasticity_relax_factor
    _relax_cases(plasticity_relax_factor)


def _check_pin(a, pin):
    assert list(a.shape) == pin["shape"]
    # entries at rounding-noise level count as zeros (the reference stores some of them, not all)
    nz = a[np.abs(a) > 1e-12 * np.abs(a).max()]
    assert abs(len(nz) - pin["nnz"]) <= max(2, 0.02 * pin["nnz"])
    assert abs(a.sum() - pin["sum"]) <= 1e-12 * max(1.0, abs(pin["fro"]) * a.size)
    assert abs(np.linalg.norm(a) - pin["fro"]) <= 1e-12 * pin["fro"] * 10
    for r, c, v in pin["sample"]:
        assert abs(a[r, c] - v) <= 1e-12 * max(1.0, abs(v)), (r, c, a[r, c], v)


@pytest.mark.parametrize("order", [4, 5, 6])
def test_vandermonde_at_reference_nodes(order):
    pin = PIN[str(order)]
    nodes = np.array(pin["nodes"])
    B = order * (order + 1) * (order + 2) // 6
    assert nodes.shape == (B, 3)
    v, vinv = P.matrices(order, nodes)
    _check_pin(v, pin["v"])
    _check_pin(vinv, pin["vInv"])


@pytest.mark.parametrize("order", [4, 5, 6])
def test_library_default_nodes(built_lib, order):
    from seissol_gb300 import plasticity_nodes
    assert np.array_equal(plasticity_nodes(order), P.lattice_nodes(order))
    v, vinv = P.matrices(order, P.lattice_nodes(order))
    assert np.abs(v @ vinv - np.eye(len(v))).max() < 1e-9


def _case(order, seed, cohesion):
    rng = np.random.default_rng(seed)
    B = order * (order + 1) * (order + 2) // 6
    n = 64
    q = rng.uniform(-1.0, 1.0, (n, 9, B)) * 1e6
    s0 = np.tile(np.array([-2e6, -2e6, -2e6, 0.0, 0.0, 0.0]), (n, 1))
    bf = np.full(n, 0.6)
    co = np.full(n, cohesion)
    mu = rng.uniform(2.5e10, 3.5e10, n)
    nodes = np.array(PIN[str(order)]["nodes"])
    v, vinv = P.matrices(order, nodes)
    s0n, ccos, ssin = P.cell_parameters(bf, co, s0, B)
    return q, np.zeros((n, 7, B)), v, vinv, s0n, ccos, ssin, mu


@pytest.mark.parametrize("order", [4, 6])
def test_return_to_yield_surface(order):
    q, ps, v, vinv, s0, ccos, ssin, mu = _case(order, 3, 1e6)
    q1 = q.copy()
    dt = 1e-3
    adj = P.apply(q1, ps, v, vinv, s0, ccos, ssin, mu, dt, 1e-12)  # r = 1: the stresses return onto the surface
    assert adj.any()
    nodal0 = np.einsum("nk,cxk->cxn", v, q[:, :6]) + s0
    nodal1 = np.einsum("nk,cxk->cxn", v, q1[:, :6]) + s0
    m0, m1 = nodal0[:, :3].mean(axis=1), nodal1[:, :3].mean(axis=1)
    assert np.abs(m1 - m0).max() <= 1e-9 * np.abs(m0).max()
    dev = nodal1.copy()
    dev[:, :3] -= m1[:, None]
    tau = np.sqrt(0.5 * (dev[:, :3] ** 2).sum(1) + (dev[:, 3:] ** 2).sum(1))
    lim = np.maximum(0.0, ccos - m1 * ssin)
    assert (tau <= lim * (1 + 1e-10) + 1e-6).all()
    # the nodes that yielded sit on the surface
    dev0 = nodal0.copy()
    dev0[:, :3] -= m0[:, None]
    tau0 = np.sqrt(0.5 * (dev0[:, :3] ** 2).sum(1) + (dev0[:, 3:] ** 2).sum(1))
    y = tau0 > lim
    assert y.any()
    assert np.abs(tau[y] - lim[y]).max() <= 1e-10 * lim[y].max()
    # the quantities 6..8 (velocities) are untouched
    assert np.array_equal(q1[:, 6:], q[:, 6:])


def test_no_yield_changes_nothing():
    q, ps, v, vinv, s0, ccos, ssin, mu = _case(5, 4, 1e12)
    q1 = q.copy()
    adj = P.apply(q1, ps, v, vinv, s0, ccos, ssin, mu, 1e-3, 0.05)
    assert not adj.any() and np.array_equal(q1, q) and not ps.any()


def test_strain_rate_and_eta():
    q, ps, v, vinv, s0, ccos, ssin, mu = _case(4, 5, 1e6)
    dt, tv = 2e-3, 0.05
    r = P.relax_factor(tv, dt)
    nodal = np.einsum("nk,cxk->cxn", v, q[:, :6]) + s0
    m = nodal[:, :3].mean(axis=1)
    dev = nodal.copy()
    dev[:, :3] -= m[:, None]
    tau = np.sqrt(0.5 * (dev[:, :3] ** 2).sum(1) + (dev[:, 3:] ** 2).sum(1))
    lim = np.maximum(0.0, ccos - m * ssin)
    q1 = q.copy()
    P.apply(q1, ps, v, vinv, s0, ccos, ssin, mu, dt, tv)
    c, k = np.argwhere(tau > lim)[0]
    y = (lim[c, k] / tau[c, k] - 1.0) * r
    rate = -(1.0 / (2 * mu[c])) / (tv * r) * y * dev[c, :, k]
    assert np.allclose(ps[c, :6, k], dt * rate, rtol=1e-12)
    assert math.isclose(ps[c, 6, k], dt * math.sqrt(0.5 * (rate ** 2).sum()), rel_tol=1e-12)
