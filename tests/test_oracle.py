"""Pins the oracle to the reference's own data and unit tests (CPU only).

* global matrices vs codegen/matrices/matrices_{20,35,56}.xml (fixture global_matrices_pin.json,
  full XML when the reference tree is present);
* Godunov states vs tests/Model/Values.h (fixture godunov_elastic.json) with the structural
  checks of tests/Model/GodunovState.t.h (Qgod_local + Qgod_neighbor = I, P^2 = P);
* monomial time basis vs tests/Numerical/TimeBasis.t.h;
* the product's exact-arithmetic matrices vs the oracle's quadrature ones;
* plane-wave convergence of the full scheme (validates orientations and flux signs).
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import cube_mesh, dg_setup, oracle_py

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
# The reference tree, when present, is named by SEI_REFERENCE_ROOT; the full-XML check is skipped without it.
REF_MATRICES = os.path.join(os.environ.get("SEI_REFERENCE_ROOT", ""), "codegen", "matrices")


@pytest.mark.parametrize("order", [4, 5, 6])
def test_global_matrices_pinned(order):
    pin = json.load(open(os.path.join(GOLD, "global_matrices_pin.json")))[str(dg_setup.nbasis3(order))]
    g = dg_setup.global_matrices(order)
    for name, spec in pin.items():
        base, idx = name[:-3], int(name[-2])
        m = g[base][idx]
        if base == "kDivMT":
            m = -m  # the reference negates kDivMT at load time; the file holds the un-negated values
        assert list(m.shape) == spec["shape"], name
        assert int((m != 0).sum()) == spec["nnz"], name
        assert math.isclose(m.sum(), spec["sum"], rel_tol=1e-12, abs_tol=1e-12), name
        assert math.isclose(np.linalg.norm(m), spec["fro"], rel_tol=1e-12), name
        for r, c, v in spec["sample"]:
            assert abs(m[r, c] - v) <= 1e-12 * max(1.0, abs(v)), (name, r, c)


@pytest.mark.skipif(not os.environ.get("SEI_REFERENCE_ROOT") or not os.path.isdir(REF_MATRICES),
                    reason="reference tree not named by SEI_REFERENCE_ROOT")
@pytest.mark.parametrize("order", [4, 6])
def test_global_matrices_full_xml(order):
    import xml.etree.ElementTree as ET
    root = ET.parse(os.path.join(REF_MATRICES, f"matrices_{dg_setup.nbasis3(order)}.xml")).getroot()
    g = dg_setup.global_matrices(order)
    for mx in root:
        name = mx.get("name")
        ref = np.zeros((int(mx.get("rows")), int(mx.get("columns"))))
        for e in mx:
            ref[int(e.get("row")) - 1, int(e.get("column")) - 1] = float(e.get("value"))
        m = g[name[:-3]][int(name[-2])]
        if name.startswith("kDivMT"):
            m = -m
        assert np.abs(m - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), name


def _godunov_gold():
    return json.load(open(os.path.join(GOLD, "godunov_elastic.json")))


@pytest.mark.parametrize("case", ["Homogeneous", "Heterogeneous"])
def test_godunov_golden(case):
    g = _godunov_gold()
    m1, m2 = tuple(g["MaterialVal1"]), tuple(g["MaterialVal2"])
    loc, nb = dg_setup.godunov_state(m1, m1 if case == "Homogeneous" else m2)
    for mat, key in ((loc, f"Solution{case}Local"), (nb, f"Solution{case}Neighbor")):
        ref = np.array(g[key]).T  # golden[j][i] == view(i, j)
        assert np.linalg.norm(mat - ref) <= 1e2 * np.finfo(np.float64).eps * np.linalg.norm(ref)
    assert np.linalg.norm(loc + nb - np.eye(9)) <= 1e-13 * 3
    assert np.linalg.norm(nb @ nb - nb) <= 1e-12 * np.linalg.norm(nb)


def test_time_basis():
    for order in range(1, 10):
        for point in (0.0, 1.0, 2.0, 0.123, 15.0):
            c = dg_setup.taylor_integrate(order, 0.0, point)
            p = dg_setup.taylor_point(order, point)
            for j in range(order):
                assert c[j] == pytest.approx(point ** (j + 1) / math.gamma(j + 2), abs=10 * np.finfo(float).eps, rel=1e-15)
                assert p[j] == pytest.approx(point ** j / math.gamma(j + 1), abs=10 * np.finfo(float).eps, rel=1e-15)


@pytest.mark.parametrize("order", [4, 5])
def test_product_matrices_match_oracle(order):
    from seissol_gb300.codegen import basis
    a = basis.global_matrices(order)
    b = dg_setup.global_matrices(order)
    for name in ("kDivM", "kDivMT", "rDivM", "rT", "fMrT", "fP"):
        for x, y in zip(a[name], b[name]):
            assert np.array_equal(x != 0, y != 0), name
            assert np.abs(x - y).max() <= 1e-13 * max(1.0, np.abs(y).max()), name


def test_face_relations_consistent():
    topo, coords = cube_mesh.periodic_cube(4, 6, 4)
    nb, side, orient = dg_setup.face_relations(topo)
    assert (nb >= 0).all()
    for c in range(topo.shape[0]):
        for f in range(4):
            d, j = nb[c, f], side[c, f]
            assert nb[d, j] == c and side[d, j] == f
            # the shared face has the same vertex set
            assert sorted(topo[c, list(dg_setup.FACE2NODES[f])]) == sorted(topo[d, list(dg_setup.FACE2NODES[j])])


def _plane_wave_error(order, n, direction=(1, 0, 0), wave="p"):
    h = 100.0
    L = n * h
    topo, coords = cube_mesh.periodic_cube(n, n, n, h)
    nc = topo.shape[0]
    rho, vp, vs = 2700.0, 6000.0, 3464.0
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    mat = np.tile([rho, mu, lam], (nc, 1))
    nb, side, orient = dg_setup.face_relations(topo)
    ops = dg_setup.cell_operators(coords, mat, nb)
    m = np.array(direction, float)
    d = m / np.linalg.norm(m)
    A = sum(d[i] * dg_setup.coefficient_matrix_T(rho, mu, lam, i).T for i in range(3))
    w, V = np.linalg.eig(A)
    w, V = w.real, V.real
    idx = np.argmax(w) if wave == "p" else np.argsort(w)[-2]
    c, r = w[idx], V[:, idx]
    k = 2 * np.pi / L * np.linalg.norm(m)
    xi, eta, zeta, W = dg_setup._quad_tet(order + 4)
    phi = np.array([dg_setup.tet_dubiner(*t, xi, eta, zeta) for t in dg_setup.basis_indices3(order)])
    Md = ((phi * W) @ phi.T).diagonal()

    def project(t):
        Q = np.zeros((nc, 9, phi.shape[0]))
        for cc in range(nc):
            v = coords[cc]
            x = v[0] + np.outer(xi, v[1] - v[0]) + np.outer(eta, v[2] - v[0]) + np.outer(zeta, v[3] - v[0])
            Q[cc] = (np.outer(r, np.sin(k * (x @ d) - k * c * t)) * W) @ phi.T / Md
        return Q

    dt = dg_setup.cfl_timestep(coords, np.full(nc, vp), order, 0.5).min()
    T = 0.2 * L / c
    ns = int(np.ceil(T / dt))
    Q = oracle_py.Oracle(order).steps(project(0.0), ops["star"], ops["AplusT"], ops["AminusT"], nb, side, orient,
                                      T / ns, ns)
    Qe = project(T)
    return math.sqrt(((Q - Qe) ** 2 * Md).sum() / (Qe ** 2 * Md).sum())


@pytest.mark.parametrize("direction,wave", [((1, 0, 0), "p"), ((1, 1, 0), "s")])
def test_plane_wave_convergence(direction, wave):
    e4 = _plane_wave_error(4, 4, direction, wave)
    e6 = _plane_wave_error(4, 6, direction, wave)
    rate = math.log(e4 / e6) / math.log(6 / 4)
    assert e6 < 2e-3
    assert rate > 3.5, (e4, e6, rate)
