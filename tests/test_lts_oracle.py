"""Oracle of rate-2 local time stepping (CPU only).

* with one cluster, one LTS cycle is one global time step of the oracle (1e-12);
* on a graded cube (cube edges log-uniform in [h, 4 h]) the clustering gives several clusters,
  neighbours at most one cluster apart, and every cell's cluster step within its CFL step;
* a plane wave advanced by LTS over two or more clusters has the accuracy of global stepping at
  the finest step (its error against the exact solution within 10 % of that of global stepping);
* with a planar fault the two cells of every fault face share a cluster;
* the viscoelastic adapter reproduces the dense viscoelastic oracle with one cluster (exactly).
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py
from tests.helpers import seeded_dofs


def _graded(order, grading, seed=4, dims=(6, 6, 6)):
    from seissol_gb300 import Context
    with Context(order, device=-1) as ctx:
        n = ctx.build_periodic_cube(*dims, perturb=0.05, seed=seed, grading=grading)
        cells = ctx.get_cells()
        coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    return n, cells, dg_setup.cfl_timestep(coords, vp, order, 0.5)


def test_one_cluster_is_global_stepping(built_lib):
    order = 4
    n, cells, dt = _graded(order, 1.0)
    cl, dt0 = oracle_py.lts_clusters(dt, cells["neighbor"], cells["face_type"], 1)
    assert (cl == 0).all()
    o = oracle_py.Oracle(order)
    q0 = seeded_dofs(n, order, 2).astype(np.float64)
    q_lts = oracle_py.lts_cycles(o, q0, cells, cl, dt0, 2)
    q_gts = o.steps(q0, *(cells[k].astype(np.float64) for k in ("star", "AplusT", "AminusT")), cells["neighbor"],
                    cells["side"], cells["orient"], dt0, 2, cells["face_type"])
    assert np.abs(q_lts - q_gts).max() <= 1e-12 * np.abs(q_gts).max()


def test_graded_clustering(built_lib):
    n, cells, dt = _graded(4, 4.0)
    cl, dt0 = oracle_py.lts_clusters(dt, cells["neighbor"], cells["face_type"], 8)
    assert cl.max() >= 1
    assert (dt0 * 2.0 ** cl <= dt * (1 + 1e-12)).all()
    reg = cells["face_type"] == 0
    diff = np.abs(cl[:, None] - cl[np.where(reg, cells["neighbor"], 0)])
    assert diff[reg].max() <= 1


def _plane_wave(order, coords, t, rho=2700.0, vp=6000.0, vs=3464.0):
    """L2 projection of a P plane wave along x with one wavelength over the periodic x extent."""
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    L = coords[..., 0].max() - coords[..., 0].min()
    A = dg_setup.coefficient_matrix_T(rho, mu, lam, 0).T
    w, V = np.linalg.eig(A)
    idx = np.argmax(w.real)
    c, r = w.real[idx], V.real[:, idx]
    k = 2 * np.pi / L
    xi, eta, zeta, W = dg_setup._quad_tet(order + 4)
    phi = np.array([dg_setup.tet_dubiner(*tt, xi, eta, zeta) for tt in dg_setup.basis_indices3(order)])
    Md = ((phi * W) @ phi.T).diagonal()
    Q = np.zeros((coords.shape[0], 9, phi.shape[0]))
    for cc in range(coords.shape[0]):
        v = coords[cc]
        x = v[0] + np.outer(xi, v[1] - v[0]) + np.outer(eta, v[2] - v[0]) + np.outer(zeta, v[3] - v[0])
        Q[cc] = (np.outer(r, np.sin(k * x[:, 0] - k * c * t)) * W) @ phi.T / Md
    return Q, Md


@pytest.mark.parametrize("order", [4, 5])
def test_lts_plane_wave_matches_global_stepping(built_lib, order):
    """A plane wave on the graded cube: after two LTS cycles the error against the exact solution
    is within 10 % of the error of global stepping at the finest step."""
    from seissol_gb300 import Context
    with Context(order, device=-1) as ctx:
        n = ctx.build_periodic_cube(6, 6, 6, perturb=0.0, seed=4, grading=4.0)
        cells = ctx.get_cells()
        coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    dt = dg_setup.cfl_timestep(coords, vp, order, 0.5)
    cl, dt0 = oracle_py.lts_clusters(dt, cells["neighbor"], cells["face_type"], 8)
    ncl = int(cl.max()) + 1
    assert ncl >= 2
    o = oracle_py.Oracle(order)
    q0, Md = _plane_wave(order, coords, 0.0)
    cycles = 2
    T = cycles * dt0 * (1 << (ncl - 1))
    qe, _ = _plane_wave(order, coords, T)
    q_lts = oracle_py.lts_cycles(o, q0, cells, cl, dt0, cycles)
    q_gts = o.steps(q0, *(cells[k].astype(np.float64) for k in ("star", "AplusT", "AminusT")), cells["neighbor"],
                    cells["side"], cells["orient"], dt0, cycles << (ncl - 1), cells["face_type"])
    err = lambda q: np.sqrt((((q - qe) ** 2) * Md).sum() / ((qe ** 2) * Md).sum())
    e_lts, e_gts = err(q_lts), err(q_gts)
    assert e_lts < 1.1 * e_gts + 1e-9, (e_lts, e_gts)


def test_clustering_keeps_fault_pairs_together(built_lib):
    """A graded cube with a planar fault: both cells of every dynamic-rupture face share one
    cluster, regular neighbours stay at most one cluster apart, and no cell is above the cluster
    of its own CFL step."""
    from seissol_gb300 import Context
    order = 4
    with Context(order, device=-1) as ctx:
        ctx.build_periodic_cube(8, 6, 6, perturb=0.05, seed=9, grading=4.0, fault_plane=4)
        cells = ctx.get_cells()
        coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    dt = dg_setup.cfl_timestep(coords, vp, order, 0.5)
    ft, nb = cells["face_type"], cells["neighbor"]
    cell_i, face_i = np.nonzero(ft == 1)
    assert cell_i.size > 0
    pairs = np.unique(np.sort(np.stack([cell_i, nb[cell_i, face_i]], axis=1), axis=1), axis=0)
    cl, dt0 = oracle_py.lts_clusters(dt, nb, ft, 8, pairs)
    assert cl.max() >= 1
    assert np.array_equal(cl[pairs[:, 0]], cl[pairs[:, 1]])
    reg = ft == 0
    assert (np.abs(cl[:, None] - cl[np.where(reg, nb, 0)])[reg] <= 1).all()
    own = np.clip(np.floor(np.log2(dt / dt0) + 1e-12).astype(np.int64), 0, 7)
    assert (cl <= own).all()


def test_visco_adapter_one_cluster_is_dense_global_stepping(built_lib):
    """The viscoelastic adapter behind lts_cycles: with one cluster, two LTS cycles equal two steps
    of the dense viscoelastic oracle exactly."""
    from oracle import cube_mesh, visco
    order = 4
    topo, coords = cube_mesh.periodic_cube(4, 4, 4)
    n = topo.shape[0]
    nb, side, orient = dg_setup.face_relations(topo)
    rho, vs, vp = 2700.0, 3464.0, 6000.0
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    mats, thetas = [], []
    for _ in range(n):
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, 100.0, 50.0, 0.5, 100.0)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    ops = visco.cell_operators(coords, np.array(mats), omega, np.array(thetas), nb)
    ft = np.zeros((n, 4), np.int8)
    vcells = {"star": np.concatenate([ops["star"], ops["ET"][:, None]], axis=1), "AplusT": ops["AplusT"],
              "AminusT": ops["AminusT"], "neighbor": nb, "side": side, "orient": orient, "face_type": ft}
    q0 = np.random.default_rng(1).uniform(-1, 1, (n, visco.NQ, dg_setup.nbasis3(order)))
    dt = 1e-3
    a = oracle_py.lts_cycles(visco.ViscoLts(order), q0, vcells, np.zeros(n, np.int64), dt, 2)
    b = visco.Visco(order).steps(q0, ops, nb, side, orient, ft, dt, 2)
    assert np.array_equal(a, b)
