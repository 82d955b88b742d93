"""GPU viscoelastic element update (27 quantities, 3 mechanisms) through the C ABI against the dense
FP64 oracle (oracle/visco.py), whose operators are rebuilt independently from the context's
geometry and relaxed material (Qp 100, Qs 50, central frequency 0.5 Hz, ratio 100).

Tolerances (per quantity, FP32 GPU vs FP64 oracle on the same inputs): one ADER 2e-5 relative L2;
one local integral and one neighbour flux: the error of the update within 2e-5 of the update plus
1e-6 of the field (the FP32 storage of Q: the memory variables of the slowest mechanism change by
~1e-4 of their value in one application); ten steps of kernel 'all' 1e-4 relative L2.
"""
import numpy as np
import pytest

from oracle import visco
from tests.helpers import rel_l2_per_quantity


def _update_errors(q_new, q_old, ref):
    """Per quantity: |q_new - ref| / (|ref - q_old| + 0.05 |q_old|), compared with 2e-5 below, i.e.
    an update error within 2e-5 of the update plus 1e-6 of the field."""
    out = []
    for k in range(q_new.shape[1]):
        num = np.linalg.norm(q_new[:, k].astype(np.float64) - ref[:, k])
        den = np.linalg.norm(ref[:, k] - q_old[:, k]) + 0.05 * np.linalg.norm(q_old[:, k])
        out.append(num / den)
    return out

pytestmark = pytest.mark.gpu

QP, QS, FC, RATIO = 100.0, 50.0, 0.5, 100.0


def _setup(order, dims=(4, 4, 4), seed=8):
    from seissol_gb300 import Context
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(*dims, perturb=0.1, seed=seed)
    ctx.visco_setup(QP, QS, FC, RATIO)
    assert ctx.nq == 27
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    mats, thetas = [], []
    for rho, mu, lam in material:
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, QP, QS, FC, RATIO)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    ops = visco.cell_operators(coords, np.array(mats), omega, np.array(thetas), cells["neighbor"])
    rng = np.random.default_rng(seed)
    q0 = rng.uniform(-1, 1, (n, 27, ctx.B)).astype(np.float32)
    ctx.set_dofs(q0)
    return ctx, n, cells, ops, q0


@pytest.mark.parametrize("order", [4, 5])
def test_visco_kernels_one_application(built_lib, order):
    ctx, n, cells, ops, q0 = _setup(order)
    o = visco.Visco(order)
    dt = ctx.cfl_timestep(0.5)
    ctx.compute_ader(dt)
    ctx.sync()
    i_gpu = ctx.get_time_integrated()
    i_ref = o.ader(q0.astype(np.float64), ops["star"], ops["ET"], dt)
    errs = rel_l2_per_quantity(i_gpu, i_ref)
    assert max(errs) < 2e-5, errs
    ctx.compute_local_integral()
    ctx.sync()
    q_loc = ctx.get_dofs()
    ref = o.local(q0.astype(np.float64), i_gpu.astype(np.float64), ops["star"], ops["ET"], ops["AplusT"],
                  cells["face_type"])
    errs = _update_errors(q_loc, q0, ref)
    assert max(errs) < 2e-5, errs
    ctx.compute_neighbors_integral()
    ctx.sync()
    ref_n = o.neighbor(q_loc.astype(np.float64), i_gpu.astype(np.float64), ops["AminusT"], cells["neighbor"],
                       cells["side"], cells["orient"], cells["face_type"])
    errs = _update_errors(ctx.get_dofs(), q_loc, ref_n)
    assert max(errs) < 2e-5, errs
    ctx.close()


@pytest.mark.parametrize("order", [4, 5])
def test_visco_ten_steps(built_lib, order):
    ctx, n, cells, ops, q0 = _setup(order, seed=9)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 10)
    ctx.sync()
    ref = visco.Visco(order).steps(q0.astype(np.float64), ops, cells["neighbor"], cells["side"], cells["orient"],
                                   cells["face_type"], dt, 10)
    errs = rel_l2_per_quantity(ctx.get_dofs(), ref)
    assert max(errs) < 1e-4, errs
    ctx.close()


def test_visco_rejects_unbuilt(built_lib):
    from seissol_gb300 import Context, SeiError
    ctx = Context(6, device=0)
    ctx.build_periodic_cube(4, 4, 4)
    with pytest.raises(SeiError, match="SEI_ERR_UNSUPPORTED"):
        ctx.visco_setup()
    ctx.close()
    ctx, *_ = _setup(4)
    with pytest.raises(SeiError, match="SEI_ERR_UNSUPPORTED"):
        ctx.run("all_dr", 1e-4, 1)
    ctx.close()


def _graded_visco(order, grading, max_clusters, seed=31):
    from seissol_gb300 import Context
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(8, 8, 8, perturb=0.05, seed=seed, grading=grading)
    ctx.visco_setup(QP, QS, FC, RATIO)
    ncl = ctx.lts_setup(0.5, max_clusters)
    return ctx, n, ncl


def test_visco_lts_single_cluster_is_global_stepping(built_lib):
    """One cluster: the LTS cycle of the viscoelastic kernels is global stepping bit for bit."""
    from seissol_gb300 import Context
    a, n, ncl = _graded_visco(4, 6.0, 1)
    assert ncl == 1
    _, dts = a.lts_clusters()
    b = Context(4, device=0)
    b.build_periodic_cube(8, 8, 8, perturb=0.05, seed=31, grading=6.0)
    b.visco_setup(QP, QS, FC, RATIO)
    q0 = np.random.default_rng(3).uniform(-1, 1, (n, 27, a.B)).astype(np.float32)
    a.set_dofs(q0)
    b.set_dofs(q0)
    a.lts_run(3)
    b.run("all", dts[0], 3)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_dofs(), b.get_dofs())
    a.close()
    b.close()


@pytest.mark.parametrize("order", [4, 5])
def test_visco_lts_matches_oracle(built_lib, order):
    """Rate-2 LTS of the viscoelastic equations on a graded cube (several clusters), one cycle,
    against the FP64 restatement driving the dense viscoelastic oracle: 1e-4 relative L2 per
    quantity."""
    from oracle import dg_setup, oracle_py
    ctx, n, ncl = _graded_visco(order, 6.0, 8)
    assert ncl >= 2
    start, _ = ctx.lts_clusters()
    cl_gpu = np.repeat(np.arange(ncl), np.diff(start))
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 8)
    assert np.array_equal(cl, cl_gpu)
    mats, thetas = [], []
    for rho, mu, lam in material:
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, QP, QS, FC, RATIO)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    ops = visco.cell_operators(coords, np.array(mats), omega, np.array(thetas), cells["neighbor"])
    vcells = {"star": np.concatenate([ops["star"], ops["ET"][:, None]], axis=1), "AplusT": ops["AplusT"],
              "AminusT": ops["AminusT"], "neighbor": cells["neighbor"], "side": cells["side"],
              "orient": cells["orient"], "face_type": cells["face_type"]}
    q0 = np.random.default_rng(5).uniform(-1, 1, (n, 27, ctx.B)).astype(np.float32)
    ctx.set_dofs(q0)
    ctx.lts_run(1)
    ctx.sync()
    ref = oracle_py.lts_cycles(visco.ViscoLts(order), q0.astype(np.float64), vcells, cl, dt0, 1)
    errs = rel_l2_per_quantity(ctx.get_dofs(), ref)
    assert max(errs) < 1e-4, errs
    ctx.close()
