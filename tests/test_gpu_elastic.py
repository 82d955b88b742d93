"""GPU parity of the elastic element update against the FP64 oracle (calls through the C ABI).

Tolerances (relative L2 per quantity, FP32 GPU vs FP64 oracle on the same inputs):
one kernel application 2e-5, ten time steps of kernel 'all' 1e-4.
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py
from tests.helpers import rel_l2, rel_l2_per_quantity, seeded_dofs

pytestmark = pytest.mark.gpu

TOL_ONE = 2e-5
TOL_STEPS = 1e-4


def _setup(order, dims=(4, 4, 4), perturb=0.1, seed=3, store_derivatives=True):
    from seissol_gb300 import Context
    ctx = Context(order, device=0, store_derivatives=store_derivatives)
    n = ctx.build_periodic_cube(*dims, perturb=perturb, seed=seed)
    cells = ctx.get_cells()
    q0 = seeded_dofs(n, order, seed)
    ctx.set_dofs(q0)
    return ctx, n, cells, q0


def _ops64(cells):
    return {k: cells[k].astype(np.float64) for k in ("star", "AplusT", "AminusT")}


@pytest.mark.parametrize("order", [4, 5, 6])
def test_ader_local_neighbor_parity(built_lib, order):
    ctx, n, cells, q0 = _setup(order)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    ops = _ops64(cells)
    coeffs = dg_setup.taylor_integrate(order, 0.0, dt)
    i_ref, d_ref = o.ader(q0.astype(np.float64), ops["star"], coeffs, want_derivs=True)
    q_ref = o.local(q0, i_ref, ops["star"], ops["AplusT"], cells["face_type"])

    ctx.compute_ader_local(dt)
    ctx.sync()
    i_gpu = ctx.get_time_integrated()
    q_gpu = ctx.get_dofs()
    d_gpu = ctx.get_derivatives()
    assert max(rel_l2_per_quantity(i_gpu, i_ref)) < TOL_ONE
    assert max(rel_l2_per_quantity(q_gpu - q0, q_ref - q0)) < TOL_ONE
    assert rel_l2(d_gpu, d_ref) < TOL_ONE

    q_ref2 = o.neighbor(q_ref, i_ref, ops["AminusT"], cells["neighbor"], cells["side"], cells["orient"],
                        cells["face_type"])
    ctx.compute_neighbors_integral()
    ctx.sync()
    q_gpu2 = ctx.get_dofs()
    assert max(rel_l2_per_quantity(q_gpu2 - q_gpu, q_ref2 - q_ref)) < TOL_ONE
    ctx.close()


@pytest.mark.parametrize("order", [4, 6])
def test_ten_steps_all(built_lib, order):
    ctx, n, cells, q0 = _setup(order, store_derivatives=False)
    dt = ctx.cfl_timestep(0.5)
    ops = _ops64(cells)
    q_ref = oracle_py.Oracle(order).steps(q0, ops["star"], ops["AplusT"], ops["AminusT"], cells["neighbor"],
                                          cells["side"], cells["orient"], dt, 10, cells["face_type"])
    ctx.run("all", dt, 10)
    ctx.sync()
    q_gpu = ctx.get_dofs()
    errs = rel_l2_per_quantity(q_gpu, q_ref)
    assert max(errs) < TOL_STEPS, errs
    assert np.isfinite(q_gpu).all()
    ctx.close()


def test_taylor_evaluation(built_lib):
    import torch
    order = 5
    ctx, n, cells, q0 = _setup(order)
    dt = ctx.cfl_timestep(0.5)
    ctx.compute_ader_local(dt)
    ctx.sync()
    d_gpu = ctx.get_derivatives()
    coeffs = dg_setup.taylor_point(order, 0.37 * dt)
    out = torch.zeros((n, 9, (dg_setup.nbasis3(order) + 3) // 4 * 4), dtype=torch.float32, device="cuda")
    import ctypes
    rc = ctx.lib.sei_evaluate_taylor(ctx.h, np.ascontiguousarray(coeffs, np.float64).ctypes.data_as(ctypes.c_void_p),
                                     ctypes.c_void_p(out.data_ptr()))
    assert rc == 0
    ctx.sync()
    got = out.cpu().numpy()[:, :, : dg_setup.nbasis3(order)]
    ref = oracle_py.Oracle(order).taylor(d_gpu.astype(np.float64), coeffs)
    assert rel_l2(got, ref) < 1e-6
    ctx.close()


def test_run_host_matches_device_path(built_lib):
    order = 4
    ctx, n, cells, q0 = _setup(order, store_derivatives=False)
    dt = ctx.cfl_timestep(0.5)
    out = np.empty_like(q0)
    ctx.run_host("all", dt, 3, q0, out)
    ctx.set_dofs(q0)
    ctx.run("all", dt, 3)
    ctx.sync()
    assert np.array_equal(out, ctx.get_dofs())
    ctx.close()


def test_set_cells_generic_mesh(built_lib):
    """Operators uploaded through sei_set_cells (oracle-built) give the same result as the host build."""
    from seissol_gb300 import Context
    order = 4
    ctx, n, cells, q0 = _setup(order, store_derivatives=False)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 2)
    ctx.sync()
    a = ctx.get_dofs()
    ctx2 = Context(order, device=0)
    ctx2.set_cells(cells["star"], cells["AplusT"], cells["AminusT"], cells["neighbor"], cells["side"],
                   cells["orient"], cells["face_type"])
    ctx2.set_dofs(q0)
    ctx2.run("all", dt, 2)
    ctx2.sync()
    assert np.array_equal(a, ctx2.get_dofs())
    ctx.close()
    ctx2.close()


def test_bad_relations_rejected(built_lib):
    from seissol_gb300 import Context, SeiError
    ctx, n, cells, q0 = _setup(4, store_derivatives=False)
    nb = cells["neighbor"].copy()
    nb[3, 1] = n + 5
    ctx2 = Context(4, device=0)
    with pytest.raises(SeiError, match="SEI_ERR_ARG"):
        ctx2.set_cells(cells["star"], cells["AplusT"], cells["AminusT"], nb, cells["side"], cells["orient"],
                       cells["face_type"])
    ctx.close()
    ctx2.close()


@pytest.mark.parametrize("order", [4, 6])
def test_ader_and_local_integral_separately(built_lib, order):
    """sei_compute_ader leaves Q unchanged and matches the oracle; sei_compute_local_integral then
    matches the oracle's volume + local flux; the fused launch gives the same bits."""
    ctx, n, cells, q0 = _setup(order, store_derivatives=False)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    ops = _ops64(cells)
    i_ref = o.ader(q0.astype(np.float64), ops["star"], dg_setup.taylor_integrate(order, 0.0, dt))
    ctx.compute_ader(dt)
    ctx.sync()
    assert np.array_equal(ctx.get_dofs(), q0)
    i_gpu = ctx.get_time_integrated()
    assert max(rel_l2_per_quantity(i_gpu, i_ref)) < TOL_ONE
    ctx.compute_local_integral()
    ctx.sync()
    q_split = ctx.get_dofs()
    q_ref = o.local(q0, i_ref, ops["star"], ops["AplusT"], cells["face_type"])
    assert max(rel_l2_per_quantity(q_split - q0, q_ref - q0)) < TOL_ONE
    ctx.set_dofs(q0)
    ctx.set_option(1, 1)  # SEI_OPT_FUSED_LOCAL
    ctx.compute_ader_local(dt)
    ctx.sync()
    assert np.array_equal(ctx.get_dofs(), q_split)
    assert np.array_equal(ctx.get_time_integrated(), i_gpu)
    ctx.close()


def test_ader_with_caller_coefficients(built_lib):
    """sei_compute_ader(ctx, coeffs, dt) integrates over the interval the caller's coefficients name
    (Spacetime::computeAder takes them from its TimeCluster): the sub-interval [dt/2, dt] of a local
    time step matches the oracle with integrate(dt/2, dt), and coeffs = NULL gives integrate(0, dt)."""
    order = 5
    ctx, n, cells, q0 = _setup(order, store_derivatives=False)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    ops = _ops64(cells)
    sub = dg_setup.taylor_integrate(order, 0.5 * dt, dt)
    ctx.compute_ader(dt, coeffs=sub)
    ctx.sync()
    i_ref = o.ader(q0.astype(np.float64), ops["star"], sub)
    assert max(rel_l2_per_quantity(ctx.get_time_integrated(), i_ref)) < TOL_ONE
    ctx.compute_ader(dt)
    ctx.sync()
    i_full = ctx.get_time_integrated()
    ctx.compute_ader(dt, coeffs=dg_setup.taylor_integrate(order, 0.0, dt))
    ctx.sync()
    assert rel_l2(ctx.get_time_integrated(), i_full) < 1e-6  # the same coefficients up to FP32 rounding
    ctx.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_graded_mesh_global_steps(built_lib, precision):
    """Five global steps of kernel 'all' (at the smallest CFL step) on a graded cube, whose cells
    span a factor of about six in edge length, against the FP64 oracle, FP32 and mixed paths."""
    from seissol_gb300 import Context
    order = 5
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(8, 8, 8, perturb=0.05, seed=11, grading=6.0)
    cells = ctx.get_cells()
    q0 = seeded_dofs(n, order, 11)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 5)
    ctx.sync()
    ops = _ops64(cells)
    ref = oracle_py.Oracle(order).steps(q0, ops["star"], ops["AplusT"], ops["AminusT"], cells["neighbor"], cells["side"],
                                        cells["orient"], dt, 5, cells["face_type"])
    errs = rel_l2_per_quantity(ctx.get_dofs(), ref)
    assert max(errs) < 1e-5, errs
    ctx.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_hundred_thousand_cells_one_step(built_lib, precision):
    """One step of kernel 'all' at order 6 on a 100,000-tet cube (20 x 20 x 50 cubes), FP32 and
    mixed paths, against the OpenMP FP64 oracle: 1e-5 relative L2 per quantity of the field."""
    from seissol_gb300 import Context
    order = 6
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(20, 20, 50, perturb=0.1, seed=13)
    assert n == 100000
    cells = ctx.get_cells()
    q0 = seeded_dofs(n, order, 13)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 1)
    ctx.sync()
    got = ctx.get_dofs()
    ctx.close()
    ops = _ops64(cells)
    ref = oracle_py.Oracle(order).steps(q0, ops["star"], ops["AplusT"], ops["AminusT"], cells["neighbor"], cells["side"],
                                        cells["orient"], dt, 1, cells["face_type"])
    errs = rel_l2_per_quantity(got, ref)
    assert max(errs) < 1e-5, errs
    upd = rel_l2_per_quantity(got - q0, ref - q0)
    assert max(upd) < 2e-5, upd  # the update itself, the single-application bar


@pytest.mark.parametrize("precision", [0, 1])
def test_benchmark_mesh_two_steps(built_lib, precision):
    """The benchmark's own workload: order 6, 400,000 tets (40 x 40 x 50 cubes, material +-10 %,
    the bench's seed), two steps of kernel 'all' on the FP32 and the mixed path against the
    OpenMP FP64 oracle: 1e-5 relative L2 per quantity of the field, 2e-5 of the update."""
    from seissol_gb300 import Context
    order = 6
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(40, 40, 50, perturb=0.1, seed=2024)
    assert n == 400000
    cells = ctx.get_cells()
    q0 = seeded_dofs(n, order, 2024)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 2)
    ctx.sync()
    got = ctx.get_dofs()
    ctx.close()
    ops = _ops64(cells)
    ref = oracle_py.Oracle(order).steps(q0, ops["star"], ops["AplusT"], ops["AminusT"], cells["neighbor"], cells["side"],
                                        cells["orient"], dt, 2, cells["face_type"])
    errs = rel_l2_per_quantity(got, ref)
    assert max(errs) < 1e-5, errs
    upd = rel_l2_per_quantity(got - q0, ref - q0)
    assert max(upd) < 2e-5, upd


@pytest.mark.parametrize("precision", [0, 1])
def test_benchmark_mesh_linearity(built_lib, precision):
    """A size-independent property at the benchmark's full size (400,000 tets, order 6): a step is
    linear in the DOFs, so step(a Q1 + b Q2) = a step(Q1) + b step(Q2) to float rounding
    (1e-6 relative L2 per quantity)."""
    from seissol_gb300 import Context
    order = 6
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(40, 40, 50, perturb=0.1, seed=2024)
    dt = ctx.cfl_timestep(0.5)
    q1, q2 = seeded_dofs(n, order, 1), seeded_dofs(n, order, 2)
    out = []
    for q in (q1, q2, (0.75 * q1.astype(np.float64) - 0.5 * q2).astype(np.float32)):
        ctx.set_dofs(q)
        ctx.run("all", dt, 1)
        ctx.sync()
        out.append(ctx.get_dofs().astype(np.float64))
    ctx.close()
    errs = rel_l2_per_quantity(out[2], 0.75 * out[0] - 0.5 * out[1])
    assert max(errs) < 1e-6, errs
