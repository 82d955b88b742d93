"""Mixed-precision path (SEI_PREC_F16X3: local integral and neighbour flux on tcgen05 tensor
cores, split FP16) against the FP64 oracle.

Tolerances: one application of the local integral or of the neighbour flux 2e-5 relative L2 of
the update per quantity (the FP32 bar); ten time steps of kernel 'all' 1e-5 relative L2 per
quantity of the field (the accuracy bar of the mixed-precision metric).
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py
from tests.helpers import rel_l2_per_quantity, seeded_dofs

pytestmark = pytest.mark.gpu

PREC_F16X3 = 1
OPT_TC_LOCAL = 3
OPT_NB_FORM = 5


def _ctx(order, precision, dims=(4, 4, 4), seed=3, tc_local=0):
    """tc_local: 0 local integral on the CUDA cores, 1 transposed tensor-core kernel, 2 rows form."""
    from seissol_gb300 import Context
    ctx = Context(order, device=0, precision=precision)
    if tc_local:
        ctx.set_option(OPT_TC_LOCAL, int(tc_local))
    n = ctx.build_periodic_cube(*dims, perturb=0.1, seed=seed)
    q0 = seeded_dofs(n, order, seed)
    ctx.set_dofs(q0)
    return ctx, n, q0


@pytest.mark.parametrize("order,form", [(4, 1), (5, 1), (6, 1), (4, 2), (6, 2)])
def test_local_integral_tensor_cores(built_lib, order, form):
    """The local integral on the tensor cores, transposed (1) and rows form (2), against the FP64
    oracle applied to the same time-integrated DOFs (the face traces these kernels store are
    checked through the neighbour flux that reads them, in the step tests)."""
    ctx, n, q0 = _ctx(order, PREC_F16X3, tc_local=form)
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    ctx.compute_ader(dt)
    ctx.sync()
    i_gpu = ctx.get_time_integrated()
    ctx.compute_local_integral()
    ctx.sync()
    q_gpu = ctx.get_dofs()
    o = oracle_py.Oracle(order)
    q_ref = o.local(q0, i_gpu.astype(np.float64), cells["star"].astype(np.float64), cells["AplusT"].astype(np.float64),
                    cells["face_type"])
    errs = rel_l2_per_quantity(q_gpu - q0, q_ref - q0)
    assert max(errs) < 2e-5, errs
    ctx.close()


@pytest.mark.parametrize("order,form", [(4, 1), (5, 1), (6, 1), (4, 0), (6, 0), (6, 2)])
def test_neighbor_tensor_cores(built_lib, order, form):
    """The neighbour flux from the stored face traces, transposed (form 1) and rows (form 0)
    kernels; after ADER alone the traces are stale and the neighbour call recomputes them from
    the new time-integrated DOFs first."""
    ctx, n, q0 = _ctx(order, PREC_F16X3)
    ctx.set_option(OPT_NB_FORM, form)
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    aminus = cells["AminusT"].astype(np.float64)
    q_prev = q0
    for rep in range(2):
        ctx.compute_ader(dt * (1.0 + 0.5 * rep))
        ctx.sync()
        i_gpu = ctx.get_time_integrated()
        ctx.compute_neighbors_integral()
        ctx.sync()
        q_gpu = ctx.get_dofs()
        q_ref = o.neighbor(q_prev.astype(np.float64), i_gpu.astype(np.float64), aminus, cells["neighbor"], cells["side"],
                           cells["orient"], cells["face_type"])
        errs = rel_l2_per_quantity(q_gpu - q_prev, q_ref - q_prev)
        assert max(errs) < 2e-5, (rep, errs)
        q_prev = q_gpu
    ctx.close()


@pytest.mark.parametrize("order,tc_local", [(4, 0), (6, 0), (4, 1), (5, 1), (6, 1), (6, 2)])
def test_ten_steps_mixed_precision(built_lib, order, tc_local):
    ctx, n, q0 = _ctx(order, PREC_F16X3, tc_local=tc_local)
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    q_ref = oracle_py.Oracle(order).steps(q0, cells["star"].astype(np.float64), cells["AplusT"].astype(np.float64),
                                          cells["AminusT"].astype(np.float64), cells["neighbor"], cells["side"],
                                          cells["orient"], dt, 10, cells["face_type"])
    ctx.run("all", dt, 10)
    ctx.sync()
    errs = rel_l2_per_quantity(ctx.get_dofs(), q_ref)
    assert max(errs) < 1e-5, errs
    ctx.close()


def test_mixed_and_fp32_agree_on_larger_mesh(built_lib):
    """Both precisions on the same 8x8x8-cube mesh for 5 steps stay within 1e-5 of each other."""
    a, n, q0 = _ctx(6, 0, dims=(8, 8, 8), seed=5)
    b, _, _ = _ctx(6, PREC_F16X3, dims=(8, 8, 8), seed=5)
    dt = a.cfl_timestep(0.5)
    a.run("all", dt, 5)
    b.run("all", dt, 5)
    a.sync()
    b.sync()
    errs = rel_l2_per_quantity(b.get_dofs(), a.get_dofs())
    assert max(errs) < 1e-5, errs
    a.close()
    b.close()


@pytest.mark.parametrize("precision,ncand", [(0, 2), (PREC_F16X3, 14)])
def test_autotune_keeps_state_and_results(built_lib, precision, ncand):
    """sei_autotune times every variant of the step, restores the DOFs, keeps the fastest variant;
    five steps with the chosen options then agree with the FP32 path within 1e-5."""
    a, n, q0 = _ctx(6, precision, dims=(8, 8, 8), seed=5)
    ref, _, _ = _ctx(6, 0, dims=(8, 8, 8), seed=5)
    dt = a.cfl_timestep(0.5)
    r = a.autotune(dt, 2)
    assert r["candidates"] == ncand
    assert 0 < r["best_ms"] <= r["worst_ms"]
    assert r["nb_ctas"] in (1, 2, 3) and r["fused_local"] in (0, 1) and r["tc_local"] in (0, 1, 2)
    assert r["nb_form"] in (0, 1, 2)
    assert np.array_equal(a.get_dofs(), q0)
    a.run("all", dt, 5)
    ref.run("all", dt, 5)
    a.sync()
    ref.sync()
    errs = rel_l2_per_quantity(a.get_dofs(), ref.get_dofs())
    assert max(errs) < 1e-5, errs
    a.close()
    ref.close()


@pytest.mark.parametrize("order", [4, 6])
def test_mixed_outflow_faces(built_lib, order):
    """Faces marked outflow (face type 2) through sei_set_cells contribute no flux on the mixed path:
    five steps of kernel 'all' against the FP64 oracle on the same inputs (1e-5 relative L2)."""
    from seissol_gb300 import Context
    base, n, q0 = _ctx(order, 0, seed=17)
    cells = base.get_cells()
    base.close()
    ft = np.array(cells["face_type"], dtype=np.int8)
    rng = np.random.default_rng(4)
    ft[rng.random(ft.shape) < 0.15] = 2
    ctx = Context(order, device=0, precision=PREC_F16X3)
    ctx.set_cells(cells["star"], cells["AplusT"], cells["AminusT"], cells["neighbor"], cells["side"], cells["orient"],
                  ft)
    ctx.set_dofs(q0)
    dt = 1e-4  # below the CFL step of these 100 m cells
    ctx.run("all", dt, 5)
    ctx.sync()
    ref = oracle_py.Oracle(order).steps(q0, cells["star"].astype(np.float64), cells["AplusT"].astype(np.float64),
                                        cells["AminusT"].astype(np.float64), cells["neighbor"], cells["side"],
                                        cells["orient"], dt, 5, ft)
    errs = rel_l2_per_quantity(ctx.get_dofs(), ref)
    assert max(errs) < 1e-5, errs
    ctx.close()


@pytest.mark.parametrize("precision,nsteps", [(0, 1), (0, 3), (PREC_F16X3, 1), (PREC_F16X3, 3)])
def test_run_host_pipelined_matches_device_run(built_lib, precision, nsteps):
    """sei_run_host pipelines the host copies with the step in chunks of cells; its result equals
    sei_set_dofs + sei_run + sei_get_dofs bit for bit."""
    a, n, q0 = _ctx(6, precision, dims=(8, 8, 8), seed=12)
    dt = a.cfl_timestep(0.5)
    out = np.empty_like(q0)
    a.run_host("all", dt, nsteps, q0, out)
    a.set_dofs(q0)
    a.run("all", dt, nsteps)
    a.sync()
    assert np.array_equal(out, a.get_dofs())
    a.close()


@pytest.mark.parametrize("order", [4, 6])
def test_neighbor_forms_agree_with_partial_tile(built_lib, order):
    """The transposed and rows forms of the tensor-core neighbour flux on a 317-cell mesh (the first
    317 cells of a periodic cube, faces towards the dropped cells made outflow), so the last 8-cell
    tile of the transposed kernel is partial: each within 2e-5 of the FP64 oracle, and within 2e-6
    of each other."""
    from seissol_gb300 import Context
    base, _, _ = _ctx(order, 0, seed=21)
    cells = base.get_cells()
    base.close()
    keep = 317
    cut = {k: np.ascontiguousarray(v[:keep]) for k, v in cells.items()}
    ft = np.array(cut["face_type"], dtype=np.int8)
    nb = np.array(cut["neighbor"])
    ft[nb >= keep] = 2
    nb[nb >= keep] = 0
    q0 = seeded_dofs(keep, order, 21)
    outs = []
    for form in (1, 0):
        ctx = Context(order, device=0, precision=PREC_F16X3)
        ctx.set_cells(cut["star"], cut["AplusT"], cut["AminusT"], nb, cut["side"], cut["orient"], ft)
        ctx.set_option(OPT_NB_FORM, form)
        ctx.set_dofs(q0)
        ctx.compute_ader(1e-4)
        ctx.sync()
        i_gpu = ctx.get_time_integrated()
        ctx.compute_neighbors_integral()
        ctx.sync()
        q_gpu = ctx.get_dofs()
        q_ref = oracle_py.Oracle(order).neighbor(q0.astype(np.float64), i_gpu.astype(np.float64),
                                                 cut["AminusT"].astype(np.float64), nb, cut["side"], cut["orient"], ft)
        errs = rel_l2_per_quantity(q_gpu - q0, q_ref - q0)
        assert max(errs) < 2e-5, (form, errs)
        outs.append(q_gpu - q0)
        ctx.close()
    assert max(rel_l2_per_quantity(outs[0], outs[1])) < 2e-6


@pytest.mark.parametrize("fused", [0, 1])
@pytest.mark.parametrize("order", [4, 5, 6])
def test_ten_steps_local_flux_in_neighbour_kernel(built_lib, order, fused):
    """SEI_OPT_NB_FORM 2: in kernel 'all' the local flux joins the neighbour flux in the transposed
    tensor-core kernel (the local integral computes the volume and the traces; with
    SEI_OPT_FUSED_LOCAL 1 one launch computes ADER, volume and traces); ten steps within 1e-5 of
    the FP64 oracle, and the pipelined host-buffer run equals the device run bit for bit."""
    ctx, n, q0 = _ctx(order, PREC_F16X3)
    ctx.set_option(OPT_NB_FORM, 2)
    ctx.set_option(1, fused)  # SEI_OPT_FUSED_LOCAL
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    q_ref = oracle_py.Oracle(order).steps(q0, cells["star"].astype(np.float64), cells["AplusT"].astype(np.float64),
                                          cells["AminusT"].astype(np.float64), cells["neighbor"], cells["side"],
                                          cells["orient"], dt, 10, cells["face_type"])
    ctx.run("all", dt, 10)
    ctx.sync()
    errs = rel_l2_per_quantity(ctx.get_dofs(), q_ref)
    assert max(errs) < 1e-5, errs
    out = np.empty_like(q0)
    ctx.run_host("all", dt, 3, q0, out)
    ctx.set_dofs(q0)
    ctx.run("all", dt, 3)
    ctx.sync()
    assert np.array_equal(out, ctx.get_dofs())
    ctx.close()


@pytest.mark.parametrize("fused", [0, 1])
@pytest.mark.parametrize("order", [4, 6])
def test_local_flux_in_neighbour_kernel_partial_blocks(built_lib, order, fused):
    """The fused-flux step (SEI_OPT_NB_FORM 2, with and without the one-launch ADER + volume +
    traces kernel) on the 317-cell cut mesh: the last 32-cell block of the cell-local kernels and
    the last 8-cell tile of the neighbour kernel are partial, and outflow faces carry no flux;
    three steps within 1e-5 of the FP64 oracle."""
    from seissol_gb300 import Context
    base, _, _ = _ctx(order, 0, seed=23)
    cells = base.get_cells()
    dt = base.cfl_timestep(0.5)
    base.close()
    keep = 317
    cut = {k: np.ascontiguousarray(v[:keep]) for k, v in cells.items()}
    ft = np.array(cut["face_type"], dtype=np.int8)
    nb = np.array(cut["neighbor"])
    ft[nb >= keep] = 2
    nb[nb >= keep] = 0
    q0 = seeded_dofs(keep, order, 23)
    ctx = Context(order, device=0, precision=PREC_F16X3)
    ctx.set_cells(cut["star"], cut["AplusT"], cut["AminusT"], nb, cut["side"], cut["orient"], ft)
    ctx.set_option(OPT_NB_FORM, 2)
    ctx.set_option(1, fused)  # SEI_OPT_FUSED_LOCAL
    ctx.set_dofs(q0)
    ctx.run("all", dt, 3)
    ctx.sync()
    q_gpu = ctx.get_dofs()
    ctx.close()
    q_ref = oracle_py.Oracle(order).steps(q0, cut["star"].astype(np.float64), cut["AplusT"].astype(np.float64),
                                          cut["AminusT"].astype(np.float64), nb, cut["side"], cut["orient"], dt, 3, ft)
    errs = rel_l2_per_quantity(q_gpu, q_ref)
    assert max(errs) < 1e-5, errs


def test_autotune_failure_restores_the_options(built_lib):
    """A candidate that fails (injected on the host through SEI_OPT_TUNE_FAIL_AT) makes sei_autotune
    return its error and leaves the context's options and DOFs as they were on entry."""
    from seissol_gb300 import SeiError
    ctx, n, q0 = _ctx(4, PREC_F16X3)
    ctx.set_option(1, 1)  # SEI_OPT_FUSED_LOCAL
    ctx.set_option(OPT_NB_FORM, 1)
    ctx.set_option(4, 2)  # SEI_OPT_NB_CTAS
    opts = (1, 3, 4, OPT_NB_FORM)
    before = {o: ctx.get_option(o) for o in opts}
    ctx.set_option(7, 3)  # SEI_OPT_TUNE_FAIL_AT: the fourth candidate fails
    dt = ctx.cfl_timestep(0.5)
    with pytest.raises(SeiError):
        ctx.autotune(dt, 2)
    assert {o: ctx.get_option(o) for o in opts} == before
    assert np.array_equal(ctx.get_dofs(), q0)
    ctx.set_option(7, -1)
    r = ctx.autotune(dt, 2)
    assert r["candidates"] == 14
    ctx.close()
