"""GPU local time stepping (rate 2) through the C ABI against the FP64 oracle restatement.

Tolerances: two LTS cycles on a graded cube, 1e-4 relative L2 per quantity (FP32 GPU vs FP64
oracle, the bar of multi-step elastic runs); with a single cluster LTS reproduces global time
stepping of the same kernels bit for bit.
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py
from tests.helpers import rel_l2_per_quantity, seeded_dofs

pytestmark = pytest.mark.gpu


def _graded_ctx(order, grading=6.0, dims=(8, 8, 8), seed=5, precision=0):
    from seissol_gb300 import Context
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(*dims, perturb=0.05, seed=seed, grading=grading)
    return ctx, n


@pytest.mark.parametrize("order", [4, 6])
def test_lts_matches_oracle(built_lib, order):
    ctx, n = _graded_ctx(order)
    coords0, _, _ = ctx.get_geometry()
    ncl = ctx.lts_setup(0.5, 8)
    assert ncl >= 2
    perm = ctx.lts_permutation()
    assert np.array_equal(np.sort(perm), np.arange(n))
    coords, material, _ = ctx.get_geometry()
    assert np.array_equal(coords, coords0[perm])
    start, dts = ctx.lts_clusters()
    cl_gpu = np.repeat(np.arange(ncl), np.diff(start))
    cells = ctx.get_cells()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 8)
    assert np.array_equal(cl, cl_gpu)
    assert np.allclose(dts, dt0 * 2.0 ** np.arange(ncl), rtol=1e-12)
    q0 = seeded_dofs(n, order, 7)
    ctx.set_dofs(q0)
    ctx.lts_run(2)
    ctx.sync()
    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dt0, 2)
    errs = rel_l2_per_quantity(ctx.get_dofs(), q_ref)
    assert max(errs) < 1e-4, errs
    ctx.close()


def test_lts_single_cluster_is_global_stepping(built_lib):
    ctx, n = _graded_ctx(5)
    q0 = seeded_dofs(n, 5, 9)
    assert ctx.lts_setup(0.5, 1) == 1
    _, dts = ctx.lts_clusters()
    ctx.set_dofs(q0)
    ctx.lts_run(3)
    ctx.sync()
    q_lts = ctx.get_dofs()
    ctx.set_dofs(q0)
    ctx.run("all", dts[0], 3)
    ctx.sync()
    assert np.array_equal(q_lts, ctx.get_dofs())
    ctx.close()


def test_lts_rejects_fault_and_repeat(built_lib):
    from seissol_gb300 import Context, RSParams, SeiError
    ctx = Context(4, device=0)
    ctx.build_periodic_cube(8, 4, 4, fault_plane=4)
    with pytest.raises(SeiError, match="SEI_ERR_STATE"):  # the fault must be set up first
        ctx.lts_setup(0.5, 4)
    ctx.dr_setup(RSParams.fault_config())
    ctx.lts_setup(0.5, 4)
    with pytest.raises(SeiError, match="SEI_ERR_STATE"):  # and not after
        ctx.dr_setup(RSParams.fault_config())
    ctx.close()
    ctx, _ = _graded_ctx(4, dims=(4, 4, 4))
    ctx.lts_setup(0.5, 4)
    with pytest.raises(SeiError, match="SEI_ERR_STATE"):
        ctx.lts_setup(0.5, 4)
    ctx.close()


def test_lts_graph_replay_matches_direct_launches(built_lib):
    """SEI_OPT_LTS_GRAPH: a recorded cycle replayed three times gives the DOFs of three directly
    launched cycles, bit for bit."""
    SEI_OPT_LTS_GRAPH = 2
    out = []
    for graph in (0, 1):
        ctx, n = _graded_ctx(5)
        ctx.lts_setup(0.5, 8)
        ctx.set_option(SEI_OPT_LTS_GRAPH, graph)
        ctx.set_dofs(seeded_dofs(n, 5, 11))
        ctx.lts_run(2)
        ctx.lts_run(1)
        ctx.sync()
        out.append(ctx.get_dofs())
        ctx.close()
    assert np.array_equal(out[0], out[1])


DR_FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
                 trac1="traction1", trac2="traction2")


def _fault_ctx(order, grading, dims=(8, 8, 8), seed=13, precision=0):
    from seissol_gb300 import Context, RSParams
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(*dims, perturb=0.05, seed=seed, grading=grading, fault_plane=4)
    rs = RSParams.fault_config(seed=seed + 2)
    ctx.dr_setup(rs)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    return ctx, n, params


def test_lts_with_fault_single_cluster_is_global_stepping(built_lib):
    """One cluster: the LTS cycle with the fault step is kernel 'all_dr' bit for bit."""
    a, n, _ = _fault_ctx(4, 1.0, dims=(8, 4, 4))
    b, _, _ = _fault_ctx(4, 1.0, dims=(8, 4, 4))
    q0 = seeded_dofs(n, 4, 21)
    assert a.lts_setup(0.5, 1) == 1
    _, dts = a.lts_clusters()
    a.set_dofs(q0)
    b.set_dofs(q0)
    a.lts_run(3)
    b.run("all_dr", dts[0], 3)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_dofs(), b.get_dofs())
    for f in DR_FIELDS.values():
        assert np.array_equal(a.dr_state(f), b.dr_state(f)), f
    a.close()
    b.close()


def test_lts_with_fault_matches_oracle(built_lib):
    """A graded cube with the fault on its fifth cube-vertex plane along x, in several clusters: the two cells of each fault face share a cluster, and one LTS cycle with the fault
    step in each cluster's correction matches the FP64 restatement (DOFs 1e-4 relative L2 per
    quantity, slip rate 1e-4 relative per point + 1e-12 m/s, state variable 1e-6)."""
    order = 4
    ctx, n, params = _fault_ctx(order, 6.0)
    ncl = ctx.lts_setup(0.5, 8)
    assert ncl >= 2
    start, dts = ctx.lts_clusters()
    cl_gpu = np.repeat(np.arange(ncl), np.diff(start))
    cells = ctx.get_cells()
    faces = ctx.dr_faces()
    coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 8, faces["cells"])
    assert np.array_equal(cl, cl_gpu)
    assert np.array_equal(cl[faces["cells"][:, 0]], cl[faces["cells"][:, 1]])
    assert len(np.unique(cl[faces["cells"][:, 0]])) >= 1
    q0 = seeded_dofs(n, order, 23)
    ctx.set_dofs(q0)
    state = {k: ctx.dr_state(v) for k, v in DR_FIELDS.items()}
    dr = {"faces": faces, "params": params, "state": state, "a": ctx.dr_state("a"),
          "init": np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)}
    ctx.lts_run(1)
    ctx.sync()
    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dt0, 1, dr=dr)
    errs = rel_l2_per_quantity(ctx.get_dofs(), q_ref)
    assert max(errs) < 1e-4, errs
    v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
    v_ref = np.hypot(state["v1"], state["v2"])
    assert (np.abs(v_gpu - v_ref) <= 1e-4 * np.abs(v_ref) + 1e-12).all()
    assert np.abs(ctx.dr_state("psi") - state["psi"]).max() < 1e-6
    ctx.close()


PREC_F16X3 = 1
OPT_NB_FORM = 5


@pytest.mark.parametrize("form", [1, 2])
@pytest.mark.parametrize("order", [4, 6])
def test_lts_mixed_precision_matches_oracle(built_lib, order, form):
    """Mixed precision under local time stepping: the tensor-core neighbour kernel reads the face
    traces of the pool blocks (cells, integration buffers, half-step integrals) through the
    cycle's source tables; with SEI_OPT_NB_FORM 2 the local flux joins it.  Two cycles within
    1e-4 of the FP64 oracle (the LTS bar) and within 1e-5 of the FP32 LTS run."""
    outs = []
    for prec in (0, PREC_F16X3):
        ctx, n = _graded_ctx(order, precision=prec)
        ncl = ctx.lts_setup(0.5, 8)
        assert ncl >= 2
        if prec:
            ctx.set_option(OPT_NB_FORM, form)
        cells = ctx.get_cells()
        start, dts = ctx.lts_clusters()
        q0 = seeded_dofs(n, order, 7)
        ctx.set_dofs(q0)
        ctx.lts_run(2)
        ctx.sync()
        outs.append(ctx.get_dofs())
        ctx.close()
    cl = np.repeat(np.arange(len(dts)), np.diff(start))
    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dts[0], 2)
    errs = rel_l2_per_quantity(outs[1], q_ref)
    assert max(errs) < 1e-4, errs
    assert max(rel_l2_per_quantity(outs[1], outs[0])) < 1e-5


def test_lts_mixed_precision_graph_and_fault(built_lib):
    """Mixed precision, local time stepping and the fault step together (the combined
    configuration's path): one recorded cycle replayed gives the DOFs and fault state of directly
    launched cycles bit for bit, and one cycle matches the FP64 restatement with the tolerances of
    the FP32 test."""
    order = 4
    out = []
    for graph in (0, 1):
        ctx, n, params = _fault_ctx(order, 6.0, precision=PREC_F16X3)
        ctx.lts_setup(0.5, 8)
        ctx.set_option(OPT_NB_FORM, 2)
        ctx.set_option(2, graph)  # SEI_OPT_LTS_GRAPH
        q0 = seeded_dofs(n, order, 23)
        ctx.set_dofs(q0)
        if graph == 0:
            cells = ctx.get_cells()
            faces = ctx.dr_faces()
            start, dts = ctx.lts_clusters()
            state = {k: ctx.dr_state(v) for k, v in DR_FIELDS.items()}
            dr = {"faces": faces, "params": params, "state": state, "a": ctx.dr_state("a"),
                  "init": np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)}
            ctx.lts_run(1)
            ctx.sync()
            cl = np.repeat(np.arange(len(dts)), np.diff(start))
            q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dts[0], 1, dr=dr)
            errs = rel_l2_per_quantity(ctx.get_dofs(), q_ref)
            assert max(errs) < 1e-4, errs
            v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
            v_ref = np.hypot(state["v1"], state["v2"])
            assert (np.abs(v_gpu - v_ref) <= 1e-4 * np.abs(v_ref) + 1e-12).all()
            ctx.lts_run(2)
        else:
            ctx.lts_run(1)
            ctx.lts_run(2)
        ctx.sync()
        out.append((ctx.get_dofs(), ctx.dr_state("psi")))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
