"""GPU parity of the dynamic-rupture step (proxy kernel all_dr) against the FP64 oracle.

Workload: orders 4-6, periodic cube 8 x 4 x 4 cubes with a planar fault at x = 4 h (32 faces x
25, 36 or 49 points), the fast-velocity-weakening parameters of the fault configuration (a ~ U[0.008, 0.02],
normal stress ~ U[-120, -40] MPa, shear ~ U[20, 75] MPa, V_init = 1e-16 m/s).
Tolerances: derivatives 2e-5 relative L2; imposed states and DOFs 1e-4 relative L2 per quantity;
slip rate 1e-4 relative per point (plus 1e-12 m/s absolute); state variable 1e-6 absolute.
"""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu

FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")


def _setup(seed=3, order=4, precision=0):
    from seissol_gb300 import Context, RSParams
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=seed, fault_plane=4)
    rs = RSParams.fault_config(seed=seed + 2)
    ctx.dr_setup(rs)
    q0 = seeded_dofs(n, order, seed)
    ctx.set_dofs(q0)
    cells = ctx.get_cells()
    faces = ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    a = ctx.dr_state("a")
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    return ctx, n, q0, cells, faces, state, a, init, params


def _compare_state(ctx, state, tol_v=1e-4):
    v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
    v_ref = np.hypot(state["v1"], state["v2"])
    assert (np.abs(v_gpu - v_ref) <= tol_v * np.abs(v_ref) + 1e-12).all(), np.max(np.abs(v_gpu - v_ref) / (v_ref + 1e-30))
    assert np.abs(ctx.dr_state("psi") - state["psi"]).max() < 1e-6
    assert rel_l2(ctx.dr_state("slip"), state["slip"]) < tol_v


@pytest.mark.parametrize("order,precision", [(4, 0), (5, 0), (6, 0), (6, 1)])
def test_dr_one_step(built_lib, order, precision):
    """precision 1: the mixed path (tensor-core neighbour flux beside the fault kernel)."""
    ctx, n, q0, cells, faces, state, a, init, params = _setup(order=order, precision=precision)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, params)
    q_ref, isp_ref, ism_ref, iters, (d_ref, _, _) = oracle_py.dr_full_step(o, dro, q0, cells, faces, state, a, init, dt)
    ctx.run("all_dr", dt, 1)
    ctx.sync()
    nf = faces["cells"].shape[0]
    slots = ctx.dr_slots()
    d_gpu = ctx.get_derivatives_slots(2 * nf)
    pc, mc = faces["cells"][:, 0], faces["cells"][:, 1]
    assert rel_l2(d_gpu[slots[pc]], d_ref[pc]) < 2e-5
    assert rel_l2(d_gpu[slots[mc]], d_ref[mc]) < 2e-5
    isp, ism = ctx.dr_imposed()
    for q in (0, 3, 5, 6, 7, 8):
        assert rel_l2(isp[:, q], isp_ref[:, q]) < 1e-4, q
        assert rel_l2(ism[:, q], ism_ref[:, q]) < 1e-4, q
    assert np.abs(isp[:, [1, 2, 4]]).max() == 0.0
    _compare_state(ctx, state)
    q_gpu = ctx.get_dofs()
    for q in range(9):
        assert rel_l2(q_gpu[:, q] - q0[:, q], q_ref[:, q] - q0[:, q]) < 1e-4, q
    it_gpu, npoints = ctx.dr_newton_iterations()
    assert npoints == nf * (order + 1) ** 2
    assert abs(it_gpu - iters.sum()) <= 0.02 * iters.sum() + 5
    ctx.close()


def test_dr_ten_steps(built_lib):
    ctx, n, q0, cells, faces, state, a, init, params = _setup(seed=11)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(4)
    dro = oracle_py.DROracle(4, faces, params)
    q = q0
    for _ in range(10):
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt)
    ctx.run("all_dr", dt, 10)
    ctx.sync()
    _compare_state(ctx, state, tol_v=1e-3)
    q_gpu = ctx.get_dofs()
    for qq in range(9):
        assert rel_l2(q_gpu[:, qq], q[:, qq]) < 1e-3, qq
    assert np.isfinite(q_gpu).all()
    ctx.close()


def test_dr_larger_fault_twenty_steps(built_lib):
    """512 faces (8 x 16 x 16 cubes, fault at x = 4 h) along 20 steps of the oracle's trajectory:
    before every step the GPU takes the oracle's DOFs and fault state, so each step is compared
    alone (rupture nucleation amplifies the float rounding of free runs).  Per step: slip rate
    1e-4 relative + 1e-12 m/s, state variable 1e-6, DOFs 1e-5 relative L2, Newton iterations
    within 1 %, every state finite.  A free 20-step GPU run stays finite."""
    from seissol_gb300 import Context, RSParams
    seed = 21
    ctx = Context(4, device=0)
    n = ctx.build_periodic_cube(8, 16, 16, perturb=0.0, seed=seed, fault_plane=4)
    rs = RSParams.fault_config(seed=seed + 2)
    nf = ctx.dr_setup(rs)
    assert nf == 512
    q = seeded_dofs(n, 4, seed)
    ctx.set_dofs(q)
    cells = ctx.get_cells()
    faces = ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    start = {k: v.copy() for k, v in state.items()}
    a = ctx.dr_state("a")
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(4)
    dro = oracle_py.DROracle(4, faces, params)
    for _ in range(20):
        q, _, _, it, _ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt)
        ctx.dr_reset_counters()
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        for name in FIELDS.values():
            assert np.isfinite(ctx.dr_state(name)).all(), name
        _compare_state(ctx, state, tol_v=1e-4)
        it_gpu, _ = ctx.dr_newton_iterations()
        assert abs(it_gpu - int(it.sum())) <= 0.01 * int(it.sum()), (it_gpu, int(it.sum()))
        assert rel_l2(ctx.get_dofs(), q) < 1e-5
        for k, v in FIELDS.items():
            ctx.dr_set_state(v, state[k])
        ctx.set_dofs(q.astype(np.float32))
    # free run from the initial state
    for k, v in FIELDS.items():
        ctx.dr_set_state(v, start[k])
    ctx.set_dofs(seeded_dofs(n, 4, seed))
    ctx.run("all_dr", dt, 20)
    ctx.sync()
    for name in FIELDS.values():
        assert np.isfinite(ctx.dr_state(name)).all(), name
    assert np.isfinite(ctx.get_dofs()).all()
    ctx.close()
