"""GPU parity of the aging, slip and severe-velocity-weakening laws (sei_dr_setup_rate_state)
against the FP64 oracle (CpuImpl/AgingLaw.h, SlipLaw.h, SevereVelocityWeakeningLaw.h).

Workload: periodic cube 8 x 4 x 4 (32 fault faces at x = 4 h), the fault configuration's
distributions (a ~ U[0.008, 0.02], sn ~ U[-120, -40] MPa, tau ~ U[20, 75] MPa, V_init 1e-16 m/s)
and the state of steady sliding at V_init.  Along the oracle's trajectory (the GPU takes the
oracle's DOFs and fault state before every step) 6 steps are compared one by one: slip rate 1e-4
relative per point + 1e-12 m/s (severe law: + 1e-5 m/s: above V0 its friction hardly depends on V,
so V = (tau - |sn| mu) / eta_s carries the float32 stress error itself, ~10 Pa / eta_s ~ 2e-6 m/s), state variable 1e-5 relative (it follows the slip rate, whose
float32 wave-field inputs carry ~1e-7, and the slip law amplifies that about twelvefold: d ln theta
/ d ln V = -1 + e^-x (1 - x ln(V theta_ref / L)), x = V dt / L; plus 1e-10 absolute, 1e-8 for the
severe law, whose update adds about 1e-3 V per step with V known to 1e-5 m/s), slip 1e-4 relative L2, friction
coefficient 1e-6, DOFs 1e-5 relative L2, Newton iterations within 2 % (+ 5).
"""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu

FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")


@pytest.mark.parametrize("law,order", [(4, 4), (5, 4), (6, 4), (4, 6), (5, 5), (6, 6)])
def test_rate_state_law_along_oracle(built_lib, law, order):
    from seissol_gb300 import Context, RSParams
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=3, fault_plane=4)
    rs = RSParams.fault_config(seed=5)
    ctx.dr_setup_rate_state(rs, law)
    assert ctx.dr_law() == law
    q = seeded_dofs(n, order, 3)
    cells, faces = ctx.get_cells(), ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    a = ctx.dr_state("a")
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, params)
    aux = {"law": law, "time": 0.0}
    moving = 0
    for _ in range(6):
        ctx.set_dofs(q.astype(np.float32))
        for k, v in FIELDS.items():
            ctx.dr_set_state(v, state[k])
        ctx.dr_reset_counters()
        q, _, _, it, _ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        v_ref = np.hypot(state["v1"], state["v2"])
        vabs = 1e-5 if law == 6 else 1e-12
        assert (np.abs(v_gpu - v_ref) <= 1e-4 * v_ref + vabs).all(), np.max(np.abs(v_gpu - v_ref) / (v_ref + 1e-30))
        th, th_ref = ctx.dr_state("psi"), state["psi"]
        bad = np.abs(th - th_ref) - (1e-5 * np.abs(th_ref) + (1e-8 if law == 6 else 1e-10))
        assert (bad <= 0).all(), (th.ravel()[bad.argmax()], th_ref.ravel()[bad.argmax()])
        assert rel_l2(ctx.dr_state("slip"), state["slip"]) < 1e-4
        assert np.abs(ctx.dr_state("mu") - state["mu"]).max() < 1e-6
        assert rel_l2(ctx.get_dofs(), q) < 1e-5
        it_gpu, _ = ctx.dr_newton_iterations()
        assert abs(it_gpu - int(it.sum())) <= 0.02 * int(it.sum()) + 5, (it_gpu, int(it.sum()))
        moving = max(moving, int((v_ref > 1e-3).sum()))
    assert moving > 0
    ctx.close()
