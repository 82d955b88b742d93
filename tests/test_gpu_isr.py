"""GPU parity of the imposed slip rates (sei_dr_setup_imposed; CpuImpl/ImposedSlipRates.h with the
regularised Yoffe, Gaussian and delta source time functions) against the FP64 oracle.

Workload: periodic cube 8 x 4 x 4 (32 fault faces), slip direction (0.8, 0.6), onset times
spread over the first three steps per face, tau_S = 2 dt, tau_R = 5 dt (Gaussian rise time 4 dt).
Along the oracle's trajectory, 10 steps: slip rate and slip within 1e-10 of their largest
magnitude (they depend on time only; the Yoffe closed form cancels near the onset, where CUDA's
and the host's asin and atan differ in the last bits), tractions 1e-5 relative L2 (float32 stresses), rupture time exact, DOFs 1e-5 relative L2.
"""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu

FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")


@pytest.mark.parametrize("law,order", [(7, 4), (8, 4), (9, 4), (7, 6), (8, 5)])
def test_imposed_slip_rate_along_oracle(built_lib, law, order):
    from seissol_gb300 import Context, ISRParams
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=3, fault_plane=4)
    dt = ctx.cfl_timestep(0.5)
    p = ISRParams(law=law, slip_dir1=0.8, slip_dir2=0.6, onset_time=0.0, tau_s=(4 if law == 8 else 2) * dt,
                  tau_r=5 * dt, sn0=-50e6, tau1_0=20e6)
    nf = ctx.dr_setup_imposed(p)
    npts = (order + 1) ** 2
    onset = np.repeat(np.linspace(0.0, 3 * dt, nf)[:, None], npts, axis=1)
    ctx.dr_set_state("onset_time", onset)
    q = seeded_dofs(n, order, 5)
    cells, faces = ctx.get_cells(), ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    aux = {"law": law, "time": 0.0, "peak": ctx.dr_state("peak_slip_rate"), "trup": ctx.dr_state("rupture_time"),
           "dir1": ctx.dr_state("slip_dir1"), "dir2": ctx.dr_state("slip_dir2"), "onset": onset,
           "taus": ctx.dr_state("tau_s"), "taur": ctx.dr_state("tau_r")}
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, {})
    a = np.zeros_like(state["v1"])
    for _ in range(10):
        ctx.set_dofs(q.astype(np.float32))
        for k, v in FIELDS.items():
            ctx.dr_set_state(v, state[k])
        ctx.dr_set_state("peak_slip_rate", aux["peak"])
        ctx.dr_set_state("rupture_time", aux["trup"])
        ctx.dr_set_time(aux["time"])
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        for k in ("v1", "v2", "slip1", "slip2", "slip"):
            g, r = ctx.dr_state(FIELDS[k]), state[k]
            assert (np.abs(g - r) <= 1e-10 * np.abs(r).max() + 1e-12 * np.abs(r)).all(), k
        assert rel_l2(ctx.dr_state("traction1"), state["trac1"]) < 1e-5
        assert rel_l2(ctx.dr_state("traction2"), state["trac2"]) < 1e-5
        assert np.array_equal(ctx.dr_state("rupture_time") >= 0, aux["trup"] >= 0)
        assert rel_l2(ctx.get_dofs(), q) < 1e-5
    assert (state["slip"] > 0.5).any()
    ctx.close()
