"""GPU parity of thermal pressurisation (sei_dr_set_thermal_pressurization) against the FP64
oracle (CpuImpl/ThermalPressurization/ThermalPressurization.cpp with RateAndState.h's coupling).

Workload: periodic cube 8 x 4 x 4 (32 fault faces, O4), the fault configuration's rate-and-state
set-up (fast velocity weakening and the aging law), thermal diffusivity 1e-6 m^2/s, heat capacity
2.7e6 J/(m^3 K), undrained response 1e6 Pa/K, shear zone half width 2 mm, hydraulic diffusivity
1e-4 m^2/s, so that the pore pressure rises by MPa in the slipping points.  Both sides run 4 steps
from the same start (the modes cannot be set through the ABI): after every step the slip rate
agrees to 1e-4 relative + 1e-9 m/s, temperature and pressure to 1e-6 relative to their change,
the state variable to 1e-6 relative, DOFs to 1e-5 relative L2.
"""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu

FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")


@pytest.mark.parametrize("law", [0, 4])
def test_thermal_pressurization_matches_oracle(built_lib, law):
    from seissol_gb300 import Context, RSParams, TPParams
    order = 4
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=3, fault_plane=4)
    rs = RSParams.fault_config(seed=5)
    ctx.dr_setup_rate_state(rs, law)
    tp = TPParams(thermal_diffusivity=1e-6, heat_capacity=2.7e6, undrained_tp_response=1e6, initial_temperature=483.15,
                  initial_pressure=0.0, half_width_shear_zone=0.002, hydraulic_diffusivity=1e-4)
    ctx.dr_set_thermal_pressurization(True, tp)
    q = seeded_dofs(n, order, 3)
    ctx.set_dofs(q)
    cells, faces = ctx.get_cells(), ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    a = ctx.dr_state("a")
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    nf, npts = a.shape
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    full = lambda v: np.full((nf, npts), float(v))
    aux = {"law": law, "time": 0.0, "tp": 1, "tp_alpha": 1e-6, "tp_rhoc": 2.7e6, "tp_lambda": 1e6, "tp_t0": 483.15,
           "tp_p0": 0.0, "tp_hw": full(0.002), "tp_hyd": full(1e-4), "tp_theta": np.zeros((nf, 60, npts)),
           "tp_sigma": np.zeros((nf, 60, npts)), "tp_temp": full(483.15), "tp_pres": full(0.0)}
    assert np.all(ctx.dr_state("tp_temperature") == 483.15) and np.all(ctx.dr_state("tp_pressure") == 0.0)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, params)
    for _ in range(4):
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        v_ref = np.hypot(state["v1"], state["v2"])
        assert (np.abs(v_gpu - v_ref) <= 1e-4 * v_ref + 1e-9).all(), np.max(np.abs(v_gpu - v_ref) / (v_ref + 1e-30))
        for name, key, base in (("tp_temperature", "tp_temp", 483.15), ("tp_pressure", "tp_pres", 0.0)):
            g, r = ctx.dr_state(name), aux[key]
            assert np.abs(g - r).max() <= 1e-6 * np.abs(r - base).max() + 1e-9, name
        assert np.allclose(ctx.dr_state("psi"), state["psi"], rtol=1e-6, atol=1e-9)
        assert rel_l2(ctx.get_dofs(), q) < 1e-5
    assert np.abs(aux["tp_pres"]).max() > 1e6  # the pore pressure moved by MPa
    ctx.close()


def test_thermal_pressurization_api(built_lib):
    from seissol_gb300 import Context, LSWParams, RSParams, SeiError, TPParams
    ctx = Context(4, device=0)
    ctx.build_periodic_cube(8, 4, 4, fault_plane=4)
    ctx.dr_setup_lsw(LSWParams.fault_config())
    tp = TPParams(1e-6, 2.7e6, 1e6, 483.15, 0.0, 0.002, 1e-4)
    with pytest.raises(SeiError):
        ctx.dr_set_thermal_pressurization(True, tp)  # not a rate-and-state law
    ctx.dr_setup(RSParams.fault_config())
    with pytest.raises(SeiError):
        ctx.dr_set_thermal_pressurization(True, TPParams(1e-4, 2.7e6, 1e6, 483.15, 0.0, 0.002, 1e-4))  # equal diffusivities
    ctx.dr_set_thermal_pressurization(True, tp)
    ctx.dr_set_thermal_pressurization(False)
    ctx.close()
