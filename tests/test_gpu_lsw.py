"""GPU parity of linear slip weakening, nucleation, the fault time and the rupture outputs against
the FP64 oracle (src/DynamicRupture/FrictionLaws/CpuImpl/LinearSlipWeakening.h, BaseFrictionLaw.h).

Workload: periodic cube 8 x 4 x 4 cubes of 100 m with a planar fault at x = 4 h (32 faces), the
slip-weakening set-up of LSWParams.fault_config (mu_s 0.677, mu_d 0.525, d_c 0.01 m, sn0 ~
U[-125, -115] MPa, tau1_0 ~ U[62, 78] MPa), forced rupture at t = 0 on the first quarter of the
faces.  Along the oracle's trajectory (the GPU takes the oracle's DOFs, fault state and time
before every step) each step is compared alone: slip rate 1e-5 relative L2 and 1e-3 m/s per
point, accumulated slip and tractions 1e-5 relative L2, friction coefficient 1e-6, peak slip rate
1e-5 relative L2, rupture and dynamic-stress times equal to 1e-12 relative (the host and the
oracle round the sub-step lengths differently) on all but 0.2 % of the points, DOFs 1e-5 relative
L2.  A free run stays within 1e-3 (slip) of the oracle's free run.
"""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu

FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")
AUX_FIELDS = dict(peak="peak_slip_rate", trup="rupture_time", tdyn="dyn_stress_time", mu_s="mu_s", mu_d="mu_d",
                  d_c="d_c", cohesion="cohesion", t_forced="forced_rupture_time", reg="reg_strength")


def _init(ctx):
    return np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)


def _setup(order=4, law=1, seed=5, precision=0, dims=(8, 4, 4), **kw):
    from seissol_gb300 import Context, LSWParams
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(*dims, perturb=0.0, seed=seed, fault_plane=dims[0] // 2)
    p = LSWParams.fault_config(law=law, seed=seed + 1, **kw)
    nf = ctx.dr_setup_lsw(p)
    assert ctx.dr_law() == law
    npts = (order + 1) ** 2
    tf = np.full((nf, npts), 1e300)
    tf[: nf // 4] = 0.0
    ctx.dr_set_state("forced_rupture_time", tf)
    q0 = seeded_dofs(n, order, seed)
    ctx.set_dofs(q0)
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    aux = {k: ctx.dr_state(v) for k, v in AUX_FIELDS.items()}
    aux.update(time=0.0, t0=p.t0, s0=0.0, nucleate=0, nuc=None, law=law, healing=p.healing_threshold,
               v_star=p.v_star, prakash_length=p.prakash_length, tp_exponent=p.tp_proxy_exponent)
    return ctx, n, q0, ctx.get_cells(), ctx.dr_faces(), state, _init(ctx), aux


def _push(ctx, q, state, init, aux):
    """The oracle's DOFs, fault state, initial stresses and time into the context."""
    ctx.set_dofs(q.astype(np.float32))
    for k, v in FIELDS.items():
        ctx.dr_set_state(v, state[k])
    for k, v in AUX_FIELDS.items():
        if aux.get(k) is not None:
            ctx.dr_set_state(v, aux[k])
    for i, name in enumerate(("sn0", "tau1_0", "tau2_0")):
        ctx.dr_set_state(name, init[:, i])
    ctx.dr_set_time(aux["time"])


def _times_agree(a, b, frac=0.002):
    same = (a == b) | (np.abs(a - b) <= 1e-12 * np.abs(b))
    return (~same).mean() <= frac


def _compare(ctx, q, state, init, aux, law):
    v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
    v_ref = np.hypot(state["v1"], state["v2"])
    assert rel_l2(v_gpu, v_ref) < 1e-5, rel_l2(v_gpu, v_ref)
    assert np.abs(v_gpu - v_ref).max() < 1e-3, np.abs(v_gpu - v_ref).max()
    for k in ("slip", "slip1", "trac1", "trac2"):
        assert rel_l2(ctx.dr_state(FIELDS[k]), state[k]) < 1e-5, k
    assert np.abs(ctx.dr_state("mu") - state["mu"]).max() < 1e-6
    assert rel_l2(ctx.dr_state("peak_slip_rate"), aux["peak"]) < 1e-5
    assert _times_agree(ctx.dr_state("rupture_time"), aux["trup"])
    assert _times_agree(ctx.dr_state("dyn_stress_time"), aux["tdyn"])
    if law == 2:
        assert rel_l2(ctx.dr_state("reg_strength"), aux["reg"]) < 1e-6
    assert np.allclose(_init(ctx), init, rtol=1e-12, atol=0)
    assert abs(ctx.dr_time() - aux["time"]) <= 1e-15 * max(1.0, aux["time"])
    assert rel_l2(ctx.get_dofs(), q) < 1e-5, rel_l2(ctx.get_dofs(), q)


@pytest.mark.parametrize("order,law,precision", [(4, 1, 0), (4, 2, 0), (4, 3, 0), (5, 1, 0), (6, 1, 0), (6, 1, 1)])
def test_lsw_steps_along_oracle(built_lib, order, law, precision):
    """precision 1: the mixed path (tensor-core neighbour flux beside the fault kernel)."""
    ctx, n, q, cells, faces, state, init, aux = _setup(order, law, precision=precision, t0=0.0)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, {})
    a = np.zeros_like(state["v1"])
    slipping = 0
    for _ in range(8):
        _push(ctx, q, state, init, aux)
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        _compare(ctx, q, state, init, aux, law)
        slipping = max(slipping, int((np.hypot(state["v1"], state["v2"]) > 1e-3).sum()))
    # the forced-rupture patch slips and the weakened points reach d_c
    assert slipping >= faces["cells"].shape[0] // 4 * (order + 1) ** 2 // 2
    assert (aux["tdyn"] >= 0).any() and (aux["trup"] >= 0).any()
    ctx.close()


def test_lsw_ramp_and_healing_along_oracle(built_lib):
    """Forced-rupture ramp over 3 steps and healing below 0.05 m/s."""
    ctx, n, q, cells, faces, state, init, aux = _setup(4, 1, seed=9)
    dt = ctx.cfl_timestep(0.5)
    ctx.close()
    ctx, n, q, cells, faces, state, init, aux = _setup(4, 1, seed=9, t0=3 * dt, healing_threshold=0.05)
    o = oracle_py.Oracle(4)
    dro = oracle_py.DROracle(4, faces, {})
    a = np.zeros_like(state["v1"])
    for _ in range(10):
        _push(ctx, q, state, init, aux)
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        _compare(ctx, q, state, init, aux, 1)
    ctx.close()


def test_lsw_free_run(built_lib):
    """15 steps at order 5 from the same start on both sides, no exchange: the float32 wave field
    and the non-smooth law keep the fault state within 1e-3 of the oracle."""
    order = 5
    ctx, n, q, cells, faces, state, init, aux = _setup(order, 1, seed=17)
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, {})
    a = np.zeros_like(state["v1"])
    for _ in range(15):
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
    ctx.run("all_dr", dt, 15)
    ctx.sync()
    assert rel_l2(ctx.dr_state("slip"), state["slip"]) < 1e-3
    assert rel_l2(ctx.get_dofs(), q) < 1e-3
    assert np.abs(ctx.dr_state("mu") - state["mu"]).max() < 1e-3
    assert _times_agree(ctx.dr_state("rupture_time"), aux["trup"], 0.02)
    assert abs(ctx.dr_time() - 15 * dt) < 1e-12
    ctx.close()


@pytest.mark.parametrize("law", [0, 1])
def test_nucleation_along_oracle(built_lib, law):
    """Gaussian nucleation of +20 MPa shear (-5 MPa normal) on the first half of the faces over
    3 steps, for rate and state (law 0) and slip weakening (law 1, no forced rupture)."""
    from seissol_gb300 import Context, RSParams
    order = 4
    if law == 0:
        ctx = Context(order, device=0)
        n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=3, fault_plane=4)
        rs = RSParams.fault_config(seed=5)
        ctx.dr_setup(rs)
        q = seeded_dofs(n, order, 3)
        ctx.set_dofs(q)
        cells, faces = ctx.get_cells(), ctx.dr_faces()
        state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
        init = _init(ctx)
        params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                              "max_newton", "max_outer")}
        a = ctx.dr_state("a")
        aux = {"peak": ctx.dr_state("peak_slip_rate"), "trup": ctx.dr_state("rupture_time"), "law": 0,
               "time": 0.0, "s0": 0.0}
    else:
        ctx, n, q, cells, faces, state, init, aux = _setup(order, 1, seed=3)
        ctx.dr_set_state("forced_rupture_time", np.full_like(state["v1"], 1e300))
        aux["t_forced"][:] = 1e300
        params, a = {}, np.zeros_like(state["v1"])
    nf, npts = state["v1"].shape
    dt = ctx.cfl_timestep(0.5)
    nuc = np.zeros((nf, 3, npts))
    nuc[: nf // 2, 1] = 20e6
    nuc[: nf // 2, 0] = -5e6
    for i, name in enumerate(("nuc_sn", "nuc_tau1", "nuc_tau2")):
        ctx.dr_set_state(name, nuc[:, i])
    ctx.dr_set_nucleation(True, 3 * dt, 0.0)
    aux.update(nucleate=1, nuc=nuc, t0=3 * dt)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, params)
    tau_start = init[:, 1].copy()
    for _ in range(5):
        ctx.set_dofs(q.astype(np.float32))
        for k, v in FIELDS.items():
            ctx.dr_set_state(v, state[k])
        for i, name in enumerate(("sn0", "tau1_0", "tau2_0")):
            ctx.dr_set_state(name, init[:, i])
        ctx.dr_set_state("peak_slip_rate", aux["peak"])
        ctx.dr_set_state("rupture_time", aux["trup"])
        ctx.dr_set_time(aux["time"])
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        assert np.allclose(_init(ctx), init, rtol=1e-12, atol=0)
        v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
        v_ref = np.hypot(state["v1"], state["v2"])
        if law == 0:
            assert (np.abs(v_gpu - v_ref) <= 1e-4 * np.abs(v_ref) + 1e-12).all()
            assert np.abs(ctx.dr_state("psi") - state["psi"]).max() < 1e-6
        else:
            assert rel_l2(v_gpu, v_ref) < 1e-5
        assert rel_l2(ctx.dr_state("peak_slip_rate"), aux["peak"]) < 1e-4
        assert _times_agree(ctx.dr_state("rupture_time"), aux["trup"])
        assert rel_l2(ctx.get_dofs(), q) < 1e-5
    # the full nucleation stress is in after the window (3 dt)
    assert np.allclose(init[: nf // 2, 1] - tau_start[: nf // 2], 20e6, rtol=1e-12)
    assert np.array_equal(init[nf // 2:, 1], tau_start[nf // 2:])
    ctx.close()


def test_lsw_under_lts_matches_oracle(built_lib):
    """Graded cube (several clusters), slip weakening with forced rupture as a ramp: one LTS cycle
    (each cluster's fault step at its own time within the cycle) against the LTS restatement."""
    from seissol_gb300 import Context, LSWParams
    from oracle import dg_setup
    order = 4
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(8, 8, 8, perturb=0.05, seed=13, grading=6.0, fault_plane=4)
    p = LSWParams.fault_config(law=1, seed=14, t0=2e-3)
    nf = ctx.dr_setup_lsw(p)
    npts = (order + 1) ** 2
    tf = np.full((nf, npts), 1e300)
    tf[: nf // 3] = 0.0
    ctx.dr_set_state("forced_rupture_time", tf)
    ncl = ctx.lts_setup(0.5, 8)
    assert ncl >= 2
    cells, faces = ctx.get_cells(), ctx.dr_faces()
    coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 8, faces["cells"])
    q0 = seeded_dofs(n, order, 23)
    ctx.set_dofs(q0)
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    aux = {k: ctx.dr_state(v) for k, v in AUX_FIELDS.items()}
    aux.update(time=0.0, t0=p.t0, s0=0.0, nucleate=0, nuc=None, law=1, healing=-1.0, v_star=p.v_star,
               prakash_length=p.prakash_length, tp_exponent=p.tp_proxy_exponent)
    dr = {"faces": faces, "params": {}, "state": state, "a": np.zeros_like(state["v1"]), "init": _init(ctx),
          "aux": aux}
    ctx.lts_run(1)
    ctx.sync()
    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dt0, 1, dr=dr)
    assert rel_l2(ctx.get_dofs(), q_ref) < 1e-4
    v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
    v_ref = np.hypot(state["v1"], state["v2"])
    assert rel_l2(v_gpu, v_ref) < 1e-4
    assert rel_l2(ctx.dr_state("slip"), state["slip"]) < 1e-4
    assert np.abs(ctx.dr_state("mu") - state["mu"]).max() < 1e-5
    assert _times_agree(ctx.dr_state("rupture_time"), aux["trup"])
    assert abs(ctx.dr_time() - aux["time"]) <= 1e-12
    assert (v_ref > 1e-3).any()
    ctx.close()


def test_lsw_api(built_lib):
    from seissol_gb300 import Context, LSWParams, SeiError
    ctx = Context(4, device=0)
    ctx.build_periodic_cube(8, 4, 4, fault_plane=4)
    for bad in (dict(law=0), dict(law=4), dict(d_c=0.0), dict(sn_max=1e6), dict(t0=-1.0),
                dict(law=2, prakash_length=0.0), dict(law=3, tp_proxy_exponent=0.0)):
        with pytest.raises(SeiError):
            ctx.dr_setup_lsw(LSWParams.fault_config(**bad))
    ctx.dr_setup_lsw(LSWParams.fault_config())
    assert ctx.dr_law() == 1 and ctx.dr_time() == 0.0
    assert np.all(ctx.dr_state("rupture_time") == -1.0) and np.all(ctx.dr_state("mu") == 0.677)
    with pytest.raises(SeiError):
        ctx.dr_set_time(-1.0)
    with pytest.raises(SeiError):
        ctx.dr_set_nucleation(True, 0.0, 0.0)
    with pytest.raises(SeiError):
        ctx.dr_warm_start(True)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all_dr", dt, 3)
    ctx.sync()
    assert ctx.dr_time() == (0.0 + dt) + dt + dt
    ctx.close()
