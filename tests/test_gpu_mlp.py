"""GPU warm start of the slip-rate Newton solve: training kernels against the oracle, training on
recorded samples, and what the trained network gains over the plain start.

Tolerances: gradient 1e-4 relative L2 and loss 1e-5 relative against the FP64 numpy gradient
(FP32 forward/backward, atomically accumulated); predicted log10 slip rate 1e-3 absolute; warm
and plain solves from the same state agree on slip rates to 1e-6 relative + 1e-12 m/s, on the
state variable to 1e-9 and on the DOFs to 1e-6 relative (Newton tolerance 1e-8 m/s); the GPU
warm-started step matches the oracle's warm-started step with the tolerances of the plain
fault step (slip rate 1e-4 relative, state 1e-6).
"""
import numpy as np
import pytest

from oracle import mlp as M
from oracle import oracle_py
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu


def _synthetic_samples(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-120e6, -40e6, n), rng.uniform(20e6, 75e6, n), rng.uniform(0.3, 0.9, n),
                     rng.uniform(0.008, 0.02, n), np.full(n, 0.014), rng.uniform(-40, 1, n)],
                    axis=1).astype(np.float32)


@pytest.mark.parametrize("n", [1, 63, 1000, 20000])
def test_gradient_matches_oracle(built_lib, n):
    from seissol_gb300 import mlp_gradient
    S = _synthetic_samples(n, n)
    p = M.glorot(7)
    norm = M.normalisation(_synthetic_samples(500, 9), 1e-6)
    g, loss = mlp_gradient(p, norm, S)
    loss_ref, g_ref = M.loss_and_grad(p, norm, S)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref, (loss, loss_ref)
    assert rel_l2(g, g_ref) < 1e-4, rel_l2(g, g_ref)


def test_predict_matches_oracle(built_lib):
    from seissol_gb300 import mlp_predict
    S = _synthetic_samples(3000, 11)
    p = M.glorot(12)
    norm = M.normalisation(S, 1e-6)
    out = mlp_predict(p, norm, S)
    ref = M.predict(p, norm, S)
    assert np.abs(out - ref).max() < 1e-3, np.abs(out - ref).max()


FIELDS = dict(psi="psi", v1="slip_rate1", v2="slip_rate2", slip1="slip1", slip2="slip2", slip="slip", mu="mu",
              trac1="traction1", trac2="traction2")


def _fault(seed):
    from seissol_gb300 import Context, RSParams
    ctx = Context(4, device=0)
    n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=seed, fault_plane=4)
    rs = RSParams.fault_config(seed=seed + 2)
    ctx.dr_setup(rs)
    ctx.set_dofs(seeded_dofs(n, 4, seed))
    return ctx, rs


def _trained(steps=6, train_steps=1500):
    """Network trained on the GPU from the samples a plain 6-step run on fault seed 3 recorded."""
    ctx, _ = _fault(3)
    ctx.dr_record_samples(200000)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all_dr", dt, steps)
    ctx.sync()
    S = ctx.dr_samples()
    first, last = ctx.mlp_train(steps=train_steps, lr=3e-3, seed=1)
    p, norm = ctx.mlp_get()
    ctx.close()
    return S, first, last, p, norm


@pytest.fixture(scope="module")
def trained():
    return _trained()


def test_recorded_samples_and_training(built_lib, trained):
    S, first, last, p, norm = trained
    assert len(S) > 10000 and np.isfinite(S).all()
    assert (S[:, 0] < 0).all() and (S[:, 1] > 0).all()
    assert last < 0.02 * first, (first, last)
    keep = M.usable(S)
    err = np.abs(M.predict(p, norm, S[keep]) - S[keep, 5])
    assert np.median(err) < 0.05, np.median(err)


def test_warm_start_gain_and_identical_slip_rates(built_lib, trained):
    _, _, _, p, norm = trained
    plain, _ = _fault(4)
    warm, _ = _fault(4)
    warm.mlp_set(p, norm)
    warm.dr_warm_start(True)
    dt = plain.cfl_timestep(0.5)
    for ctx in (plain, warm):
        ctx.dr_reset_counters()
        ctx.run("all_dr", dt, 6)
        ctx.sync()
    tot_p, npts, first_p = plain.dr_newton_iterations(first=True)
    tot_w, _, first_w = warm.dr_newton_iterations(first=True)
    print(f"Newton iterations over 6 steps x {npts} points: plain {tot_p} (first solves {first_p}), "
          f"warm {tot_w} (first solves {first_w}); first-solve ratio {first_p / first_w:.2f}, "
          f"total ratio {tot_p / tot_w:.2f}")
    assert first_p >= 2.0 * first_w
    assert tot_w < tot_p
    vp = np.hypot(plain.dr_state("slip_rate1"), plain.dr_state("slip_rate2"))
    vw = np.hypot(warm.dr_state("slip_rate1"), warm.dr_state("slip_rate2"))
    assert (np.abs(vp - vw) <= 1e-6 * vp + 1e-12).all(), np.max(np.abs(vp - vw) / (vp + 1e-30))
    assert np.abs(plain.dr_state("psi") - warm.dr_state("psi")).max() < 1e-9
    qp, qw = plain.get_dofs(), warm.get_dofs()
    assert np.abs(qp - qw).max() <= 1e-6 * np.abs(qp).max()
    plain.close()
    warm.close()


def test_warm_step_matches_oracle(built_lib, trained):
    _, _, _, p, norm = trained
    ctx, rs = _fault(5)
    ctx.mlp_set(p, norm)
    ctx.dr_warm_start(True)
    n = ctx.get_dofs().shape[0]
    q0 = seeded_dofs(n, 4, 5)
    cells = ctx.get_cells()
    faces = ctx.dr_faces()
    state = {k: ctx.dr_state(v) for k, v in FIELDS.items()}
    a = ctx.dr_state("a")
    init = np.stack([ctx.dr_state("sn0"), ctx.dr_state("tau1_0"), ctx.dr_state("tau2_0")], axis=1)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(4)
    dro = oracle_py.DROracle(4, faces, params)
    first = np.zeros((faces["cells"].shape[0], 25), np.int64)
    q_ref, _, _, iters, _ = oracle_py.dr_full_step(o, dro, q0, cells, faces, state, a, init, dt, mlp=(p, norm),
                                                   first_iters=first)
    ctx.dr_reset_counters()
    ctx.run("all_dr", dt, 1)
    ctx.sync()
    v_gpu = np.hypot(ctx.dr_state("slip_rate1"), ctx.dr_state("slip_rate2"))
    v_ref = np.hypot(state["v1"], state["v2"])
    assert (np.abs(v_gpu - v_ref) <= 1e-4 * np.abs(v_ref) + 1e-12).all()
    assert np.abs(ctx.dr_state("psi") - state["psi"]).max() < 1e-6
    q_gpu = ctx.get_dofs()
    for q in range(9):
        assert rel_l2(q_gpu[:, q] - q0[:, q], q_ref[:, q] - q0[:, q]) < 1e-4, q
    # the kernel evaluates the network and the start comparison in float32 (tanh.approx), the
    # oracle in float64: a start can flip where the two residuals are close
    tot, _, fst = ctx.dr_newton_iterations(first=True)
    assert abs(fst - first.sum()) <= 0.1 * first.sum() + 5, (fst, first.sum())
    assert abs(tot - iters.sum()) <= 0.1 * iters.sum() + 5, (tot, iters.sum())
    ctx.close()


OPT_DR_REFINE32 = 6
STATE_FIELDS = ("psi", "slip_rate1", "slip_rate2", "slip1", "slip2", "slip", "mu", "traction1", "traction2")


def _same_solution(a, b):
    va = np.hypot(a.dr_state("slip_rate1"), a.dr_state("slip_rate2"))
    vb = np.hypot(b.dr_state("slip_rate1"), b.dr_state("slip_rate2"))
    assert (np.abs(va - vb) <= 1e-6 * va + 1e-12).all(), np.max(np.abs(va - vb) / (va + 1e-30))
    assert np.abs(a.dr_state("psi") - b.dr_state("psi")).max() < 1e-9
    qa, qb = a.get_dofs(), b.get_dofs()
    assert np.abs(qa - qb).max() <= 1e-6 * np.abs(qa).max()


@pytest.mark.parametrize("warm", [False, True])
def test_float32_presolve_keeps_the_solution(built_lib, trained, warm):
    """SEI_OPT_DR_REFINE32 (with and without the network's first guess): six steps give the plain
    solve's slip rates, state and DOFs to the Newton tolerance, with fewer float64 Newton
    iterations (the measured ratio over 200 steps of the fault workload is in the benchmark)."""
    _, _, _, p, norm = trained
    plain, _ = _fault(4)
    ref, _ = _fault(4)
    ref.set_option(OPT_DR_REFINE32, 1)
    if warm:
        ref.mlp_set(p, norm)
        ref.dr_warm_start(True)
    dt = plain.cfl_timestep(0.5)
    for ctx in (plain, ref):
        ctx.dr_reset_counters()
        ctx.run("all_dr", dt, 6)
        ctx.sync()
    tot_p, npts = plain.dr_newton_iterations()
    tot_r, _ = ref.dr_newton_iterations()
    it32 = ref.dr_newton_iterations32()
    print(f"float64 Newton iterations per point and step over 6 steps x {npts} points: plain {tot_p / npts / 6:.2f}, "
          f"refined {tot_r / npts / 6:.2f} (+{it32 / npts / 6:.2f} float32); ratio {tot_p / max(tot_r, 1):.2f}")
    assert plain.dr_newton_iterations32() == 0 and it32 > 0
    assert tot_r < tot_p
    _same_solution(plain, ref)
    plain.close()
    ref.close()


def test_late_step_warm_and_plain_solves_agree(built_lib, trained):
    """One state taken after 100 plain steps; the next step solved plain and warm-started (network
    guess and float32 pre-solve) from that same state agrees point by point: the warm start
    changes where each solve begins, not what it converges to."""
    _, _, _, p, norm = trained
    ctx, _ = _fault(4)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all_dr", dt, 100)
    ctx.sync()
    q100 = ctx.get_dofs()
    s100 = {f: ctx.dr_state(f) for f in STATE_FIELDS}
    assert np.hypot(s100["slip_rate1"], s100["slip_rate2"]).max() > 1e-6  # the fault is slipping
    other, _ = _fault(4)
    other.set_dofs(q100)
    for f, v in s100.items():
        other.dr_set_state(f, v)
    other.mlp_set(p, norm)
    other.dr_warm_start(True)
    other.set_option(OPT_DR_REFINE32, 1)
    for c in (ctx, other):
        c.dr_reset_counters()
        c.run("all_dr", dt, 1)
        c.sync()
    tot_p, npts, first_p = ctx.dr_newton_iterations(first=True)
    tot_w, _, first_w = other.dr_newton_iterations(first=True)
    print(f"step 101, {npts} points: float64 Newton iterations plain {tot_p} (first solves {first_p}), "
          f"warm {tot_w} (first solves {first_w}, +{other.dr_newton_iterations32()} float32)")
    _same_solution(ctx, other)
    ctx.close()
    other.close()


def test_warm_start_needs_a_network(built_lib):
    from seissol_gb300 import SeiError
    ctx, _ = _fault(6)
    with pytest.raises(SeiError):
        ctx.dr_warm_start(True)
    with pytest.raises(SeiError):
        ctx.mlp_train(samples=np.zeros((4, 6), np.float32))
    ctx.close()
