"""Oracle of the slip-rate warm start (CPU only).

* the numpy gradient of the training loss vs central finite differences (relative 1e-5);
* the C restatement of the network's guess (used inside the oracle's friction solve) vs the
  numpy one (1e-9 in ln V, both evaluate the network in float32);
* the warm start inside the oracle's fault step: a network trained (numpy Adam) on samples the
  plain solve recorded on one seeded fault, applied to a fault drawn with another seed, needs at
  least 2x fewer Newton iterations in the solves it starts and converges to the plain solve's
  slip rates (1e-6 relative + 1e-12 m/s; the Newton tolerance is 1e-8 m/s on the residual).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp as M
from oracle import oracle_py


def _synthetic_samples(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-120e6, -40e6, n), rng.uniform(20e6, 75e6, n), rng.uniform(0.3, 0.9, n),
                     rng.uniform(0.008, 0.02, n), np.full(n, 0.014), rng.uniform(-40, 1, n)], axis=1)


def test_gradient_finite_differences():
    S = _synthetic_samples(300, 1)
    p = M.glorot(2).astype(np.float64)
    norm = M.normalisation(S, 1e-6).astype(np.float64)
    loss, g = M.loss_and_grad(p, norm, S)
    assert g.shape == (M.NUM_PARAMS,) and np.isfinite(loss)
    rng = np.random.default_rng(3)
    # one index from every parameter block plus random ones
    blocks = [0, 320, 384, 384 + 4096, 384 + 4096 + 64, M.NUM_PARAMS - 1]
    for i in list(blocks) + list(rng.choice(M.NUM_PARAMS, 30, replace=False)):
        eps = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (M.loss_and_grad(pp, norm, S)[0] - M.loss_and_grad(pm, norm, S)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(g[i]), 1e-3 * np.abs(g).max()), (i, fd, g[i])


def test_c_and_numpy_guess_agree():
    S = _synthetic_samples(200, 4)
    p = M.glorot(5)
    norm = M.normalisation(S, 1e-6)
    L = oracle_py.lib(np.float64)
    L.oracle_mlp_forward.restype = C.c_double
    L.oracle_mlp_forward.argtypes = [C.c_void_p, C.c_void_p] + [C.c_double] * 5
    ref = M.predict(p, norm, S) * M.LN10
    for k in range(len(S)):
        lnv = L.oracle_mlp_forward(p.ctypes.data, norm.ctypes.data, *S[k, :5])
        assert abs(lnv - ref[k]) < 1e-9 * max(1.0, abs(ref[k])) + 2e-5, (k, lnv, ref[k])


def _fault(seed):
    """Oracle fault step inputs on the 8 x 4 x 4 periodic cube with a planar fault (the device
    set-up draws a, sn0, tau0 on the GPU; here they are drawn with numpy from the same ranges)."""
    from seissol_gb300 import Context, RSParams
    from tests.helpers import seeded_dofs
    with Context(4, device=-1) as ctx:
        n = ctx.build_periodic_cube(8, 4, 4, perturb=0.0, seed=seed, fault_plane=4)
        cells = ctx.get_cells()
        faces = ctx.dr_faces()
        dt = ctx.cfl_timestep(0.5)
    rs = RSParams.fault_config(seed=seed + 2)
    nf, npts = faces["cells"].shape[0], 25
    rng = np.random.default_rng(seed)
    a = rng.uniform(rs.a_min, rs.a_max, (nf, npts))
    lowv = np.maximum(rs.f0 - (rs.b - a) * np.log(rs.v_init / rs.v0), 0)
    fss = rs.muw + (lowv - rs.muw) / (1 + (rs.v_init / rs.vw) ** 8) ** 0.125
    c = fss / a
    psi = a * (np.abs(c) + np.log(rs.v0 / rs.v_init * -np.sign(c) * np.expm1(-2 * np.abs(c))))
    z = np.zeros((nf, npts))
    state = dict(psi=psi, v1=np.full((nf, npts), rs.v_init), v2=z.copy(), slip1=z.copy(), slip2=z.copy(),
                 slip=z.copy(), mu=z.copy(), trac1=z.copy(), trac2=z.copy())
    init = np.stack([rng.uniform(rs.sn_min, rs.sn_max, (nf, npts)), rng.uniform(rs.tau_min, rs.tau_max, (nf, npts)),
                     z.copy()], axis=1)
    params = {k: getattr(rs, k) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                          "max_newton", "max_outer")}
    return dict(q=seeded_dofs(n, 4, seed), cells=cells, faces=faces, state=state, a=a, init=init, dt=dt,
                o=oracle_py.Oracle(4), dro=oracle_py.DROracle(4, faces, params), v0=rs.v0, nf=nf)


def _run(env, steps, mlp=None, record=None):
    total = 0
    first = np.zeros((env["nf"], 25), np.int64)
    for _ in range(steps):
        env["q"], _, _, it, _ = oracle_py.dr_full_step(env["o"], env["dro"], env["q"], env["cells"], env["faces"],
                                                      env["state"], env["a"], env["init"], env["dt"], mlp=mlp,
                                                      record=record, first_iters=first)
        total += int(it.sum())
    return total, int(first.sum())


@pytest.mark.timeout(600)
def test_oracle_warm_start_gain(built_lib):
    train = _fault(3)
    rec = (np.zeros((60000, 6), np.float32), np.zeros(1, np.int64))
    _run(train, 6, record=rec)
    S = rec[0][:int(min(rec[1][0], rec[0].shape[0]))]
    assert len(S) > 10000 and np.isfinite(S).all()
    sub = S[np.random.default_rng(0).choice(len(S), 6000, replace=False)]
    p, norm, losses = M.train_adam(sub, train["v0"], steps=400, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]
    plain, warm = _fault(4), _fault(4)
    tot_p, first_p = _run(plain, 6)
    tot_w, first_w = _run(warm, 6, mlp=(p, norm))
    assert first_p >= 2.0 * first_w, (first_p, first_w)
    assert tot_w < tot_p
    vp = np.hypot(plain["state"]["v1"], plain["state"]["v2"])
    vw = np.hypot(warm["state"]["v1"], warm["state"]["v2"])
    assert (np.abs(vp - vw) <= 1e-6 * vp + 1e-12).all(), np.max(np.abs(vp - vw) / (vp + 1e-30))
    assert np.abs(plain["state"]["psi"] - warm["state"]["psi"]).max() < 1e-9
    assert np.abs(plain["q"] - warm["q"]).max() <= 1e-9 * np.abs(plain["q"]).max()
