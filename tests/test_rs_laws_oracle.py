"""The oracle's aging, slip and severe-velocity-weakening laws (CPU only).

No reference unit test covers these laws; the restatement of CpuImpl/AgingLaw.h, SlipLaw.h,
SevereVelocityWeakeningLaw.h and the generic Newton of RateAndState.h:327-385 is checked for
(a) steady sliding: a face at rest in the state of steady sliding at V_init, with the shear
traction equal to the steady friction, keeps V and theta (1e-9 relative), and (b) on an overstressed
face the final friction coefficient and slip rate satisfy V = (tau - |sn| mu(V)) / eta_s to
1e-8 (1 + V) and mu is the law's at the final state.  One order-4 face, no wave field.
"""
import math

import numpy as np
import pytest

from oracle import oracle_py

NPTS = 25
RHO, VP, VS = 2700.0, 6000.0, 3464.0
P = dict(f0=0.6, b=0.014, v0=1e-6, l=0.02, muw=0.1, vw=0.1, newton_tol=1e-8, state_tol=1e-8, max_newton=60,
         max_outer=10)


def _faces():
    zp, zs = RHO * VP, RHO * VS
    return {"imp": np.array([[zp, zs, zp, zs, zp / 2, zs / 2, 2 / zs, 0.0]])}


def _mu(law, a, theta, v):
    if law == 6:
        return P["f0"] + a * v / (v + P["v0"]) - P["b"] * theta / (theta + P["l"])
    psi = P["f0"] + P["b"] * math.log(P["v0"] * theta / P["l"])
    return a * math.asinh(v / (2 * P["v0"]) * math.exp(psi / a))


def _run(law, v_init, tau_of, a=0.01, sn=-50e6):
    dro = oracle_py.DROracle(4, _faces(), P)
    tp, tw, deltat, _ = oracle_py.dr_collocation(4, 1e-3)
    qi = np.zeros((1, len(tp), 9, NPTS))
    theta = P["l"] / v_init if law in (4, 5) else v_init * P["l"] / P["v0"]
    state = {k: np.zeros((1, NPTS)) for k in oracle_py.STATE_FIELDS}
    state["psi"][:] = theta
    state["v1"][:] = v_init
    init = np.zeros((1, 3, NPTS))
    init[:, 0] = sn
    init[:, 1] = tau_of(law, a, theta, v_init, sn)
    aa = np.full((1, NPTS), a)
    dro.friction(qi, qi, state, aa, init, deltat, tw, aux={"law": law})
    return state, init, theta


@pytest.mark.parametrize("law", [4, 5, 6])
def test_steady_sliding_is_kept(law):
    v = 1e-9
    state, _, theta = _run(law, v, lambda law, a, th, v, sn: abs(sn) * _mu(law, a, th, v) + RHO * VS / 2 * v)
    assert np.allclose(np.hypot(state["v1"], state["v2"]), v, rtol=1e-9)
    assert np.allclose(state["psi"], theta, rtol=1e-9)


@pytest.mark.parametrize("law", [4, 5, 6])
def test_converged_rate_satisfies_the_law(law):
    sn = -50e6
    state, init, _ = _run(law, 1e-12, lambda law, a, th, v, s: 0.8 * abs(s), sn=sn)
    v = np.hypot(state["v1"], state["v2"])[0]
    etas = RHO * VS / 2
    g = (init[0, 1] - abs(sn) * state["mu"][0]) / etas - v
    assert (v > 1e-7).all()  # the overstressed face accelerates
    assert np.abs(g).max() < 1e-8 * (1 + v.max())
    th = state["psi"][0]
    mu = np.array([_mu(law, 0.01, t, x) for t, x in zip(th, v)])
    assert np.allclose(mu, state["mu"][0], rtol=1e-9)
