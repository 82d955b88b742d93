"""Linear-slip-weakening oracle against closed forms (CPU only).

The reference holds no unit test of its slip-weakening laws (tests/DynamicRupture covers the
shared precompute / postcompute, pinned in test_dr_oracle.py), so the restatement of
src/DynamicRupture/FrictionLaws/CpuImpl/LinearSlipWeakening.h is checked here on cases whose
answer follows from the law by hand: one order-4 face (25 points, 4 time points) with no wave
field (QInterpolated = 0), so that the fault stresses are the initial ones.

* locked fault: shear below the static strength -> no slip, mu stays mu_s, zero imposed state;
* forced rupture as a step (t0 = 0): mu drops to mu_d after the first time point, the later
  ones slip at (tau0 - mu_d |sn0|) / eta_s, tractions -eta_s V, the rupture time is the start
  of the second time point, the dynamic-stress time the start of the point where the
  accumulated slip reaches d_c;
* forced-rupture ramp (t0 > 0): mu = mu_s - (mu_s - mu_d) (t_end / t0);
* TP proxy state 1 - (1 + |slip| / d_c)^-p; bimaterial regularised strength relaxing towards the
  strength with exp(-v_star dt / L); healing back to mu_s;
* Gaussian nucleation: the increments over a window telescope to smoothStep(t_end - s0).
Tolerance: 1e-12 relative.
"""
import math

import numpy as np
import pytest

from oracle import oracle_py

ORDER = 4
NPTS = 25
RHO, VP, VS = 2700.0, 6000.0, 3464.0


def _faces(nf=1):
    zp, zs = RHO * VP, RHO * VS
    imp = np.tile(np.array([zp, zs, zp, zs, zp / 2, zs / 2, 2 / zs, 0.0]), (nf, 1))
    return {"imp": imp}


def _run(law, sn0, tau0, dt=1e-3, time=0.0, steps=1, **kw):
    """Runs `steps` fault steps of one face with no wave field; returns state, init, aux, deltat."""
    nf = 1
    dro = oracle_py.DROracle(ORDER, _faces(nf), dict(f0=0, b=0, v0=1, l=1, muw=0, vw=1, newton_tol=1, state_tol=1,
                                                     max_newton=1, max_outer=1))
    tp, tw, deltat, coll = oracle_py.dr_collocation(ORDER, dt)
    nts = len(tp)
    qi = np.zeros((nf, nts, 9, NPTS))
    state = {k: np.zeros((nf, NPTS)) for k in oracle_py.STATE_FIELDS}
    state["mu"][:] = kw.get("mu_s", 0.677)
    if "slip" in kw:
        state["slip"][:] = kw["slip"]
    init = np.zeros((nf, 3, NPTS))
    init[:, 0], init[:, 1] = sn0, tau0
    full = lambda v: np.full((nf, NPTS), float(v))
    aux = dict(time=time, t0=kw.get("t0", 0.0), s0=kw.get("s0", 0.0), nucleate=int("nuc" in kw),
               nuc=kw.get("nuc"), peak=full(kw.get("peak", 0.0)), trup=full(-1), tdyn=full(-1), law=law,
               healing=kw.get("healing", -1.0), v_star=kw.get("v_star", 0.1), prakash_length=kw.get("L", 1.0),
               tp_exponent=kw.get("p", 1.0 / 3.0), mu_s=full(kw.get("mu_s", 0.677)), mu_d=full(kw.get("mu_d", 0.525)),
               d_c=full(kw.get("d_c", 0.4)), cohesion=full(kw.get("cohesion", 0.0)),
               t_forced=full(kw.get("t_forced", 1e300)), reg=full(kw.get("reg", 0.0)))
    isp = ism = None
    for _ in range(steps):
        isp, ism = dro.friction_lsw(qi, qi, state, init, deltat, tw, aux)
        aux["time"] += dt
    return state, init, aux, deltat, (isp, ism)


def close(a, b, rtol=1e-12):
    return np.allclose(a, b, rtol=rtol, atol=0.0)


@pytest.mark.parametrize("law", [1, 2, 3])
def test_locked_fault(law):
    sn, tau = -120e6, 70e6  # static strength 81.24 MPa
    state, init, aux, _, (isp, ism) = _run(law, sn, tau, reg=0.677 * 120e6)
    for k in ("v1", "v2", "slip1", "slip2", "slip", "trac1", "trac2"):
        assert np.abs(state[k]).max() == 0.0, k
    assert (state["mu"] == 0.677).all()
    assert (aux["trup"] == -1).all() and (aux["peak"] == 0).all()
    assert np.abs(isp).max() == 0.0 and np.abs(ism).max() == 0.0


def test_forced_rupture_step():
    sn, tau, mud, dt = -120e6, 70e6, 0.525, 1e-3
    etas = RHO * VS / 2
    dc = 5e-4
    state, init, aux, deltat, (isp, _) = _run(1, sn, tau, dt=dt, t_forced=0.0, d_c=dc)
    v = (tau - mud * 120e6) / etas
    assert close(state["v1"], v) and np.abs(state["v2"]).max() == 0.0
    assert close(state["trac1"], -etas * v)
    assert close(state["mu"], mud)
    # slip from time points 1.. (the first one still sees mu_s); the resample matrix keeps a constant
    assert close(state["slip1"], v * deltat[1:].sum())
    assert close(state["slip"], v * deltat[1:].sum(), rtol=1e-10)
    starts = np.concatenate([[0.0], np.cumsum(deltat)[:-1]])
    assert close(aux["trup"], starts[1]) and close(aux["peak"], v)
    reach = np.nonzero(v * np.cumsum(np.concatenate([[0.0], deltat[1:]])) >= dc)[0]
    assert reach.size and close(aux["tdyn"], starts[reach[0]], rtol=1e-12)
    # imposed traction: time-weighted tractions of the slipping points
    tp, tw, _, _ = oracle_py.dr_collocation(ORDER, dt)
    assert close(isp[0, 3], -etas * v * tw[1:].sum(), rtol=1e-10)


def test_forced_rupture_ramp():
    """d_c so large that the slip term stays below the ramp; shear below the dynamic strength."""
    sn, tau, dt, t0 = -120e6, 20e6, 1e-3, 4e-3
    state, _, aux, deltat, _ = _run(1, sn, tau, dt=dt, t_forced=0.0, t0=t0, d_c=1e9, steps=2)
    t_end = 2 * dt
    assert close(state["mu"], 0.677 - (0.677 - 0.525) * t_end / t0)
    assert np.abs(state["v1"]).max() == 0.0


def test_tp_proxy_state():
    sn, tau, s, dc, p = -120e6, 10e6, 0.3, 0.4, 1.0 / 3.0
    state, *_ = _run(3, sn, tau, slip=s, d_c=dc, p=p)
    assert close(state["slip"], s)
    assert close(state["mu"], 0.677 - (0.677 - 0.525) * (1 - (1 + s / dc) ** -p))


def test_linear_state_from_slip():
    sn, tau, s, dc = -120e6, 10e6, 0.1, 0.4
    state, *_ = _run(1, sn, tau, slip=s, d_c=dc)
    assert close(state["mu"], 0.677 - (0.677 - 0.525) * s / dc)


def test_bimaterial_regularised_strength():
    sn, tau, vstar, L, dt = -120e6, 10e6, 0.2, 0.5, 1e-3
    r0 = 50e6
    state, _, aux, deltat, _ = _run(2, sn, tau, dt=dt, reg=r0, v_star=vstar, L=L)
    target = 0.677 * 120e6
    r = r0
    for d in deltat:
        e = -vstar * d / L
        r = r * math.exp(e) + target * -math.expm1(e)
    assert close(aux["reg"], r)
    # the regularised strength stays above the shear: locked
    assert np.abs(state["v1"]).max() == 0.0


@pytest.mark.parametrize("healing,expect", [(0.1, 0.677), (-1.0, 0.525)])
def test_healing(healing, expect):
    """Forced rupture (state 1) on a locked point whose peak slip rate passed the threshold."""
    state, *_ = _run(1, -120e6, 10e6, t_forced=0.0, peak=1.0, healing=healing)
    assert close(state["mu"], expect)


def test_nucleation_telescopes():
    sn, tau, dt, t0, n = -120e6, 10e6, 1e-3, 5e-3, 3e6
    nuc = np.zeros((1, 3, NPTS))
    nuc[:, 1] = n
    nuc[:, 0] = -n
    _, init, *_ = _run(1, sn, tau, dt=dt, t0=t0, s0=0.0, nuc=nuc, steps=3)

    def smooth(t):
        if t <= 0:
            return 0.0
        if t < t0:
            return math.exp((t - t0) ** 2 / (t * (t - 2 * t0)))
        return 1.0

    g = smooth(3 * dt)
    assert close(init[:, 1], tau + n * g) and close(init[:, 0], sn - n * g)
    assert 0 < g < 1
