"""Imposed slip rates in the oracle, pinned to the reference's unit tests (CPU only).

* regularised Yoffe closed form vs the convolution of the Yoffe function with a triangle
  (tests/Numerical/RegularizedYoffe.t.h restated: Tinti et al. 2005 eqs 1-3; the integral by the
  midpoint rule after x = s^2, which removes the onset singularity), at the test's rise and
  acceleration times, 1e-6 absolute (the reference test allows 1e-2; the gap is below 1e-8);
* the Gaussian source time function: slip rate = direction x (step(t) - step(t - dt)) / dt with the
  step of tests/Numerical/GaussianNucleation.t.h, 1e-12 relative;
* the delta pulse puts the whole unit slip into the sub-step after the onset; the Yoffe and
  Gaussian slips integrate to one over their duration (2 % and 1e-9).
One order-4 face with no wave field.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle_py

NPTS = 25
RHO, VP, VS = 2700.0, 6000.0, 3464.0


def _yoffe(t, rise):
    eps = 10 * np.finfo(float).eps
    out = np.zeros_like(t)
    m = (t >= eps) & (t <= rise - eps)
    out[m] = 2 / (math.pi * rise) * np.sqrt((rise - t[m]) / t[m])
    return out


def _triangle(t, half):
    out = np.zeros_like(t)
    a = (t > 0) & (t < half)
    b = (t > half) & (t < 2 * half)
    out[a] = t[a] / half ** 2
    out[b] = (2 * half - t[b]) / half ** 2
    return out


def _convolved(time, tS, tR, n=200000):
    """The test's convolution integral over the Yoffe support [0, tR], with x = s^2 so that the
    1 / sqrt(x) singularity at the onset becomes a smooth integrand (2 s yoffe(s^2) is finite)."""
    if time < -2 * tS or time > tR + 2 * tS:
        return 0.0
    s = (np.arange(n) + 0.5) * (math.sqrt(tR) / n)  # midpoints
    x = s * s
    f = 2 / (math.pi * tR) * np.sqrt(np.maximum(tR - x, 0.0)) * 2.0 * _triangle(time - x, tS)
    return float(f.sum() * math.sqrt(tR) / n)


def test_regularized_yoffe_matches_convolution():
    L = oracle_py.lib()
    L.oracle_regularized_yoffe.restype = C.c_double
    L.oracle_regularized_yoffe.argtypes = [C.c_double] * 3
    for acc in (0.2, 0.3):
        for rise in (0.9, 1.1):
            tS = acc / 1.27
            tR = rise - 2 * tS
            for i in range(-10, 111):
                t = i * 0.01
                assert abs(L.oracle_regularized_yoffe(t, tS, tR) - _convolved(t, tS, tR)) < 1e-6, (t, tS, tR)


def _run(law, steps, dt=1e-3, **kw):
    zp, zs = RHO * VP, RHO * VS
    dro = oracle_py.DROracle(4, {"imp": np.array([[zp, zs, zp, zs, zp / 2, zs / 2, 2 / zs, 0.0]])}, {})
    tp, tw, deltat, _ = oracle_py.dr_collocation(4, dt)
    qi = np.zeros((1, len(tp), 9, NPTS))
    state = {k: np.zeros((1, NPTS)) for k in oracle_py.STATE_FIELDS}
    init = np.zeros((1, 3, NPTS))
    full = lambda v: np.full((1, NPTS), float(v))
    aux = dict(time=0.0, law=law, peak=full(0), trup=full(-1), dir1=full(kw.get("d1", 0.8)), dir2=full(kw.get("d2", 0.6)),
               onset=full(kw.get("onset", 2.5e-3)), taus=full(kw.get("tS", 4e-3)), taur=full(kw.get("tR", 1e-2)))
    rates = []
    for _ in range(steps):
        dro.friction_isr(qi, qi, state, init, deltat, tw, aux)
        rates.append(np.hypot(state["v1"], state["v2"])[0, 0])
        aux["time"] += dt
    return state, aux, deltat, rates


def test_gaussian_rate_is_the_step_increment():
    t0, onset, dt = 4e-3, 2.5e-3, 1e-3

    def step(t):
        if t < 0:
            return 0.0
        if t > t0:
            return 1.0
        return math.exp((t - t0) ** 2 / (t * (t - 2 * t0)))

    state, aux, deltat, rates = _run(8, 5, dt=dt, tS=t0, onset=onset)
    t_end = 5 * dt  # the last time point of the last step ends there
    want = (step(t_end - onset) - step(t_end - onset - deltat[-1])) / deltat[-1]
    assert abs(rates[-1] - want) <= 1e-12 * max(want, 1e-300)
    state, aux, _, _ = _run(8, 12, dt=dt, tS=t0, onset=onset)
    assert abs(math.hypot(state["slip1"][0, 0], state["slip2"][0, 0]) - 1.0) < 1e-9
    assert abs(state["slip"][0, 0] - 1.0) < 1e-9


def test_delta_pulse_slip():
    state, aux, _, _ = _run(9, 4, onset=1.5e-3)
    assert np.allclose(state["slip1"], 0.8, rtol=1e-12) and np.allclose(state["slip2"], 0.6, rtol=1e-12)
    assert aux["trup"][0, 0] >= 1e-3 and aux["peak"][0, 0] > 0


def test_yoffe_slip_integrates_to_one():
    state, _, _, _ = _run(7, 40, dt=1e-3, tS=3e-3, tR=2e-2, onset=1e-3)
    assert abs(state["slip"][0, 0] - 1.0) < 2e-2
