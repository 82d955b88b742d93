"""Thermal pressurisation in the oracle (CPU only): the spectral update of
CpuImpl/ThermalPressurization/ThermalPressurization.cpp:27-107 against analytic limits.

* no slip: temperature and pressure stay at their initial values;
* a short heating step (every mode's diffusion factor below 1e-4): the inverse transform of the
  Gaussian heat source gives the shear-zone centre's temperature rise tau V dt / (rho c sqrt(2 pi) w)
  (the 60-mode log grid integrates it to 1e-3), and the pressure falls by Lambda times that rise
  (undrained limit), 1e-6 relative to the rise;
* after the heating stops, diffusion lowers the centre's temperature monotonically.
"""
import ctypes as C
import math

import numpy as np

from oracle import oracle_py


def _aux(hw=0.02, hyd=1e-4):
    nm = 60
    a = dict(tp=1, tp_alpha=1e-6, tp_rhoc=2.7e6, tp_lambda=0.1e6, tp_t0=483.15, tp_p0=-80e6,
             tp_hw=np.full((1, 1), hw), tp_hyd=np.full((1, 1), hyd), tp_theta=np.zeros((1, nm, 1)),
             tp_sigma=np.zeros((1, nm, 1)), tp_temp=np.zeros((1, 1)), tp_pres=np.zeros((1, 1)))
    return a, oracle_py._aux_struct(a)


def _step(ax, sn, mu, v, dt, save=1):
    L = oracle_py.lib()
    L.oracle_dr_tp_point.restype = C.c_double
    L.oracle_dr_tp_point.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_int]
    return L.oracle_dr_tp_point(C.addressof(ax), 0, 1, 0, sn, mu, v, dt, save)


def test_no_slip_keeps_initial_state():
    a, ax = _aux()
    p = _step(ax, -100e6, 0.6, 0.0, 1e-3)
    assert p == -80e6 and a["tp_temp"][0, 0] == 483.15


def test_short_heating_limit():
    a, ax = _aux()
    sn, mu, v, dt, hw = -100e6, 0.6, 1.0, 1e-7, 0.02
    p = _step(ax, sn, mu, v, dt)
    rise = a["tp_temp"][0, 0] - 483.15
    want = (-mu * sn * v) * dt / (2.7e6 * math.sqrt(2 * math.pi) * hw)
    assert abs(rise - want) < 1e-3 * want, (rise, want)
    assert abs((-80e6 - p) - 0.1e6 * rise) < 1e-6 * 0.1e6 * rise


def test_diffusion_cools_the_centre():
    a, ax = _aux()
    _step(ax, -100e6, 0.6, 1.0, 1e-2)
    temps = [a["tp_temp"][0, 0]]
    for _ in range(5):
        _step(ax, -100e6, 0.6, 0.0, 1.0)
        temps.append(a["tp_temp"][0, 0])
    assert all(t1 < t0 for t0, t1 in zip(temps, temps[1:])) and temps[-1] > 483.15
