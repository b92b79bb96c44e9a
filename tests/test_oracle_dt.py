"""The oracle's dt under DT_CORRECTION_DYNAMIC (UpdateAcceleration.cpp:15-29,
104-121): the OpenMP build compiles the maxima out, so dt = CFL*h/c; with
dt_dynamic_reduce the maxima of |a_j| and arvmu_j over the step give
dt = CFL*min(sqrt(h/amax), h/(c + mumax))."""

import ctypes

import numpy as np
import pytest

from sph2d_gb300 import capi


def _case():
    from sph2d_gb300 import cases

    case = cases.dam_break_2d(nx=30, ny=15)
    p = case.params()
    p.dt_correction_method = 2
    p.CFL_coef = 0.2
    return case, p


def test_dynamic_dt_of_the_openmp_build():
    from oracle import binding as O

    case, p = _case()
    c = float(np.sqrt(O.lib().orc_eos_c_sqr(ctypes.byref(p))))
    run = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=4)
    assert run["time"] == pytest.approx(4 * 0.2 * p.hsml / c, rel=1e-14)


def test_dynamic_dt_with_the_true_maxima():
    from oracle import binding as O

    case, p = _case()
    p.dt_dynamic_reduce = 1
    c = float(np.sqrt(O.lib().orc_eos_c_sqr(ctypes.byref(p))))
    run = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=1)
    # the first step's forces see r0, v_predict = v0 (a = 0) and the summation density of r0
    rho, pres = O.density(p, case.r, case.v, case.rho, case.itype)
    a, _, mu = O.forces(p, capi.TERM_ALL, case.r, case.v, rho, pres, case.itype)
    assert np.array_equal(a, run["a"])
    amax = float(np.sqrt((a * a).sum(axis=1)).max())
    dt = 0.2 * min(np.sqrt(p.hsml / amax), p.hsml / (c + float(mu.max())))
    assert run["time"] == pytest.approx(dt, rel=1e-14)
    assert dt < 0.2 * p.hsml / c
