"""Ensembles of tanks packed into one solver (rrsph_set_wave_makers) and the
gather autotuner (rrsph_autotune / rrsph_set_gather_threads)."""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tanks():
    from sph2d_gb300 import cases

    return cases.ensemble_tanks(ntanks=5, seed=9, n_lo=400, n_hi=3000, steps=40)


def _run_tank(c, precision, steps):
    from sph2d_gb300 import Solver

    p = c.params()
    with Solver(p, precision) as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        s.set_wave_makers([c.notes["wave_maker"]])
        s.step(steps, 0.0)
        return s.download(), s.pair_count()[0]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_packed_ensemble_equals_the_tanks_run_one_by_one(gpu_available, tanks, precision, tol):
    from sph2d_gb300 import Solver, cases

    ens = cases.pack_tanks(tanks)
    p = ens.params()
    steps = 30
    with Solver(p, precision) as s:
        s.upload(ens.r, ens.v, ens.rho, ens.itype)
        s.set_wave_makers(ens.notes["wave_makers"])
        s.step(steps, 0.0)
        st = s.download()
        pairs = s.pair_count()[0]
    tank_pairs = 0
    for c, (a, b), (ox, oy) in zip(tanks, ens.notes["ranges"], ens.notes["offsets"]):
        ref, pc = _run_tank(c, precision, steps)
        tank_pairs += pc
        assert rel_l2(st["r"][a:b] - np.array([ox, oy]), ref["r"]) < tol
        assert rel_l2(st["v"][a:b], ref["v"]) < tol * 10
        assert rel_l2(st["rho"][a:b], ref["rho"]) < tol
        assert np.array_equal(st["itype"][a:b], ref["itype"])
    assert pairs == tank_pairs
    # the pistons moved
    for c, (a, b) in zip(tanks, ens.notes["ranges"]):
        m = c.notes["wave_maker"]
        i = a + m["particles_start"]
        assert st["v"][i, 0] != 0.0


def test_a_one_piston_table_is_the_params_piston(gpu_available):
    """The flume's own piston (params nwm = 2, depth 0.5) and the same piston
    given as a one-entry wave-maker table move the particles identically."""
    import math

    from sph2d_gb300 import Solver, cases

    c = cases.piston_flume_2d(nx=200, ny=100)
    p = c.params()
    out = []
    for table in (False, True):
        with Solver(p, "fp64") as s:
            s.upload(c.r, c.v, c.rho, c.itype)
            if table:
                s.set_wave_makers([{"particles_start": p.nwm_particles_start, "particles_end": p.nwm_particles_end,
                                    "nwm": 2, "time_start": p.nwm_time_start, "phase": p.nwm_phase,
                                    "wave_length": p.nwm_wave_length, "wave_magnitude": p.nwm_wave_magnitude,
                                    "depth": p.depth}])
            s.step(20, 0.0)
            out.append(s.download())
    for k in ("r", "v", "rho", "p"):
        assert np.array_equal(out[0][k], out[1][k]), k
    assert math.isfinite(out[0]["v"][p.nwm_particles_start, 0]) and out[0]["v"][p.nwm_particles_start, 0] != 0


def test_wave_maker_ranges_are_checked(gpu_available, tanks):
    from sph2d_gb300 import RrsphError, Solver, capi

    c = tanks[0]
    m = c.notes["wave_maker"]
    with Solver(c.params(), "fp64") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        with pytest.raises(RrsphError) as e:
            s.set_wave_makers([m, m])
        assert e.value.code == capi.ERR_INVALID_ARGUMENT
        with pytest.raises(RrsphError):
            s.set_gather_threads(100, 128)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_the_state_and_the_results(gpu_available, precision):
    from sph2d_gb300 import Solver, cases

    c = cases.dam_break_2d(nx=60, ny=30)
    p = c.params()
    with Solver(p, precision) as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        s.step(3, 0.0)
        before = s.download()
        choice = s.autotune(steps=3)
        assert all(x in (64, 128, 256) for x in choice)
        after = s.download()
        for k in ("r", "v", "rho", "p", "itype"):
            assert np.array_equal(before[k], after[k]), k
        s.step(10, 0.0)
        tuned = s.download()
    with Solver(p, precision) as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        s.step(3, 0.0)
        s.step(10, 0.0)
        plain = s.download()
    for k in ("r", "v", "rho"):
        if precision == "fp64":
            assert np.array_equal(tuned[k], plain[k]), k
        else:
            assert rel_l2(tuned[k], plain[k]) < 1e-6, k


def test_autotune_skin_keeps_the_state(gpu_available):
    """rrsph_autotune_skin times skins of 0.2-0.8 h on the uploaded state, puts
    the state back and keeps the fastest; the steps after it equal a run with
    that skin set directly (the pair counts exactly, the state to float
    rounding)."""
    from sph2d_gb300 import RrsphError, Solver, capi, cases

    c = cases.dam_break_2d(nx=60, ny=30)
    p = c.params()
    with Solver(p, "mixed") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        t = s.step(3, 0.0)
        before = s.download()
        skin = s.autotune_skin(steps=12)
        assert skin in (0.2, 0.3, 0.4, 0.5, 0.6, 0.8)
        after = s.download()
        for k in ("r", "v", "rho", "p", "itype"):
            assert np.array_equal(before[k], after[k]), k
        tuned_pairs = []
        for _ in range(8):
            t = s.step(1, t)
            tuned_pairs.append(s.pair_count()[0])
        tuned = s.download()
    with Solver(p, "mixed") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        t = s.step(3, 0.0)
        s.set_neighbour_reuse(True, skin)
        plain_pairs = []
        for _ in range(8):
            t = s.step(1, t)
            plain_pairs.append(s.pair_count()[0])
        plain = s.download()
    assert tuned_pairs == plain_pairs
    for k in ("r", "v", "rho"):
        assert rel_l2(tuned[k], plain[k]) < 1e-6, k
    with Solver(p, "fp64") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        with pytest.raises(RrsphError) as e:
            s.autotune_skin(steps=2)
        assert e.value.code == capi.ERR_UNSUPPORTED
