"""The C oracle against the reference's own compute core on the same inputs.

oracle/_ref/rrsph_ref is the reference's RRSPH_OMP code compiled from its
sources (oracle/build_ref.sh). Integer outputs must be identical; the oracle
restates the double arithmetic operation by operation, so floating outputs
are compared bit for bit as well, with a 1e-12 relative fallback noted where a
libm call may differ between builds. Skipped where the reference core is absent.
"""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.skipif(
    not __import__("oracle.binding", fromlist=["ref_available"]).ref_available(),
    reason="reference core not built (reference sources absent)",
)


def _small_cases():
    from sph2d_gb300 import cases

    out = []
    c = cases.dam_break_2d(nx=60, ny=30, density_treatment=1)
    out.append(("dam_break_con", c))
    c = cases.dam_break_2d(nx=60, ny=30, density_treatment=0)
    out.append(("dam_break_sum", c))
    c = cases.piston_flume_2d(nx=300, ny=40, density_treatment=0)
    out.append(("flume_sum", c))
    return out


CASES = _small_cases()


@pytest.mark.parametrize("name,case", CASES, ids=[n for n, _ in CASES])
def test_grid_identical(name, case):
    from oracle import binding as O

    p = case.params()
    counts, lst, keys, grid, cs = O.neighbours(p, case.r, case.itype)
    ref = O.ref_run(p, "grid", case.r, case.v, case.rho, case.itype)
    assert np.array_equal(ref["keys"], keys)
    assert np.array_equal(ref["grid"], grid)
    assert np.array_equal(ref["cells_start"], cs)
    assert np.array_equal(ref["counts"], counts)
    flat = np.concatenate([lst[j, :counts[j]] for j in range(len(counts))])
    assert np.array_equal(ref["list"], flat)


@pytest.mark.parametrize("name,case", CASES, ids=[n for n, _ in CASES])
def test_density_identical(name, case):
    from oracle import binding as O

    p = case.params()
    out, pres = O.density(p, case.r, case.v, case.rho, case.itype)
    ref = O.ref_run(p, "density", case.r, case.v, case.rho, case.itype)
    assert np.array_equal(ref["density"], out)
    assert np.array_equal(ref["pout"], pres)


SWITCHES = [
    dict(),
    dict(intf_sph_approximation=1),
    dict(artificial_pressure=1),
    dict(average_velocity=1, average_velocity_coef=0.05),
    dict(boundary_treatment=0),
    dict(artificial_bulk_visc=0.2),
    dict(density_treatment=2, density_delta_sph_coef=0.1),
]


@pytest.mark.parametrize("sw", SWITCHES, ids=[",".join(f"{k}={v}" for k, v in s.items()) or "base" for s in SWITCHES])
def test_force_terms_identical(sw):
    from oracle import binding as O
    from sph2d_gb300 import capi, cases

    case = cases.dam_break_2d(nx=60, ny=30, seed=11)
    p = case.params()
    for k, v in sw.items():
        setattr(p, k, v)
    p.dt_correction_method = 2  # the reference tracks max |mu| only under dynamic dt
    rng = np.random.default_rng(5)
    v = rng.normal(0, 0.3, size=case.r.shape)
    pres = O.eos_p(p, case.rho) - 200.0  # some negative pressures for the artificial pressure
    a, av, mu = O.forces(p, capi.TERM_ALL, case.r, v, case.rho, pres, case.itype)
    ref = O.ref_run(p, f"terms:{capi.TERM_ALL}", case.r, v, case.rho, case.itype, pres=pres)
    assert np.array_equal(ref["a"], a)
    assert np.array_equal(ref["mu"], mu)
    if p.average_velocity:
        assert np.array_equal(ref["av"], av)


@pytest.mark.parametrize("name,case", CASES, ids=[n for n, _ in CASES])
def test_time_loop_matches(name, case):
    """20 steps of the loop body (piston enabled for the flume)."""
    from oracle import binding as O

    p = case.params()
    n = 20
    mine = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=n)
    ref = O.ref_run(p, f"run:{n}", case.r, case.v, case.rho, case.itype)
    for k, rk in (("r", "r_out"), ("v", "v_out"), ("rho", "rho_out"), ("p", "p_out"), ("a", "a_out")):
        e = rel_l2(mine[k], ref[rk])
        assert e <= 1e-12, (k, e)
    assert np.array_equal(mine["itype"], ref["itype_out"])
    assert mine["time"] == pytest.approx(ref["timing"]["time"], rel=1e-12)


@pytest.mark.parametrize("nwm, extra", [(3, {}), (4, {"nwm_time_start": 0.0005}), (5, {"nwm_wave_magnitude": 0.05})],
                         ids=["piston_2nd_order", "wall_disappear", "solitary_rayleigh"])
def test_wave_makers_match(nwm, extra):
    """25 steps of the loop with the second-order piston (the OMP sum of
    WaveMaker.cpp:70), the disappearing wall (WaveMaker.cpp:136-157, which
    turns itself off after its call) and the solitary-wave piston
    (WaveMaker.cpp:84-134), against the reference's own make_waves."""
    from oracle import binding as O
    from sph2d_gb300 import cases

    case = cases.piston_flume_2d(nx=150, ny=20)
    p = case.params()
    p.nwm = nwm
    for k, v in extra.items():
        setattr(p, k, v)
    n = 25
    mine = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=n)
    ref = O.ref_run(p, f"run:{n}", case.r, case.v, case.rho, case.itype)
    for k, rk in (("r", "r_out"), ("v", "v_out"), ("rho", "rho_out"), ("p", "p_out"), ("a", "a_out")):
        e = rel_l2(mine[k], ref[rk])
        assert e <= 1e-12, (k, e)
    assert np.array_equal(mine["itype"], ref["itype_out"])
    if nwm == 4:
        assert np.all(mine["itype"][p.nwm_particles_start:p.nwm_particles_end] == 0)
    else:  # the piston column moved
        assert not np.array_equal(mine["r"][p.nwm_particles_start:p.nwm_particles_end],
                                  case.r[p.nwm_particles_start:p.nwm_particles_end])
