"""The oracle against the reference's golden per-particle CSVs.

Reproduces the reference's computing tests (sources/RRSPH_COMMON/tests/
test*OMP.cpp) on its own case (tests/caseDamBreak: 23,030 particles, loaded
through this library's JSON and CSV readers and derivations) and compares with
caseDamBreak/test/OMP/*.csv. The golden files are printed with 6 or 8 decimals,
so the tolerance is the print rounding plus 1e-9 relative; the reference's own
tests use checkDouble<2> (1e-2). Skipped where the reference is absent.
"""

import csv

import numpy as np
import pytest

from conftest import GOLDEN_CASE, needs_reference

pytestmark = needs_reference


def _golden(name):
    with open(GOLDEN_CASE / "test" / "OMP" / name) as f:
        rows = list(csv.DictReader(f))
    idx = np.array([int(r["particle"]) for r in rows])
    cols = {k: np.array([float(r[k]) for r in rows]) for k in rows[0] if k != "particle"}
    return idx, cols


def _close(got, want, decimals, extra=0.0):
    tol = 0.51 * 10.0 ** (-decimals) + 1e-9 * np.abs(want) + extra
    bad = np.abs(got - want) > tol
    return int(bad.sum()), float(np.max(np.abs(got - want) - tol))


def _p_slack(p):
    """Pressure tolerance from a 2e-11 relative density difference: the golden
    generator's own double arithmetic differs from the reference code compiled
    here at that level, and the EOS slope 7B/rho0 amplifies it."""
    c2 = 200 * p.g * p.depth * p.eos_sound_vel_coef if p.eos_sound_vel_method == 0 else p.eos_sound_vel
    B = c2 * p.rho0 / 7.0
    return 7.0 * B / p.rho0 * 2e-11 * p.rho0


@pytest.fixture(scope="module")
def case():
    from sph2d_gb300 import derive, load_params, read_layer

    p0 = load_params(GOLDEN_CASE)
    r, v, rho, pres, itype = read_layer(GOLDEN_CASE / "dump" / "0.00.csv", p0)
    p = derive(p0, r)
    return p, r, v, rho, itype


def test_case_loading(case):
    p, r, v, rho, itype = case
    assert p.ntotal == 23030 and p.nfluid == 20000
    assert p.hsml == pytest.approx(0.02, rel=1e-7)
    assert p.max_cells > 0 and p.maxn == 32768
    assert p.eos_sound_vel == pytest.approx(np.sqrt(200 * 9.81 * 2.0 * 2.0))


@pytest.mark.parametrize("treatment,name,col", [(0, "sum_density_target.csv", "rho"),
                                                (1, "con_density_target.csv", "drho")])
def test_density(case, treatment, name, col):
    from oracle import binding as O

    p, r, v, rho, itype = case
    q = p.copy()
    q.density_treatment = treatment
    out, pres = O.density(q, r, v, rho, itype)
    idx, g = _golden(name)
    assert _close(out[idx], g[col], 8)[0] == 0
    assert _close(pres[idx], g["p"], 8, _p_slack(q))[0] == 0


@pytest.mark.parametrize("form,artp,name", [(1, 0, "intf1_no_artp_target.csv"), (2, 0, "intf2_no_artp_target.csv"),
                                            (1, 1, "intf1_artp_target.csv"), (2, 1, "intf2_artp_target.csv")])
def test_internal_force(case, form, artp, name):
    """testInternalForceOMP.cpp:46-98: p from density_con (= EOS of rho), then
    the sum of find_internal_changes_part."""
    from oracle import binding as O
    from sph2d_gb300 import capi

    p, r, v, rho, itype = case
    q = p.copy()
    q.intf_sph_approximation = form
    q.artificial_pressure = artp
    q.density_treatment = 1
    _, pres = O.density(q, r, v, rho, itype)
    a, _, _ = O.forces(q, capi.TERM_INTERNAL, r, v, rho, pres, itype)
    idx, g = _golden(name)
    nbad, worst = _close(a[idx, 0], g["ax"], 6)
    nbad2, worst2 = _close(a[idx, 1], g["ay"], 6)
    assert nbad == 0 and nbad2 == 0, (worst, worst2)


def test_artificial_viscosity(case):
    from oracle import binding as O
    from sph2d_gb300 import capi

    p, r, v, rho, itype = case
    q = p.copy()
    q.artificial_viscosity = 1
    q.dt_correction_method = 2
    a, _, mu = O.forces(q, capi.TERM_ART_VISC, r, v, rho, np.zeros_like(rho), itype)
    idx, g = _golden("art_visc_target.csv")
    assert _close(a[idx, 0], g["ax"], 8)[0] == 0
    assert _close(a[idx, 1], g["ay"], 8)[0] == 0
    assert _close(mu[idx], g["mu"], 8)[0] == 0


def test_external_force_dynamic(case):
    from oracle import binding as O
    from sph2d_gb300 import capi

    p, r, v, rho, itype = case
    q = p.copy()
    q.boundary_treatment = 0
    a, _, _ = O.forces(q, capi.TERM_GRAVITY | capi.TERM_EXTERNAL, r, v, rho, np.zeros_like(rho), itype)
    idx, g = _golden("exdvdt_dynamic.csv")
    assert _close(a[idx, 0], g["exdvdt_x"], 6)[0] == 0
    assert _close(a[idx, 1], g["exdvdt_y"], 6)[0] == 0


def test_external_force_repulsive(case):
    """testExternalForceOMP.cpp:64-68 (which the reference notes as failing by a
    small error) with SBT_REPULSIVE, against the golden file and the
    reference's compiled external_force_part."""
    from oracle import binding as O
    from sph2d_gb300 import capi

    p, r, v, rho, itype = case
    q = p.copy()
    q.boundary_treatment = 1
    terms = capi.TERM_GRAVITY | capi.TERM_EXTERNAL
    a, _, _ = O.forces(q, terms, r, v, rho, np.zeros_like(rho), itype)
    idx, g = _golden("exdvdt_repulsive.csv")
    assert _close(a[idx, 0], g["exdvdt_x"], 6)[0] == 0
    assert _close(a[idx, 1], g["exdvdt_y"], 6)[0] == 0
    if O.ref_available():
        ref = O.ref_run(q, f"terms:{terms}", r, v, rho, itype)
        assert np.array_equal(a, ref["a"])


def test_average_velocity(case):
    """testAverageVelocityOMP.cpp:26-62: coef 0.05, cubic, fluid particles only."""
    from oracle import binding as O
    from sph2d_gb300 import capi

    p, r, v, rho, itype = case
    q = p.copy()
    q.average_velocity = 1
    q.average_velocity_skf = 1
    q.average_velocity_coef = 0.05
    _, av, _ = O.forces(q, capi.TERM_AVERAGE_VELOCITY, r, v, rho, np.zeros_like(rho), itype)
    av[int(q.nfluid):] = 0.0
    idx, g = _golden("average_velocity_target.csv")
    assert _close(av[idx, 0], g["av_x"], 6)[0] == 0
    assert _close(av[idx, 1], g["av_y"], 6)[0] == 0


def test_neighbours_against_reference_core(case):
    """The golden neighbour list is not in the reference checkout
    (.MISSING_LARGE_BLOBS); the pair lists are compared with the reference's
    compiled find_neighbours instead, entry by entry."""
    from oracle import binding as O

    p, r, v, rho, itype = case
    counts, lst, keys, grid, cs = O.neighbours(p, r, itype)
    if not O.ref_available():
        pytest.skip("reference core not built")
    ref = O.ref_run(p, "grid", r, v, rho, itype)
    assert np.array_equal(ref["keys"], keys)
    assert np.array_equal(ref["grid"], grid)
    assert np.array_equal(ref["cells_start"], cs)
    assert np.array_equal(ref["counts"], counts)
    flat = np.concatenate([lst[j, :counts[j]] for j in range(len(counts))])
    assert np.array_equal(ref["list"], flat)
    assert int(counts.sum()) == 1004398
