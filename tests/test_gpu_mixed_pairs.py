"""The FP32-mixed step's own neighbour pairs against the oracle's find_neighbours.

The mixed step with neighbour reuse decides each step's pairs in its density
pass: the candidates of a particle's list (built with the cutoff widened by a
skin, reused while no particle has moved more than half the skin) that pass
the reference's test `dist^2 < (2h)^2` (GridFind.cpp:124, 150-156), computed
in float with cell-relative offsets and re-tested in double within 1e-5 of
the cutoff; a particle with more candidates than a list holds is searched by
stencil instead. ``rrsph_step_neighbours`` returns the pairs that pass wrote;
these tests compare them, particle by particle as sets, with the oracle's
find_neighbours on the same double positions (the pair sets must be
bit-exact), and the step's pair count with the oracle's:

- right after upload (the first step builds the lists);
- on every step of the next few, which reuse lists built several steps
  earlier or rebuild them as the motion asks;
- on the step after a forced rebuild;
- for the full 409k-particle flume, the full 2D dam break (summation and
  continuity density), a small 3D dam break, and particles whose candidate
  lists overflow (the stencil branch), 2D and 3D.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair_keys(counts, lst, n):
    """Sorted (j, i) pair keys j * n + i of a neighbour table."""
    counts = np.asarray(counts, dtype=np.int64)
    mask = np.arange(lst.shape[1])[None, :] < counts[:, None]
    rows = np.broadcast_to(np.arange(len(counts), dtype=np.int64)[:, None], lst.shape)[mask]
    keys = rows * n + lst[mask].astype(np.int64)
    keys.sort()
    return keys


def _check_step_pairs(s, p, r, itype, what):
    from oracle import binding as O

    n = int(p.ntotal)
    c_o, l_o, *_ = O.neighbours(p, r, itype)
    c, lst, tot = s.step_neighbours()
    assert np.array_equal(c, c_o), (what, int(np.sum(c != c_o)))
    ko = _pair_keys(c_o, l_o, n)
    kg = _pair_keys(c, lst, n)
    assert np.array_equal(kg, ko), (what, kg.size, ko.size)
    # a row holds no particle twice
    assert np.unique(kg).size == kg.size, what
    last, _ = s.pair_count()
    assert tot == int(c_o.sum()) == last, (what, tot, int(c_o.sum()), last)
    return tot


def _run_checks(case, p, steps: int = 8):
    """Upload, the first step, then `steps` steps one at a time (reuse steps,
    whose lists are several steps old, and the rebuilds the motion asks for),
    a forced rebuild and two steps after it; checks the pairs of each
    (positions from a download: the state the next step's pairs come from).
    Returns the ages, in steps, of the lists that the checked reuse steps used."""
    from sph2d_gb300 import Solver

    reuse_ages = []
    with Solver(p, "mixed") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        t = s.step(1, 0.0)
        _check_step_pairs(s, p, case.r, case.itype, "first step")
        assert s.neighbour_rebuilds() == 1
        age = 1
        for _ in range(steps):
            st = s.download()
            b0 = s.neighbour_rebuilds()
            t = s.step(1, t)
            reused = s.neighbour_rebuilds() == b0
            age = age + 1 if reused else 1
            if reused:
                reuse_ages.append(age)
            _check_step_pairs(s, p, st["r"], st["itype"], f"reuse step (lists {age} steps old)" if reused
                              else "step with rebuild")
        st = s.download()
        s.set_neighbour_reuse(True)  # forces a rebuild on the next step
        b0 = s.neighbour_rebuilds()
        t = s.step(1, t)
        assert s.neighbour_rebuilds() == b0 + 1
        _check_step_pairs(s, p, st["r"], st["itype"], "forced rebuild")
        # two more reuse steps after the rebuild
        for _ in range(2):
            st = s.download()
            t = s.step(1, t)
            _check_step_pairs(s, p, st["r"], st["itype"], "after rebuild")
        return reuse_ages


def test_flume_full_size_step_pairs(gpu_available):
    """The 409k-particle piston flume: ~8 million directed pairs a step."""
    from sph2d_gb300 import cases

    case = cases.piston_flume_2d()
    p = case.params()
    ages = _run_checks(case, p, steps=8)
    assert ages and max(ages) >= 3, ages  # lists several steps old were checked


@pytest.mark.parametrize("treatment", [0, 1, 2])
def test_dam_break_full_size_step_pairs(gpu_available, treatment):
    from sph2d_gb300 import cases

    case = cases.dam_break_2d(density_treatment=min(treatment, 1))
    p = case.params()
    if treatment == 2:
        p.density_treatment = 2
        p.density_delta_sph_coef = 0.1
    _run_checks(case, p, steps=6)


@pytest.mark.parametrize("treatment", [0, 1])
def test_dam_break_3d_step_pairs(gpu_available, treatment):
    from sph2d_gb300 import cases

    case = cases.dam_break_3d(dx=0.02, tank=(0.5, 0.2, 0.3), block=(0.2, 0.2, 0.15), max_neighbours=400,
                              density_treatment=treatment)
    p = case.params()
    _run_checks(case, p, steps=4)


@pytest.mark.parametrize("dim", [2, 3])
def test_over_full_candidate_lists_step_pairs(gpu_available, dim):
    """Particles with more candidates than a list holds (64 in 2D, 256 in 3D,
    from a lattice laid out for a shorter h) take the stencil branch of the
    density pass; their pairs are the oracle's too."""
    from sph2d_gb300 import Solver, cases

    if dim == 2:
        case = cases.dam_break_2d(nx=40, ny=20)
        case.model["intf_hsml_coef"] = 2.0
        case.model["max_neighbours"] = 65
    else:
        case = cases.dam_break_3d(dx=0.02, block=(0.3, 0.3, 0.3), density_treatment=0)
        case.model["intf_hsml_coef"] = 1.75
        case.model["max_neighbours"] = 400
    p = case.params()
    with Solver(p, "mixed") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        t = 0.0
        for k in range(3):
            st = s.download() if k else {"r": case.r, "itype": case.itype}
            t = s.step(1, t)
            _check_step_pairs(s, p, st["r"], st["itype"], f"step {k}")
        # every step rebuilt: an over-full list asks for a fresh grid
        assert s.neighbour_rebuilds() == 3


def test_step_neighbours_refuses_without_a_step(gpu_available):
    from sph2d_gb300 import RrsphError, Solver, capi, cases

    case = cases.dam_break_2d(nx=20, ny=10)
    p = case.params()
    with Solver(p, "mixed") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        with pytest.raises(RrsphError) as e:
            s.step_neighbours()
        assert e.value.code == capi.ERR_INVALID_ARGUMENT
        s.step(1, 0.0)
        s.step_neighbours()
        s.grid_find()  # replaces the grid the list refers to
        with pytest.raises(RrsphError):
            s.step_neighbours()
    with Solver(p, "fp64") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        s.step(1, 0.0)
        with pytest.raises(RrsphError) as e:
            s.step_neighbours()
        assert e.value.code == capi.ERR_UNSUPPORTED
