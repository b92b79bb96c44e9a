"""The C oracle reproduces the committed reference fixtures.

tests/golden/reference_fixtures.npz holds the outputs of the reference's own
compute core on seeded cases (made by tests/golden/make_golden.py). This test
needs no reference sources, so it also pins the oracle on machines where only
the fixture is available. Integer results must be identical; floating results
within 1e-11 relative L2 (the case inputs are regenerated from seeds, and libm
may differ by an ulp between machines).
"""

import hashlib

import numpy as np
import pytest

from conftest import rel_l2

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def fx():
    return np.load(GOLDEN / "reference_fixtures.npz")


def _cases():
    import sys

    sys.path.insert(0, str(GOLDEN))
    import make_golden

    return make_golden


@pytest.mark.parametrize("name", ["dam", "flume"])
def test_oracle_reproduces_reference_fixture(fx, name):
    from oracle import binding as O
    from sph2d_gb300 import capi

    mg = _cases()
    case = mg.fixture_cases()[name]
    p = case.params()
    counts, lst, keys, grid, cs = O.neighbours(p, case.r, case.itype)
    flat = np.concatenate([lst[j, :counts[j]] for j in range(len(counts))])
    assert mg.digest(keys, grid, cs) == str(fx[f"{name}/grid_sha"])
    assert mg.digest(counts, flat) == str(fx[f"{name}/pairs_sha"])
    out, pres = O.density(p, case.r, case.v, case.rho, case.itype)
    assert rel_l2(out, fx[f"{name}/density"]) < 1e-11
    assert rel_l2(pres, fx[f"{name}/density_p"]) < 1e-11
    v = mg.velocity_field(case)
    q = p.copy()
    q.dt_correction_method = 2
    pr = O.eos_p(q, case.rho)
    a, _, mu = O.forces(q, capi.TERM_ALL, case.r, v, case.rho, pr, case.itype)
    assert rel_l2(a, fx[f"{name}/terms_a"]) < 1e-11
    assert rel_l2(mu, fx[f"{name}/terms_mu"]) < 1e-11
    n = mg.RUN_STEPS[name]
    run = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=n)
    for k in ("r", "v", "rho", "p"):
        assert rel_l2(run[k], fx[f"{name}/run_{k}"]) < 1e-10, k
    assert np.array_equal(run["itype"], fx[f"{name}/run_itype"])
    assert run["time"] == pytest.approx(float(fx[f"{name}/run_time"]), rel=1e-13)


def test_fixture_script_is_consistent():
    mg = _cases()
    assert set(mg.RUN_STEPS) == {"dam", "flume"}
    h = hashlib.sha256(b"x").hexdigest()
    assert mg.digest(np.frombuffer(b"x", dtype=np.uint8)) == h
