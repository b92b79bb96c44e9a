"""The oracle's forward-mode reference for the piston adjoint
(oracle/rrsph_tangent.c): its forward run is orc_run's, and its derivatives of
the gauge series by the Fourier coefficients match central finite differences
of that forward run."""

import numpy as np
import pytest

STEPS = 200
GAUGE_X = 0.15


@pytest.fixture(scope="module")
def small():
    from sph2d_gb300 import cases

    c = cases.adjoint_flume_2d(nx=60, ny=15, dx=0.01, steps=STEPS, gauge_x=GAUGE_X, window=0.005, sample_every=5)
    return c, c.params()


def _run(c, p, coef):
    from oracle import binding as O

    return O.piston_tangent_run(p, c.r, c.v, c.rho, c.itype, STEPS, c.notes["omega"], coef, GAUGE_X,
                                sample_from=c.notes["sample_from"], sample_every=c.notes["sample_every"])


def test_forward_is_the_loop_of_orc_run(small):
    """With all coefficients 0 the piston rests, as with no wave maker."""
    from oracle import binding as O

    c, p = small
    g, dg, st = _run(c, p, np.zeros(8))
    q = p.copy()
    q.nwm = 0
    ref = O.run(q, c.r, c.v, c.rho, c.itype, nsteps=STEPS)
    for k in ("r", "v", "rho", "p", "itype"):
        assert np.array_equal(st[k], ref[k]), k
    assert st["time"] == ref["time"]
    assert len(g) == (STEPS - c.notes["sample_from"]) // c.notes["sample_every"] + 1
    assert g[-1] == O.gauge(q, ref["r"], ref["itype"], GAUGE_X, 3.0, 2)


def test_tangents_match_central_differences(small):
    c, p = small
    coef = c.notes["coef"]
    g, dg, _ = _run(c, p, coef)
    assert dg.shape == (len(g), len(coef)) and np.abs(dg).max() > 1e-3
    eps = 1e-6
    fd = np.zeros_like(dg)
    for k in range(len(coef)):
        cp, cm = coef.copy(), coef.copy()
        cp[k] += eps
        cm[k] -= eps
        fd[:, k] = (_run(c, p, cp)[0] - _run(c, p, cm)[0]) / (2 * eps)
    assert np.abs(dg - fd).max() < 1e-6 * np.abs(dg).max()


def test_method_set_is_checked(small):
    from oracle import binding as O

    c, p = small
    q = p.copy()
    q.density_treatment = 1
    with pytest.raises(O.OracleError):
        O.piston_tangent_run(q, c.r, c.v, c.rho, c.itype, 2, 1.0, [0.01], GAUGE_X)
