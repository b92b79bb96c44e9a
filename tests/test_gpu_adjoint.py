"""The adjoint of the FP64 loop with a Fourier piston (rrsph_adjoint_forward /
rrsph_adjoint_reverse): forward parity with the oracle, the gradient against
the oracle's forward-mode reference and against central finite differences
on the GPU, checkpoint-interval independence, and the torch.autograd wrapper
used by this harness."""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

STEPS = 200
GX = 0.15


@pytest.fixture(scope="module")
def small():
    from sph2d_gb300 import cases

    c = cases.adjoint_flume_2d(nx=60, ny=15, dx=0.01, steps=STEPS, gauge_x=GX, window=0.005, sample_every=5)
    return c, c.params()


def _forward(s, c, coef, K=50):
    s.upload(c.r, c.v, c.rho, c.itype)
    s.set_piston_fourier(c.notes["omega"], coef)
    return s.adjoint_forward(STEPS, GX, sample_from=c.notes["sample_from"], sample_every=c.notes["sample_every"],
                             checkpoint_every=K)[0]


def _oracle(c, p, coef):
    from oracle import binding as O

    return O.piston_tangent_run(p, c.r, c.v, c.rho, c.itype, STEPS, c.notes["omega"], coef, GX,
                                sample_from=c.notes["sample_from"], sample_every=c.notes["sample_every"])


def test_fourier_forward_matches_the_oracle(gpu_available, small):
    from sph2d_gb300 import Solver

    c, p = small
    g_ref, _, st_ref = _oracle(c, p, c.notes["coef"])
    with Solver(p, "fp64") as s:
        g = _forward(s, c, c.notes["coef"])
        st = s.download()
    assert g.shape == g_ref.shape
    assert np.abs(g - g_ref).max() < 1e-10 * np.abs(g_ref).max()
    for k in ("r", "v", "rho"):
        assert rel_l2(st[k], st_ref[k]) < 1e-10, k


def test_adjoint_matches_the_forward_mode_reference(gpu_available, small):
    from sph2d_gb300 import Solver

    c, p = small
    _, dg_ref, _ = _oracle(c, p, c.notes["coef"])
    w = np.random.default_rng(11).standard_normal(dg_ref.shape[0])
    with Solver(p, "fp64") as s:
        _forward(s, c, c.notes["coef"])
        dcoef, dvx = s.adjoint_reverse(w)
    want = dg_ref.T @ w
    assert np.linalg.norm(dcoef - want) < 1e-8 * np.linalg.norm(want)
    assert np.count_nonzero(dvx) > 0


def test_checkpoint_interval_does_not_change_the_gradient(gpu_available, small):
    """Recomputed segments reproduce the forward states bit for bit."""
    from sph2d_gb300 import Solver

    c, p = small
    out = []
    for K in (1, 7, STEPS):
        with Solver(p, "fp64") as s:
            g = _forward(s, c, c.notes["coef"], K=K)
            end = s.download()
            dcoef, dvx = s.adjoint_reverse(np.linspace(1.0, 2.0, len(g)))
            after = s.download()
        for k in ("r", "v", "rho"):  # the reverse sweep leaves the forward end state
            assert np.array_equal(end[k], after[k]), k
        out.append((g, dcoef, dvx))
    for g, dcoef, dvx in out[1:]:
        assert np.array_equal(g, out[0][0])
        assert np.array_equal(dcoef, out[0][1]) and np.array_equal(dvx, out[0][2])


def test_misfit_gradient_matches_central_differences(gpu_available, small):
    """d(mean squared gauge misfit)/d(coefficients) against central
    differences of the FP64 GPU forward run (eps = 1e-6)."""
    from sph2d_gb300 import Solver

    c, p = small
    with Solver(p, "fp64") as s:
        target = _forward(s, c, c.notes["target_coef"])
        coef = c.notes["coef"]
        g = _forward(s, c, coef)
        dcoef, _ = s.adjoint_reverse(2.0 * (g - target) / len(g))

        def loss(cf):
            return float(np.mean((_forward(s, c, cf) - target) ** 2))

        eps = 1e-6
        fd = np.zeros_like(coef)
        for k in range(len(coef)):
            cp, cm = coef.copy(), coef.copy()
            cp[k] += eps
            cm[k] -= eps
            fd[k] = (loss(cp) - loss(cm)) / (2 * eps)
    assert np.linalg.norm(dcoef - fd) < 1e-5 * np.linalg.norm(fd)


def test_torch_autograd_function(gpu_available, small):
    """The harness's torch.autograd.Function around the C-ABI reverse call."""
    torch = pytest.importorskip("torch")
    from sph2d_gb300 import Solver

    c, p = small

    class PistonGauges(torch.autograd.Function):
        @staticmethod
        def forward(ctx, coef, solver):
            ctx.solver = solver
            ctx.coef = coef.detach().numpy().copy()
            return torch.from_numpy(_forward(solver, c, ctx.coef).copy())

        @staticmethod
        def backward(ctx, grad):
            # the solver keeps one recorded run: record this evaluation point again
            _forward(ctx.solver, c, ctx.coef)
            dcoef, _ = ctx.solver.adjoint_reverse(grad.detach().numpy())
            return torch.from_numpy(dcoef.copy()), None

    with Solver(p, "fp64") as s:
        target = torch.from_numpy(_forward(s, c, c.notes["target_coef"]).copy())
        coef = torch.tensor(c.notes["coef"], dtype=torch.float64, requires_grad=True)
        loss = ((PistonGauges.apply(coef, s) - target) ** 2).mean()
        loss.backward()
        g = _forward(s, c, c.notes["coef"])
        direct, _ = s.adjoint_reverse(2.0 * (g - target.numpy()) / len(g))
        assert np.allclose(coef.grad.numpy(), direct, rtol=1e-12, atol=0)
        # Jacobian of the gauge series against torch's own finite differences
        x = torch.tensor(c.notes["coef"][:8], dtype=torch.float64, requires_grad=True)
        assert torch.autograd.gradcheck(lambda cf: PistonGauges.apply(cf, s), (x,), eps=1e-6, atol=1e-7, rtol=1e-4)


def test_adjoint_rejects_unsupported_methods(gpu_available, small):
    from sph2d_gb300 import RrsphError, Solver, capi

    c, p = small
    with Solver(p, "mixed") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        with pytest.raises(RrsphError) as e:
            s.adjoint_forward(10, GX)
        assert e.value.code == capi.ERR_UNSUPPORTED
    q = p.copy()
    q.density_treatment = 1
    with Solver(q, "fp64") as s:
        s.upload(c.r, c.v, c.rho, c.itype)
        with pytest.raises(RrsphError) as e:
            s.adjoint_forward(10, GX)
        assert e.value.code == capi.ERR_UNSUPPORTED
        with pytest.raises(RrsphError):
            s.adjoint_reverse(np.zeros(1))
