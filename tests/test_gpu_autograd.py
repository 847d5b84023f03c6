"""Differentiation: the solve as a torch.autograd.Function whose backward is an
adjoint BDDC solve reusing the forward factors plus the per-element gradient
kernel.  The gradient of J = 1/2 |u - u*|^2 with respect to the element
coefficients is checked against central finite differences of GPU solves and
against the gradient assembled from CPU oracle forward + adjoint solves."""
import numpy as np
import pytest

from oracle_gradient import oracle_gradient

pytestmark = pytest.mark.gpu

NE, NS = 3, 2


def _setup(precision):
    torch = pytest.importorskip("torch")
    from bddcml_gb300 import problems
    from bddcml_gb300.autograd import PoissonCube
    op = PoissonCube(NE, NS, precision=precision, tol=1e-12)
    n = NE * NS
    kappa = torch.tensor(problems.lognormal_kappa(n, 1.0, seed=3), dtype=torch.float64, device="cuda")
    ustar = torch.tensor(problems.smooth_target(n, seed=4), dtype=torch.float64, device="cuda")
    return torch, op, kappa, ustar


def _grad(torch, op, kappa, ustar):
    k = kappa.clone().requires_grad_(True)
    u = op.solve(k)
    J = 0.5 * torch.sum((u - ustar) ** 2)
    J.backward()
    return u.detach(), k.grad.detach()


@pytest.mark.parametrize("precision", [0, 1])
def test_gradient_matches_oracle(built_lib, oracle_mod, precision):
    torch, op, kappa, ustar = _setup(precision)
    u, g = _grad(torch, op, kappa, ustar)
    u_o, g_o = oracle_gradient(oracle_mod, NE, NS, kappa.cpu().numpy(), ustar.cpu().numpy())
    tol = 1e-8 if precision == 0 else 1e-7
    assert np.linalg.norm(u.cpu().numpy() - u_o) <= tol * np.linalg.norm(u_o)
    assert np.linalg.norm(g.cpu().numpy() - g_o) <= tol * np.linalg.norm(g_o)


def test_gradient_matches_finite_differences(built_lib):
    torch, op, kappa, ustar = _setup(0)
    _, g = _grad(torch, op, kappa, ustar)
    rng = np.random.default_rng(11)
    eps = 1e-6
    with torch.no_grad():
        for _ in range(4):
            d = torch.tensor(rng.standard_normal(kappa.numel()), dtype=torch.float64, device="cuda")
            jp = 0.5 * torch.sum((op.solve(kappa * torch.exp(eps * d)) - ustar) ** 2).item()
            jm = 0.5 * torch.sum((op.solve(kappa * torch.exp(-eps * d)) - ustar) ** 2).item()
            fd = (jp - jm) / (2 * eps)
            an = torch.dot(g, kappa * d).item()
            assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)), (fd, an)
    import bddcml_gb300 as B
    B.bddcml_finalize()
