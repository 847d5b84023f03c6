"""Gradient of the differentiation example from CPU oracle solves.

TEST INFRASTRUCTURE ONLY (imported by tests/ and by the CPU leg of bench.py):
J = 1/2 |u - u*|^2 for the Poisson cube with per-element coefficients kappa_e,
and dJ/dkappa_e = -lambda_e^T K_e^0 u_e assembled from an oracle forward solve
K u = f and an oracle adjoint solve K lambda = u - u* (same SPD operator,
homogeneous Dirichlet values).  The problem is the one of
examples/poisson_on_cube.f90:729-901 with kappa_e scaling each element matrix.
"""
import copy

import numpy as np


def oracle_solution(oracle_mod, prob, tol=1e-12, nthreads=None):
    o = oracle_mod.Oracle(prob, nthreads=nthreads)
    o.setup(1, 1, 0)
    it, reason, _ = o.solve(tol, 500, 50)
    assert reason == 0
    return o.global_solution(), it


def objective(u, ustar):
    return 0.5 * float(np.dot(u - ustar, u - ustar))


def oracle_gradient(oracle_mod, ne, ns, kappa, ustar, tol=1e-12, nthreads=None, with_iterations=False):
    """(u, dJ/dkappa) of the ne^3-element subdomains, ns per cube edge."""
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns, kappa=kappa)
    u, it_f = oracle_solution(oracle_mod, prob, tol, nthreads)
    g = u - ustar
    adj = copy.deepcopy(prob)
    for s in adj.subdomains:
        s.rhs = np.where(s.ifix != 0, 0.0, g[s.isvgvn])
        s.fixv = np.zeros(s.ndofs)
    lam, it_a = oracle_solution(oracle_mod, adj, tol, nthreads)
    n = ne * ns
    conn = problems.cube_connectivity(n)
    ke0 = problems.q1_laplace_reference_matrix() / n
    ue, le = u[conn], lam[conn]
    grad = -np.einsum("ea,ab,eb->e", le, ke0, ue)
    if with_iterations:
        return u, grad, it_f, it_a
    return u, grad
