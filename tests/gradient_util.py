"""Differentiation example helpers: J = 1/2 |u - u*|^2 and its gradient with
respect to element coefficients, dJ/dkappa_e = -lambda_e^T K_e^0 u_e, assembled
from CPU oracle solves (forward and adjoint)."""
import copy

import numpy as np


def oracle_solution(oracle_mod, prob, tol=1e-12):
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    _, reason, _ = o.solve(tol, 500, 50)
    assert reason == 0
    return o.global_solution()


def objective(u, ustar):
    return 0.5 * float(np.dot(u - ustar, u - ustar))


def oracle_gradient(oracle_mod, ne, ns, kappa, ustar):
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns, kappa=kappa)
    u = oracle_solution(oracle_mod, prob)
    g = u - ustar
    adj = copy.deepcopy(prob)
    for s in adj.subdomains:
        s.rhs = np.where(s.ifix != 0, 0.0, g[s.isvgvn])
        s.fixv = np.zeros(s.ndofs)
    lam = oracle_solution(oracle_mod, adj)
    n = ne * ns
    conn = problems.cube_connectivity(n)
    ke0 = problems.q1_laplace_reference_matrix() / n
    ue, le = u[conn], lam[conn]
    return u, -np.einsum("ea,ab,eb->e", le, ke0, ue)
