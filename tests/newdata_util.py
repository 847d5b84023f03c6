"""Changed loads and Dirichlet values for a Poisson problem (one dof per node):
a seeded global load field and the boundary values g = 0.1 + x + 2y - z, each
restricted consistently to the subdomains."""
import copy

import numpy as np


def changed_data(prob, seed):
    rng = np.random.default_rng(seed)
    scale = max(float(np.abs(s.rhs).max()) for s in prob.subdomains)
    load = rng.uniform(0.5, 1.5, prob.ndof) * scale
    p2 = copy.deepcopy(prob)
    for s in p2.subdomains:
        x, y, z = s.xyz[0], s.xyz[1], s.xyz[2]
        fixed = s.ifix != 0
        s.fixv = np.where(fixed, 0.1 + x + 2.0 * y - z, 0.0)
        s.rhs = np.where(fixed, 0.0, load[s.isvgvn])
        s.sol = np.zeros(s.ndofs)
    return p2


def direct_solution(prob):
    """Direct solve of the assembled global system with the Dirichlet values."""
    import scipy.sparse.linalg as spla
    from bddcml_gb300 import problems
    K, f, fixed = problems.global_matrix_and_rhs(prob)
    ub = np.zeros(prob.ndof)
    for s in prob.subdomains:
        ub[s.isvgvn[s.ifix != 0]] = s.fixv[s.ifix != 0]
    free = ~fixed
    u = ub.copy()
    rhs = f[free] - K[free][:, fixed] @ ub[fixed]
    u[free] = spla.spsolve(K[free][:, free].tocsc(), rhs)
    return u
