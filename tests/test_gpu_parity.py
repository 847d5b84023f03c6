"""GPU parity: the C-ABI solve against the CPU oracle (restatement of the
reference BDDC-PCG) on seeded/deterministic inputs.

Tolerances (from the spec of the path): iteration count within +-2 of the
oracle; solution relative error <= 1e-8 for the plain FP64 path and <= 1e-7
for the mixed-precision path, at PCG relative residual 1e-8.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-8
TOL_MIXED = 1e-7


def _run(prob, precision, weights_type=0, numbase=0):
    import bddcml_gb300 as B
    return B.solve_problem(prob, precision=precision, tol=1e-8, maxit=300, ndecrmax=50,
                           weights_type=weights_type, numbase=numbase)


def _oracle(oracle_mod, prob, weights_type=0):
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, weights_type)
    it, reason, cond = o.solve(1e-8, 300, 50)
    return o, it, reason, cond, o.global_solution()


CASES = [(4, 2), (4, 3), (6, 3), (5, 4), (8, 4)]


@pytest.mark.parametrize("ne,ns", CASES)
@pytest.mark.parametrize("precision", [0, 1])
def test_poisson_cube_parity(built_lib, oracle_mod, ne, ns, precision):
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns)
    o, it_o, reason_o, cond_o, u_o = _oracle(oracle_mod, prob)
    u, it, reason, cond, st = _run(prob, precision)
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert err <= (TOL_FP64 if precision == 0 else TOL_MIXED), err
    assert abs(cond - cond_o) <= 0.05 * cond_o + 1e-6, (cond, cond_o)


@pytest.mark.parametrize("precision", [0, 1])
def test_heterogeneous_coefficients_weights_stiffness(built_lib, oracle_mod, precision):
    from bddcml_gb300 import problems
    kappa = problems.lognormal_kappa(16, 1.0, seed=3)
    prob = problems.poisson_on_cube(4, 4, kappa=kappa)
    o, it_o, reason_o, cond_o, u_o = _oracle(oracle_mod, prob, weights_type=1)
    u, it, reason, cond, st = _run(prob, precision, weights_type=1)
    assert reason == 0 and reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert err <= (TOL_FP64 if precision == 0 else TOL_MIXED), err


@pytest.mark.parametrize("precision", [0, 1])
def test_uneven_box_partition(built_lib, oracle_mod, precision):
    from bddcml_gb300 import problems
    boxes = problems.random_box_partition(24, 5, 10, seed=17)
    prob = problems.poisson_boxes(24, boxes, name="uneven")
    o, it_o, reason_o, cond_o, u_o = _oracle(oracle_mod, prob)
    u, it, reason, cond, st = _run(prob, precision)
    assert reason == 0 and reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert err <= (TOL_FP64 if precision == 0 else TOL_MIXED), err


def test_fortran_numbering(built_lib, oracle_mod):
    """numbase = 1 shifts every index array and isub (module_levels.f90:249,718)."""
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 3)
    u0, it0, *_ = _run(prob, 1, numbase=0)
    u1, it1, *_ = _run(prob, 1, numbase=1)
    assert it0 == it1
    assert np.allclose(u0, u1, rtol=0, atol=1e-13)


def test_solution_matches_direct_solve(built_lib):
    import scipy.sparse.linalg as spla
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(6, 3)
    K, f, fixed = problems.global_matrix_and_rhs(prob)
    free = ~fixed
    ud = np.zeros(prob.ndof)
    ud[free] = spla.spsolve(K[free][:, free].tocsc(), f[free])
    for precision in (0, 1):
        u, it, reason, cond, st = _run(prob, precision)
        assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-7


@pytest.mark.parametrize("ne,ns", [(3, 2), (4, 3)])
@pytest.mark.parametrize("precision", [0, 1])
def test_elasticity_parity(built_lib, oracle_mod, ne, ns, precision):
    """Three dofs per node (Q1 elasticity, clamped at x = 0, body force)."""
    from bddcml_gb300 import problems
    prob = problems.elasticity_on_cube(ne, ns)
    o, it_o, reason_o, cond_o, u_o = _oracle(oracle_mod, prob)
    u, it, reason, cond, st = _run(prob, precision)
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2
    tol = TOL_FP64 if precision == 0 else TOL_MIXED
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= tol
