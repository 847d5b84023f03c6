"""GPU parity of the other Krylov methods of bddcml_solve_c against the oracle:
BiCGSTAB (method 1, module_krylov.f90:948-1505), steepest descent (method 2,
module_krylov.f90:1508-1840) and the defaults of method -1
(module_bddcml.f90:515-520: BiCGSTAB, tol 1e-6, maxit 1000, ndecrmax 30).

Tolerances as for PCG: iteration count within +-2 of the oracle; solution
relative error <= 1e-8 (FP64) or 1e-7 (mixed precision) against the oracle at
relative residual 1e-8.  The condition number is -1 for these methods.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


def _problem(kind):
    from bddcml_gb300 import problems
    from newdata_util import changed_data
    if kind == "dirichlet":  # non-zero initial guess from the boundary values
        return changed_data(problems.poisson_on_cube(4, 3), seed=11)
    boxes = problems.random_box_partition(20, 4, 9, seed=5)
    return problems.poisson_boxes(20, boxes, kappa=problems.lognormal_kappa(20, 1.0, seed=7))


@pytest.mark.parametrize("kind", ["dirichlet", "uneven"])
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_method_parity(built_lib, oracle_mod, kind, method, precision):
    import bddcml_gb300 as B
    prob = _problem(kind)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_o, reason_o, cond_o = o.solve(1e-8, 300, 50, method=method)
    u_o = o.global_solution()
    u, it, reason, cond, st = B.solve_problem(prob, precision=precision, tol=1e-8, maxit=300, ndecrmax=50,
                                              method=method)
    assert reason == reason_o == 0
    assert cond == cond_o == -1.0
    assert abs(it - it_o) <= 2, (it, it_o)
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert err <= TOL[precision], err


@pytest.mark.parametrize("precision", [0, 1])
def test_default_method_ignores_passed_parameters(built_lib, oracle_mod, precision):
    """method -1: BiCGSTAB at tol 1e-6 whatever tol/maxit/ndecrmax are passed."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(5, 4)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_o, reason_o, _ = o.solve(1e-6, 1000, 30, method=1)
    u_o = o.global_solution()
    u, it, reason, cond, st = B.solve_problem(prob, precision=precision, tol=1e-14, maxit=1, ndecrmax=1,
                                              method=-1)
    assert reason == reason_o == 0 and cond == -1.0
    assert abs(it - it_o) <= 2, (it, it_o)
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= 1e-5


def test_bicgstab_maxit_reason(built_lib, oracle_mod):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(5, 4)
    u, it, reason, cond, st = B.solve_problem(prob, precision=1, tol=1e-14, maxit=2, ndecrmax=50, method=1)
    assert (it, reason) == (2, -1)


def test_unimplemented_and_unknown_methods_are_rejected(built_lib):
    """method 5 (direct solve by backsubstitution) is outside the implemented
    path; methods outside -1, 0, 1, 2, 5 are an argument error."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        with pytest.raises(B.BddcmlError) as e5:
            B.bddcml_solve(0, 5, 1e-8, 100, 50, 0, 0)
        assert e5.value.code == 4  # UNSUPPORTED
        with pytest.raises(B.BddcmlError) as e3:
            B.bddcml_solve(0, 3, 1e-8, 100, 50, 0, 0)
        assert e3.value.code == 1  # ARGUMENT
        it, reason, cond = B.bddcml_solve(0, 1, 1e-8, 100, 50, 0, 0)  # still usable afterwards
        assert reason == 0 and cond == -1.0
    finally:
        B.bddcml_finalize()
