"""Global solution and reactions through the C ABI against the oracle
(bddcml_download_global_solution_c, bddcml_download_local_reactions_c,
bddcml_download_global_reactions_c; module_levels.f90:4617-4914,
module_dd.f90:1258-1374): every subdomain's reaction vector within 1e-8 of
the oracle's (relative to its largest entry), the global vectors likewise, and
the calls refused before a solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_reactions_and_global_solution(built_lib, oracle_mod, precision):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    from newdata_util import changed_data
    prob = changed_data(problems.poisson_on_cube(5, 3), seed=5)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    o.solve(1e-10, 300, 50)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(precision)
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        with pytest.raises(B.BddcmlError):
            B.bddcml_download_global_reactions(prob.ndof)
        it, reason, cond = B.bddcml_solve(0, 0, 1e-10, 300, 50, 0, 0)
        assert reason == 0
        tol = 1e-8 if precision == 0 else 1e-7
        for s in prob.subdomains:
            r = B.bddcml_download_local_reactions(s.isub, s.ndofs)
            ro = o.reactions(s.isub)
            assert np.abs(r - ro).max() <= tol * max(1e-300, np.abs(ro).max()), s.isub
        u = B.bddcml_download_global_solution(prob.ndof)
        uo = o.global_solution()
        assert np.linalg.norm(u - uo) <= tol * np.linalg.norm(uo)
        rg = B.bddcml_download_global_reactions(prob.ndof)
        rgo = o.global_reactions()
        assert np.abs(rg - rgo).max() <= tol * np.abs(rgo).max()
        with pytest.raises(B.BddcmlError):
            B.bddcml_download_global_solution(prob.ndof + 1)
    finally:
        B.bddcml_finalize()
