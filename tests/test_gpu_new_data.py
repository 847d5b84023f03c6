"""New loads and boundary values after setup: bddcml_change_subdomain_data_c +
bddcml_setup_new_data_c (module_levels.f90:785-903) re-solve with the factors and
preconditioner of the first setup.  Each re-solve must match the oracle's fresh
solve of the changed problem within the path's tolerances (iterations +-2,
solution 1e-8 plain FP64 / 1e-7 mixed), on two changes in a row."""
import numpy as np
import pytest

from newdata_util import changed_data

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


@pytest.mark.parametrize("ne,ns", [(4, 3), (8, 2)])
@pytest.mark.parametrize("precision", [0, 1])
def test_new_data_matches_fresh_solve(built_lib, oracle_mod, ne, ns, precision):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns)
    B.solve_problem(prob, precision=precision, finalize=False)
    try:
        for seed in (1, 2):
            p2 = changed_data(prob, seed)
            for s in p2.subdomains:
                B.bddcml_change_subdomain_data(s.isub, s.ifix, s.fixv, s.rhs, 1, s.sol)
            B.bddcml_setup_new_data()
            it, reason, cond = B.bddcml_solve(0, 0, 1e-8, 300, 50, 0, 0)
            u = np.zeros(prob.ndof)
            for s in p2.subdomains:
                u[s.isvgvn] = B.bddcml_download_local_solution(s.isub, s.ndofs)
            o = oracle_mod.Oracle(p2)
            o.setup(1, 1, 0)
            it_o, reason_o, _ = o.solve(1e-8, 300, 50)
            uo = o.global_solution()
            assert reason == reason_o == 0
            assert abs(it - it_o) <= 2
            assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= TOL[precision]
        # changing which dofs are fixed needs a new setup and is refused
        s = prob.subdomains[0]
        ifix2 = s.ifix.copy()
        ifix2[int(np.argmax(ifix2 == 0))] = 1
        with pytest.raises(B.BddcmlError):
            B.bddcml_change_subdomain_data(s.isub, ifix2, s.fixv, s.rhs, 1, s.sol)
    finally:
        B.bddcml_finalize()
