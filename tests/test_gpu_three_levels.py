"""Three-level BDDC through the C ABI against the oracle (nl = 3:
levels_corsub_standard_level / levels_solve_last_level /
levels_add_standard_level, module_levels.f90:3849-4250; the level-2 problem of
levels_prepare_standard_level, :1297-3000).  The level-2 subdomains come from
the same coordinate bisection of the level-1 subdomain centroids in both.
Tolerances as for two levels: iterations +-2, solution 1e-8 (FP64) / 1e-7
(mixed) against the oracle; the solution also matches a direct solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


def _run(prob, precision, nsub2, weights=0):
    import bddcml_gb300 as B
    B.bddcml_init(3, [prob.nsub, nsub2, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(precision)
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(prob.matrixtype, 0, 1, 1, 1, 0, 0, weights)
        it, reason, cond = B.bddcml_solve(0, 0, 1e-8, 500, 50, 0, 0)
        u = np.zeros(prob.ndof)
        for s in prob.subdomains:
            u[s.isvgvn] = B.bddcml_download_local_solution(s.isub, s.ndofs)
    finally:
        B.bddcml_finalize()
    return u, it, reason, cond


@pytest.mark.parametrize("case", ["poisson", "elasticity"])
@pytest.mark.parametrize("precision", [0, 1])
def test_three_levels_parity(built_lib, oracle_mod, case, precision):
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    if case == "poisson":
        prob, nsub2 = problems.poisson_on_cube(4, 6), 27
    else:
        prob, nsub2 = problems.elasticity_on_cube(3, 4), 8
    o = oracle_mod.Oracle(prob)
    o.set_levels(3, nsub2)
    o.setup(1, 1, 0)
    it_o, reason_o, cond_o = o.solve(1e-8, 500, 50)
    u_o = o.global_solution()
    u, it, reason, cond = _run(prob, precision, nsub2)
    print(f"{case} precision {precision}: iterations {it} (oracle {it_o}), cond {cond:.3f} (oracle {cond_o:.3f})")
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= TOL[precision]
    ud = direct_solution(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-6


def test_level_count_validation(built_lib):
    import bddcml_gb300 as B
    with pytest.raises(B.BddcmlError):
        B.bddcml_init(4, [64, 8, 2, 1], -1, 0, 0, 0, 0)
    with pytest.raises(B.BddcmlError):
        B.bddcml_init(3, [8, 16, 1], -1, 0, 0, 0, 0)
