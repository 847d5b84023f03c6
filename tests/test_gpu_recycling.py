"""Krylov recycling through bddcml_solve_c (recycling_int = 1,
max_number_of_stored_vectors; module_krylov.f90:313-484, 663-726) over load
cases changed with bddcml_change_subdomain_data_c + bddcml_setup_new_data_c,
against the oracle running the same sequence: iterations within +-1 of the
oracle's for every case, solutions within 1e-8 (FP64) / 1e-7 (mixed) of it,
and no iteration for a case the stored directions already resolve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


@pytest.mark.parametrize("precision", [0, 1])
def test_recycling_matches_oracle_sequence(built_lib, oracle_mod, precision):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_boxes(15, problems.uniform_boxes(15, 3), kappa=problems.lognormal_kappa(15, 1.0, 3))
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 1)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(precision)
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 1)
        rng = np.random.default_rng(2)
        loads = [None, rng.uniform(0.5, 1.5, prob.ndof), rng.uniform(0.5, 1.5, prob.ndof), "repeat"]
        its = []
        for case, load in enumerate(loads):
            if load is not None:
                for s in prob.subdomains:
                    if not isinstance(load, str):
                        s.rhs = np.where(s.ifix != 0, 0.0, load[s.isvgvn] / prob.n_el_edge ** 3)
                    zero = np.zeros(s.ndofs)
                    B.bddcml_change_subdomain_data(s.isub, s.ifix, s.fixv, s.rhs, 1, zero)
                    o.new_loads(s.isub, s.rhs)
                B.bddcml_setup_new_data()
            it, reason, cond = B.bddcml_solve(0, 0, 1e-8, 300, 50, 1, 40)
            it_o, reason_o, _ = o.solve_recycling(1e-8, 300, 50, True, 40)
            u = np.zeros(prob.ndof)
            for s in prob.subdomains:
                u[s.isvgvn] = B.bddcml_download_local_solution(s.isub, s.ndofs)
            uo = o.global_solution()
            assert reason == reason_o == 0, (case, reason, reason_o)
            assert abs(it - it_o) <= 1, (case, it, it_o)
            assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= TOL[precision], case
            its.append(it)
        assert its[-1] <= 1  # the repeated load case is resolved by the projection
        assert its[1] < its[0] and its[2] <= its[1]
    finally:
        B.bddcml_finalize()


def test_recycling_off_and_other_methods_unchanged(built_lib):
    """recycling_int = 0 keeps plain PCG; BiCGSTAB ignores the recycling
    arguments as the reference does."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(5, 3)
    _, it0, *_ = B.solve_problem(prob, precision=1)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        it, reason, _ = B.bddcml_solve(0, 0, 1e-8, 500, 50, 0, 30)
        assert it == it0 and reason == 0
        it1, reason1, cond1 = B.bddcml_solve(0, 1, 1e-8, 500, 50, 1, 30)
        assert reason1 == 0 and cond1 == -1.0
    finally:
        B.bddcml_finalize()
