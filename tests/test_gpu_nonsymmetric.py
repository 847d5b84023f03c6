"""General (nonsymmetric, matrixtype 0) matrices through the C ABI: LU
factors of the interior and preconditioner blocks, the dual coarse basis of
the adjoint problem for the restriction (module_dd.f90:5687-5757, 6126-6206),
a general coarse problem, BiCGSTAB (module_krylov.f90:948-1505).  Checked
against the oracle restatement (iterations +-2, solution within 1e-8 in FP64
and 1e-7 in mixed precision) and a direct solve of the assembled system."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


def _run(prob, precision, tol=1e-10, method=1, weights=0):
    import bddcml_gb300 as B
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(precision)
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(0, 0, 1, 1, 1, 0, 0, weights)
        it, reason, cond = B.bddcml_solve(0, method, tol, 500, 50, 0, 0)
        u = np.zeros(prob.ndof)
        for s in prob.subdomains:
            u[s.isvgvn] = B.bddcml_download_local_solution(s.isub, s.ndofs)
    finally:
        B.bddcml_finalize()
    return u, it, reason


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", [(3, 2, (10.0, 7.0, 4.0)), (4, 3, (20.0, 10.0, 5.0)), (8, 2, (24.0, -9.0, 6.0))])
def test_nonsymmetric_matches_oracle(built_lib, oracle_mod, precision, case):
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    ne, ns, b = case
    prob = problems.convection_diffusion_on_cube(ne, ns, b)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_o, reason_o, _ = o.solve(1e-10, 500, 50, method=1)
    u_o = o.global_solution()
    u, it, reason = _run(prob, precision)
    print(f"{prob.name} precision {precision}: iterations {it} (oracle {it_o})")
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= TOL[precision]
    ud = direct_solution(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-7


def test_nonsymmetric_inhomogeneous_dirichlet(built_lib, oracle_mod):
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    prob = problems.convection_diffusion_on_cube(4, 2)
    for s in prob.subdomains:
        x = s.xyz
        s.fixv = np.where(s.ifix != 0, 1.0 + x[0] + 2.0 * x[1] * x[2], 0.0)
    u, it, reason = _run(prob, 1)
    ud = direct_solution(prob)
    assert reason == 0
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-7


def test_nonsymmetric_unsupported_paths(built_lib):
    """Three levels, adaptive constraints, batched loads and reactions are
    built for symmetric matrices; a general matrix gets BDDCML_ERR_UNSUPPORTED."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.convection_diffusion_on_cube(3, 2)
    B.bddcml_init(3, [prob.nsub, 2, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_setup_preconditioner(0, 0, 1, 1, 1, 0, 0, 0)
        assert e.value.code == 4
    finally:
        B.bddcml_finalize()
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_setup_preconditioner(0, 0, 1, 1, 1, 1, 0, 0)
        assert e.value.code == 4
        B.bddcml_setup_preconditioner(0, 0, 1, 1, 1, 0, 0, 0)
        B.bddcml_solve(0, 1, 1e-8, 200, 50, 0, 0)
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_download_local_reactions(prob.subdomains[0].isub, prob.subdomains[0].ndofs)
        assert e.value.code == 4
        for s in prob.subdomains:
            B.bddcml_upload_subdomain_rhs_batch(s.isub, np.ones((2, s.ndofs)))
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_solve_batch(2, 0, 0, 1e-8, 100, 50)
        assert e.value.code == 4
    finally:
        B.bddcml_finalize()
