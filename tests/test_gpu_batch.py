"""Batched loads through bddcml_upload_subdomain_rhs_batch_c /
bddcml_solve_batch_c: every column is checked against the oracle solving that
load alone (bddcml_change_subdomain_data + bddcml_setup_new_data semantics,
module_levels.f90:785-853, then krylov_bddcpcg, module_krylov.f90:545-888,
from the zero initial guess).  Per column: the same stop reason, iterations
within +-1 of the oracle's, solution within 1e-8 (FP64) / 1e-7 (mixed) of it.
Two and three levels, padded batches (nrhs not a power of two), a zero load,
the maximum batch of 64, and the single-load state after a batched solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


def _loads(prob, nrhs, seed, zero_column=None):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nrhs):
        g = rng.standard_normal(prob.ndof) if k != zero_column else np.zeros(prob.ndof)
        out.append(g)
    return out


def _subdomain_rhs(prob, s, g):
    return np.where(s.ifix != 0, 0.0, g[s.isvgvn])


def _batch_solve(prob, precision, loads, levels=2, nsub2=1, tol=1e-8, maxit=500, operator=None):
    import bddcml_gb300 as B
    nrhs = len(loads)
    if levels == 2:
        B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    else:
        B.bddcml_init(3, [prob.nsub, nsub2, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(precision)
        if operator is not None:
            B.set_batch_operator(operator)
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(prob.matrixtype, 0, 1, 1, 1, 0, 0, 0)
        for s in prob.subdomains:
            B.bddcml_upload_subdomain_rhs_batch(s.isub, np.stack([_subdomain_rhs(prob, s, g) for g in loads]), 1)
        it, reason, cond = B.bddcml_solve_batch(nrhs, 0, 0, tol, maxit, 50)
        u = np.zeros((nrhs, prob.ndof))
        for s in prob.subdomains:
            u[:, s.isvgvn] = B.bddcml_download_local_solution_batch(s.isub, nrhs, s.ndofs)
        # the subdomains' own loads are still the single-load problem
        it1, reason1, _ = B.bddcml_solve(0, 0, tol, maxit, 50, 0, 0)
        u1 = np.zeros(prob.ndof)
        for s in prob.subdomains:
            u1[s.isvgvn] = B.bddcml_download_local_solution(s.isub, s.ndofs)
    finally:
        B.bddcml_finalize()
    return u, it, reason, cond, (u1, it1, reason1)


def _oracle_columns(oracle_mod, prob, loads, levels=2, nsub2=1):
    o = oracle_mod.Oracle(prob)
    if levels == 3:
        o.set_levels(3, nsub2)
    o.setup(1, 1, 0)
    it_s, _, _ = o.solve(1e-8, 500, 50)
    u_s = o.global_solution()
    res = []
    for g in loads:
        for s in prob.subdomains:
            o.new_loads(s.isub, _subdomain_rhs(prob, s, g))
        it, reason, cond = o.solve(1e-8, 500, 50)
        res.append((o.global_solution(), it, reason, cond))
    return res, (u_s, it_s)


def _check(u, it, reason, ref, precision, zero_column=None):
    for k, (uo, it_o, reason_o, _) in enumerate(ref):
        if k == zero_column:
            assert it[k] == 0 and np.abs(u[k]).max() == 0.0
            continue
        assert reason[k] == reason_o == 0, (k, reason[k], reason_o)
        assert abs(int(it[k]) - it_o) <= 1, (k, it[k], it_o)
        err = np.linalg.norm(u[k] - uo) / np.linalg.norm(uo)
        assert err <= TOL[precision], (k, err)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_two_levels_matches_oracle(built_lib, oracle_mod, precision):
    from bddcml_gb300 import problems
    prob = problems.poisson_boxes(15, problems.uniform_boxes(15, 3), kappa=problems.lognormal_kappa(15, 1.0, 3))
    loads = _loads(prob, 5, seed=11, zero_column=3)
    u, it, reason, cond, (u1, it1, reason1) = _batch_solve(prob, precision, loads)
    ref, (u_s, it_s) = _oracle_columns(oracle_mod, prob, loads)
    print(f"precision {precision}: iterations {list(it)} oracle {[r[1] for r in ref]}")
    _check(u, it, reason, ref, precision, zero_column=3)
    for k in (0, 1, 2, 4):
        assert cond[k] > 1.0 and abs(cond[k] - ref[k][3]) <= 0.05 * ref[k][3]
    assert reason1 == 0 and abs(it1 - it_s) <= 1
    assert np.linalg.norm(u1 - u_s) / np.linalg.norm(u_s) <= TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_three_levels_elasticity_matches_oracle(built_lib, oracle_mod, precision):
    from bddcml_gb300 import problems
    prob = problems.elasticity_on_cube(3, 4)
    loads = _loads(prob, 3, seed=5)
    u, it, reason, cond, _ = _batch_solve(prob, precision, loads, levels=3, nsub2=8)
    ref, _ = _oracle_columns(oracle_mod, prob, loads, levels=3, nsub2=8)
    print(f"precision {precision}: iterations {list(it)} oracle {[r[1] for r in ref]}")
    _check(u, it, reason, ref, precision)


def test_batch_of_64_matches_single_solves(built_lib, oracle_mod):
    """The largest batch, on a small problem: every column against the oracle."""
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 3)
    loads = _loads(prob, 64, seed=23)
    u, it, reason, cond, _ = _batch_solve(prob, 1, loads)
    ref, _ = _oracle_columns(oracle_mod, prob, loads)
    _check(u, it, reason, ref, 1)


def test_batch_argument_errors(built_lib):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(3, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        s0 = prob.subdomains[0]
        B.bddcml_upload_subdomain_rhs_batch(s0.isub, np.ones((2, s0.ndofs)))
        with pytest.raises(B.BddcmlError) as e:  # other subdomains have no batch
            B.bddcml_solve_batch(2, 0, 0, 1e-8, 100, 50)
        assert e.value.code == 1
        for s in prob.subdomains:
            B.bddcml_upload_subdomain_rhs_batch(s.isub, np.ones((2, s.ndofs)))
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_solve_batch(2, 0, 1, 1e-8, 100, 50)
        assert e.value.code == 4
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_download_local_solution_batch(s0.isub, 2, s0.ndofs)
        assert e.value.code == 1
        it, reason, _ = B.bddcml_solve_batch(2, 0, 0, 1e-8, 100, 50)
        assert list(reason) == [0, 0] and it[0] == it[1] > 0
        a = B.bddcml_download_local_solution_batch(s0.isub, 2, s0.ndofs)
        assert np.array_equal(a[0], a[1])
    finally:
        B.bddcml_finalize()


@pytest.mark.parametrize("levels", [2, 3])
def test_batch_operators_agree(built_lib, oracle_mod, levels):
    """Mixed precision with the double-float SIMT Schur apply (operator 0), the
    sliced bf16 tensor-core Schur apply with 3xTF32 preconditioner products
    (operator 1) and with sliced preconditioner products (operator 2): all
    match the oracle per column, and their solutions agree far below the
    solver tolerance."""
    from bddcml_gb300 import problems
    if levels == 2:
        prob, nsub2 = problems.poisson_boxes(15, problems.uniform_boxes(15, 3),
                                             kappa=problems.lognormal_kappa(15, 1.0, 3)), 1
    else:
        prob, nsub2 = problems.elasticity_on_cube(3, 4), 8
    loads = _loads(prob, 6, seed=31)
    ref, _ = _oracle_columns(oracle_mod, prob, loads, levels=levels, nsub2=nsub2)
    res = {}
    for op in (0, 1, 2):
        u, it, reason, cond, _ = _batch_solve(prob, 1, loads, levels=levels, nsub2=nsub2, operator=op)
        _check(u, it, reason, ref, 1)
        res[op] = (u, it)
    print(f"levels {levels}: iterations " + " ".join(f"op{op} {list(res[op][1])}" for op in res))
    for op in (1, 2):
        assert np.max(np.abs(res[0][1] - res[op][1])) <= 1
        for k in range(len(loads)):
            d = np.linalg.norm(res[0][0][k] - res[op][0][k]) / np.linalg.norm(res[0][0][k])
            assert d <= 1e-8, (op, k, d)
