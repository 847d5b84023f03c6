"""CPU oracle: pinned against the reference's known-answer vectors for the set
operations it uses, against direct sparse solves of the assembled global
system, against structural invariants of the coarse space, and against its own
golden regression fixtures (tests/golden/)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_reference_set_operations_known_answers(oracle_mod):
    """test/test_module_utils.f90:29-47 / :154-166 of the reference."""
    with open(os.path.join(GOLDEN, "reference_utils_known_answers.json")) as f:
        ka = json.load(f)
    inter = oracle_mod.array_intersection(ka["array1"], ka["array2"])
    assert list(inter) == ka["intersection_check"]
    uni = oracle_mod.array_union(ka["array1"], ka["array2"])
    assert list(uni) == ka["union_check"]
    # get_array_norepeat on a sorted array = union with an empty array
    assert list(oracle_mod.array_union(ka["array3"], [])) == ka["array3_check"]


def _direct(prob):
    import scipy.sparse.linalg as spla
    from bddcml_gb300 import problems
    K, f, fixed = problems.global_matrix_and_rhs(prob)
    free = ~fixed
    u = np.zeros(prob.ndof)
    u[free] = spla.spsolve(K[free][:, free].tocsc(), f[free])
    return u


@pytest.mark.parametrize("ne,ns", [(4, 2), (4, 3), (5, 4)])
def test_oracle_matches_direct_solve(oracle_mod, ne, ns):
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-10, 300, 50)
    assert reason == 0
    u = o.global_solution()
    ud = _direct(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-9


def test_oracle_heterogeneous_uneven_matches_direct(oracle_mod):
    from bddcml_gb300 import problems
    boxes = problems.random_box_partition(20, 4, 9, seed=5)
    kappa = problems.lognormal_kappa(20, 1.0, seed=7)
    prob = problems.poisson_boxes(20, boxes, kappa=kappa)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 1)
    it, reason, cond = o.solve(1e-10, 300, 50)
    assert reason == 0
    u = o.global_solution()
    ud = _direct(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-9


def test_coarse_space_hand_count(oracle_mod):
    """2 x 2 x 2 subdomains: 19 corners (1 centre vertex, 6 boundary-edge
    vertices, 12 face-corner selections merged) + 6 edges + 12 faces = 37."""
    from bddcml_gb300 import problems
    o = oracle_mod.Oracle(problems.poisson_on_cube(4, 2))
    o.setup(1, 1, 0)
    st = o.stats()
    assert (st["ncorner"], st["nedge"], st["nface"], st["ndofc"]) == (19, 6, 12, 37)


def test_weights_partition_of_unity(oracle_mod):
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 3, kappa=problems.lognormal_kappa(12, 1.0, seed=1))
    for wt in (0, 1):
        o = oracle_mod.Oracle(prob)
        o.setup(1, 1, wt)
        tot = {}
        cnt = np.zeros(prob.nnod, dtype=int)
        for s in prob.subdomains:
            cnt[s.isngn] += 1
        for s in prob.subdomains:
            w = o.weights(s.isub)
            iface = [g for g in s.isvgvn if cnt[g] > 1]
            for g, wi in zip(iface, w):
                tot[g] = tot.get(g, 0.0) + wi
        assert max(abs(v - 1.0) for v in tot.values()) < 1e-14


def test_zero_rhs_returns_without_iterations(oracle_mod):
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 2)
    for s in prob.subdomains:
        s.rhs[:] = 0.0
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-8, 100, 50)
    assert it == 0 and reason == 0


def test_maxit_reason(oracle_mod):
    """maxit reached -> converged_reason -1 (module_krylov.f90:785-795)."""
    from bddcml_gb300 import problems
    o = oracle_mod.Oracle(problems.poisson_on_cube(5, 4))
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-14, 3, 50)
    assert it == 3 and reason == -1


def test_oracle_golden_regression(oracle_mod):
    from bddcml_gb300 import problems
    with open(os.path.join(GOLDEN, "oracle_small.json")) as f:
        gold = json.load(f)
    specs = {
        "cube_4x2": lambda: problems.poisson_on_cube(4, 2),
        "cube_4x3": lambda: problems.poisson_on_cube(4, 3),
        "cube_5x4": lambda: problems.poisson_on_cube(5, 4),
        "boxes_24_seed17": lambda: problems.poisson_boxes(24, problems.random_box_partition(24, 5, 10, seed=17)),
        "lognormal_16_seed3_w1": lambda: problems.poisson_on_cube(4, 4, kappa=problems.lognormal_kappa(16, 1.0, 3)),
    }
    for name, mk in specs.items():
        g = gold[name]
        o = oracle_mod.Oracle(mk())
        o.setup(1, 1, g["weights_type"])
        it, reason, cond = o.solve(1e-8, 300, 50)
        assert it == g["iterations"] and reason == g["reason"], name
        assert abs(cond - g["cond"]) < 1e-8 * g["cond"], name
        assert o.stats() == g["coarse"], name
        u = o.global_solution()
        assert abs(np.linalg.norm(u) - g["solution_norm2"]) < 1e-10 * g["solution_norm2"], name


def test_oracle_inhomogeneous_dirichlet_matches_direct(oracle_mod):
    """Nonzero boundary values and a varying load: the eliminated Dirichlet
    contributions (module_sm.f90:431-600, module_dd.f90:1081-1256) against a
    direct solve of the assembled system."""
    from bddcml_gb300 import problems
    from newdata_util import changed_data, direct_solution
    prob = changed_data(problems.poisson_on_cube(4, 3), seed=3)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-10, 300, 50)
    assert reason == 0
    u = o.global_solution()
    ud = direct_solution(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-9


def test_oracle_adjoint_gradient_matches_finite_differences(oracle_mod):
    """The differentiation formula dJ/dkappa_e = -lambda_e^T K_e^0 u_e with the
    adjoint solve, against central differences of J = 1/2 |u - u*|^2."""
    from bddcml_gb300 import problems
    from oracle_gradient import objective, oracle_gradient, oracle_solution
    ne, ns = 3, 2
    n = ne * ns
    kappa = problems.lognormal_kappa(n, 1.0, seed=3)
    ustar = problems.smooth_target(n, seed=4)
    _, grad = oracle_gradient(oracle_mod, ne, ns, kappa, ustar)
    rng = np.random.default_rng(11)
    eps = 1e-6
    for _ in range(4):
        d = rng.standard_normal(kappa.size)
        jp = objective(oracle_solution(oracle_mod, problems.poisson_on_cube(ne, ns, kappa=kappa * np.exp(eps * d)))[0],
                       ustar)
        jm = objective(oracle_solution(oracle_mod, problems.poisson_on_cube(ne, ns, kappa=kappa * np.exp(-eps * d)))[0],
                       ustar)
        fd = (jp - jm) / (2 * eps)           # directional derivative along kappa * d
        an = float(np.dot(grad, kappa * d))
        assert abs(fd - an) <= 1e-6 * max(abs(fd), abs(an)), (fd, an)


def test_oracle_elasticity_matches_direct(oracle_mod):
    """Q1 linear elasticity (3 dofs per node, clamped face, body force)."""
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    prob = problems.elasticity_on_cube(3, 2)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-10, 300, 50)
    assert reason == 0
    u = o.global_solution()
    ud = direct_solution(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-9


@pytest.mark.parametrize("method,tol", [(1, 1e-10), (2, 1e-9)])
def test_oracle_bicgstab_and_steepest_descent_match_direct(oracle_mod, method, tol):
    """BiCGSTAB (module_krylov.f90:948-1505) and steepest descent
    (module_krylov.f90:1508-1840) from a non-zero initial guess (the Dirichlet
    values) reach the direct solution; neither estimates a condition number."""
    from bddcml_gb300 import problems
    from newdata_util import changed_data, direct_solution
    prob = changed_data(problems.poisson_on_cube(4, 3), seed=3)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(tol, 400, 50, method=method)
    assert reason == 0 and cond == -1.0 and 0 < it < 400
    u = o.global_solution()
    ud = direct_solution(prob)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e3 * tol


def test_oracle_default_method_is_bicgstab_with_default_parameters(oracle_mod):
    """method -1 ignores the passed tol/maxit/ndecrmax (module_bddcml.f90:515-520)."""
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 3)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_d, reason_d, cond_d = o.solve(1e-14, 2, 1, method=-1)
    hist_d = o.relres_history()
    o2 = oracle_mod.Oracle(prob)
    o2.setup(1, 1, 0)
    it_b, reason_b, _ = o2.solve(1e-6, 1000, 30, method=1)
    assert (it_d, reason_d, cond_d) == (it_b, 0, -1.0) and reason_b == 0
    assert hist_d[-1] < 1e-6 and np.allclose(hist_d, o2.relres_history(), rtol=0, atol=1e-15)


def test_oracle_bicgstab_maxit_reason(oracle_mod):
    from bddcml_gb300 import problems
    o = oracle_mod.Oracle(problems.poisson_on_cube(5, 4))
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-14, 2, 50, method=1)
    assert it == 2 and reason == -1


def test_oracle_dense_eigensolver_matches_numpy(oracle_mod):
    """The oracle's Householder + implicit-QR eigensolver (stands in for
    LAPACK DSYEV/DSYGV of module_adaptivity.f90) on random and degenerate
    symmetric matrices."""
    rng = np.random.default_rng(4)
    for n in (1, 3, 17, 64, 120):
        a = rng.standard_normal((n, n))
        a = a + a.T
        w, z = oracle_mod.sym_eig(a)
        assert np.abs(w - np.linalg.eigvalsh(a)).max() < 1e-12 * max(1.0, np.abs(w).max())
        assert np.abs(z.T @ z - np.eye(n)).max() < 1e-12
        assert np.abs(a @ z - z * w).max() < 1e-11 * max(1.0, np.abs(w).max())
    w, z = oracle_mod.sym_eig(np.diag([3.0, 1.0, 1.0, 2.0]))
    assert np.allclose(w, [1, 1, 2, 3])


def _channel_problem():
    from bddcml_gb300 import problems
    kappa = problems.channel_kappa(15, nchannels=4, width=1, contrast=1e4, sigma=1.0, seed=17)
    return problems.poisson_boxes(15, problems.uniform_boxes(15, 3), kappa=kappa)


def test_oracle_adaptive_constraints(oracle_mod):
    """Adaptive face constraints (module_adaptivity.f90:296-2514,
    module_levels.f90:2826-2938) on a high-contrast channel problem with
    rho-scaling: with an infinite threshold only the face rows are
    orthonormalised, which leaves the preconditioner unchanged; with tau = 10
    the largest pair eigenvalues above tau become constraints, the PCG
    condition number falls below the pair estimate and the solution still
    matches a direct solve."""
    prob = _channel_problem()
    ud = _direct(prob)
    o0 = oracle_mod.Oracle(prob)
    o0.setup(1, 1, 1)
    it0, r0, cond0 = o0.solve(1e-10, 500, 50)
    oi = oracle_mod.Oracle(prob)
    oi.set_adaptive(True, 1e30)
    oi.setup(1, 1, 1)
    iti, ri, condi = oi.solve(1e-10, 500, 50)
    info_i = oi.adaptive_info()
    assert len(info_i["pairs"]) == 54 and info_i["nadaptive"].sum() == 0
    assert (info_i["face_ncdof"] == 1).all()
    assert abs(iti - it0) <= 1 and abs(condi - cond0) <= 1e-6 * cond0
    oa = oracle_mod.Oracle(prob)
    oa.set_adaptive(True, 10.0)
    oa.setup(1, 1, 1)
    ita, ra, conda = oa.solve(1e-10, 500, 50)
    info = oa.adaptive_info()
    assert ra == 0 and info["nadaptive"].sum() > 0
    assert ita < 0.7 * it0 and conda < 0.1 * cond0
    assert conda <= 1.05 * info["est"] and info["est"] < 10.0
    eigs = info["eigs"]
    for p in range(len(eigs)):
        k = info["neig"][p]
        assert (np.diff(eigs[p, :k]) <= 1e-12 * max(1.0, eigs[p, 0])).all()  # descending
        assert info["nadaptive"][p] == (eigs[p, :k] >= 10.0).sum()
    err = np.linalg.norm(oa.global_solution() - ud) / np.linalg.norm(ud)
    assert err < 1e-9


def test_oracle_krylov_recycling(oracle_mod):
    """PCG with Krylov recycling (module_krylov.f90:313-484, 663-726) over
    consecutive load cases on one preconditioner: every solution matches a
    direct solve, the stored S-orthonormal basis grows by the iterations of
    each solve up to its capacity, and solving the same loads again needs no
    iteration after the projection."""
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    prob = problems.poisson_boxes(15, problems.uniform_boxes(15, 3), kappa=problems.lognormal_kappa(15, 1.0, 3))
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 1)
    rng = np.random.default_rng(2)
    its, total = [], 0
    for case in range(3):
        if case > 0:
            load = rng.uniform(0.5, 1.5, prob.ndof)
            for s in prob.subdomains:
                s.rhs = np.where(s.ifix != 0, 0.0, load[s.isvgvn] / prob.n_el_edge ** 3)
                o.new_loads(s.isub, s.rhs)
        it, reason, cond = o.solve_recycling(1e-10, 300, 50, True, 40)
        assert reason == 0
        total += it
        its.append(it)
        assert o.recycling_size() == min(40, total)
        ud = direct_solution(prob)
        assert np.linalg.norm(o.global_solution() - ud) / np.linalg.norm(ud) < 1e-8
    for s in prob.subdomains:  # the same loads again, from a zero initial guess
        o.new_loads(s.isub, s.rhs)
    it, reason, cond = o.solve_recycling(1e-10, 300, 50, True, 40)
    assert reason == 0 and it <= 1


def test_oracle_reactions_balance_the_loads(oracle_mod):
    """Reactions (dd_compute_reactions, module_dd.f90:1258-1374) on the fixed
    dofs are K u - f there.  The Q1 Laplace matrix has zero row sums, so they
    sum to minus the total load; they also equal K u - f of the assembled
    global system at every fixed dof."""
    from bddcml_gb300 import problems
    from newdata_util import changed_data
    prob = changed_data(problems.poisson_on_cube(4, 3), seed=5)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-12, 300, 50)
    assert reason == 0
    u = o.global_solution()
    rea = o.global_reactions()
    fixed = np.zeros(prob.ndof, dtype=bool)
    f = np.zeros(prob.ndof)
    for s in prob.subdomains:
        fixed[s.isvgvn[s.ifix != 0]] = True
        f[s.isvgvn] = s.rhs  # loads are given complete at shared dofs
    import scipy.sparse as sp
    rows, cols, vals = [], [], []
    for s in prob.subdomains:
        g = s.isvgvn
        rows.append(g[s.i_sparse]); cols.append(g[s.j_sparse]); vals.append(s.a_sparse)
        off = s.i_sparse != s.j_sparse
        rows.append(g[s.j_sparse[off]]); cols.append(g[s.i_sparse[off]]); vals.append(s.a_sparse[off])
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(prob.ndof, prob.ndof))
    r_true = K @ u - f
    assert np.abs(rea[fixed] - r_true[fixed]).max() <= 1e-9 * np.abs(r_true[fixed]).max()
    assert abs(rea[fixed].sum() + f.sum()) <= 1e-9 * np.abs(f).sum()


@pytest.mark.parametrize("ne,ns,b", [(3, 2, (10.0, 7.0, 4.0)), (4, 3, (20.0, 10.0, 5.0)), (5, 2, (30.0, -12.0, 6.0))])
def test_oracle_nonsymmetric_matches_direct(oracle_mod, ne, ns, b):
    """matrixtype 0 (convection-diffusion, full element matrices): LU factors,
    the dual coarse basis of the adjoint problem (module_dd.f90:5687-5757) for
    the restriction, Phi_dual^T A Phi as local coarse matrix; BiCGSTAB matches
    the direct solve of the assembled nonsymmetric system."""
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    prob = problems.convection_diffusion_on_cube(ne, ns, b)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, _ = o.solve(1e-10, 500, 50, method=1)
    u = o.global_solution()
    ud = direct_solution(prob)
    assert reason == 0 and it <= 20
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-9


def test_oracle_nonsymmetric_inhomogeneous_dirichlet(oracle_mod):
    """Fixed columns of a general matrix go into the rhs, fixed rows do not
    (module_sm.f90:528-560): nonzero boundary values match the direct solve."""
    from bddcml_gb300 import problems
    from newdata_util import direct_solution
    prob = problems.convection_diffusion_on_cube(3, 2)
    for s in prob.subdomains:
        x = s.xyz
        g = 1.0 + x[0] + 2.0 * x[1] * x[2]
        s.fixv = np.where(s.ifix != 0, g, 0.0)
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it, reason, _ = o.solve(1e-10, 500, 50, method=1)
    u = o.global_solution()
    ud = direct_solution(prob)
    assert reason == 0
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-9
