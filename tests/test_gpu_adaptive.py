"""Adaptive face constraints through the C ABI against the oracle
(module_adaptivity.f90:296-2514, module_levels.f90:2826-2938).

The GPU computes the face-pair eigenpairs with batched LOBPCG (15 iterations,
FP32 products with S and Z, FP64 Rayleigh-Ritz); the oracle solves the same
pencils exactly.  Checked: the eigenvalues above the threshold (relative 1e-3),
the number of constraints they give, and the PCG iteration count (+-2) and
solution (1e-8 FP64 / 1e-7 mixed) of the resulting preconditioner.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-8, 1: 1e-7}


def _problem():
    from bddcml_gb300 import problems
    kappa = problems.channel_kappa(15, nchannels=4, width=1, contrast=1e4, sigma=1.0, seed=17)
    return problems.poisson_boxes(15, problems.uniform_boxes(15, 3), kappa=kappa)


def _oracle(oracle_mod, prob, tau):
    o = oracle_mod.Oracle(prob)
    if tau is not None:
        o.set_adaptive(True, tau)
    o.setup(1, 1, 1)
    it, reason, cond = o.solve(1e-8, 300, 50)
    return o, it, reason, cond


@pytest.mark.parametrize("precision", [0, 1])
def test_adaptive_parity(built_lib, oracle_mod, precision):
    import bddcml_gb300 as B
    prob = _problem()
    tau = 10.0
    o, it_o, reason_o, cond_o = _oracle(oracle_mod, prob, tau)
    info_o = o.adaptive_info()
    u_o = o.global_solution()
    u, it, reason, cond, st = B.solve_problem(prob, precision=precision, tol=1e-8, maxit=300, ndecrmax=50,
                                              weights_type=1, adaptive_tau=tau, finalize=False)
    try:
        info = B.get_adaptive_info()
    finally:
        B.bddcml_finalize()
    assert len(info["pairs"]) == len(info_o["pairs"]) == 54
    ref = {(int(a), int(b)): p for p, (f, a, b) in enumerate(info_o["pairs"])}
    worst = 0.0
    nad = 0
    for p, (a, b) in enumerate(info["pairs"]):
        q = ref[(int(a), int(b))]
        k = info["k"][p]
        assert k == info_o["neig"][q]
        eo = info_o["eigs"][q, :k]
        eg = info["eigs"][p, :k]
        sel = eo >= 0.5 * tau
        if sel.any():
            worst = max(worst, float(np.max(np.abs(eg[sel] - eo[sel]) / eo[sel])))
        nad += int((eg >= tau).sum())
    print(f"precision {precision}: worst eigenvalue error {worst:.2e}, constraints {nad} "
          f"(oracle {info_o['nadaptive'].sum()}), iterations {it} (oracle {it_o}), "
          f"lobpcg residual {st['lobpcg_resid']:.1e}, est {st['adapt_est']:.3g} (oracle {info_o['est']:.3g})")
    assert worst <= 1e-3
    assert nad == info_o["nadaptive"].sum() == st["nadaptive"]
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert err <= TOL[precision], err


def test_adaptive_infinite_threshold_keeps_the_standard_preconditioner(built_lib, oracle_mod):
    """With no eigenvalue above the threshold only the face rows are
    orthonormalised: iterations equal those without adaptivity (+-1)."""
    import bddcml_gb300 as B
    prob = _problem()
    u0, it0, r0, c0, _ = B.solve_problem(prob, precision=1, tol=1e-8, maxit=300, ndecrmax=50, weights_type=1)
    u1, it1, r1, c1, st = B.solve_problem(prob, precision=1, tol=1e-8, maxit=300, ndecrmax=50, weights_type=1,
                                          adaptive_tau=1e30)
    assert st["nadaptive"] == 0 and st["npair"] == 54
    assert abs(it1 - it0) <= 1 and abs(c1 - c0) <= 1e-3 * c0
    assert np.linalg.norm(u1 - u0) / np.linalg.norm(u0) <= 1e-7
