"""Bounded waits of the tensor-core sweeps (failure detection without a GPU
fault).  With a spin limit of one poll, the first wait of every sweep CTA runs
out: the CTA drains its bulk copies in flight, frees its tensor memory and
records the timeout, and the setup fails with BDDCML_ERR_NUMERIC instead of
hanging.  With the default limit restored, the same process then sets up and
solves normally, and the result matches the oracle.  The reference has no
such path: its errors abort the process (module_utils.f90:296-298)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sweep_wait_timeout_is_reported_and_recoverable(built_lib, oracle_mod):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.set_precision(1)  # the sweeps run in the mixed-precision setup
        B.upload_problem(prob)
        B.set_wait_limit(1)
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        assert e.value.code == 3
        assert "bounded wait" in str(e.value)
    finally:
        B.set_wait_limit(0)
        B.bddcml_finalize()
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_o, _, _ = o.solve(1e-8, 200, 50)
    u_o = o.global_solution()
    u, it, reason, cond, st = B.solve_problem(prob, precision=1, tol=1e-8, maxit=200, ndecrmax=50)
    assert reason == 0 and abs(it - it_o) <= 2
    assert np.linalg.norm(u - u_o) <= 1e-7 * np.linalg.norm(u_o)
