"""Allocation-free subdomain dot product on device-resident vectors.

bddcml_dotprod_subdomain_dev_c must give the weighted subdomain dot product of
bddcml_dotprod_subdomain_c (module_dd.f90:12736-12788) for the same vectors held
in device memory, on consecutive calls, and reject a wrong length with a status.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dotprod_dev_matches_host_entry_point(built_lib):
    torch = pytest.importorskip("torch")
    import bddcml_gb300 as B
    from bddcml_gb300 import problems

    prob = problems.poisson_on_cube(4, 3)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        rng = np.random.default_rng(5)
        for isub in (0, prob.nsub // 2, prob.nsub - 1):
            n = prob.subdomains[isub].ndofs
            for _ in range(2):  # two calls in a row on fresh vectors
                v1 = rng.standard_normal(n)
                v2 = rng.standard_normal(n)
                ref = B.bddcml_dotprod_subdomain(isub, v1, v2)
                d1 = torch.from_numpy(v1).cuda()
                d2 = torch.from_numpy(v2).cuda()
                torch.cuda.synchronize()
                got = B.dotprod_subdomain_dev(isub, d1.data_ptr(), d2.data_ptr(), n)
                scale = float(np.dot(np.abs(v1), np.abs(v2)))
                assert abs(got - ref) <= 1e-12 * scale, (isub, got, ref)
        # after the first call (which loads the static scratch on the device),
        # further calls leave the free device memory unchanged
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        last = prob.nsub - 1  # d1 and d2 hold vectors of this subdomain
        for _ in range(5):
            B.dotprod_subdomain_dev(last, d1.data_ptr(), d2.data_ptr(), prob.subdomains[last].ndofs)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        with pytest.raises(B.BddcmlError):
            B.dotprod_subdomain_dev(0, d1.data_ptr(), d2.data_ptr(), prob.subdomains[0].ndofs + 1)
    finally:
        B.bddcml_finalize()
