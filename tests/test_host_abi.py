"""C ABI and host-side logic without a GPU: the library loads and exports every
entry point the header declares, the integer/geometric setup (interface,
globs, corners, coarse numbering, weights) equals the oracle's, and errors are
reported through status codes instead of aborting."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    with open(os.path.join(ROOT, "include", "bddcml_gb300.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^\s*(?:void|int)\s+(bddcml_\w+)\s*\(", src, re.M)))


def test_exports_every_header_symbol(built_lib):
    lib = C.CDLL(built_lib)
    syms = header_symbols()
    assert len(syms) >= 22
    for name in syms:
        assert hasattr(lib, name), name
    import bddcml_gb300 as B
    assert sorted(B.EXPORTS) == syms


def test_reference_signatures_present():
    """Every function of the reference header src/bddcml_interface_c.h is
    declared with the same argument list."""
    with open(os.path.join(ROOT, "include", "bddcml_gb300.h")) as f:
        src = f.read()
    for name, nargs in [("bddcml_init_c", 8), ("bddcml_upload_global_data_c", 25),
                        ("bddcml_upload_subdomain_data_c", 50), ("bddcml_setup_preconditioner_c", 8),
                        ("bddcml_solve_c", 10), ("bddcml_download_local_solution_c", 3),
                        ("bddcml_download_global_solution_c", 2), ("bddcml_download_local_reactions_c", 3),
                        ("bddcml_download_global_reactions_c", 2), ("bddcml_change_global_data_c", 8),
                        ("bddcml_change_subdomain_data_c", 10), ("bddcml_setup_new_data_c", 0),
                        ("bddcml_dotprod_subdomain_c", 6), ("bddcml_finalize_c", 0)]:
        m = re.search(name + r"\s*\(([^)]*)\)", src)
        assert m, name
        args = [a for a in m.group(1).split(",") if a.strip() and a.strip() != "void"]
        assert len(args) == nargs, (name, len(args))


@pytest.mark.parametrize("ne,ns,numbase", [(4, 2, 0), (4, 3, 1), (5, 4, 0)])
def test_host_coarse_space_equals_oracle(built_lib, oracle_mod, ne, ns, numbase):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(ne, ns)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, numbase, 0)
    B.upload_problem(prob, numbase=numbase)
    try:
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
    except B.BddcmlError as e:  # no GPU in this container: the host part has run
        assert e.code == 2
    info = B.get_coarse_info()
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    assert info == o.stats()
    for s in prob.subdomains:
        w_o = o.weights(s.isub)
        w_g = B.get_interface_weights(s.isub + numbase, len(w_o))
        assert np.array_equal(w_o, w_g)
    B.bddcml_finalize()


def test_host_uneven_partition_stiffness_weights(built_lib, oracle_mod):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_boxes(24, problems.random_box_partition(24, 5, 10, seed=17),
                                  kappa=problems.lognormal_kappa(24, 1.0, seed=2))
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    B.upload_problem(prob)
    try:
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 1)
    except B.BddcmlError as e:
        assert e.code == 2
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 1)
    assert B.get_coarse_info() == o.stats()
    for s in prob.subdomains:
        w_o = o.weights(s.isub)
        assert np.array_equal(w_o, B.get_interface_weights(s.isub, len(w_o)))
    B.bddcml_finalize()


def test_errors_are_status_codes(built_lib):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    with pytest.raises(B.BddcmlError) as ei:
        B.bddcml_init(1, [1], -1, 0, 0, 0, 0)         # fewer than 2 levels
    assert ei.value.code == 1
    with pytest.raises(B.BddcmlError) as ei:
        B.bddcml_init(2, [4, 2], -1, 0, 0, 0, 0)      # last level must have 1 subdomain
    assert ei.value.code == 1
    prob = problems.poisson_on_cube(4, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    s = prob.subdomains[0]
    bad_i = s.i_sparse.copy()
    bad_i[0], bad_j = s.j_sparse[0] + 1, s.j_sparse.copy()
    with pytest.raises(B.BddcmlError) as ei:              # lower-triangle entry for a symmetric matrix
        B.bddcml_upload_subdomain_data(prob.nelem, prob.nnod, prob.ndof, 3, 3, 0, s.nelems, s.nnods, s.ndofs,
                                       s.inet, s.nnet, s.nndf, s.isngn, s.isvgvn, s.isegn, s.xyz, s.ifix, s.fixv,
                                       s.rhs, 1, s.sol, 1, bad_i, bad_j, s.a_sparse, 0)
    assert ei.value.code == 1
    with pytest.raises(B.BddcmlError) as ei:              # solve before setup
        B.bddcml_solve(0, 0, 1e-8, 10, 10, 0, 0)
    assert ei.value.code == 1
    with pytest.raises(B.BddcmlError) as ei:              # subdomain not uploaded
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
    assert ei.value.code == 1
    with pytest.raises(B.BddcmlError) as ei:
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 1, 0, 0)  # adaptive constraints
    assert ei.value.code in (1, 4)
    # changing global data without global loading is reported unsupported, not aborted
    z = np.zeros(prob.ndof)
    with pytest.raises(B.BddcmlError) as ei:
        B.bddcml_change_global_data(np.zeros(prob.ndof, dtype=np.int32), z, z, z)
    assert ei.value.code == 4
    B.bddcml_finalize()
    # the global solution needs an initialised solver
    B.lib().bddcml_download_global_solution_c(None, None)
    assert B.last_error()[0] == 1


def test_general_matrix_indices_checked_on_both_bounds(built_lib):
    """General storage (matrixtype 0) allows row > column, so a row index past
    ndofs or a negative column index must be caught by the range check itself."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.convection_diffusion_on_cube(3, 2)
    s = prob.subdomains[0]
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        for which, value in (("i", s.ndofs), ("j", -1)):
            bi, bj = s.i_sparse.copy(), s.j_sparse.copy()
            (bi if which == "i" else bj)[7] = value
            with pytest.raises(B.BddcmlError) as ei:
                B.bddcml_upload_subdomain_data(prob.nelem, prob.nnod, prob.ndof, 3, 3, 0, s.nelems, s.nnods,
                                               s.ndofs, s.inet, s.nnet, s.nndf, s.isngn, s.isvgvn, s.isegn, s.xyz,
                                               s.ifix, s.fixv, s.rhs, 1, s.sol, 0, bi, bj, s.a_sparse, 0)
            assert ei.value.code == 1 and "out of range" in str(ei.value)
        B.bddcml_upload_subdomain_data(prob.nelem, prob.nnod, prob.ndof, 3, 3, 0, s.nelems, s.nnods, s.ndofs,
                                       s.inet, s.nnet, s.nndf, s.isngn, s.isvgvn, s.isegn, s.xyz, s.ifix, s.fixv,
                                       s.rhs, 1, s.sol, 0, s.i_sparse, s.j_sparse, s.a_sparse, 0)
    finally:
        B.bddcml_finalize()


def test_zero_weight_denominator_is_a_status(built_lib):
    """Stiffness weights (weights_type 1) of a subdomain whose matrix was negated
    cancel those of its neighbour on the dofs the two share alone: the setup
    reports a numeric error (status 3) instead of aborting the process."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(2, 2)
    prob.subdomains[0].a_sparse = -prob.subdomains[0].a_sparse
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        with pytest.raises(B.BddcmlError) as ei:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 1)
        assert ei.value.code == 3 and "zero denominator" in str(ei.value)
    finally:
        B.bddcml_finalize()


def test_setup_without_gpu_reports_an_error(built_lib):
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(4, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    B.upload_problem(prob)
    with pytest.raises(B.BddcmlError):
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)  # no GPU here -> CUDA error after host setup
    B.bddcml_finalize()


def test_host_coarse_space_equals_oracle_elasticity(built_lib, oracle_mod):
    """Three dofs per node: corners carry three coarse dofs, edge and face
    averages one per component (module_dd.f90:4298-4384)."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.elasticity_on_cube(3, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    B.upload_problem(prob)
    try:
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
    except B.BddcmlError as e:  # no GPU in this container: the host part has run
        assert e.code == 2
    info = B.get_coarse_info()
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    assert info == o.stats()
    assert info["ndofc"] == 3 * (info["ncorner"] + info["nedge"] + info["nface"])
    for s in prob.subdomains:
        w_o = o.weights(s.isub)
        assert np.array_equal(w_o, B.get_interface_weights(s.isub, len(w_o)))
    B.bddcml_finalize()


def test_batch_upload_validation_without_gpu(built_lib):
    """bddcml_upload_subdomain_rhs_batch_c checks its sizes on the host; the
    batched solve and download refuse to run before a setup / batched solve."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(3, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        s = prob.subdomains[0]
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_upload_subdomain_rhs_batch(s.isub, np.zeros((65, s.ndofs)))
        assert e.value.code == 1
        lib = B.lib()
        r = np.zeros(2 * s.ndofs - 1)
        lib.bddcml_upload_subdomain_rhs_batch_c(C.byref(C.c_int(s.isub)), C.byref(C.c_int(2)),
                                                r.ctypes.data_as(C.POINTER(C.c_double)),
                                                C.byref(C.c_int(r.size)), C.byref(C.c_int(1)))
        assert B.last_error()[0] == 1
        B.bddcml_upload_subdomain_rhs_batch(s.isub, np.ones((3, s.ndofs)))
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_solve_batch(3)
        assert e.value.code == 1
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_download_local_solution_batch(s.isub, 3, s.ndofs)
        assert e.value.code == 1
    finally:
        B.bddcml_finalize()


def test_host_general_matrix_upload_and_coarse_space(built_lib, oracle_mod):
    """matrixtype 0 uploads full element matrices (no upper-triangle check); the
    coarse space does not depend on symmetry and equals the oracle's."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.convection_diffusion_on_cube(3, 2)
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        with pytest.raises(B.BddcmlError) as e:  # the uploads say general, the setup says SPD
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        assert e.value.code == 1
        try:
            B.bddcml_setup_preconditioner(0, 0, 1, 1, 1, 0, 0, 0)
        except B.BddcmlError as e:  # no GPU in this container: the host part has run
            assert e.code == 2
        o = oracle_mod.Oracle(prob)
        o.setup(1, 1, 0)
        assert B.get_coarse_info() == o.stats()
    finally:
        B.bddcml_finalize()


def test_interior_band_of_dirichlet_subdomains(built_lib):
    """The fixed dofs of a Dirichlet face are interior dofs whose couplings were
    removed (explicit zeros); the interior ordering leaves them out of the band,
    so every 16^3 subdomain of the cube, with or without Dirichlet faces, has
    block bandwidth 4 (64-row blocks over 15^3 coupled nodes) instead of 5."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(16, 3)  # corner, edge, face and interior subdomains
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        try:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        except B.BddcmlError as e:  # no GPU in this container: the host part has run
            assert e.code == 2
        assert B.get_stats()["band_w"] == 4
    finally:
        B.bddcml_finalize()


def _merged_subdomain(parts, isub):
    """One subdomain holding the elements of several box subdomains (local
    numbering in ascending global node id)."""
    from bddcml_gb300 import problems
    g = np.unique(np.concatenate([s.isngn for s in parts]))
    n = len(g)

    def loc(s, a):
        return np.searchsorted(g, s.isngn[a]).astype(np.int32)
    xyz, ifix, rhs = np.zeros((3, n)), np.zeros(n, np.int32), np.zeros(n)
    for s in parts:
        idx = loc(s, np.arange(s.nnods))
        xyz[:, idx], ifix[idx], rhs[idx] = s.xyz, s.ifix, s.rhs
    cat = np.concatenate
    return problems.Subdomain(
        isub=isub, nelems=sum(s.nelems for s in parts), nnods=n, ndofs=n, inet=cat([loc(s, s.inet) for s in parts]),
        nnet=cat([s.nnet for s in parts]), nndf=np.ones(n, np.int32), isngn=g.astype(np.int32),
        isvgvn=g.astype(np.int32), isegn=cat([s.isegn for s in parts]), xyz=xyz, ifix=ifix, fixv=np.zeros(n),
        rhs=rhs, sol=np.zeros(n), i_sparse=cat([loc(s, s.i_sparse) for s in parts]),
        j_sparse=cat([loc(s, s.j_sparse) for s in parts]), a_sparse=cat([s.a_sparse for s in parts]))


def test_host_coarse_space_of_disconnected_subdomains(built_lib, oracle_mod):
    """The 27 boxes of a 6^3 cube regrouped by (x + y + z) parity and z layer:
    most subdomains are boxes that touch only along edges, so their dual mesh
    graph (elements sharing 3 nodes) falls into up to 5 components.  Globs are
    split by component (module_dd.f90:2680-2720, 9160-9175); the coarse space
    and the weights equal the oracle's."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(2, 3)
    groups = {}
    for k, s in enumerate(prob.subdomains):
        groups.setdefault(((k % 3 + (k // 3) % 3 + k // 9) % 2, k // 9), []).append(s)
    prob.subdomains = [_merged_subdomain(v, i) for i, v in enumerate(groups.values())]
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        try:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        except B.BddcmlError as e:  # no GPU in this container: the host part has run
            assert e.code == 2
        info = B.get_coarse_info()
        o = oracle_mod.Oracle(prob)
        o.setup(1, 1, 0)
        assert info == o.stats()
        assert info["nedge"] > 0 and info["ncorner"] > 8 * prob.nsub
        for s in prob.subdomains:
            w_o = o.weights(s.isub)
            assert np.array_equal(w_o, B.get_interface_weights(s.isub, len(w_o)))
    finally:
        B.bddcml_finalize()


def test_mesh_indices_checked_at_upload(built_lib):
    """INET must index the subdomain's own nodes and the global numbers must not
    be negative: a bad entry is a status 1 at upload, not a bad access at setup."""
    import bddcml_gb300 as B
    from bddcml_gb300 import problems
    prob = problems.poisson_on_cube(3, 2)
    s = prob.subdomains[0]
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    try:
        for field, k, value in (("inet", 5, s.nnods), ("inet", 0, -1), ("isngn", 3, -1), ("isvgvn", 2, -4)):
            arrs = {f: getattr(s, f).copy() for f in ("inet", "isngn", "isvgvn")}
            arrs[field][k] = value
            with pytest.raises(B.BddcmlError) as ei:
                B.bddcml_upload_subdomain_data(prob.nelem, prob.nnod, prob.ndof, 3, 3, 0, s.nelems, s.nnods,
                                               s.ndofs, arrs["inet"], s.nnet, s.nndf, arrs["isngn"],
                                               arrs["isvgvn"], s.isegn, s.xyz, s.ifix, s.fixv, s.rhs, 1, s.sol, 1,
                                               s.i_sparse, s.j_sparse, s.a_sparse, 0)
            assert ei.value.code == 1, field
        B.upload_problem(prob)
    finally:
        B.bddcml_finalize()


_DIGEST_RUN = r"""
import sys
sys.path.insert(0, sys.argv[1])
import bddcml_gb300 as B
from bddcml_gb300 import problems
case = sys.argv[2]
if case == "uneven":
    prob = problems.poisson_boxes(24, problems.random_box_partition(24, 5, 10, seed=17),
                                  kappa=problems.lognormal_kappa(24, 1.0, seed=2))
    weights = 1
else:
    prob = problems.elasticity_on_cube(8, 2, nu=0.3, young=problems.inclusions_young(16))
    weights = 0
B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
B.upload_problem(prob)
try:
    B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, weights)
except B.BddcmlError as e:
    assert e.code == 2, e  # no GPU: the host part has run
print(B.get_setup_digest())
B.bddcml_finalize()
"""


@pytest.mark.parametrize("case", ["uneven", "elasticity"])
def test_host_setup_independent_of_thread_count(built_lib, case):
    """Every host-side setup result (assembled matrices, components, globs,
    constraints, eliminated values, weights, numbering, orderings) is bit for bit
    the same with 1, 3 and 8 OpenMP threads: the parallel steps split work by
    subdomain or by ranges of global ids and keep the serial orders."""
    import subprocess
    import sys
    digests = set()
    for nt in (1, 3, 8):
        env = dict(os.environ, OMP_NUM_THREADS=str(nt))
        out = subprocess.run([sys.executable, "-c", _DIGEST_RUN, ROOT, case], env=env, capture_output=True,
                             text=True, timeout=300)
        assert out.returncode == 0, out.stderr[-2000:]
        digests.add(out.stdout.strip().splitlines()[-1])
    assert len(digests) == 1, digests
