"""Global loading on the GPU (bddcml_upload_global_data_file_c with the
reference example's files): the solution matches a direct solve of the
assembled problem, and with the cube partition the iteration count equals the
subdomain upload's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _direct(gp):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    rows, cols, vals = [], [], []
    k = 0
    for e in range(gp.nelem):
        nodes = gp.inet[k:k + gp.nnet[e]]
        k += gp.nnet[e]
        ke = gp.elements[e]
        rows.append(np.repeat(nodes, len(nodes))); cols.append(np.tile(nodes, len(nodes))); vals.append(ke.ravel())
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(gp.ndof, gp.ndof))
    fixed = gp.ifix != 0
    free = ~fixed
    u = np.where(fixed, gp.fixv, 0.0)
    u[free] = spla.spsolve(K[free][:, free].tocsc(), gp.rhs[free] - K[free][:, fixed] @ gp.fixv[fixed])
    return u


@pytest.mark.parametrize("precision", [0, 1])
def test_global_poisson(built_lib, tmp_path, precision):
    import bddcml_gb300 as B
    from bddcml_gb300 import pmd, problems
    gp = pmd.poisson_global(8)
    prefix = str(tmp_path / "p8")
    pmd.write_problem(prefix, gp, [8, 1], tol=1e-10)
    u, it, reason, cond = pmd.solve_global(prefix, precision=precision)
    assert reason == 0
    ud = _direct(gp)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-8
    _, it_sub, _, _, _ = B.solve_problem(problems.poisson_on_cube(4, 2), precision=precision, tol=1e-10)
    assert it == it_sub


def test_global_convection_diffusion(built_lib, tmp_path):
    from bddcml_gb300 import pmd
    gp = pmd.convection_diffusion_global(9)
    prefix = str(tmp_path / "cd9")
    pmd.write_problem(prefix, gp, [6, 1], tol=1e-10)
    u, it, reason, cond = pmd.solve_global(prefix, precision=1, matrixtype=0)
    assert reason == 0
    ud = _direct(gp)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-7


def test_change_global_data(built_lib, tmp_path):
    """bddcml_change_global_data_c + bddcml_setup_new_data_c on globally loaded
    data (levels_change_global_data): new loads and nonzero boundary values."""
    import bddcml_gb300 as B
    from bddcml_gb300 import pmd
    gp = pmd.poisson_global(8)
    prefix = str(tmp_path / "p8")
    pmd.write_problem(prefix, gp, [8, 1], tol=1e-10)
    par, d = pmd.read_problem(prefix)
    B.bddcml_init(2, [8, 1], -1, 0, 0, 0, 0)
    try:
        B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"], d["nnet"],
                                         d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"], np.zeros(par["ndof"]),
                                         prefix + ".ELM")
        B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        B.bddcml_solve(0, 0, 1e-10, 500, 50, 0, 0)
        rng = np.random.default_rng(4)
        x = gp.xyz
        gp.fixv = np.where(gp.ifix != 0, 1.0 + x[:, 0] + x[:, 1] * x[:, 2], 0.0)
        gp.rhs = np.where(gp.ifix != 0, 0.0, rng.uniform(0.5, 1.5, gp.ndof) / 8 ** 3)
        B.bddcml_change_global_data(gp.ifix, gp.fixv, gp.rhs, np.zeros(gp.ndof))
        B.bddcml_setup_new_data()
        it, reason, _ = B.bddcml_solve(0, 0, 1e-10, 500, 50, 0, 0)
        u = B.bddcml_download_global_solution(gp.ndof)
    finally:
        B.bddcml_finalize()
    assert reason == 0
    ud = _direct(gp)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) <= 1e-8
