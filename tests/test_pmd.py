"""Global problem files of the reference's global example (.PAR, .ML, .GMIS,
.FVS, .RHS, .ELM; examples/bddcml_global.f90:223-362) and global loading
(bddcml_upload_global_data_file_c): element-matrix packing order, file round
trips, and the host-side division and localisation (no GPU needed)."""
import struct

import numpy as np
import pytest


def test_pack_element_order():
    """sm_pmd_make_element_numbering (module_sm.f90:272-380): columns outer,
    rows 1..j (symmetric storage) or 1..n (general)."""
    from bddcml_gb300 import pmd
    k = np.arange(9, dtype=float).reshape(3, 3)
    assert list(pmd.pack_element(k, 1)) == [k[0, 0], k[0, 1], k[1, 1], k[0, 2], k[1, 2], k[2, 2]]
    assert list(pmd.pack_element(k, 0)) == list(k.T.ravel())


def test_problem_files_round_trip(tmp_path):
    from bddcml_gb300 import pmd
    gp = pmd.convection_diffusion_global(3)
    prefix = str(tmp_path / "cd3")
    pmd.write_problem(prefix, gp, [4, 1], tol=1e-9, maxit=77, ndecrmax=12)
    par, d = pmd.read_problem(prefix)
    assert (par["ndim"], par["nsub"], par["nelem"], par["ndof"], par["nnod"]) == (3, 4, 27, 64, 64)
    assert par["tol"] == pytest.approx(1e-9) and par["maxit"] == 77 and par["ndecrmax"] == 12
    assert pmd.read_ml(prefix) == (2, [4, 1])
    assert np.array_equal(d["inet"], gp.inet) and np.array_equal(d["nnet"], gp.nnet)
    assert np.array_equal(d["ifix"], gp.ifix) and np.allclose(d["xyz"], gp.xyz, rtol=0, atol=1e-15)
    assert np.array_equal(d["rhs"], gp.rhs)
    with open(prefix + ".ELM", "rb") as f:
        raw = f.read()
    (n0,) = np.frombuffer(raw[:4], dtype="<i4")
    assert n0 == 4 + 8 * 64 and len(raw) == 27 * (8 + 4 + 8 * 64)


def test_global_loading_host_division_matches_subdomain_upload(built_lib, tmp_path):
    """A 8^3 cube in 8 subdomains: the coordinate bisection of the element
    centroids gives the 2x2x2 cube partition, so the host setup finds the same
    coarse space as the subdomain upload of that partition."""
    import bddcml_gb300 as B
    from bddcml_gb300 import pmd, problems
    gp = pmd.poisson_global(8)
    prefix = str(tmp_path / "p8")
    pmd.write_problem(prefix, gp, [8, 1])
    par, d = pmd.read_problem(prefix)
    B.bddcml_init(2, [8, 1], -1, 0, 0, 0, 0)
    try:
        B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"], d["nnet"],
                                         d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"], np.zeros(par["ndof"]),
                                         prefix + ".ELM")
        try:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        except B.BddcmlError as e:  # no GPU in this container: the host part has run
            assert e.code == 2
        info_global = B.get_coarse_info()
    finally:
        B.bddcml_finalize()
    prob = problems.poisson_on_cube(4, 2)
    B.bddcml_init(2, [8, 1], -1, 0, 0, 0, 0)
    try:
        B.upload_problem(prob)
        try:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        except B.BddcmlError as e:
            assert e.code == 2
        info_sub = B.get_coarse_info()
    finally:
        B.bddcml_finalize()
    assert info_global == info_sub


def test_global_loading_errors(built_lib, tmp_path):
    import bddcml_gb300 as B
    from bddcml_gb300 import pmd
    gp = pmd.poisson_global(2)
    prefix = str(tmp_path / "p2")
    pmd.write_problem(prefix, gp, [2, 1])
    par, d = pmd.read_problem(prefix)
    B.bddcml_init(2, [2, 1], -1, 0, 0, 0, 0)
    try:
        with pytest.raises(B.BddcmlError) as e:  # NNET does not sum to LINET
            B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"][:-1],
                                             d["nnet"], d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"],
                                             np.zeros(par["ndof"]), prefix + ".ELM")
        assert e.value.code == 1
        with pytest.raises(B.BddcmlError) as e:  # a stored division is not implemented
            B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"], d["nnet"],
                                             d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"],
                                             np.zeros(par["ndof"]), prefix + ".ELM", load_division_int=1)
        assert e.value.code == 4
        # a damaged element file is reported at setup
        with open(prefix + ".ELM", "rb") as f:
            good = f.read()
        with open(prefix + "_bad.ELM", "wb") as f:
            f.write(good[:-20])
        B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"], d["nnet"],
                                         d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"], np.zeros(par["ndof"]),
                                         prefix + "_bad.ELM")
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        assert e.value.code == 1
    finally:
        B.bddcml_finalize()
    # a record marker claiming a huge payload is refused before anything is allocated
    B.bddcml_init(2, [2, 1], -1, 0, 0, 0, 0)
    try:
        with open(prefix + "_huge.ELM", "wb") as f:
            f.write(struct.pack("<I", 0x7FFFFFF0) + good[4:])
        B.bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], 3, 3, d["inet"], d["nnet"],
                                         d["nndf"], d["xyz"], d["ifix"], d["fixv"], d["rhs"], np.zeros(par["ndof"]),
                                         prefix + "_huge.ELM")
        with pytest.raises(B.BddcmlError) as e:
            B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        assert e.value.code == 1
    finally:
        B.bddcml_finalize()
