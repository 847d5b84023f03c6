"""GB300-native BDDC interface solver: Python binding over the C ABI.

The functions below mirror the reference Fortran/C API of BDDCML
(module_bddcml.f90, src/bddcml_interface_c.h): same names without the ``_c``
suffix, same argument meaning, same call order.  They call the in-tree shared
library ``libbddcgpu.so`` (built by :mod:`bddcml_gb300.build`) through ctypes;
there is no CPU fallback - if the library or the GPU is missing, the calls
raise :class:`BddcmlError`.

Indices passed here use the ``numbase`` given to :func:`bddcml_init`.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libbddcgpu.so")
_lib = None

STATUS = {0: "OK", 1: "ARGUMENT", 2: "CUDA", 3: "NUMERIC", 4: "UNSUPPORTED", 5: "MEMORY"}

# fields of bddcml_get_stats_c
STAT_FIELDS = ["t_host_setup", "t_device_setup", "t_solve", "t_iterations", "t_postprocess", "num_iter",
               "bytes_per_iteration", "ncorner", "nedge", "nface", "ndofc", "sum_ndofi", "sum_ndofo",
               "ninterface", "precision", "h2d_bytes", "d2h_bytes", "t_upload", "t_host_assemble",
               "t_host_iface", "t_host_globs", "t_host_blocks", "refine1", "refine2",
               "flop_sweep_oo", "flop_sweep_s", "bytes_residual", "bytes_schur_apply", "bytes_pc_local",
               "launches_setup", "launches_solve", "t_dev_alloc", "t_dev_h2d", "npair", "nadaptive",
               "adapt_est", "t_adaptive", "lobpcg_resid", "lobpcg_iter", "batch_bytes_schur",
               "batch_flop_schur_mma", "batch_flop_schur", "batch_flop_pc", "batch_nk",
               "bytes_assemble_dot", "bytes_assemble_z", "bytes_coarse_apply", "refine_steps", "band_w"]

EXPORTS = ["bddcml_init_c", "bddcml_upload_global_data_c", "bddcml_upload_subdomain_data_c",
           "bddcml_setup_preconditioner_c", "bddcml_solve_c", "bddcml_download_local_solution_c",
           "bddcml_download_global_solution_c", "bddcml_download_local_reactions_c",
           "bddcml_download_global_reactions_c", "bddcml_change_global_data_c", "bddcml_change_subdomain_data_c",
           "bddcml_setup_new_data_c", "bddcml_dotprod_subdomain_c", "bddcml_finalize_c",
           "bddcml_get_last_error_c", "bddcml_set_precision_c", "bddcml_get_stats_c",
           "bddcml_get_residual_history_c", "bddcml_get_interface_weights_c", "bddcml_get_coarse_info_c",
           "bddcml_set_profiling_c", "bddcml_get_profile_c", "bddcml_release_device_memory_c",
           "bddcml_dotprod_subdomain_dev_c", "bddcml_element_gradient_dev_c", "bddcml_set_adaptive_threshold_c",
           "bddcml_get_adaptive_info_c", "bddcml_upload_subdomain_rhs_batch_c", "bddcml_solve_batch_c",
           "bddcml_download_local_solution_batch_c", "bddcml_set_batch_operator_c",
           "bddcml_upload_global_data_file_c", "bddcml_set_wait_limit_c", "bddcml_get_setup_digest_c"]

# phases of bddcml_get_profile_c (CUDA events on the solver stream)
PHASES = ["numeric_total", "solve_total", "factor_interior", "solve_interior", "refine_residual", "schur",
          "precond_factor", "precond_solve", "precond_blocks", "coarse", "pcg", "schur_apply", "precond_local",
          "postprocess", "assemble_dot", "assemble_z", "coarse_apply"]


class BddcmlError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS.get(code, code)}] {msg}")
        self.code = code


def lib():
    """Loads libbddcgpu.so (build it with ``python -m bddcml_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise BddcmlError(2, f"{LIBPATH} is missing: run bddcml_gb300.build.build() first")
        _lib = C.CDLL(LIBPATH)
        _lib.bddcml_get_last_error_c.restype = C.c_int
    return _lib


def _i(v):
    return C.byref(C.c_int(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _pi(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def _pd(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _ci(a):
    """a as a C-contiguous int32 array (no copy when it is one already)."""
    if type(a) is np.ndarray and a.dtype == np.int32 and a.flags.c_contiguous:
        return a
    return np.ascontiguousarray(a, dtype=np.int32)


def _cd(a):
    """a as a C-contiguous float64 array (no copy when it is one already)."""
    if type(a) is np.ndarray and a.dtype == np.float64 and a.flags.c_contiguous:
        return a
    return np.ascontiguousarray(a, dtype=np.float64)


_EMPTY = np.zeros(1)
_upload_c = None


def _upload_fn():
    """bddcml_upload_subdomain_data_c with its 50 pointer arguments declared as
    addresses (a prototype of its own: the library's attribute keeps no argtypes)."""
    global _upload_c
    if _upload_c is None:
        _upload_c = C.CFUNCTYPE(None, *([C.c_void_p] * 50))(("bddcml_upload_subdomain_data_c", lib()))
    return _upload_c


def last_error():
    buf = C.create_string_buffer(1024)
    code = lib().bddcml_get_last_error_c(buf, _i(1024))
    return code, buf.value.decode(errors="replace")


def _check():
    if lib().bddcml_get_last_error_c(None, None) != 0:  # status only; the message on failure
        code, msg = last_error()
        raise BddcmlError(code, msg)


# ------------------------------------------------------------- reference API
def bddcml_init(nl: int, nsublev, nsub_loc_1: int = -1, comm_init: int = 0, verbose_level: int = 0,
                numbase: int = 0, just_direct_solve_int: int = 0) -> int:
    """module_bddcml.f90:36-101; returns nsub_loc_1 (all subdomains are local)."""
    ns, pns = _pi(nsublev)
    loc = C.c_int(nsub_loc_1)
    lib().bddcml_init_c(_i(nl), pns, _i(len(ns)), C.byref(loc), _i(comm_init), _i(verbose_level), _i(numbase),
                        _i(just_direct_solve_int))
    _check()
    return loc.value


def bddcml_upload_subdomain_data(nelem, nnod, ndof, ndim, meshdim, isub, nelems, nnods, ndofs,
                                 inet, nnet, nndf, isngn, isvgvn, isegn, xyz, ifix, fixv, rhs, is_rhs_complete,
                                 sol, matrixtype, i_sparse, j_sparse, a_sparse, is_assembled,
                                 find_components_int=1, use_dual_mesh_graph_int=1, neighbouring=3):
    """module_bddcml.f90:186-356.  ``xyz`` is (nnods, ndim) or its Fortran
    (column-major) flattening."""
    xyz = np.asarray(xyz, dtype=np.float64)
    if xyz.ndim == 2:
        if xyz.shape == (ndim, nnods):
            xyzf = np.ascontiguousarray(xyz).ravel()      # rows = coordinates -> already column-major order
        else:
            xyzf = np.ascontiguousarray(xyz.T).ravel()
    else:
        xyzf = xyz
    # every argument is a pointer: arrays by their data address, the scalars
    # as consecutive entries of one int32 array (one ctypes conversion per call
    # instead of one object per argument; the call is made once per subdomain)
    inet, nnet, nndf, isngn, isvgvn, isegn, ifix, i_sparse, j_sparse = (
        _ci(a) for a in (inet, nnet, nndf, isngn, isvgvn, isegn, ifix, i_sparse, j_sparse))
    xyzf, fixv, rhs, sol, a_sparse = (_cd(a) for a in (xyzf, fixv, rhs, sol, a_sparse))
    sc = np.array([nelem, nnod, ndof, ndim, meshdim, isub, nelems, nnods, ndofs,            # 0-8
                   len(inet), len(nnet), len(nndf), len(isngn), len(isvgvn), len(isegn),   # 9-14
                   nnods, ndim, len(ifix), len(fixv), len(rhs), is_rhs_complete, len(sol),  # 15-21
                   matrixtype, len(i_sparse), is_assembled, 0, find_components_int,        # 22-26
                   use_dual_mesh_graph_int, neighbouring], dtype=np.int32)                 # 27-28
    s0 = sc.ctypes.data

    def s(k):
        return s0 + 4 * k
    e = _EMPTY.ctypes.data
    _upload_fn()(
        s(0), s(1), s(2), s(3), s(4), s(5), s(6), s(7), s(8),
        inet.ctypes.data, s(9), nnet.ctypes.data, s(10), nndf.ctypes.data, s(11), isngn.ctypes.data, s(12),
        isvgvn.ctypes.data, s(13), isegn.ctypes.data, s(14), xyzf.ctypes.data, s(15), s(16), ifix.ctypes.data,
        s(17), fixv.ctypes.data, s(18), rhs.ctypes.data, s(19), s(20), sol.ctypes.data, s(21), s(22),
        i_sparse.ctypes.data, j_sparse.ctypes.data, a_sparse.ctypes.data, s(23), s(24),
        e, s(25), s(25), e, s(25), s(25), e, s(25),
        s(26), s(27), s(28))
    _check()


def bddcml_upload_global_data_file(nelem, nnod, ndof, ndim, meshdim, inet, nnet, nndf, xyz, ifix, fixv, rhs, sol,
                                   elm_file: str, neighbouring: int = 1, load_division_int: int = 0):
    """Global loading with the element matrices in a Fortran unformatted file
    (extension of module_levels.f90:422-612); xyz is (nnod, ndim)."""
    i_, pi = _pi(inet)
    nn, pnn = _pi(nnet)
    nd, pnd = _pi(nndf)
    xyz_f = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).T)  # column-major (nnod x ndim)
    fx, pfx = _pi(ifix)
    fv, pfv = _pd(fixv)
    r, pr = _pd(rhs)
    x, px = _pd(sol)
    lib().bddcml_upload_global_data_file_c(
        _i(nelem), _i(nnod), _i(ndof), _i(ndim), _i(meshdim), pi, _i(len(i_)), pnn, _i(len(nn)), pnd, _i(len(nd)),
        xyz_f.ctypes.data_as(C.POINTER(C.c_double)), _i(nnod), _i(ndim), pfx, _i(len(fx)), pfv, _i(len(fv)),
        pr, _i(len(r)), px, _i(len(x)), C.c_char_p(elm_file.encode()), _i(neighbouring), _i(load_division_int))
    _check()


def bddcml_setup_preconditioner(matrixtype=1, use_defaults_int=0, parallel_division_int=1,
                                use_corner_constraints_int=1, use_arithmetic_constraints_int=1,
                                use_adaptive_constraints_int=0, use_user_constraints_int=0, weights_type=0):
    """module_bddcml.f90:359-455."""
    lib().bddcml_setup_preconditioner_c(_i(matrixtype), _i(use_defaults_int), _i(parallel_division_int),
                                        _i(use_corner_constraints_int), _i(use_arithmetic_constraints_int),
                                        _i(use_adaptive_constraints_int), _i(use_user_constraints_int),
                                        _i(weights_type))
    _check()


def bddcml_solve(comm_all=0, method=0, tol=1e-6, maxit=1000, ndecrmax=30, recycling_int=0,
                 max_number_of_stored_vectors=100):
    """module_bddcml.f90:459-567; returns (num_iter, converged_reason, condition_number)."""
    it, reason, cond = C.c_int(), C.c_int(), C.c_double()
    lib().bddcml_solve_c(_i(comm_all), _i(method), _d(tol), _i(maxit), _i(ndecrmax), _i(recycling_int),
                         _i(max_number_of_stored_vectors), C.byref(it), C.byref(reason), C.byref(cond))
    _check()
    return it.value, reason.value, cond.value


def bddcml_download_local_solution(isub: int, lsols: int) -> np.ndarray:
    out = np.zeros(lsols)
    lib().bddcml_download_local_solution_c(_i(isub), out.ctypes.data_as(C.POINTER(C.c_double)), _i(lsols))
    _check()
    return out


def bddcml_download_global_solution(lsol: int) -> np.ndarray:
    """Global solution gathered from the subdomains (module_levels.f90:4617-4744)."""
    out = np.zeros(lsol)
    lib().bddcml_download_global_solution_c(out.ctypes.data_as(C.POINTER(C.c_double)), _i(lsol))
    _check()
    return out


def bddcml_download_local_reactions(isub: int, lreas: int) -> np.ndarray:
    """Reactions of one subdomain after a solve (module_dd.f90:1258-1374, 3364-3395)."""
    out = np.zeros(lreas)
    lib().bddcml_download_local_reactions_c(_i(isub), out.ctypes.data_as(C.POINTER(C.c_double)), _i(lreas))
    _check()
    return out


def bddcml_download_global_reactions(lrea: int) -> np.ndarray:
    """Global reactions gathered from the subdomains (module_levels.f90:4785-4914)."""
    out = np.zeros(lrea)
    lib().bddcml_download_global_reactions_c(out.ctypes.data_as(C.POINTER(C.c_double)), _i(lrea))
    _check()
    return out


def bddcml_dotprod_subdomain(isub: int, vec1, vec2) -> float:
    a, pa = _pd(vec1)
    b, pb = _pd(vec2)
    d = C.c_double()
    lib().bddcml_dotprod_subdomain_c(_i(isub), pa, _i(len(a)), pb, _i(len(b)), C.byref(d))
    _check()
    return d.value


def bddcml_change_subdomain_data(isub: int, ifix, fixv, rhs, is_rhs_complete: int, sol):
    i, pi = _pi(ifix)
    f, pf = _pd(fixv)
    r, pr = _pd(rhs)
    x, px = _pd(sol)
    lib().bddcml_change_subdomain_data_c(_i(isub), pi, _i(len(i)), pf, _i(len(f)), pr, _i(len(r)),
                                         _i(is_rhs_complete), px, _i(len(x)))
    _check()


def bddcml_change_global_data(ifix, fixv, rhs, sol):
    """New global fixed values, loads and initial guess (globally loaded data)."""
    i, pi = _pi(ifix)
    f, pf = _pd(fixv)
    r, pr = _pd(rhs)
    x, px = _pd(sol)
    lib().bddcml_change_global_data_c(pi, _i(len(i)), pf, _i(len(f)), pr, _i(len(r)), px, _i(len(x)))
    _check()


def bddcml_setup_new_data():
    lib().bddcml_setup_new_data_c()
    _check()


def bddcml_upload_subdomain_rhs_batch(isub: int, rhss, is_rhs_complete: int = 1):
    """Batched loads of one subdomain: rhss is (nrhs, ndof), one load per row
    (stored column-major as ndof x nrhs for the C call)."""
    r = np.ascontiguousarray(np.atleast_2d(rhss), dtype=np.float64)
    nrhs = r.shape[0]
    lib().bddcml_upload_subdomain_rhs_batch_c(_i(isub), _i(nrhs), r.ctypes.data_as(C.POINTER(C.c_double)),
                                              _i(r.size), _i(is_rhs_complete))
    _check()


def bddcml_solve_batch(nrhs: int, comm_all=0, method=0, tol=1e-8, maxit=1000, ndecrmax=30):
    """PCG on the uploaded batch; returns per-column (num_iter, converged_reason, condition_number) arrays."""
    it = np.zeros(nrhs, dtype=np.int32)
    reason = np.zeros(nrhs, dtype=np.int32)
    cond = np.zeros(nrhs)
    lib().bddcml_solve_batch_c(_i(comm_all), _i(method), _d(tol), _i(maxit), _i(ndecrmax), _i(nrhs),
                               it.ctypes.data_as(C.POINTER(C.c_int)), reason.ctypes.data_as(C.POINTER(C.c_int)),
                               cond.ctypes.data_as(C.POINTER(C.c_double)))
    _check()
    return it, reason, cond


def set_batch_operator(mode: int) -> None:
    """Products of the batched solve in mixed mode: -1 automatic (default), 0 SIMT
    (double-float Schur apply, FP32 preconditioner), 1 sliced bf16 tensor-core Schur
    apply with 3xTF32 preconditioner products, 2 sliced Schur apply and sliced
    (exact) preconditioner products."""
    lib().bddcml_set_batch_operator_c(_i(mode))
    _check()


def bddcml_download_local_solution_batch(isub: int, nrhs: int, ndof: int) -> np.ndarray:
    """Solutions of the last batched solve for one subdomain, shape (nrhs, ndof)."""
    out = np.zeros((nrhs, ndof))
    lib().bddcml_download_local_solution_batch_c(_i(isub), _i(nrhs), out.ctypes.data_as(C.POINTER(C.c_double)),
                                                 _i(out.size))
    _check()
    return out


def bddcml_finalize():
    lib().bddcml_finalize_c()
    _check()


# ---------------------------------------------------------------- extensions
def set_precision(mode: int):
    """0 = plain FP64, 1 = mixed precision (default)."""
    lib().bddcml_set_precision_c(_i(mode))
    _check()


def get_stats() -> dict:
    buf = (C.c_double * 64)()
    n = C.c_int(64)
    lib().bddcml_get_stats_c(buf, C.byref(n))
    _check()
    return {k: buf[i] for i, k in enumerate(STAT_FIELDS[: n.value])}


def set_adaptive_threshold(tau: float) -> None:
    """Eigenvalue threshold of the adaptive face constraints (default 1.5)."""
    lib().bddcml_set_adaptive_threshold_c(_d(tau))
    _check()


def get_adaptive_info() -> dict:
    """Face pairs of the last adaptive setup: 'pairs' (npair x 2 subdomains),
    'k' (eigenvalues computed per pair) and 'eigs' (npair x 10, descending)."""
    n = C.c_int(0)
    lib().bddcml_get_adaptive_info_c(None, None, C.byref(n))
    _check()
    pairs = np.zeros(3 * max(1, n.value), dtype=np.int32)
    eigs = np.zeros(10 * max(1, n.value))
    m = C.c_int(n.value)
    lib().bddcml_get_adaptive_info_c(pairs.ctypes.data_as(C.POINTER(C.c_int)),
                                     eigs.ctypes.data_as(C.POINTER(C.c_double)), C.byref(m))
    _check()
    pairs = pairs[:3 * n.value].reshape(n.value, 3)
    return {"pairs": pairs[:, :2].copy(), "k": pairs[:, 2].copy(), "eigs": eigs[:10 * n.value].reshape(n.value, 10)}


def get_residual_history() -> np.ndarray:
    n = C.c_int(0)
    lib().bddcml_get_residual_history_c(None, C.byref(n))
    _check()
    out = np.zeros(n.value)
    m = C.c_int(n.value)
    lib().bddcml_get_residual_history_c(out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(m))
    _check()
    return out


def get_interface_weights(isub: int, ndofi: int) -> np.ndarray:
    out = np.zeros(ndofi)
    lib().bddcml_get_interface_weights_c(_i(isub), out.ctypes.data_as(C.POINTER(C.c_double)), _i(ndofi))
    _check()
    return out


def dotprod_subdomain_dev(isub: int, vec1_ptr: int, vec2_ptr: int, lvec: int) -> float:
    """Weighted subdomain dot product of two device-resident vectors (raw
    device addresses, float64, length lvec); allocates nothing."""
    out = C.c_double()
    lib().bddcml_dotprod_subdomain_dev_c(_i(isub), C.c_void_p(vec1_ptr), C.c_void_p(vec2_ptr), _i(lvec),
                                         C.byref(out))
    _check()
    return out.value


def element_gradient_dev(nelem: int, nne: int, inet_ptr: int, ke0_ptr: int, per_element: bool, u_ptr: int,
                         lam_ptr: int, grad_ptr: int):
    """grad[e] = -lam_e^T K_e^0 u_e on device arrays (raw device addresses)."""
    lib().bddcml_element_gradient_dev_c(_i(nelem), _i(nne), C.c_void_p(inet_ptr), C.c_void_p(ke0_ptr),
                                        _i(1 if per_element else 0), C.c_void_p(u_ptr), C.c_void_p(lam_ptr),
                                        C.c_void_p(grad_ptr))
    _check()


def release_device_memory():
    """Hand the pooled device memory that no solver uses back to the driver."""
    lib().bddcml_release_device_memory_c()
    _check()


def set_wait_limit(spins: int) -> None:
    """Spin limit of the waits inside the tensor-core sweeps (0: default)."""
    lib().bddcml_set_wait_limit_c(C.byref(C.c_longlong(int(spins))))
    _check()


def set_profiling(on: bool):
    lib().bddcml_set_profiling_c(_i(1 if on else 0))
    _check()


def get_profile() -> dict:
    """{phase: (total ms, launches)} from the library's CUDA-event timers."""
    ms = (C.c_double * 64)()
    cnt = (C.c_int * 64)()
    n = C.c_int(64)
    lib().bddcml_get_profile_c(ms, cnt, C.byref(n))
    _check()
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PHASES[: n.value])}


def get_coarse_info() -> dict:
    buf = (C.c_int * 6)()
    n = C.c_int(6)
    lib().bddcml_get_coarse_info_c(buf, C.byref(n))
    _check()
    keys = ["ncorner", "nedge", "nface", "ndofc", "sum_ndofi", "sum_ndofo"]
    return {k: int(buf[i]) for i, k in enumerate(keys)}


def get_setup_digest() -> int:
    """64-bit digest of the host-side setup results (independent of the thread count)."""
    d = C.c_ulonglong(0)
    lib().bddcml_get_setup_digest_c(C.byref(d))
    _check()
    return d.value


# ------------------------------------------------------------ convenience
def upload_problem(prob, numbase: int = 0, find_components_int: int = 1, neighbouring: int = 3):
    """Uploads every subdomain of a :class:`bddcml_gb300.problems.Problem`
    (0-based arrays) through the C ABI, shifting indices to ``numbase``."""
    nb = numbase

    def sh(a):  # index arrays in the caller's numbering (no copy for numbase 0)
        return a + nb if nb else a
    for s in prob.subdomains:
        bddcml_upload_subdomain_data(
            prob.nelem, prob.nnod, prob.ndof, prob.ndim, prob.meshdim, s.isub + nb, s.nelems, s.nnods, s.ndofs,
            sh(s.inet), s.nnet, s.nndf, sh(s.isngn), sh(s.isvgvn), sh(s.isegn), s.xyz, s.ifix, s.fixv,
            s.rhs, s.is_rhs_complete, s.sol, prob.matrixtype, sh(s.i_sparse), sh(s.j_sparse), s.a_sparse,
            s.is_assembled, find_components_int=find_components_int, neighbouring=neighbouring)


def solve_problem(prob, precision: int = 1, tol: float = 1e-8, maxit: int = 500, ndecrmax: int = 50,
                  weights_type: int = 0, numbase: int = 0, finalize: bool = True, method: int = 0,
                  adaptive_tau=None):
    """init -> upload -> setup -> solve -> download (-> finalize) through the
    C ABI, the sequence of the reference example poisson_on_cube.f90:373-672.
    method: 0 PCG, 1 BiCGSTAB, 2 steepest descent, -1 reference defaults.
    adaptive_tau: adaptive face constraints with this eigenvalue threshold.
    Returns (global solution, num_iter, reason, cond, stats)."""
    bddcml_init(2, [prob.nsub, 1], -1, 0, 0, numbase, 0)
    set_precision(precision)
    upload_problem(prob, numbase=numbase)
    if adaptive_tau is not None:
        set_adaptive_threshold(adaptive_tau)
    bddcml_setup_preconditioner(prob.matrixtype, 0, 1, 1, 1, 1 if adaptive_tau is not None else 0, 0, weights_type)
    it, reason, cond = bddcml_solve(0, method, tol, maxit, ndecrmax, 0, 0)
    u = np.zeros(prob.ndof)
    for s in prob.subdomains:
        u[s.isvgvn] = bddcml_download_local_solution(s.isub + numbase, s.ndofs)
    st = get_stats()
    if finalize:
        bddcml_finalize()
    return u, it, reason, cond, st
