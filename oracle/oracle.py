"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU legs of ``bench.py``.  The GPU library never imports this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def sym_eig(a):
    """The oracle's dense symmetric eigensolver: (ascending eigenvalues, eigenvectors in columns)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = a.shape[0]
    w = np.zeros(n)
    z = np.zeros((n, n))
    lib().oracle_sym_eig(n, a.ctypes.data, w.ctypes.data, z.ctypes.data)
    return w, z


def build(force: bool = False) -> str:
    path = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "bddc_oracle.cpp")
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return path


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        L = _LIB
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_int, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_error.restype = C.c_char_p
        L.oracle_error.argtypes = [C.c_void_p]
        L.oracle_setup.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.oracle_solve.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.oracle_solve_method.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int,
                                          C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.oracle_download.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.oracle_set_adaptive.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.oracle_solve_recycling.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.oracle_new_loads.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.oracle_recycling_size.argtypes = [C.c_void_p]
        L.oracle_reactions.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_set_levels.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_adaptive_info.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_sym_eig.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_stats.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_sub_stats.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_relres_history.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_weights.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.oracle_dotprod_subdomain.restype = C.c_double
        L.oracle_dotprod_subdomain.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        for fn in (L.oracle_array_intersection, L.oracle_array_union):
            fn.restype = C.c_int
            fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    return _LIB


def array_intersection(a, b):
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    out = np.zeros(len(a) + len(b), np.int32)
    n = lib().oracle_array_intersection(_p(a), len(a), _p(b), len(b), _p(out))
    return out[:n]


def array_union(a, b):
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    out = np.zeros(len(a) + len(b), np.int32)
    n = lib().oracle_array_union(_p(a), len(a), _p(b), len(b), _p(out))
    return out[:n]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """BDDC interface PCG restated on the CPU (see bddc_oracle.cpp)."""

    def __init__(self, prob, nthreads: int | None = None, find_components: int = 1, neighbouring: int = 3):
        self.L = lib()
        self.prob = prob
        self.h = self.L.oracle_create(prob.nsub, int(nthreads or os.cpu_count() or 1))
        self._keep = []
        for s in prob.subdomains:
            arrs = dict(
                inet=np.ascontiguousarray(s.inet, np.int32), nnet=np.ascontiguousarray(s.nnet, np.int32),
                nndf=np.ascontiguousarray(s.nndf, np.int32), isngn=np.ascontiguousarray(s.isngn, np.int32),
                isvgvn=np.ascontiguousarray(s.isvgvn, np.int32), isegn=np.ascontiguousarray(s.isegn, np.int32),
                xyz=np.ascontiguousarray(s.xyz, np.float64), ifix=np.ascontiguousarray(s.ifix, np.int32),
                fixv=np.ascontiguousarray(s.fixv, np.float64), rhs=np.ascontiguousarray(s.rhs, np.float64),
                sol=np.ascontiguousarray(s.sol, np.float64), i=np.ascontiguousarray(s.i_sparse, np.int32),
                j=np.ascontiguousarray(s.j_sparse, np.int32), a=np.ascontiguousarray(s.a_sparse, np.float64))
            rc = self.L.oracle_upload(
                C.c_void_p(self.h), C.c_int(s.isub), C.c_int(s.nelems), C.c_int(s.nnods), C.c_int(s.ndofs),
                C.c_int(prob.ndim), _p(arrs["inet"]), C.c_int(len(s.inet)), _p(arrs["nnet"]), _p(arrs["nndf"]),
                _p(arrs["isngn"]), _p(arrs["isvgvn"]), _p(arrs["isegn"]), _p(arrs["xyz"]), _p(arrs["ifix"]),
                _p(arrs["fixv"]), _p(arrs["rhs"]), C.c_int(s.is_rhs_complete), _p(arrs["sol"]),
                C.c_int(prob.matrixtype), C.c_int(len(s.a_sparse)), _p(arrs["i"]), _p(arrs["j"]), _p(arrs["a"]),
                C.c_int(find_components), C.c_int(neighbouring))
            if rc != 0:
                raise RuntimeError(self.L.oracle_error(self.h).decode())

    def __del__(self):
        try:
            self.L.oracle_destroy(self.h)
        except Exception:
            pass

    def setup(self, use_corner_constraints=1, use_arithmetic_constraints=1, weights_type=0):
        rc = self.L.oracle_setup(self.h, use_corner_constraints, use_arithmetic_constraints, weights_type)
        if rc != 0:
            raise RuntimeError(self.L.oracle_error(self.h).decode())

    def solve_recycling(self, tol=1e-8, maxit=500, ndecrmax=50, recycling=True, maxvec=100):
        """PCG with Krylov recycling; the stored basis persists between calls."""
        it, reason, cond = C.c_int(), C.c_int(), C.c_double()
        rc = self.L.oracle_solve_recycling(self.h, tol, maxit, ndecrmax, int(recycling), maxvec, C.byref(it),
                                           C.byref(reason), C.byref(cond))
        if rc != 0:
            raise RuntimeError(self.L.oracle_error(self.h).decode())
        return it.value, reason.value, cond.value

    def set_levels(self, nlevels=2, nsub2=1):
        """Three-level BDDC with nsub2 level-2 subdomains at the next setup."""
        self.L.oracle_set_levels(self.h, nlevels, nsub2)

    def reactions(self, isub):
        """Reactions of subdomain isub after a solve (ndofs values)."""
        out = np.zeros(self.prob.subdomains[isub].ndofs)
        self.L.oracle_reactions(self.h, isub, out.ctypes.data)
        return out

    def global_reactions(self):
        r = np.zeros(self.prob.ndof)
        for s in self.prob.subdomains:
            r[s.isvgvn] = self.reactions(s.isub)
        return r

    def recycling_size(self):
        return self.L.oracle_recycling_size(self.h)

    def new_loads(self, isub, rhs, sol=None):
        """New loads and initial guess (default zero) of one subdomain (same
        Dirichlet data) after setup."""
        r = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros_like(r) if sol is None else np.ascontiguousarray(sol, dtype=np.float64)
        if self.L.oracle_new_loads(self.h, isub, r.ctypes.data, x.ctypes.data) != 0:
            raise RuntimeError(self.L.oracle_error(self.h).decode())

    def set_adaptive(self, on=True, tau=1.5):
        """Adaptive face constraints at the next setup (module_adaptivity.f90),
        eigenvalue threshold tau."""
        self.L.oracle_set_adaptive(self.h, int(on), float(tau))

    def adaptive_info(self, maxpair=100000):
        """Pairs of the last adaptive setup: dict with 'pairs' (face, isub, jsub),
        'neig', 'nadaptive', 'face_ncdof' (arrays) and 'eigs' (npair x 10,
        descending, zero-padded), plus the estimate 'est'."""
        info = np.zeros(6 * maxpair, dtype=np.int32)
        eigs = np.zeros(10 * maxpair)
        est = C.c_double()
        n = self.L.oracle_adaptive_info(self.h, info.ctypes.data, eigs.ctypes.data, maxpair, C.byref(est))
        info = info[:6 * n].reshape(n, 6)
        return {"pairs": info[:, :3].copy(), "neig": info[:, 3].copy(), "nadaptive": info[:, 4].copy(),
                "face_ncdof": info[:, 5].copy(), "eigs": eigs[:10 * n].reshape(n, 10).copy(), "est": est.value}

    def solve(self, tol=1e-8, maxit=500, ndecrmax=50, method=0):
        """method 0 PCG, 1 BiCGSTAB, 2 steepest descent, -1 reference defaults."""
        it, reason, cond = C.c_int(), C.c_int(), C.c_double()
        rc = self.L.oracle_solve_method(self.h, method, tol, maxit, ndecrmax, C.byref(it), C.byref(reason),
                                        C.byref(cond))
        if rc != 0:
            raise RuntimeError(self.L.oracle_error(self.h).decode())
        return it.value, reason.value, cond.value

    def download(self, isub):
        s = self.prob.subdomains[isub]
        out = np.zeros(s.ndofs)
        if self.L.oracle_download(self.h, isub, _p(out), s.ndofs) != 0:
            raise RuntimeError("download size mismatch")
        return out

    def global_solution(self):
        u = np.zeros(self.prob.ndof)
        for s in self.prob.subdomains:
            u[s.isvgvn] = self.download(s.isub)
        return u

    def stats(self):
        out = np.zeros(6, dtype=np.int32)
        self.L.oracle_stats(self.h, _p(out))
        return dict(ncorner=int(out[0]), nedge=int(out[1]), nface=int(out[2]), ndofc=int(out[3]),
                    sum_ndofi=int(out[4]), sum_ndofo=int(out[5]))

    def sub_stats(self, isub):
        out = np.zeros(5, dtype=np.int32)
        self.L.oracle_sub_stats(self.h, isub, _p(out))
        return dict(ndofi=int(out[0]), ndofo=int(out[1]), nconstr=int(out[2]), ncorner=int(out[3]), nadj=int(out[4]))

    def relres_history(self):
        n = self.L.oracle_relres_history(self.h, None, 0)
        out = np.zeros(n)
        self.L.oracle_relres_history(self.h, _p(out), n)
        return out

    def weights(self, isub):
        st = self.sub_stats(isub)
        out = np.zeros(st["ndofi"])
        self.L.oracle_weights(self.h, isub, _p(out), st["ndofi"])
        return out

    def dotprod_subdomain(self, isub, v1, v2):
        v1 = np.ascontiguousarray(v1, np.float64)
        v2 = np.ascontiguousarray(v2, np.float64)
        return self.L.oracle_dotprod_subdomain(self.h, isub, _p(v1), _p(v2))
