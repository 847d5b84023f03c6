"""Global problem files of the reference's global example and global loading.

The reference example ``examples/bddcml_global.f90:223-362`` reads a problem
from files named after it:

* ``.PAR``: ``ndim nsub nelem ndof nnod nnodc linet tol maxit ndecrmax`` and,
  optionally on the next line, ``meshdim`` (``pp_read_par_file``,
  ``src/module_pp.f90:655-704``);
* ``.ML``: the number of levels, then the subdomain counts of the levels;
* ``.GMIS``: ``inet`` (1-based), ``nnet``, ``nndf``, ``xyz`` (column-major
  nnod x ndim), list-directed (``pp_read_pmd_mesh``, ``module_pp.f90:989-1019``);
* ``.FVS``: ``ifix`` then ``fixv`` (``pp_read_pmd_bc``, ``module_pp.f90:796-818``);
* ``.RHS``: the assembled load, one Fortran unformatted record
  (``pp_read_pmd_rhs``, ``module_pp.f90:892-917``);
* ``.ELM``: one unformatted record ``lelm, elm(1:lelm)`` per element, each
  matrix packed column by column, upper triangle for symmetric storage
  (``sm_pmd_make_element_numbering``, ``src/module_sm.f90:272-380``).

Unformatted records use 4-byte length markers before and after the payload.
The element matrices go to the library as a file
(``bddcml_upload_global_data_file_c``), which divides the mesh at setup.
"""
from __future__ import annotations

import dataclasses
import struct
from typing import List, Optional

import numpy as np

from . import problems


@dataclasses.dataclass
class GlobalProblem:
    nelem: int
    nnod: int
    ndof: int
    ndim: int
    meshdim: int
    inet: np.ndarray      # int32, 0-based node numbers, element by element
    nnet: np.ndarray      # int32, nodes per element
    nndf: np.ndarray      # int32, dofs per node
    xyz: np.ndarray       # float64 (nnod, ndim)
    ifix: np.ndarray      # int32, ndof
    fixv: np.ndarray      # float64, ndof
    rhs: np.ndarray       # float64, ndof (assembled)
    elements: List[np.ndarray]  # element matrices (nve x nve), element order
    matrixtype: int = 1


def pack_element(k: np.ndarray, matrixtype: int) -> np.ndarray:
    """Element matrix in the order of sm_pmd_make_element_numbering: columns
    jve = 1..nve, rows ive = 1..jve (symmetric storage) or 1..nve (general)."""
    nve = k.shape[0]
    out = []
    for j in range(nve):
        rows = range(j + 1) if matrixtype != 0 else range(nve)
        out.extend(k[i, j] for i in rows)
    return np.asarray(out, dtype=np.float64)


def _write_record(f, payload: bytes) -> None:
    n = struct.pack("<i", len(payload))
    f.write(n + payload + n)


def _read_record(f) -> bytes:
    head = f.read(4)
    if len(head) != 4:
        raise EOFError("unformatted file ends early")
    (n,) = struct.unpack("<i", head)
    payload = f.read(n)
    (n2,) = struct.unpack("<i", f.read(4))
    if n2 != n or len(payload) != n:
        raise ValueError("damaged unformatted record")
    return payload


def _write_list(f, values, fmt: str, per_line: int = 8) -> None:
    for i in range(0, len(values), per_line):
        f.write(" ".join(fmt % v for v in values[i:i + per_line]) + "\n")


def write_problem(prefix: str, gp: GlobalProblem, nsublev, tol: float = 1e-8, maxit: int = 500,
                  ndecrmax: int = 50) -> None:
    """Writes the files of a global problem under the path prefix."""
    nsublev = list(nsublev)
    linet = int(gp.nnet.sum())
    with open(prefix + ".PAR", "w") as f:
        f.write(f"{gp.ndim} {nsublev[0]} {gp.nelem} {gp.ndof} {gp.nnod} 0 {linet} {tol:.6e} {maxit} {ndecrmax}\n")
        f.write(f"{gp.meshdim}\n")
    with open(prefix + ".ML", "w") as f:
        f.write(f"{len(nsublev)}\n" + " ".join(str(x) for x in nsublev) + "\n")
    with open(prefix + ".GMIS", "w") as f:
        _write_list(f, (gp.inet + 1).tolist(), "%d", 16)
        _write_list(f, gp.nnet.tolist(), "%d", 16)
        _write_list(f, gp.nndf.tolist(), "%d", 16)
        _write_list(f, np.asarray(gp.xyz).T.ravel().tolist(), "%.17e", 4)
    with open(prefix + ".FVS", "w") as f:
        _write_list(f, gp.ifix.tolist(), "%d", 16)
        _write_list(f, gp.fixv.tolist(), "%.17e", 4)
    with open(prefix + ".RHS", "wb") as f:
        _write_record(f, np.asarray(gp.rhs, dtype="<f8").tobytes())
    with open(prefix + ".ELM", "wb") as f:
        for k in gp.elements:
            e = pack_element(np.asarray(k), gp.matrixtype)
            _write_record(f, struct.pack("<i", len(e)) + e.astype("<f8").tobytes())


def _read_numbers(path: str):
    with open(path) as f:
        return f.read().replace(",", " ").split()


def read_par(prefix: str) -> dict:
    with open(prefix + ".PAR") as f:
        lines = f.read().split("\n")
    w = lines[0].replace(",", " ").split()
    ndim, nsub, nelem, ndof, nnod, nnodc, linet = (int(x) for x in w[:7])
    tol, maxit, ndecrmax = float(w[7].replace("d", "e").replace("D", "e")), int(w[8]), int(w[9])
    meshdim = ndim
    if len(lines) > 1 and lines[1].strip():
        meshdim = int(lines[1].split()[0])
    return dict(ndim=ndim, nsub=nsub, nelem=nelem, ndof=ndof, nnod=nnod, nnodc=nnodc, linet=linet, tol=tol,
                maxit=maxit, ndecrmax=ndecrmax, meshdim=meshdim)


def read_ml(prefix: str):
    w = _read_numbers(prefix + ".ML")
    nl = int(w[0])
    return nl, [int(x) for x in w[1:1 + nl]]


def read_problem(prefix: str):
    """The arrays of the global example files (element matrices stay in .ELM)."""
    par = read_par(prefix)
    w = _read_numbers(prefix + ".GMIS")
    o = 0
    inet = np.array(w[o:o + par["linet"]], dtype=np.int32) - 1; o += par["linet"]
    nnet = np.array(w[o:o + par["nelem"]], dtype=np.int32); o += par["nelem"]
    nndf = np.array(w[o:o + par["nnod"]], dtype=np.int32); o += par["nnod"]
    xyz = np.array([float(x.replace("d", "e").replace("D", "e")) for x in w[o:o + par["nnod"] * par["ndim"]]])
    xyz = xyz.reshape(par["ndim"], par["nnod"]).T
    w = _read_numbers(prefix + ".FVS")
    ifix = np.array(w[:par["ndof"]], dtype=np.int32)
    fixv = np.array([float(x.replace("d", "e").replace("D", "e")) for x in w[par["ndof"]:2 * par["ndof"]]])
    with open(prefix + ".RHS", "rb") as f:
        rhs = np.frombuffer(_read_record(f), dtype="<f8").copy()
    return par, dict(inet=inet, nnet=nnet, nndf=nndf, xyz=xyz, ifix=ifix, fixv=fixv, rhs=rhs)


# ------------------------------------------------------------- generators
def _cube_global(n: int, km_of_element, matrixtype: int) -> GlobalProblem:
    nng = n + 1
    h = 1.0 / n
    conn = problems.cube_connectivity(n)            # (n^3, 8) global node numbers
    k, j, i = np.meshgrid(np.arange(nng), np.arange(nng), np.arange(nng), indexing="ij")
    xyz = np.stack([i.ravel() * h, j.ravel() * h, k.ravel() * h], axis=1)
    onb = np.any((xyz < 0.5 * h) | (xyz > 1.0 - 0.5 * h), axis=1)
    nnod = nng ** 3
    rhs = np.where(onb, 0.0, h ** 3)
    return GlobalProblem(nelem=n ** 3, nnod=nnod, ndof=nnod, ndim=3, meshdim=3,
                         inet=conn.astype(np.int32).ravel(), nnet=np.full(n ** 3, 8, dtype=np.int32),
                         nndf=np.ones(nnod, dtype=np.int32), xyz=xyz, ifix=onb.astype(np.int32),
                         fixv=np.zeros(nnod), rhs=rhs, elements=[km_of_element(e) for e in range(n ** 3)],
                         matrixtype=matrixtype)


def poisson_global(n: int, kappa: Optional[np.ndarray] = None) -> GlobalProblem:
    """-Laplace(u) = 1 on the unit cube with n^3 Q1 elements, u = 0 on the boundary."""
    km = (1.0 / n) * problems.q1_laplace_reference_matrix()
    return _cube_global(n, lambda e: km * (kappa[e] if kappa is not None else 1.0), 1)


def convection_diffusion_global(n: int, b=(10.0, 7.0, 4.0)) -> GlobalProblem:
    """-Laplace(u) + b . grad(u) = 1 on the unit cube (general matrix)."""
    h = 1.0 / n
    km = h * problems.q1_laplace_reference_matrix() + h * h * problems.q1_convection_reference_matrix(b)
    return _cube_global(n, lambda e: km, 0)


# ------------------------------------------------------------------ solve
def solve_global(prefix: str, precision: int = 1, method: Optional[int] = None, matrixtype: int = 1,
                 numbase: int = 0, weights_type: int = 0):
    """The sequence of the reference's global example: read the files, upload
    the global data with the element matrix file, set up, solve with the
    tolerances of .PAR, return (global solution, num_iter, reason, cond)."""
    from . import (bddcml_download_global_solution, bddcml_finalize, bddcml_init, bddcml_setup_preconditioner,
                   bddcml_solve, bddcml_upload_global_data_file, set_precision)
    par, d = read_problem(prefix)
    nl, nsublev = read_ml(prefix)
    if method is None:
        method = 0 if matrixtype == 1 else 1
    bddcml_init(nl, nsublev, -1, 0, 0, numbase, 0)
    try:
        set_precision(precision)
        bddcml_upload_global_data_file(par["nelem"], par["nnod"], par["ndof"], par["ndim"], par["meshdim"],
                                       d["inet"] + numbase, d["nnet"], d["nndf"], d["xyz"], d["ifix"], d["fixv"],
                                       d["rhs"], np.zeros(par["ndof"]), prefix + ".ELM")
        bddcml_setup_preconditioner(matrixtype, 0, 1, 1, 1, 0, 0, weights_type)
        it, reason, cond = bddcml_solve(0, method, par["tol"], par["maxit"], par["ndecrmax"], 0, 0)
        u = bddcml_download_global_solution(par["ndof"])
    finally:
        bddcml_finalize()
    return u, it, reason, cond
