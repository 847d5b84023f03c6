"""The drop-in boundary from C: tests/abi_driver.c calls the solver through
the reference's C API only (src/bddcml_interface_c.h:6-60), in the call order
of examples/poisson_on_cube.f90:373-672.

- Without a GPU: the driver is compiled with the reference's unmodified header
  and include/bddcml_gb300.h in one translation unit (a C compiler rejects any
  redeclaration whose types differ) and linked against libbddcgpu.so.  This
  needs the reference sources and is skipped where they are absent.
- On the GPU: the driver, compiled against include/bddcml_gb300.h and linked
  against libbddcgpu.so, solves the 32^3 Poisson problem in 2 x 2 x 2
  subdomains (seeded load) as a separate process; its solution is checked
  against the oracle.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "abi_driver.c")
OUR_HEADER = os.path.join(ROOT, "include", "bddcml_gb300.h")
LIBDIR = os.path.join(ROOT, "bddcml_gb300")
REFERENCE_HEADER = os.path.join(os.environ.get("BDDCML_REFERENCE", "/root/reference"), "src",
                                "bddcml_interface_c.h")


def _compile(out, header, extra=()):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Werror", f'-DBDDCML_HEADER="{header}"', *extra, DRIVER,
           "-L", LIBDIR, "-lbddcgpu", f"-Wl,-rpath,{LIBDIR}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def write_problem(prob, path, tol):
    """The problem file read by abi_driver.c (its header comment gives the layout)."""
    with open(path, "wb") as f:
        f.write(struct.pack("7i", prob.nelem, prob.nnod, prob.ndof, prob.ndim, prob.meshdim, prob.nsub,
                            prob.matrixtype))
        f.write(struct.pack("d", tol))
        for s in prob.subdomains:
            f.write(struct.pack("7i", s.isub, s.nelems, s.nnods, s.ndofs, len(s.inet), len(s.a_sparse),
                                s.is_rhs_complete))
            xyz = np.asarray(s.xyz, dtype=np.float64)
            xyz_cm = np.ascontiguousarray(xyz).ravel() if xyz.shape == (prob.ndim, s.nnods) else \
                np.ascontiguousarray(xyz.T).ravel()
            for a, t in ((s.inet, np.int32), (s.nnet, np.int32), (s.nndf, np.int32), (s.isngn, np.int32),
                         (s.isvgvn, np.int32), (s.isegn, np.int32), (xyz_cm, np.float64), (s.ifix, np.int32),
                         (s.fixv, np.float64), (s.rhs, np.float64), (s.sol, np.float64), (s.i_sparse, np.int32),
                         (s.j_sparse, np.int32), (s.a_sparse, np.float64)):
                f.write(np.ascontiguousarray(a, dtype=t).tobytes())


def read_solution(prob, path):
    with open(path, "rb") as f:
        it, reason = struct.unpack("2i", f.read(8))
        (cond,) = struct.unpack("d", f.read(8))
        u = np.zeros(prob.ndof)
        for s in prob.subdomains:
            u[s.isvgvn] = np.frombuffer(f.read(8 * s.ndofs), dtype=np.float64)
    return it, reason, cond, u


def test_driver_compiles_against_the_reference_header(built_lib, tmp_path):
    if not os.path.exists(REFERENCE_HEADER):
        pytest.skip("reference sources not present")
    _compile(str(tmp_path / "drv_ref"), REFERENCE_HEADER, extra=("-include", OUR_HEADER))


@pytest.mark.gpu
def test_driver_solves_through_the_c_abi(built_lib, oracle_mod, tmp_path):
    from bddcml_gb300 import problems
    exe = _compile(str(tmp_path / "drv"), OUR_HEADER)
    prob = problems.poisson_on_cube(16, 2)
    g = np.random.default_rng(3).standard_normal(prob.ndof)
    for s in prob.subdomains:
        s.rhs = np.where(s.ifix != 0, 0.0, g[s.isvgvn])
    write_problem(prob, str(tmp_path / "problem.bin"), 1e-8)
    r = subprocess.run([exe, str(tmp_path / "problem.bin"), str(tmp_path / "solution.bin")], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    it, reason, cond, u = read_solution(prob, str(tmp_path / "solution.bin"))
    o = oracle_mod.Oracle(prob)
    o.setup(1, 1, 0)
    it_o, reason_o, cond_o = o.solve(1e-8, 500, 50)
    u_o = o.global_solution()
    err = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    print(f"C driver: iterations {it} (oracle {it_o}), cond {cond:.4f} (oracle {cond_o:.4f}), error {err:.2e}")
    assert reason == reason_o == 0
    assert abs(it - it_o) <= 2
    assert err <= 1e-7
