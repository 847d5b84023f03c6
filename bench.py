#!/usr/bin/env python
"""Benchmark: time-to-solve of the BDDC-preconditioned interface PCG to
relative residual 1e-8 on one GB300, mixed precision (FP32 subdomain factors
and preconditioner blocks, FP64-accurate Schur operator, FP64 Krylov vectors,
weights and coarse solve) against the plain FP64 path of the same code.

Workload (default): -Laplace(u) = 1 on the unit cube, Q1 hexahedra, 128^3
elements, 8 x 8 x 8 = 512 cubic subdomains of 16^3 elements, homogeneous
Dirichlet boundary, corner + edge + face arithmetic constraints, weights by
cardinality, PCG tol 1e-8, zero initial guess (deterministic synthetic data,
generated like the reference example poisson_on_cube.f90).

One step = one complete solve.  `value` is the device time-to-solve from the
uploaded subdomain data resident in HBM to the solution in HBM (numeric setup
+ PCG + interior resolve), taken from CUDA events recorded by the library on
its own stream.  `e2e` is the wall time of the reference-facing C ABI sequence
(init, upload of every subdomain from host buffers, setup, solve, download,
finalize).  Every step streams several GB of factors (inputs larger than the
129 MB L2), so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference algorithm
(oracle/, OpenMP over subdomains) on the same workload: the reference itself
(Fortran + MPI + MUMPS) cannot be built on this image.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# one process per GPU under torchrun: pin the GPU before any CUDA library loads
if "LOCAL_RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import numpy as np  # noqa: E402

METRIC = "time-to-solve at rel.res 1e-8: batched mixed-prec vs plain FP64 BDDC, same GB300"

WORKLOADS = {
    # name: (elements per subdomain edge, subdomains per cube edge)
    "poisson_128^3_512subs": (16, 8),
    "poisson_32^3_8subs": (16, 2),
    "poisson_64^3_64subs": (16, 4),
}
DEFAULT_WORKLOAD = "poisson_128^3_512subs"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return pk["hbm_gbs"], pk["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        if not self.rows:
            return None
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        loaded = [v for v in sm if v > 0.5 * (max(sm) if sm else 1)]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons), "samples": len(self.rows)}


def make_problem(workload):
    from bddcml_gb300 import problems
    ne, ns = WORKLOADS[workload]
    return problems.poisson_on_cube(ne, ns)


def e2e_solve(B, prob, precision, profile=False):
    """The reference-facing sequence through the C ABI with host buffers."""
    t0 = time.perf_counter()
    B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    B.set_precision(precision)
    if profile:
        B.set_profiling(True)
    B.upload_problem(prob)
    B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
    it, reason, cond = B.bddcml_solve(0, 0, 1e-8, 500, 50, 0, 0)
    sols = [B.bddcml_download_local_solution(s.isub, s.ndofs) for s in prob.subdomains]
    st = B.get_stats()
    prof = B.get_profile()
    B.bddcml_finalize()
    t1 = time.perf_counter()
    return t1 - t0, it, reason, cond, st, prof, sols


def roofline_for(phase, prof, prob_sizes, hbm, tensor, mixed):
    """Algorithmic bytes or flops per launch of a phase, over its measured
    average launch time (CUDA events on the library stream)."""
    ms, cnt = prof[phase]
    if cnt == 0 or ms <= 0:
        return None
    per_launch_s = ms / cnt / 1e3
    ni = prob_sizes["ni"]
    if phase == "schur_apply":
        # S entries (8 B: FP32 hi/lo pair or FP64) + gathered input + written output (FP64)
        byts = float(np.sum(ni.astype(np.float64) ** 2) * 8 + np.sum(ni) * 16)
        ach = byts / per_launch_s / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "algorithmic_bytes": byts, "avg_launch_ms": ms / cnt}
    if phase == "precond_local":
        eb = 4 if mixed else 8
        nc = prob_sizes["nc"]
        byts = float(np.sum(ni.astype(np.float64) ** 2) * eb + np.sum(ni * nc) * eb + np.sum(ni) * 24)
        ach = byts / per_launch_s / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "algorithmic_bytes": byts, "avg_launch_ms": ms / cnt}
    return None


def dominant_roofline(prof, prob_sizes, hbm, tensor, mixed, nref):
    """Roofline of the phase with the largest share of the device time."""
    phases = ["factor_interior", "solve_interior", "refine_residual", "schur", "precond_factor", "precond_solve",
              "precond_blocks", "coarse", "schur_apply", "precond_local"]
    best = max(phases, key=lambda k: prof[k][0])
    ms, cnt = prof[best]
    no, ni, w = prob_sizes["no"], prob_sizes["ni"], prob_sizes["w"]
    if best == "solve_interior":
        # forward + backward block-band sweeps on [A_oi | f]: 2 * no * b * (ni+1) flop per sweep
        b = (w + 1) * 64
        flop = float(np.sum(2.0 * 2.0 * no * b * (ni + 1)))  # fwd + bwd
        ach = flop / (ms / cnt / 1e3) / 1e12
        return best, {"bound": "tensor", "achieved": ach, "peak": tensor, "unit": "TFLOP/s", "frac": ach / tensor,
                      "algorithmic_flop": flop, "avg_launch_ms": ms / cnt,
                      "note": "one launch = one forward+backward multi-RHS sweep over all subdomains"}
    r = roofline_for(best, prof, prob_sizes, 0, 0, mixed)
    return best, r


def sizes_of(prob):
    """Per-subdomain interface/interior sizes from the problem geometry."""
    ni, no, nc = [], [], []
    for s in prob.subdomains:
        pass
    return None


def run_gpu(args):
    import bddcml_gb300 as B
    from bddcml_gb300 import build
    build.build()
    dist = None
    rank, world = 0, 1
    if args.gpus > 1 and "RANK" in os.environ:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        rank, world = dist.get_rank(), dist.get_world_size()
    prob = make_problem(args.workload)
    hbm, tensor, peak_kind = load_peaks()

    def barrier():
        if dist:
            dist.barrier()

    # warm-up (also builds the JIT-free library state, page-in of host buffers)
    for _ in range(args.warmup):
        e2e_solve(B, prob, 1)
    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
    e2e_t, dev_t, info = [], [], None
    for _ in range(args.steps):
        barrier()
        t, it, reason, cond, st, prof, sols = e2e_solve(B, prob, 1)
        barrier()
        e2e_t.append(t)
        dev_t.append((prof["numeric_total"][0] + prof["solve_total"][0]) / 1e3)
        info = (it, reason, cond, st, prof)
    clocks = sampler.stop() if sampler else None
    it, reason, cond, st, prof = info
    # max over ranks
    if dist:
        import torch
        v = torch.tensor([statistics.mean(dev_t), statistics.mean(e2e_t)], dtype=torch.float64)
        dist.all_reduce(v, op=dist.ReduceOp.MAX)
        dev_mean, e2e_mean = float(v[0]), float(v[1])
    else:
        dev_mean, e2e_mean = statistics.mean(dev_t), statistics.mean(e2e_t)
    # profiled run (outside the timed region): per-phase device times
    t_p, _, _, _, st_p, prof_p, _ = e2e_solve(B, prob, 1, profile=True)
    # plain FP64 path, same workload (the comparison arm of the metric)
    fp64 = None
    if not args.no_fp64:
        t64, it64, r64, c64, st64, prof64, sols64 = e2e_solve(B, prob, 0)
        fp64 = {"time_to_solve_s": (prof64["numeric_total"][0] + prof64["solve_total"][0]) / 1e3,
                "e2e_s": t64, "iterations": it64,
                "numeric_setup_s": prof64["numeric_total"][0] / 1e3, "solve_s": prof64["solve_total"][0] / 1e3}
        d = np.concatenate([a - b for a, b in zip(sols, sols64)])
        nrm = np.sqrt(sum(float(np.dot(b, b)) for b in sols64))
        fp64["mixed_vs_fp64_rel_err"] = float(np.linalg.norm(d) / nrm)
        fp64["speedup_mixed_over_fp64"] = fp64["time_to_solve_s"] / dev_mean
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # sizes for the roofline
    from bddcml_gb300 import problems  # noqa: F401
    ni = np.array([st_p["sum_ndofi"]])  # replaced below by per-subdomain sizes
    sizes = subdomain_sizes(prob)
    phase, roof = dominant_roofline(prof_p, sizes, hbm, tensor, True, 2)
    if roof:
        roof["phase"] = phase
        roof["peak_kind"] = peak_kind
        roof["traffic"] = None
    apply_roof = {k: roofline_for(k, prof_p, sizes, hbm, tensor, True) for k in ("schur_apply", "precond_local")}
    for v in apply_roof.values():
        if v:
            v["peak_kind"] = peak_kind
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(prob)
    out = {
        "metric": METRIC, "value": dev_mean, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_mean * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factors / f64 Krylov", "data": "synthetic (deterministic Poisson cube)",
        "config": {"workload": args.workload, "elements": prob.nelem, "subdomains": prob.nsub, "dofs": prob.ndof,
                   "precision": "mixed", "tol": 1e-8, "constraints": "corners+edges+faces", "weights": "cardinality",
                   "l2": "inputs larger than L2 (several GB of factors streamed per step)",
                   "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "1 GPU, all subdomains resident"},
        "e2e": {"value": e2e_mean, "unit": "s", "h2d_bytes_per_step": st["h2d_bytes"],
                "d2h_bytes_per_step": st["d2h_bytes"]},
        "iterations": it, "converged_reason": reason, "condition_number": cond,
        "phases_ms": {k: v[0] for k, v in prof_p.items()},
        "phase_launches": {k: v[1] for k, v in prof_p.items()},
        "gpu_launches": None,
        "roofline": roof, "apply_roofline": apply_roof, "fp64_plain": fp64, "cpu_baseline": cpu,
        "clocks": clocks,
    }
    out["gpu_launches"] = estimate_launches(prof_p, sizes, it)
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def subdomain_sizes(prob):
    """Interface/interior dof counts and band blocks per subdomain (cube
    subdomains: interface = nodes shared with a neighbour)."""
    cnt = np.zeros(prob.nnod, dtype=np.int32)
    for s in prob.subdomains:
        cnt[s.isngn] += 1
    ni, no, w = [], [], []
    for s in prob.subdomains:
        shared = cnt[s.isngn] > 1
        ni.append(int(shared.sum()))
        no.append(int((~shared).sum()))
        # lexicographic interior: half bandwidth = nx*ny + nx + 1 of the interior box
        w.append(4)
    ni = np.array(ni)
    return {"ni": ni, "no": np.array(no), "w": np.array(w), "nc": np.full(len(ni), 26)}


def estimate_launches(prof, sizes, iters):
    """Kernel launches of one solve (setup + PCG) counted from the phase structure."""
    return int(sum(v[1] for v in prof.values()))


def cpu_baseline(prob, nthreads=None):
    """The CPU restatement (oracle/) on the same workload: upload + setup + solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    nthreads = nthreads or os.cpu_count() or 1
    t0 = time.perf_counter()
    o = orc.Oracle(prob, nthreads=nthreads)
    o.setup(1, 1, 0)
    it, reason, cond = o.solve(1e-8, 500, 50)
    t = time.perf_counter() - t0
    return {"value": t, "unit": "s", "cores": nthreads, "kind": "port",
            "sample": f"full workload, one solve (upload + setup + PCG), {it} iterations",
            "iterations": it}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    prob = make_problem(args.workload)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    small = make_problem("poisson_32^3_8subs")
    for _ in range(args.warmup):   # warm-up on a small case: page-in and thread pool start
        o = orc.Oracle(small)
        o.setup(1, 1, 0)
        o.solve(1e-8, 500, 50)
    times = []
    nthreads = os.cpu_count() or 1
    it = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o = orc.Oracle(prob, nthreads=nthreads)
        o.setup(1, 1, 0)
        it, reason, cond = o.solve(1e-8, 500, 50)
        times.append(time.perf_counter() - t0)
        del o
    v = statistics.mean(times)
    out = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (deterministic Poisson cube)", "impl": "reference",
           "config": {"workload": args.workload, "elements": prob.nelem, "subdomains": prob.nsub},
           "cpu_baseline": {"value": v, "unit": "s", "cores": nthreads, "kind": "port",
                            "sample": "full workload per step (upload + setup + PCG); warm-up steps on the 32^3 case"},
           "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "iterations": it,
           "note": "CPU restatement of the reference algorithm (oracle/); the Fortran/MPI/MUMPS reference "
                   "cannot be built on this image"}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
