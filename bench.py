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
+ PCG + interior resolve), from CUDA events the library records on its own
stream.  `e2e` is the wall time of the reference-facing C ABI sequence (init,
upload of every subdomain from host buffers, setup, solve, download,
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


def visible_device_for_rank(local_rank, visible):
    """The CUDA_VISIBLE_DEVICES value for one rank of a multi-rank launch: the
    LOCAL_RANK-th entry of a list the launcher already set (so that a job given
    GPUs 4,5 stays on them), else the bare local rank."""
    if visible:
        ids = [v.strip() for v in visible.split(",") if v.strip()]
        if local_rank >= len(ids):
            raise ValueError(f"LOCAL_RANK {local_rank} but CUDA_VISIBLE_DEVICES lists {len(ids)} GPUs")
        return ids[local_rank]
    return str(local_rank)


# one process per GPU under torchrun: pin the GPU before any CUDA library loads
if "LOCAL_RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
    os.environ["CUDA_VISIBLE_DEVICES"] = visible_device_for_rank(int(os.environ["LOCAL_RANK"]),
                                                                 os.environ.get("CUDA_VISIBLE_DEVICES"))

import numpy as np  # noqa: E402

METRIC = "time-to-solve at rel.res 1e-8: batched mixed-prec vs plain FP64 BDDC, same GB300"

WORKLOADS = {
    # name: problem generator, weights type, adaptive threshold (None: no adaptive constraints)
    "poisson_128^3_512subs": ("cube", (16, 8), 0, None),
    "poisson_64^3_64subs": ("cube", (16, 4), 0, None),
    "poisson_32^3_8subs": ("cube", (16, 2), 0, None),
    # 96^3, kappa = exp(2 g) (seed 17) with 20 channels of 1e4 (width 2), 300 boxes
    # of sides 8..24 (6 x 5 x 10), rho-scaling, adaptive face constraints tau = 10
    "poisson_96^3_300boxes_channels_adaptive": ("channels", (96, (6, 5, 10)), 1, 10.0),
    "poisson_96^3_300boxes_channels": ("channels", (96, (6, 5, 10)), 1, None),
    # 96^3 Q1 elasticity (E = 1, nu = 0.3) with 10 % of spherical inclusions of E = 1e3
    # (radius 3..6, seed 5), clamped at x = 0, body force -z; 512 subdomains, three levels
    # with 8 level-2 subdomains, rho-scaling; one right-hand side
    "elasticity_96^3_512subs_3levels": ("elasticity", (12, 8, 8), 1, None),
    # the same problem with 64 load cases (every element's body force scaled by
    # its own iid N(0, 1) factor per case, seed 5) solved by one batched PCG
    "elasticity_96^3_512subs_3levels_64rhs": ("elasticity", (12, 8, 8, 64), 1, None),
    # the same subdomain size on 48^3 with 64 subdomains (8 level-2 subdomains): the
    # small case of the batched kernels for parity runs and full profiler captures
    "elasticity_48^3_64subs_3levels_64rhs": ("elasticity", (12, 4, 8, 64), 1, None),
    # differentiation: 64^3 Poisson, 64 subdomains of 16^3, log-normal kappa (sigma 1,
    # seed 3), J = 1/2 |u - u*|^2 with u* from 8 seeded Fourier modes (seed 4); one step
    # = forward solve + adjoint solve + per-element gradient through torch.autograd
    "poisson_64^3_64subs_gradient": ("gradient", (16, 4), 0, None),
}
DEFAULT_WORKLOAD = "poisson_128^3_512subs"

SETUP_PHASES = ["factor_interior", "solve_interior", "refine_residual", "schur", "precond_factor", "precond_solve",
                "precond_blocks", "coarse"]


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
        self.rows, self.proc, self.th = [], None, None

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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in self.rows if len(r) > 2) if v is not None]
        mx = [v for v in (num(r[2]) for r in self.rows if len(r) > 2) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        loaded = [v for v in sm if sm and v > 0.5 * max(sm)]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons), "samples": len(self.rows)}


def make_problem(workload):
    from bddcml_gb300 import problems
    kind, par, _, _ = WORKLOADS[workload]
    if kind == "cube":
        return problems.poisson_on_cube(*par)
    if kind == "gradient":
        return problems.poisson_on_cube(*par, kappa=problems.lognormal_kappa(par[0] * par[1], 1.0, seed=3))
    if kind == "elasticity":
        nes, nss = par[0], par[1]
        return problems.elasticity_on_cube(nes, nss, nu=0.3, young=problems.inclusions_young(nes * nss))
    ne, counts = par
    kappa = problems.channel_kappa(ne, nchannels=20, width=2, contrast=1e4, sigma=2.0, seed=17)
    return problems.poisson_boxes(ne, problems.random_box_counts(ne, counts, 8, 24, seed=17), kappa=kappa)


def make_loads(prob, workload):
    """Batched load cases of a workload (None: the problem's own single load)."""
    from bddcml_gb300 import problems
    kind, par, _, _ = WORKLOADS[workload]
    if kind == "elasticity" and len(par) > 3:
        return problems.body_force_loads(prob, par[3], seed=5)
    return None


def e2e_solve(B, prob, precision, profile=False, workload=DEFAULT_WORKLOAD, loads=None):
    """The reference-facing sequence through the C ABI with host buffers
    (poisson_on_cube.f90:373-672); with loads, the batched upload, solve and
    download of all load cases in place of the single solve."""
    kind, par, weights, tau = WORKLOADS[workload]
    tp = [time.perf_counter()]
    if kind == "elasticity":
        B.bddcml_init(3, [prob.nsub, par[2], 1], -1, 0, 0, 0, 0)
    else:
        B.bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
    B.set_precision(precision)
    if profile:
        B.set_profiling(True)
    if tau is not None:
        B.set_adaptive_threshold(tau)
    tp.append(time.perf_counter())
    B.upload_problem(prob)
    tp.append(time.perf_counter())
    B.bddcml_setup_preconditioner(1, 0, 1, 1, 1, 1 if tau is not None else 0, 0, weights)
    tp.append(time.perf_counter())
    if loads is None:
        it, reason, cond = B.bddcml_solve(0, 0, 1e-8, 1000, 1000, 0, 0)
        tp.append(time.perf_counter())
        sols = [B.bddcml_download_local_solution(s.isub, s.ndofs) for s in prob.subdomains]
    else:
        nrhs = loads[0].shape[0]
        for s, ld in zip(prob.subdomains, loads):
            B.bddcml_upload_subdomain_rhs_batch(s.isub, ld, 1)
        it, reason, cond = B.bddcml_solve_batch(nrhs, 0, 0, 1e-8, 1000, 1000)
        tp.append(time.perf_counter())
        sols = [B.bddcml_download_local_solution_batch(s.isub, nrhs, s.ndofs) for s in prob.subdomains]
    tp.append(time.perf_counter())
    st = B.get_stats()
    prof = B.get_profile()
    B.bddcml_finalize()
    tp.append(time.perf_counter())
    names = ["init", "upload", "setup", "solve", "download", "finalize"]
    st["e2e_phases_ms"] = {n: 1e3 * (tp[i + 1] - tp[i]) for i, n in enumerate(names)}
    return tp[-1] - tp[0], it, reason, cond, st, prof, sols


def phase_roofline(phase, prof, st, hbm, tensor, peak_kind):
    """Algorithmic work per launch of a phase (reported by the library from the
    exact block structure) over its average launch time (CUDA events on the
    library stream)."""
    ms, cnt = prof[phase]
    if cnt == 0 or ms <= 0:
        return None
    t = ms / cnt / 1e3
    if phase in ("solve_interior", "precond_solve"):
        # one launch = forward + backward block-band sweep over all subdomains.
        # 3xTF32: each algorithmic FP32 flop costs three TF32 MMA flops and the
        # dense TF32 rate is half the bf16 rate: attainable = bf16 peak / 6
        flop = st["flop_sweep_oo"] if phase == "solve_interior" else st["flop_sweep_s"]
        ach = flop / t / 1e12
        return {"bound": "tensor", "achieved": ach, "peak": tensor, "unit": "TFLOP/s", "frac": ach / tensor,
                "algorithmic_flop": flop, "avg_launch_ms": ms / cnt, "peak_kind": peak_kind,
                "attainable_3xtf32": tensor / 6.0, "frac_of_3xtf32_ceiling": ach / (tensor / 6.0)}
    byts = {"schur_apply": st["bytes_schur_apply"], "precond_local": st["bytes_pc_local"],
            "refine_residual": st["bytes_residual"], "assemble_dot": st.get("bytes_assemble_dot"),
            "assemble_z": st.get("bytes_assemble_z"), "coarse_apply": st.get("bytes_coarse_apply")}.get(phase)
    if byts is None:
        return None
    ach = byts / t / 1e9
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "algorithmic_bytes": byts, "avg_launch_ms": ms / cnt, "peak_kind": peak_kind}


def roofline_traffic(workload, phase, roof):
    """DRAM bytes per launch of the roofline kernel, from the committed ncu
    captures of smaller cases of the same kernels, scaled by the units processed
    (full-size captures would exceed the capture size limit); None elsewhere."""
    if workload == "poisson_128^3_512subs" and phase == "solve_interior" and "algorithmic_flop" in roof:
        # k_band_sweep_tc forward + backward sweep at 64^3 with 64 subdomains of 16^3
        # (profiles/k_band_sweep_tc_poisson64.md): 6.151 GB for 3.756e11 flop, scaled by
        # the algorithmic flop (block rows x window blocks x columns processed)
        return (1.845567 + 1.173766 + 1.959529 + 1.172174) * 1e9 * roof["algorithmic_flop"] / 375641866240.0, \
            "ncu capture at 64^3 (64 subdomains of 16^3), scaled by the sweeps' algorithmic flop"
    if phase == "schur_apply" and "algorithmic_bytes" in roof:
        # kb_schur_oz at 48^3 (profiles/kb_schur_oz_elasticity48_64subs_64rhs.md):
        # 4.675 GB read + 0.063 GB written for 4.5068 GB of slice bytes
        return roof["algorithmic_bytes"] * (4.675 + 0.063) / 4.506779648, \
            "ncu capture at 48^3 (64 subdomains), scaled by slice bytes"
    return None, None


def batch_schur_roofline(prof, st, hbm, tensor, peak_kind):
    """Batched Schur apply: the sliced operator (6-bit bf16 slices of S, made at
    the batch setup) is streamed once per apply for all columns, so the bound is
    its bytes over HBM; the tensor-core view (bf16 MMA flops executed for the 36
    slice pairs) and the FP64-equivalent rate of S X are reported beside it."""
    ms, cnt = prof["schur_apply"]
    if cnt == 0 or ms <= 0:
        return None
    t = ms / cnt / 1e3
    byts = st["batch_bytes_schur"]
    ach = byts / t / 1e9
    out = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
           "algorithmic_bytes": byts, "avg_launch_ms": ms / cnt, "peak_kind": peak_kind}
    if st["batch_flop_schur_mma"] > 0:
        mma = st["batch_flop_schur_mma"] / t / 1e12
        out["tensor_bf16_tflops"] = mma
        out["tensor_frac"] = mma / tensor
    out["fp64_equivalent_tflops"] = st["batch_flop_schur"] / t / 1e12
    return out


def cpu_baseline(prob, nthreads=None, weights=0):
    """The CPU restatement (oracle/) on the same workload: upload + setup + solve.
    Returns the baseline record and the oracle's global solution (the parity
    reference of the GPU solution)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    nthreads = nthreads or os.cpu_count() or 1
    t0 = time.perf_counter()
    o = orc.Oracle(prob, nthreads=nthreads)
    o.setup(1, 1, weights)
    it, reason, cond = o.solve(1e-8, 1000, 1000)
    t = time.perf_counter() - t0
    return {"value": t, "unit": "s", "cores": nthreads, "kind": "port",
            "sample": f"full workload, one solve (upload + setup + PCG, {it} iterations)", "iterations": it,
            "note": "band-Cholesky restatement (A11 and the constrained local problem factored in band form in "
                    "the subdomain's dof order), not the reference's MUMPS sparse LDL^T"}, \
        (o.global_solution(), it, reason)


def global_vector(prob, sols):
    u = np.zeros(prob.ndof)
    for s, v in zip(prob.subdomains, sols):
        u[s.isvgvn] = v
    return u


def oracle_parity(prob, sols, it, reason, sols64, it64, oracle_result):
    """GPU solutions (mixed, and plain FP64 when run) against the oracle's on
    the same workload: iterations within +-2 and relative error <= 1e-7
    (mixed) / 1e-8 (FP64), the bar of the path's specification."""
    u_o, it_o, reason_o = oracle_result
    nrm = np.linalg.norm(u_o)
    out = {"iterations_oracle": int(it_o), "iterations": int(it), "converged_reason_oracle": int(reason_o),
           "rel_err_vs_oracle": float(np.linalg.norm(global_vector(prob, sols) - u_o) / nrm),
           "tolerance": 1e-7}
    ok = reason == reason_o == 0 and abs(int(it) - int(it_o)) <= 2 and out["rel_err_vs_oracle"] <= 1e-7
    if sols64 is not None:
        out["fp64_iterations"] = int(it64)
        out["fp64_rel_err_vs_oracle"] = float(np.linalg.norm(global_vector(prob, sols64) - u_o) / nrm)
        out["fp64_tolerance"] = 1e-8
        ok = ok and abs(int(it64) - int(it_o)) <= 2 and out["fp64_rel_err_vs_oracle"] <= 1e-8
    out["ok"] = bool(ok)
    return out


def replica_max(values, dist=None):
    """Per-rank figures (lists of floats) -> their maximum over the ranks of the
    process group (the replicas of `--gpus N`); the values themselves on one rank."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def run_gpu(args):
    import bddcml_gb300 as B
    from bddcml_gb300 import build
    build.build()
    dist = None
    rank = 0
    if args.gpus > 1 and "RANK" in os.environ:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        rank = dist.get_rank()
    prob = make_problem(args.workload)
    loads = make_loads(prob, args.workload)
    hbm, tensor, peak_kind = load_peaks()

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        e2e_solve(B, prob, 1, workload=args.workload, loads=loads)
    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
    e2e_t, dev_t = [], []
    for _ in range(args.steps):
        barrier()
        t, it, reason, cond, st, prof, sols = e2e_solve(B, prob, 1, workload=args.workload, loads=loads)
        barrier()
        e2e_t.append(t)
        dev_t.append((prof["numeric_total"][0] + prof["solve_total"][0]) / 1e3)
    clocks = sampler.stop() if sampler else None
    dev_mean, e2e_mean = replica_max([statistics.mean(dev_t), statistics.mean(e2e_t)], dist)  # max over ranks
    # profiled run outside the timed region: per-phase device times
    _, _, _, _, st_p, prof_p, _ = e2e_solve(B, prob, 1, profile=True, workload=args.workload, loads=loads)
    fp64 = None
    if not args.no_fp64:
        t64, it64, r64, c64, st64, prof64, sols64 = e2e_solve(B, prob, 0, workload=args.workload, loads=loads)
        fp64 = {"time_to_solve_s": (prof64["numeric_total"][0] + prof64["solve_total"][0]) / 1e3,
                "e2e_s": t64, "iterations": int(np.max(it64)),
                "numeric_setup_s": prof64["numeric_total"][0] / 1e3, "solve_s": prof64["solve_total"][0] / 1e3}
        # per load case: |u_mixed - u_fp64| / |u_fp64| over all subdomain dofs (max over cases)
        d2 = sum(np.sum(np.atleast_2d(a - b) ** 2, axis=1) for a, b in zip(sols, sols64))
        n2 = sum(np.sum(np.atleast_2d(b) ** 2, axis=1) for b in sols64)
        fp64["mixed_vs_fp64_rel_err"] = float(np.max(np.sqrt(d2 / n2)))
        fp64["speedup_mixed_over_fp64"] = fp64["time_to_solve_s"] / dev_mean
    batch = None
    if loads is not None:
        # one load at a time through the same solver (single-load ABI), for the
        # gain of batching: numeric setup + nrhs x the single solve
        _, it1, _, _, _, prof1, _ = e2e_solve(B, prob, 1, workload=args.workload)
        nrhs = loads[0].shape[0]
        batch = {"nrhs": nrhs, "iterations_min": int(np.min(it)), "iterations_max": int(np.max(it)),
                 "iterations_mean": float(np.mean(it)), "condition_number_max": float(np.max(cond)),
                 "all_converged": bool(np.all(reason == 0)),
                 "single_load_solve_s": prof1["solve_total"][0] / 1e3, "single_load_iterations": it1,
                 "sequential_estimate_s": (prof1["numeric_total"][0] + nrhs * prof1["solve_total"][0]) / 1e3}
        batch["speedup_over_sequential"] = batch["sequential_estimate_s"] / dev_mean
        it, reason, cond = int(np.max(it)), int(np.min(reason)), float(np.max(cond))
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    dominant = max(SETUP_PHASES + ["pcg"], key=lambda k: prof_p[k][0])
    roof = phase_roofline(dominant, prof_p, st_p, hbm, tensor, peak_kind)
    if loads is not None:
        # batched solve: the Schur apply is the largest single kernel (kb_schur_oz)
        dominant = "schur_apply"
        roof = batch_schur_roofline(prof_p, st_p, hbm, tensor, peak_kind)
    if roof is None:  # dominant phase without a single-kernel roofline: largest phase that has one
        cands = [k for k in ("solve_interior", "precond_solve", "refine_residual", "schur_apply", "precond_local")
                 if phase_roofline(k, prof_p, st_p, hbm, tensor, peak_kind)]
        dominant = max(cands, key=lambda k: prof_p[k][0])
        roof = phase_roofline(dominant, prof_p, st_p, hbm, tensor, peak_kind)
    roof["phase"] = dominant
    roof["traffic"], src = roofline_traffic(args.workload, dominant, roof)
    if src:
        roof["traffic_source"] = src
    all_roof = {k: phase_roofline(k, prof_p, st_p, hbm, tensor, peak_kind)
                for k in ("solve_interior", "precond_solve", "refine_residual", "schur_apply", "precond_local",
                          "assemble_dot", "assemble_z", "coarse_apply")}
    kind, _, weights, tau = WORKLOADS[args.workload]
    # the oracle solves the adaptive pair eigenproblems densely, and takes minutes on the
    # three-level elasticity: both far beyond a bounded sample
    cpu, parity = None, None
    if not (args.no_cpu_baseline or tau is not None or kind == "elasticity"):
        cpu, oracle_result = cpu_baseline(prob, weights=weights)
        parity = oracle_parity(prob, sols, it, reason, sols64 if fp64 else None, fp64["iterations"] if fp64 else 0,
                               oracle_result)
    out = {
        "metric": METRIC, "value": dev_mean, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_mean * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factors / f64 Krylov",
        "data": {"cube": "synthetic (deterministic Poisson cube)",
                 "channels": "synthetic (seeded coefficients, channels and box partition)",
                 "elasticity": "synthetic (seeded spherical inclusions)"}[WORKLOADS[args.workload][0]],
        "config": {"workload": args.workload, "elements": prob.nelem, "subdomains": prob.nsub, "dofs": prob.ndof,
                   "precision": "mixed", "tol": 1e-8,
                   "constraints": "corners+edges+faces" + (f" + adaptive faces (tau {tau:g})" if tau else ""),
                   "weights": "cardinality" if weights == 0 else "diagonal stiffness",
                   "l2": "inputs larger than L2 (several GB of factors streamed per step)",
                   "timing": "CUDA events on the library stream (value); host wall clock around the ABI calls (e2e)",
                   "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "1 GPU, all subdomains resident"},
        "e2e": {"value": e2e_mean, "unit": "s", "h2d_bytes_per_step": st["h2d_bytes"],
                "d2h_bytes_per_step": st["d2h_bytes"]},
        "iterations": it, "converged_reason": reason, "condition_number": cond, "batch": batch,
        "phases_ms": {k: v[0] for k, v in prof_p.items()},
        "phase_launches": {k: v[1] for k, v in prof_p.items()},
        "gpu_launches": int(args.steps * (st["launches_setup"] + st["launches_solve"])),
        "gpu_launches_per_step": {"setup": int(st["launches_setup"]), "solve": int(st["launches_solve"])},
        "roofline": roof, "phase_rooflines": all_roof, "fp64_plain": fp64, "cpu_baseline": cpu,
        "parity": parity,
        "refinement": {"max_correction_ratio_first": st_p["refine1"], "max_correction_ratio_last": st_p["refine2"],
                       "steps": int(st_p.get("refine_steps", 0))},
        "adaptive": None if tau is None else {k: st_p[k] for k in ("npair", "nadaptive", "adapt_est", "t_adaptive",
                                                                  "lobpcg_resid", "lobpcg_iter", "ndofc")},
        "host_ms": {k: 1e3 * st_p[k] for k in ("t_upload", "t_host_assemble", "t_host_iface", "t_host_globs",
                                                "t_host_blocks", "t_device_setup", "t_dev_alloc", "t_dev_h2d")},
        "e2e_phases_ms": st["e2e_phases_ms"],
        "clocks": clocks,
    }
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    if parity is not None and not parity["ok"]:
        print(f"parity with the oracle failed: {parity}", file=sys.stderr)
        sys.exit(3)


def run_gradient(args):
    """Differentiation workload: dJ/dkappa through the torch.autograd binding
    (forward BDDC solve, adjoint solve reusing the forward factors, per-element
    gradient kernel).  `value` is the device time: the library's CUDA events of
    the forward setup and solve and of the adjoint's new data and solve, plus
    the gradient kernel.  `e2e` is the wall time of the user call from kappa in
    pinned host memory to the gradient back in host memory.  Outside the timed
    steps the gradient is compared with the oracle's forward + adjoint gradient
    (same tolerance), and plain-FP64 solves to relres 1e-12 give central
    differences along 32 seeded directions (step 1e-6)."""
    import torch
    import bddcml_gb300 as B
    from bddcml_gb300 import build, problems
    from bddcml_gb300.autograd import PoissonCube
    build.build()
    ne, ns = WORKLOADS[args.workload][1]
    n = ne * ns
    hbm, tensor, peak_kind = load_peaks()
    kappa = problems.lognormal_kappa(n, 1.0, seed=3)
    ustar = problems.smooth_target(n, seed=4)
    k_host = torch.tensor(kappa, dtype=torch.float64).pin_memory()
    us = torch.tensor(ustar, dtype=torch.float64, device="cuda")
    op = PoissonCube(ne, ns, precision=1, tol=1e-8, maxit=1000)

    def step(profile=False):
        op.profile = profile
        t0 = time.perf_counter()
        k = k_host.to("cuda", non_blocking=True).requires_grad_(True)
        u = op.solve(k)
        J = 0.5 * torch.sum((u - us) ** 2)
        J.backward()
        g = k.grad.to("cpu")
        t = time.perf_counter() - t0
        dev = (op.last_profile["numeric_total"][0] + op.last_profile["solve_total"][0] + op.last_gradient_ms) / 1e3
        return t, dev, u.detach(), g

    for _ in range(args.warmup):
        step()
    sampler = ClockSampler()
    sampler.start()
    e2e_t, dev_t = [], []
    for _ in range(args.steps):
        t, dev, u, g = step()
        e2e_t.append(t)
        dev_t.append(dev)
    clocks = sampler.stop()
    dev_mean, e2e_mean = statistics.mean(dev_t), statistics.mean(e2e_t)
    st = op.last_stats
    it_f, it_a = op.last_iterations, op.last_adjoint_iterations
    step(profile=True)
    prof_p, st_p = op.last_profile, op.last_stats
    dominant = max(SETUP_PHASES + ["pcg"], key=lambda k: prof_p[k][0])
    roof = phase_roofline(dominant, prof_p, st_p, hbm, tensor, peak_kind)
    if roof is None:
        cands = [k for k in ("solve_interior", "precond_solve", "refine_residual", "schur_apply", "precond_local")
                 if phase_roofline(k, prof_p, st_p, hbm, tensor, peak_kind)]
        dominant = max(cands, key=lambda k: prof_p[k][0])
        roof = phase_roofline(dominant, prof_p, st_p, hbm, tensor, peak_kind)
    roof["phase"] = dominant
    roof["traffic"] = None
    # the oracle's forward + adjoint gradient at the same tolerance (CPU leg)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from oracle_gradient import oracle_gradient
    orc.build()
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    u_o, g_o, it_fo, it_ao = oracle_gradient(orc, ne, ns, kappa, ustar, tol=1e-8, nthreads=nthreads,
                                             with_iterations=True)
    t_cpu = time.perf_counter() - t0
    u_np, g_np = u.cpu().numpy(), g.numpy()
    err_u = float(np.linalg.norm(u_np - u_o) / np.linalg.norm(u_o))
    err_g = float(np.linalg.norm(g_np - g_o) / np.linalg.norm(g_o))
    # central differences along 32 seeded directions, plain FP64 solves to relres 1e-12
    fd_op = PoissonCube(ne, ns, precision=0, tol=1e-12, maxit=1000)
    kt = torch.tensor(kappa, dtype=torch.float64, device="cuda")
    kg = kt.clone().requires_grad_(True)
    J = 0.5 * torch.sum((fd_op.solve(kg) - us) ** 2)
    J.backward()
    g_acc = kg.grad.cpu().numpy()
    err_g64 = float(np.linalg.norm(g_np - g_acc) / np.linalg.norm(g_acc))
    rng = np.random.default_rng(11)
    eps, worst = 1e-6, 0.0
    with torch.no_grad():
        for _ in range(32):
            d = rng.standard_normal(kappa.size)
            dt = torch.tensor(d, dtype=torch.float64, device="cuda")
            jp = 0.5 * torch.sum((fd_op.solve(kt * torch.exp(eps * dt)) - us) ** 2).item()
            jm = 0.5 * torch.sum((fd_op.solve(kt * torch.exp(-eps * dt)) - us) ** 2).item()
            fd = (jp - jm) / (2 * eps)
            an = float(np.dot(g_acc, kappa * d))
            worst = max(worst, abs(fd - an) / max(abs(fd), abs(an)))
    B.bddcml_finalize()
    parity = {"iterations": [int(it_f), int(it_a)], "iterations_oracle": [int(it_fo), int(it_ao)],
              "rel_err_vs_oracle": err_u, "gradient_rel_err_vs_oracle": err_g, "tolerance": 1e-7,
              "gradient_rel_diff_vs_fp64_tol1e-12": err_g64,
              "fd_directions": 32, "fd_step": eps, "fd_worst_rel_diff": worst, "fd_tolerance": 1e-5,
              "fd_solves": "plain FP64, relres 1e-12"}
    parity["ok"] = bool(abs(it_f - it_fo) <= 2 and abs(it_a - it_ao) <= 2 and err_u <= 1e-7 and err_g <= 1e-7
                        and worst <= 1e-5)
    h2d = st["h2d_bytes"] + kappa.nbytes
    d2h = st["d2h_bytes"] + kappa.nbytes
    out = {
        "metric": METRIC, "value": dev_mean, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_mean * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 factors / f64 Krylov", "data": "synthetic (seeded log-normal coefficients and target)",
        "config": {"workload": args.workload, "elements": n ** 3, "subdomains": ns ** 3, "dofs": (n + 1) ** 3,
                   "precision": "mixed", "tol": 1e-8, "objective": "1/2 |u - u*|^2",
                   "gradient_entries": n ** 3,
                   "step": "forward solve + adjoint solve (forward factors) + element gradient",
                   "l2": "inputs larger than L2 (factors streamed per step)",
                   "timing": "CUDA events of the library (setup, new data, solves) and of the gradient kernel "
                             "(value); host wall clock around the autograd call (e2e)",
                   "parallelism": "1 GPU, all subdomains resident"},
        "e2e": {"value": e2e_mean, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(args.steps * (st["launches_setup"] + st["launches_solve"] + 1)),
        "phases_ms": {k: v[0] for k, v in prof_p.items()}, "roofline": roof, "parity": parity,
        "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": nthreads, "kind": "port",
                         "sample": "full workload: oracle forward + adjoint solve and gradient, one step"},
        "clocks": clocks,
    }
    print(json.dumps(out))
    if not parity["ok"]:
        print(f"parity with the oracle failed: {parity}", file=sys.stderr)
        sys.exit(3)


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
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
    times, it = [], None
    nthreads = os.cpu_count() or 1
    kind, par, _, _ = WORKLOADS[args.workload]
    for _ in range(args.steps):
        t0 = time.perf_counter()
        if kind == "gradient":  # forward + adjoint solve and the element gradient
            from bddcml_gb300 import problems
            from oracle_gradient import oracle_gradient
            n = par[0] * par[1]
            _, _, it, _ = oracle_gradient(orc, par[0], par[1], problems.lognormal_kappa(n, 1.0, seed=3),
                                          problems.smooth_target(n, seed=4), tol=1e-8, nthreads=nthreads,
                                          with_iterations=True)
        else:
            o = orc.Oracle(prob, nthreads=nthreads)
            o.setup(1, 1, 0)
            it, reason, cond = o.solve(1e-8, 500, 50)
            del o
        times.append(time.perf_counter() - t0)
    v = statistics.mean(times)
    out = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (deterministic Poisson cube)", "impl": "reference",
           "config": {"workload": args.workload, "elements": prob.nelem, "subdomains": prob.nsub},
           "cpu_baseline": {"value": v, "unit": "s", "cores": nthreads, "kind": "port",
                            "sample": "full workload per step (upload + setup + PCG); warm-up steps on the 32^3 case"},
           "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "iterations": it,
           "note": "CPU restatement of the reference algorithm (oracle/), with band Cholesky factors of A11 and "
                   "of the constrained local problem in place of MUMPS's sparse LDL^T; the Fortran/MPI/MUMPS "
                   "reference cannot be built on this image"}
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
    elif WORKLOADS[args.workload][0] == "gradient":
        run_gradient(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
