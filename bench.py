#!/usr/bin/env python
"""Benchmark of the GB300 DOUG solve path.

Metric: time to relative residual 1e-8 (seconds per solve) on the 128^3
log-normal diffusion problem (2,097,152 unknowns, 14,581,760 nonzeros;
kappa = exp(g), g Gaussian with std 1 and correlation length 8 cells),
two-level additive Schwarz with 64 subdomains (4x4x4 boxes of the grid, the
stand-in for a METIS partition), overlap 2 and a smoothed-aggregation coarse
grid, solved by PCG on one GB300.

A step is one complete solve from a right-hand side already in HBM: the
numeric factorisations of the 64 subdomain matrices and of the coarse matrix,
then PCG to ||r||/||r0|| <= 1e-8.  The headline `value` is the mixed-precision
solve (FP32 subdomain factors and solves, flexible CG with FP64 recurrences,
FP64 residual replacement, FP64 coarse Cholesky); the plain FP64 solve of the
same system is timed beside it (`fp64_s`, `mixed_vs_fp64`).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun each rank solves its own replica (the path does not shard
across GPUs here: replicas only); rank 0 prints one JSON line.
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

import numpy as np  # noqa: E402

N = 128
PARTS_PER_DIM = 4
SEED = 0
TOL = "1.0e-8"
CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=2, smoothers=1,
           strong1="0.08", radius1=5, maxasize1=400, solve_tolerance=TOL, solve_maxiters=2000)
METRIC = "time to rel. residual 1e-8 (s), mixed+batched vs plain FP64 PCG, 1 GB300"
SUBSOLVE_TRAFFIC_BYTES = 4.620e9  # ncu, one PCG iteration of the 128^3 mixed solve
WORKLOAD = ("128^3 log-normal diffusion (sigma 1, corr. length 8), 7-point FV, 2,097,152 unknowns; "
            "PCG + 2-level additive Schwarz: 64 subdomains (4x4x4 boxes), overlap 2, "
            "smoothed-aggregation coarse grid")


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def _problem(grid=None):
    from doug_gb300 import problems as P
    g = grid or N
    n, r, c, v, b = P.diffusion3d_fv(g, sigma=1.0, corr=8.0, seed=SEED)
    part = P.block_partition(g, PARTS_PER_DIM)
    return n, r, c, v, b, part


def _solver(n, r, c, v, b, part, precision):
    import doug_gb300 as D
    s = D.DougSolver(CTL)
    s.set_option("precision", precision)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.set_partition(part)
    s.setup()
    return s


def _ctl_text(ctl):
    return "".join(f"{k} {v}\n" for k, v in ctl.items())


def _config(n, nnz, nsub, ncoarse):
    """The workload description both arms print (the same dict)."""
    return {"workload": WORKLOAD, "n": int(n), "nnz": int(nnz), "subdomains": int(nsub),
            "coarse_unknowns": int(ncoarse), "controls": CTL,
            "l2": "working set (factors ~2 GB) far larger than the 129 MB L2; no flush needed"}


def host_threads():
    """Host threads the CPU legs use: every core of this process's affinity set."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def oracle_whole_run(n, r, c, v, b, part, threads, steps, warmup):
    """The oracle's whole solve of the workload on `threads` host threads:
    its setup once (aggregation, R, AC, subdomains), then per step what a GPU
    step does: numeric factorisations of every subdomain matrix and of the
    coarse matrix (exact nested-dissection multifrontal Cholesky, standing in
    for the reference's UMFPACK) and the two-level PCG to 1e-8."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.set_threads(threads)
    t0 = time.perf_counter()
    sess = O.Session(n, r, c, v, _ctl_text(CTL), part)
    setup_s = time.perf_counter() - t0
    for _ in range(warmup):
        sess.solve(b)
    times, res = [], None
    for _ in range(steps):
        t = time.perf_counter()
        res = sess.solve(b)
        times.append(time.perf_counter() - t)
        if res["status"] != 0:
            raise RuntimeError("oracle solve failed: " + res["errmsg"])
    info = {"setup_s": setup_s, "factor_s": res["t_factor"], "pcg_s": res["t_solve"],
            "iterations": res["iterations"], "subdomains": len(sess.setup["subdomains"]),
            "coarse_unknowns": sess.setup["AC"][0]}
    sess.close()
    return times, res, info


def _oracle_sample(threads, info):
    return (f"the whole workload every step: numeric factorisations of the {info['subdomains']} subdomain "
            f"matrices and the coarse matrix ({info['coarse_unknowns']} unknowns) by the oracle's exact "
            f"nested-dissection multifrontal Cholesky, then its two-level PCG to 1e-8 "
            f"({info['iterations']} iterations), on {threads} host threads; the oracle's setup "
            f"(aggregation, R, AC, subdomains: {info['setup_s']:.2f} s) once before, like the GPU's")


def max_over_ranks(t, world, device="cuda"):
    """The slowest rank's time: with N GPUs every rank solves its own replica
    of the workload, and the step takes as long as the slowest one."""
    if world <= 1:
        return t
    import torch
    tt = torch.tensor([t], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def run_reference(args, rank, world):
    """The CPU arm: the oracle's restatement of DOUG's solve (the reference
    itself needs gfortran, MPI, METIS and UMFPACK, none of which the GPU host
    has) on the same workload, one whole solve per step on all host threads."""
    if rank != 0:
        return 0
    n, r, c, v, b, part = _problem()
    threads = host_threads()
    times, res, info = oracle_whole_run(n, r, c, v, b, part, threads, args.steps, args.warmup)
    value = float(np.mean(times))
    line = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, doug_gb300/problems.py)",
            "config": _config(n, len(v), info["subdomains"], info["coarse_unknowns"]),
            "iterations": info["iterations"], "setup_s": info["setup_s"],
            "phases": {"factor_s": info["factor_s"], "pcg_s": info["pcg_s"]},
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                             "sample": _oracle_sample(threads, info)},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, rank, world):
    import torch
    import doug_gb300 as D

    D.build_library()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n, r, c, v, b, part = _problem()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    # ---- mixed precision (headline) ----
    t0 = time.perf_counter()
    sm = _solver(n, r, c, v, b, part, precision=1)
    setup_s = time.perf_counter() - t0
    setup_phases = sm.setup_phases()
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    xd = torch.empty_like(bd)
    for _ in range(args.warmup):
        st = sm.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    its = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            st = sm.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
            launches += st.gpu_launches
            its.append(st.iterations)
        e1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_mixed = max_over_ranks(e0.elapsed_time(e1) * 1e-3 / args.steps, world)
    last = st
    # accuracy of the mixed solve against the FP64 path (below)
    x_mixed = xd.cpu().numpy()

    # ---- end to end through the host-buffer API (pinned host memory) ----
    bh = torch.tensor(b, dtype=torch.float64).pin_memory()
    xh = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes
    L = D.load_library()
    stats = D._Stats()
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = L.dg_solve(sm._h, ctypes.cast(bh.data_ptr(), ctypes.POINTER(ctypes.c_double)),
                        ctypes.cast(xh.data_ptr(), ctypes.POINTER(ctypes.c_double)), ctypes.byref(stats))
        e2e.append(time.perf_counter() - t)
        assert rc == D.DG_OK, L.dg_last_error(sm._h)
    t_e2e = float(np.mean(e2e))

    # ---- phase profile of one extra solve (not timed) ----
    sm.set_option("profile", 1)
    prof = sm.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
    sm.set_option("profile", 0)
    del sm
    torch.cuda.empty_cache()

    # ---- plain FP64 path ----
    sf = _solver(n, r, c, v, b, part, precision=0)
    for _ in range(1):
        sf.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    f0.record(stream)
    for _ in range(args.fp64_steps):
        stf = sf.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
    f1.record(stream)
    torch.cuda.synchronize()
    t_fp64 = f0.elapsed_time(f1) * 1e-3 / args.fp64_steps
    x64 = xd.cpu().numpy()
    err_mixed_vs_fp64 = float(np.linalg.norm(x_mixed - x64) / np.linalg.norm(x64))
    del sf
    torch.cuda.empty_cache()
    small = None
    if not args.no_small:
        try:
            small = run_small(args, max(args.steps, 3), max(args.warmup, 3))
        except Exception as ex:
            small = {"error": repr(ex)}
    batched = None
    if not args.no_batched:
        try:
            batched = run_batched(args, args.steps, args.warmup)
        except Exception as ex:  # reported in the line; the headline stands on its own
            batched = {"error": repr(ex)}
    adjoint = None
    if not args.no_adjoint:
        try:
            adjoint = run_adjoint(args, 0)
        except Exception as ex:
            adjoint = {"error": repr(ex)}
    elasticity = None
    if not args.no_elasticity:
        try:
            elasticity = run_elasticity(args, 1, 1)
        except Exception as ex:
            elasticity = {"error": repr(ex)}

    if rank != 0:
        return 0
    hbm, peak_kind = _peaks()
    # roofline of the dominant kernel group: the subdomain triangular solves
    # (multifrontal forward + backward over all levels), HBM-bound
    per_solve_s = prof.t_subsolve_s / max(prof.iterations, 1)
    achieved = prof.subsolve_bytes / per_solve_s / 1e9 if per_solve_s > 0 else None
    roofline = {"kernel": "mf_fwd_small+mf_fwd_big+mf_bwd_big+mf_bwd_small (FP32 subdomain solves, all levels)",
                "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None,
                # DRAM bytes (read + write) of the group per application, from one
                # ncu capture of this workload (dram__bytes_read.sum + dram__bytes_write.sum
                # summed over one iteration's subdomain-solve launches)
                "traffic": SUBSOLVE_TRAFFIC_BYTES,
                "peak_source": f"{peak_kind} hbm_gbs",
                "bytes_per_launch_group": prof.subsolve_bytes, "launch_group_s": per_solve_s}
    phases = {"factor_s": prof.t_factor_s, "iterate_s": prof.t_iterate_s,
              "subsolve_s": prof.t_subsolve_s, "coarse_s": prof.t_coarse_s, "spmv_s": prof.t_spmv_s,
              "spmv_GBps": (prof.spmv_bytes * prof.iterations / prof.t_spmv_s / 1e9) if prof.t_spmv_s else None}
    cpu = None
    vs_oracle = None
    if not args.no_cpu_baseline:
        threads = host_threads()
        times, ores, info = oracle_whole_run(n, r, c, v, b, part, threads, 1, 0)
        cpu = {"value": times[0], "unit": "s", "cores": threads, "kind": "port",
               "sample": _oracle_sample(threads, info), "detail": info}
        xo = ores["x"]
        vs_oracle = {"fp64_rel_err": float(np.linalg.norm(x64 - xo) / np.linalg.norm(xo)),
                     "fp64_iterations": stf.iterations,
                     "mixed_rel_err": float(np.linalg.norm(x_mixed - xo) / np.linalg.norm(xo)),
                     "mixed_iterations": last.iterations, "oracle_iterations": ores["iterations"]}
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": t_mixed, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 outer / f32 subdomain factors",
        "data": "synthetic (seeded generator, doug_gb300/problems.py)",
        "config": _config(n, len(v), last.nsubdomains, last.ncoarse),
        "parallelism": "replicas" if world > 1 else "1 GPU",
        "iterations": last.iterations, "true_rel_residual": last.true_rel_residual,
        "vs_oracle": vs_oracle,
        "fp64_s": t_fp64, "fp64_iterations": stf.iterations, "mixed_vs_fp64": t_mixed / t_fp64,
        "mixed_rel_err_vs_fp64_solution": err_mixed_vs_fp64,
        "setup_host_s": setup_s, "setup_phases": setup_phases, "phases_mixed": phases,
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "api": "dg_solve (host buffers, pinned)"},
        "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": int(launches),
        "small": small,
        "batched": batched,
        "elasticity": elasticity,
        "adjoint": adjoint,
    }
    print(json.dumps(line), flush=True)
    return 0


BATCH_SYSTEMS = 256
BATCH_CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1,
                 strong1="0.08", radius1=2, solve_tolerance=TOL, solve_maxiters=2000)
BATCH_WORKLOAD = ("256 independent jittered 2-D P1 Poisson systems, unknowns log-uniform in [2k, 200k] "
                  "(seeded), each with its own two-level additive Schwarz (its own aggregation, "
                  "coarse-aggregate subdomains with overlap 1, smoothed-aggregation coarse grid), all "
                  "solved in one batch")


SMALL_NODES = 129
SMALL_CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08",
                 radius1=2, solve_tolerance=TOL, solve_maxiters=1000, omega=repr(2.0 / 3.0))
SMALL_WORKLOAD = ("2-D P1 Poisson on a 129x129 jittered node grid (16,129 unknowns), 4 subdomains (2x2 quadrants, "
                  "imported), overlap 1, smoothed-aggregation coarse grid with omega 2/3")


def run_small(args, steps, warmup):
    """The small plain case: the whole solve on the GPU (FP64 and mixed) and
    the oracle's whole setup + solve on one host core beside it."""
    import torch
    import doug_gb300 as D
    from doug_gb300 import problems as P

    D.build_library()
    n, r, c, v, b, xy = P.poisson2d_p1(SMALL_NODES, seed=SEED)
    part = (1 + (xy[:, 0] >= 0.5) * 2 + (xy[:, 1] >= 0.5)).astype(np.int32)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    xd = torch.empty_like(bd)
    out = {"config": {"workload": SMALL_WORKLOAD, "n": n, "nnz": int(len(v)), "subdomains": 4,
                      "controls": SMALL_CTL}}
    xs = {}
    for prec, key in ((0, "fp64"), (1, "mixed")):
        s = D.DougSolver(SMALL_CTL)
        s.set_option("precision", prec)
        s.set_matrix_coo(n, r, c, v)
        s.set_rhs(b)
        s.set_partition(part)
        t0 = time.perf_counter()
        s.setup()
        setup_s = time.perf_counter() - t0
        for _ in range(warmup):
            st = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            st = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        xs[key] = xd.cpu().numpy()
        out[key] = {"solve_s": e0.elapsed_time(e1) * 1e-3 / steps, "iterations": st.iterations,
                    "true_rel_residual": st.true_rel_residual, "setup_host_s": setup_s}
        del s
    out["mixed_rel_err_vs_fp64_solution"] = float(np.linalg.norm(xs["mixed"] - xs["fp64"]) / np.linalg.norm(xs["fp64"]))
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        ctl = "".join(f"{k} {v_}\n" for k, v_ in SMALL_CTL.items())
        t0 = time.perf_counter()
        ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, part=part)
        wall = time.perf_counter() - t0
        out["cpu_reference_port"] = {"value": wall, "unit": "s", "cores": 1, "kind": "port",
                                     "sample": "the whole workload: the oracle's setup, exact subdomain and "
                                               "coarse factorisations and PCG to 1e-8, one host core",
                                     "iterations": ro["iterations"], "setup_s": ro["t_setup"],
                                     "factor_s": ro["t_factor"], "solve_s": ro["t_solve"],
                                     "gpu_fp64_rel_err_vs_oracle": float(np.linalg.norm(xs["fp64"] - ro["x"]) /
                                                                         np.linalg.norm(ro["x"]))}
    return out


def _batched_vs_oracle(systems, x64, xmixed, gpu_iters, sample=8):
    """The oracle's own solve of a seeded sample of the systems (the smallest,
    the largest and six drawn at random), each against its slice of the GPU
    batch: FP64 and mixed relative errors and FP64 iteration counts."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    ns = np.array([t[0] for t in systems])
    rng = np.random.default_rng(1)
    pick = sorted(set([int(ns.argmin()), int(ns.argmax())]
                      + [int(i) for i in rng.choice(len(systems), sample, replace=False)]))[:sample]
    O.set_threads(host_threads())
    rows = []
    try:
        for i in pick:
            n, r, c, v, b = systems[i]
            ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(BATCH_CTL))
            xo = ro["x"]
            rows.append({"system": i, "n": int(n), "oracle_iterations": ro["iterations"],
                         "fp64_iterations": int(gpu_iters[i]),
                         "fp64_rel_err": float(np.linalg.norm(x64[i] - xo) / np.linalg.norm(xo)),
                         "mixed_rel_err": float(np.linalg.norm(xmixed[i] - xo) / np.linalg.norm(xo))})
    finally:
        O.set_threads(1)
    return {"systems": rows, "fp64_rel_err_max": max(r["fp64_rel_err"] for r in rows),
            "mixed_rel_err_max": max(r["mixed_rel_err"] for r in rows),
            "iterations_max_diff": max(abs(r["oracle_iterations"] - r["fp64_iterations"]) for r in rows)}


def run_batched(args, steps, warmup):
    """The batched uneven-systems workload: every step solves all systems
    (factorisations + per-system PCG to 1e-8) from right-hand sides in HBM."""
    import torch
    import doug_gb300 as D
    from doug_gb300 import problems as P

    D.build_library()
    systems = P.batched_poisson2d_p1(BATCH_SYSTEMS, seed=SEED)
    ns = np.array([t[0] for t in systems])
    b = np.concatenate([t[4] for t in systems])
    n = int(ns.sum())
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    xd = torch.empty_like(bd)
    out = {}
    for prec in (1, 0):
        s = D.DougSolver(BATCH_CTL)
        s.set_option("precision", prec)
        s.set_systems([t[:4] for t in systems], [t[4] for t in systems])
        t0 = time.perf_counter()
        s.setup()
        setup_s = time.perf_counter() - t0
        for _ in range(warmup if prec == 1 else 1):
            s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        k = steps if prec == 1 else 1
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches = 0
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            st = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
            launches += st.gpu_launches
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3 / k
        ss = s.system_stats()
        sec = ss["seconds"].copy()
        s.set_option("profile", 1)  # phase split of one extra solve (not timed)
        pr = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        s.set_option("profile", 0)
        res = {"batch_s": t, "solves_per_s": BATCH_SYSTEMS / t, "setup_host_s": setup_s,
               "p50_system_s": float(np.percentile(sec, 50)), "p99_system_s": float(np.percentile(sec, 99)),
               "iterations_max": int(ss["iterations"].max()),
               "iterations_p50": float(np.median(ss["iterations"])),
               "worst_true_rel_residual": float(ss["rel_residual"].max()),
               "all_converged": bool(np.all(ss["status"] == D.DG_OK)), "gpu_launches": int(launches // k),
               "phases": {"factor_s": pr.t_factor_s, "iterate_s": pr.t_iterate_s, "subsolve_s": pr.t_subsolve_s,
                          "coarse_s": pr.t_coarse_s, "spmv_s": pr.t_spmv_s,
                          "subsolve_GBps": pr.subsolve_bytes * pr.iterations / pr.t_subsolve_s / 1e9
                          if pr.t_subsolve_s else None}}
        if prec == 1:
            x_mixed = xd.cpu().numpy()
            # end to end through dg_solve (pinned host buffers)
            bh = torch.tensor(b, dtype=torch.float64).pin_memory()
            xh = torch.empty(n, dtype=torch.float64).pin_memory()
            import ctypes
            L = D.load_library()
            stats = D._Stats()
            e2e = []
            for _ in range(k):
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                rc = L.dg_solve(s._h, ctypes.cast(bh.data_ptr(), ctypes.POINTER(ctypes.c_double)),
                                ctypes.cast(xh.data_ptr(), ctypes.POINTER(ctypes.c_double)), ctypes.byref(stats))
                e2e.append(time.perf_counter() - t1)
                assert rc == D.DG_OK, L.dg_last_error(s._h)
            res["e2e"] = {"value": BATCH_SYSTEMS / float(np.mean(e2e)), "unit": "solves/s",
                          "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n}
            sz = s.sizes()
            out["config"] = {"workload": BATCH_WORKLOAD, "systems": BATCH_SYSTEMS, "n_total": n,
                             "n_min": int(ns.min()), "n_median": float(np.median(ns)), "n_max": int(ns.max()),
                             "subdomains": sz["nsubdomains"], "coarse_unknowns": sz["nagr_fine"],
                             "controls": BATCH_CTL}
            out["mixed"] = res
        else:
            x64 = xd.cpu().numpy()
            out["fp64"] = res
            err = [np.linalg.norm(a - c) / np.linalg.norm(c) for a, c in zip(s.split(x_mixed), s.split(x64))]
            out["mixed_rel_err_vs_fp64_solution_max"] = float(max(err))
            if not args.no_cpu_baseline:
                out["vs_oracle"] = _batched_vs_oracle(systems, s.split(x64), s.split(x_mixed), ss["iterations"])
        del s
        torch.cuda.empty_cache()
    out["mixed_vs_fp64"] = out["mixed"]["batch_s"] / out["fp64"]["batch_s"]
    return out


ELAS_N = 64
ELAS_CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08",
                radius1=2, maxasize1=100, solve_tolerance=TOL, solve_maxiters=5000)
ELAS_WORKLOAD = ("3-D linear elasticity, P1 tetrahedra: 64^3 hexes x 6 tets (1,572,864 elements, 12x12 element "
                 "matrices), nodes jittered +-0.15h, E = 1 with 20 seeded boxes of E = 1e3, nu = 0.3, bottom "
                 "face clamped, body force (0,0,-1): 811,200 freedoms; elemental input; 128 box subdomains "
                 "(4x4x8), overlap 1, smoothed-aggregation coarse grid over 3x3 nodal blocks with the six "
                 "rigid-body modes as near-nullspace (coarse_method 3; *_scalar_coarse: the reference's scalar "
                 "aggregation)")


def run_elasticity(args, steps, warmup):
    """The elemental elasticity workload: mixed and FP64 solves with the
    assembled products, and the mixed solve with the matrix-free element
    products (elemental_matvec 1); every step is a full solve from the
    element right-hand side in HBM."""
    import torch
    import doug_gb300 as D
    from doug_gb300 import problems as P

    D.build_library()
    ngf, eptr, efree, emat, erhs, info = P.elasticity3d_p1_elements(ELAS_N, seed=SEED)
    part = P.dof_box_partition(info["node_ijk"], ELAS_N)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    out = {"config": {"workload": ELAS_WORKLOAD, "n": int(ngf), "elements": int(len(eptr) - 1),
                      "element_values": int(len(emat)), "controls": ELAS_CTL}}
    xs = {}
    # the configuration's coarse space: smoothed aggregation over 3x3 nodal
    # blocks with the rigid-body near-nullspace (coarse_method 3); the
    # reference's scalar aggregation (coarse_method 1) beside it
    runs = (("mixed", 1, 0, 3), ("fp64", 0, 0, 3), ("mixed_matrix_free", 1, 1, 3),
            ("mixed_scalar_coarse", 1, 0, 1), ("fp64_scalar_coarse", 0, 0, 1))
    for name, prec, emv, cm in runs:
        s = D.DougSolver(dict(ELAS_CTL, coarse_method=cm))
        s.set_option("precision", prec)
        s.set_option("elemental_matvec", emv)
        s.set_elements(ngf, eptr, efree, emat, erhs)
        if cm == 3:  # smoothed aggregation over nodal blocks with rigid-body modes
            s.set_node_geometry(info["coords"], info["freemap"])
        s.set_partition(part)
        t0 = time.perf_counter()
        s.setup()
        setup_s = time.perf_counter() - t0
        b = s.input_matrix()[4]
        bd = torch.tensor(b, dtype=torch.float64, device="cuda")
        xd = torch.empty_like(bd)
        k = steps if name == "mixed" else 1
        for _ in range(warmup if name == "mixed" else 1):
            s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            st = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3 / k
        s.set_option("profile", 1)
        pr = s.solve_device(bd.data_ptr(), xd.data_ptr(), sptr)
        s.set_option("profile", 0)
        xs[name] = xd.cpu().numpy()
        res = {"solve_s": t, "iterations": st.iterations, "true_rel_residual": st.true_rel_residual,
               "setup_host_s": setup_s, "gpu_launches": st.gpu_launches, "coarse_unknowns": st.ncoarse,
               "phases": {"factor_s": pr.t_factor_s, "iterate_s": pr.t_iterate_s, "subsolve_s": pr.t_subsolve_s,
                          "coarse_s": pr.t_coarse_s, "product_s": pr.t_spmv_s,
                          "product_ms_per_iteration": 1e3 * pr.t_spmv_s / max(pr.iterations, 1)}}
        if name == "mixed":
            sz = s.sizes()
            out["config"].update({"nnz": int(len(s.input_matrix()[3])), "subdomains": sz["nsubdomains"],
                                  "coarse_unknowns": int(st.ncoarse), "node_aggregates": sz["nagr_fine"]})
        out[name] = res
        del s
        torch.cuda.empty_cache()
    x64 = xs["fp64"]
    for name in ("mixed", "mixed_matrix_free", "mixed_scalar_coarse", "fp64_scalar_coarse"):
        out[name]["rel_err_vs_fp64_solution"] = float(np.linalg.norm(xs[name] - x64) / np.linalg.norm(x64))
    out["mixed_vs_fp64"] = out["mixed"]["solve_s"] / out["fp64"]["solve_s"]
    out["scalar_coarse_vs_rigid_body"] = out["mixed_scalar_coarse"]["solve_s"] / out["mixed"]["solve_s"]
    return out


ADJ_NODES = 513
ADJ_RHS = 32
ADJ_CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08",
               radius1=2, solve_tolerance="1.0e-10", solve_maxiters=3000)
ADJ_WORKLOAD = ("2-D P1 diffusion on a 513x513 jittered node grid (261,121 unknowns, 524,288 triangles), one "
                "conductivity per element (log-normal, sigma 0.5), 32 right-hand sides U[-1,1], loss "
                "sum ||x - x_target||^2 with x_target from the conductivities perturbed by 10 %; mixed-precision "
                "PCG to 1e-10, adjoint gradients dL/dkappa and dL/db")


def run_adjoint(args, fd_elements):
    """Forward solve of the 32 right-hand sides and the adjoint backward pass
    (doug_gb300.autograd.element_solve); optional central finite differences
    of the loss on seeded elements (each two full forward solves, FP64 to 1e-12)."""
    import torch
    import doug_gb300 as D
    from doug_gb300 import problems as P
    from doug_gb300.autograd import element_solve

    D.build_library()
    rng = np.random.default_rng(SEED + 4)
    ntri = 2 * (ADJ_NODES - 1) ** 2
    kappa = np.exp(0.5 * rng.standard_normal(ntri))
    ngf, eptr, efree, Kb, erhs, _ = P.poisson2d_p1_elements(nodes=ADJ_NODES, seed=SEED + 4)
    B = torch.tensor(rng.uniform(-1.0, 1.0, (ngf, ADJ_RHS)), device="cuda")
    k_target = kappa * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, ntri))
    s = D.DougSolver(ADJ_CTL)
    s.set_option("precision", 1)
    with torch.no_grad():
        Xt = element_solve(s, ngf, eptr, efree, Kb, erhs, torch.tensor(k_target), B).detach()
    # one untimed forward + backward pass (first use of the torch kernels of the loss)
    kw = torch.tensor(kappa, requires_grad=True)
    ((element_solve(s, ngf, eptr, efree, Kb, erhs, kw, B) - Xt) ** 2).sum().backward()
    k = torch.tensor(kappa, requires_grad=True)
    bt = B.clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    X = element_solve(s, ngf, eptr, efree, Kb, erhs, k, bt)
    L = ((X - Xt) ** 2).sum()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    g = k.grad.numpy().copy()
    out = {"config": {"workload": ADJ_WORKLOAD, "n": int(ngf), "elements": ntri, "rhs": ADJ_RHS,
                      "controls": ADJ_CTL},
           "forward_s": t1 - t0, "backward_s": t2 - t1, "loss": float(L.item()),
           "note": "forward = element assembly + host setup + numeric factorisations + 32 PCG solves; "
                   "backward = 32 adjoint solves with the kept factors + dg_grad_elements"}
    if fd_elements:
        sf = D.DougSolver(dict(ADJ_CTL, solve_tolerance="1.0e-12"))
        sf.set_option("precision", 0)

        def loss(kap):
            with torch.no_grad():
                Xk = element_solve(sf, ngf, eptr, efree, Kb, erhs, torch.tensor(kap), B)
                return float(((Xk - Xt) ** 2).sum().item())

        sel = rng.choice(ntri, fd_elements, replace=False)
        errs = []
        gmax = float(np.abs(g).max())
        for e in sel:
            h = 1e-4 * kappa[e]
            kp, km = kappa.copy(), kappa.copy()
            kp[e] += h
            km[e] -= h
            fd = (loss(kp) - loss(km)) / (2 * h)
            errs.append(abs(fd - g[e]) / max(gmax, 1e-300))
        out["fd_elements"] = int(fd_elements)
        out["fd_max_err_rel_to_max_grad"] = float(max(errs))
    return out


def run_profile_solve(args):
    """One solve of the workload (grid args.grid^3) inside a
    cudaProfilerStart/Stop range, after one warm-up solve: the command the
    kernel summaries are captured from (`ncu --profile-from-start off`)."""
    import torch
    import doug_gb300 as D

    D.build_library()
    torch.cuda.set_device(0)
    if args.workload == "elasticity":
        from doug_gb300 import problems as P
        ngf, eptr, efree, emat, erhs, info = P.elasticity3d_p1_elements(args.grid, seed=SEED)
        s = D.DougSolver(ELAS_CTL)
        s.set_option("precision", args.precision)
        s.set_option("elemental_matvec", 1)
        s.set_elements(ngf, eptr, efree, emat, erhs)
        s.set_partition(P.dof_box_partition(info["node_ijk"], args.grid))
        s.setup()
        b = s.input_matrix()[4]
        n = b.shape[0]
    elif args.workload == "batched":
        from doug_gb300 import problems as P
        systems = P.batched_poisson2d_p1(BATCH_SYSTEMS, seed=SEED)
        b = np.concatenate([t[4] for t in systems])
        n = b.shape[0]
        s = D.DougSolver(BATCH_CTL)
        s.set_option("precision", args.precision)
        s.set_systems([t[:4] for t in systems], [t[4] for t in systems])
        s.setup()
    else:
        n, r, c, v, b, part = _problem(args.grid)
        if args.ctl:  # control-word overrides (e.g. fine_method=0 levels=1: the SpMV alone)
            s = D.DougSolver(dict(CTL, **dict(kv.split("=", 1) for kv in args.ctl)))
            s.set_option("precision", args.precision)
            s.set_matrix_coo(n, r, c, v)
            s.set_rhs(b)
            s.set_partition(part)
            s.setup()
        else:
            s = _solver(n, r, c, v, b, part, precision=args.precision)
    stream = torch.cuda.current_stream()
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    xd = torch.empty_like(bd)
    s.solve_device(bd.data_ptr(), xd.data_ptr(), stream.cuda_stream, allow_not_converged=bool(args.ctl))
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    st = s.solve_device(bd.data_ptr(), xd.data_ptr(), stream.cuda_stream, allow_not_converged=bool(args.ctl))
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"grid": args.grid, "n": n, "precision": args.precision, "iterations": st.iterations,
                      "true_rel_residual": st.true_rel_residual, "gpu_launches": st.gpu_launches,
                      "t_factor_s": st.t_factor_s, "t_iterate_s": st.t_iterate_s}), flush=True)
    return 0 if (args.ctl or st.true_rel_residual < 1e-7) else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched uneven-systems workload")
    ap.add_argument("--no-small", action="store_true", help="skip the small 129x129 P1 workload")
    ap.add_argument("--no-elasticity", action="store_true", help="skip the elemental elasticity workload")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiation workload")
    ap.add_argument("--fd-elements", type=int, default=50, help="finite-difference checks of --workload adjoint")
    ap.add_argument("--workload", default="diffusion128",
                    choices=["diffusion128", "batched", "elasticity", "adjoint"],
                    help="batched / elasticity / adjoint: print only that workload's line")
    ap.add_argument("--profile-solve", action="store_true",
                    help="one solve inside a profiler range (for ncu), no timing line")
    ap.add_argument("--grid", type=int, default=N, help="grid size of --profile-solve")
    ap.add_argument("--precision", type=int, default=1, help="precision of --profile-solve")
    ap.add_argument("--ctl", action="append", default=[], metavar="WORD=VALUE",
                    help="control-word override of --profile-solve (repeatable)")
    args = ap.parse_args()
    if args.profile_solve:
        return run_profile_solve(args)
    if args.workload == "adjoint" and args.impl == "gb300" and not args.profile_solve:
        import torch
        torch.cuda.set_device(0)
        with ClockSampler(0) as clk:
            ad = run_adjoint(args, args.fd_elements)
        print(json.dumps({"metric": "forward + adjoint time (s), 32 right-hand sides, 1 GB300",
                          "value": ad["forward_s"] + ad["backward_s"], "unit": "s", "n_gpus": 1, "steps": 1,
                          "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64 outer / f32 subdomain factors",
                          "data": "synthetic (seeded generator, doug_gb300/problems.py)",
                          "config": ad["config"], "adjoint": ad, "clocks": clk.summary()}), flush=True)
        return 0
    if args.workload == "elasticity" and args.impl == "gb300" and not args.profile_solve:
        import torch
        torch.cuda.set_device(0)
        with ClockSampler(0) as clk:
            el = run_elasticity(args, args.steps, args.warmup)
        m = el["mixed"]
        print(json.dumps({"metric": "time to rel. residual 1e-8 (s), elemental elasticity, 1 GB300",
                          "value": m["solve_s"], "unit": "s", "n_gpus": 1, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": m["solve_s"] * 1e3, "higher_is_better": False,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64 outer / f32 subdomain factors",
                          "data": "synthetic (seeded generator, doug_gb300/problems.py)",
                          "config": el["config"], "elasticity": el, "clocks": clk.summary()}), flush=True)
        return 0
    if args.workload == "batched" and args.impl == "gb300" and not args.profile_solve:
        import torch
        torch.cuda.set_device(0)
        with ClockSampler(0) as clk:
            bt = run_batched(args, args.steps, args.warmup)
        m = bt["mixed"]
        print(json.dumps({"metric": "aggregate solves/s, 256 uneven systems to rel. residual 1e-8, 1 GB300",
                          "value": m["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": m["batch_s"] * 1e3, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64 outer / f32 subdomain factors",
                          "data": "synthetic (seeded generator, doug_gb300/problems.py)",
                          "config": bt["config"], "batched": bt, "e2e": m["e2e"], "clocks": clk.summary(),
                          "gpu_launches": m["gpu_launches"] * args.steps}), flush=True)
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if args.impl == "gb300":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
    else:
        rc = run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
