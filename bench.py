#!/usr/bin/env python
"""Benchmark of the two-scale Richards hot path on GB300.

Workload (default): the GPU-scale plain method -- 201 x 201 macro nodes
(80,000 triangles), a 21 x 21-node micro mesh per cell with per-cell
inclusion size U(0.3, 0.7), N = 35,320,401 FP64 unknowns, EXPREM with
tol 1e-6 and Krylov dimension <= 40 (seeded synthetic inputs; the reference
publishes no dataset).

A step is one accepted EXPREM step (the unit of the reference's driver loop,
src/main.cpp:313-341): a G evaluation at the new state, m finite-difference
Jacobian-vector products, modified Gram-Schmidt, phi_1(dt H_m) on the host
and the update.  The metric is the reference's own instrument -- right-hand-
side evaluations per second (FuncEvals / runtime, src/main.cpp:350-351) --
over the timed steps.

  value  device-resident stepping (u, G(u) and the Krylov basis in HBM);
  e2e    the reference-facing call exprem(...) with u0 in (pinned) host
         memory, copied in and out on every step (tsr_exprem_step).

--impl reference times the CPU implementation of the same path on the host
cores: the oracle's OpenMP form of Gfunc_parallel and its EXPREM step (C
library log/exp) over the same workload, whose geometry the oracle's own
mesh preprocessing builds, so that arm loads nothing of the GB300 library
(the reference's own Gfunc_parallel and exprem sources are not in its tree).

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORLD = int(os.environ.get("WORLD_SIZE", "1"))
RANK = int(os.environ.get("RANK", "0"))
GS = {"mgs": 0, "cgs2": 1}          # Arnoldi orthogonalisation variants (tsr_set_gram_schmidt)
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1:
    # one GPU per rank: the library's CUDA runtime sees only this rank's GPU
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

import ctypes as C  # noqa: E402

import numpy as np  # noqa: E402

METRIC = "G-evals/s (EXPREM FuncEvals per second)"
UNIT = "G-evals/s"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            if vis is not None and vis.isdigit() and f[0] != vis:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                   "reasons": sorted(reasons), "samples": len(sm)}
        return out


def dist_init():
    if WORLD == 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def make_problem(args, lib=None):
    """The workload; lib: the mesh preprocessing that builds its geometry
    (None: the GB300 library's; the CPU arm passes the oracle's)."""
    from twoscalerich_gb300 import problem as P
    if args.config == 4:
        p = P.config4(scenarios=args.scenarios, n_macro=args.n_macro, n_micro=args.n_micro, lib=lib)
    elif args.config == 3:
        p = P.config3(n_macro=args.n_macro, lib=lib)
    else:
        p = P.config2(n_macro=args.n_macro, n_micro=args.n_micro, lib=lib)
    p.options.MaxKrylov = args.max_krylov
    return p


def l2_statement(args, N):
    """No L2 flush: each step streams the Krylov basis and state vectors,
    a working set far above the 129 MB L2 at the benchmark sizes."""
    vec = N * 8 / 1e6
    ws = vec * (7 + 1 + 5)
    head = "inputs larger than L2" if ws > 129.0 else "working set within L2 (small case, no flush)"
    return ("%s: one unknown vector is %.0f MB; an EXPREM step streams the Krylov basis and 5 state "
            "vectors, %.0f MB at Krylov dimension 7 (L2 129 MB)" % (head, vec, ws))


def workload(args, N):
    w = _workload(args, N)
    w["orthogonalisation"] = {"mgs": "modified Gram-Schmidt", "cgs2": "classical Gram-Schmidt twice"}[args.gs]
    return w


def _workload(args, N):
    if args.config == 4:
        return {"workload": "two-scale Richards ensemble, independent EXPREM per scenario",
                "scenarios": args.scenarios,
                "macro_nodes": "%dx%d per scenario" % (args.n_macro, args.n_macro),
                "micro_nodes_per_cell": "%dx%d" % (args.n_micro, args.n_micro),
                "cells": args.scenarios * 2 * (args.n_macro - 1) ** 2, "unknowns": N,
                "max_krylov": args.max_krylov, "tol": 1e-6, "t_end_days": 1.0,
                "per_scenario": "Ks_A ~ LogNormal(ln 0.054, 0.5), Ks_B ~ LogNormal(ln 0.001, 0.5), "
                                "alpha_A ~ U(1.5, 4), n_A ~ U(1.8, 2.6), h0 ~ U(-10, -1) m",
                "inputs_vs_l2": l2_statement(args, N),
                "parallelism": "replicas" if WORLD > 1 else "1 GPU", "packing": "autotuned"}
    if args.config == 3:
        return {"workload": "two-scale Richards, batched uneven micro meshes, EXPREM steps",
                "macro_nodes": "%dx%d" % (args.n_macro, args.n_macro),
                "micro_nodes_per_cell": "5..41 per side (p .30/.25/.20/.12/.08/.05), square or disk",
                "cells": 2 * (args.n_macro - 1) ** 2, "unknowns": N,
                "max_krylov": args.max_krylov, "tol": 1e-6,
                "inputs_vs_l2": l2_statement(args, N),
                "parallelism": "replicas" if WORLD > 1 else "1 GPU", "packing": "autotuned"}
    return {"workload": "two-scale Richards, plain method, EXPREM steps",
            "macro_nodes": "%dx%d" % (args.n_macro, args.n_macro),
            "micro_nodes_per_cell": "%dx%d" % (args.n_micro, args.n_micro),
            "cells": 2 * (args.n_macro - 1) ** 2, "unknowns": N, "max_krylov": args.max_krylov,
            "tol": 1e-6, "inputs_vs_l2": l2_statement(args, N),
            "parallelism": "replicas" if WORLD > 1 else "1 GPU"}


def cell_plan(lib, h):
    """The cell kernel's plan after autotuning."""
    from twoscalerich_gb300 import capi
    out = (C.c_int * 6)()
    capi.check(lib.tsr_cell_plan(h, out), "tsr_cell_plan")
    return {"tables_in_shared_memory": bool(out[2]), "cells_per_bundle_max": out[3], "grid": out[4],
            "smem_per_cta": out[5]}


def repo_libraries():
    """Shared libraries of this repository mapped into the process (Linux)."""
    found = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if line.strip() else ""
                if path.endswith(".so") and path.startswith(ROOT):
                    found.add(os.path.relpath(path, ROOT))
    except OSError:
        return None
    return sorted(found)


def cpu_exprem_rate(p, u, t, stats, threads, min_seconds=10.0, min_steps=2):
    """G evaluations per second of the oracle's OpenMP EXPREM (C-library
    log/exp) stepping the workload on from state u at time t with the step
    size in stats: at least min_steps accepted steps and min_seconds of work
    (the first step evaluates G(u) once more, as any restart does)."""
    import oracle
    from twoscalerich_gb300 import capi
    o = oracle.Oracle(p, nthreads=threads, libm=True)
    u = np.array(u, dtype=np.float64)
    st = capi.ExpremStats()
    C.memmove(C.byref(st), C.byref(stats), C.sizeof(st))
    tspan = np.array([0.0])
    solns = np.zeros(1)
    ev0, n0 = st.FuncEvals, st.NumSteps
    t0 = time.perf_counter()
    while st.NumSteps - n0 < min_steps or time.perf_counter() - t0 < min_seconds:
        t = o.exprem_step(t, u, tspan, solns, p.options, st)
        if t >= p.tend:
            break
    el = time.perf_counter() - t0
    o.close()
    return (st.FuncEvals - ev0) / el, el, st.NumSteps - n0, st.FuncEvals - ev0


def run_reference(args):
    """CPU arm: the oracle's OpenMP EXPREM (Gfunc_parallel form, C-library
    log/exp) on all host cores over the same workload, geometry from the
    oracle's own mesh preprocessing.  Like the GPU arm, W untimed accepted
    steps from t = 0, then K timed accepted steps; value = G evaluations per
    second over the timed steps.  Ensembles (config 4): each step advances
    the first 8 scenarios by one accepted step each."""
    if RANK != 0:
        return
    import oracle
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    threads = os.cpu_count() or 1
    meshlib = oracle.MeshLib(libm=True)
    if args.config == 4:
        ens = make_problem(args, lib=meshlib)
        probs = [P.scenario_problem(ens, s, lib=meshlib) for s in range(min(8, ens.S))]
    else:
        probs = [make_problem(args, lib=meshlib)]
    runs = []
    for p in probs:
        runs.append(dict(o=oracle.Oracle(p, nthreads=threads, libm=True), p=p, u=p.u0.copy(),
                         st=capi.ExpremStats(), t=0.0))
    tspan = np.array([0.0])
    solns = np.zeros(1)

    def step():
        for r in runs:
            if r["t"] < r["p"].tend:
                r["t"] = r["o"].exprem_step(r["t"], r["u"], tspan, solns, r["p"].options, r["st"])
    for _ in range(args.warmup):
        step()
    ev0 = sum(r["st"].FuncEvals for r in runs)
    n0 = sum(r["st"].NumSteps for r in runs)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    total = time.perf_counter() - t0
    evals = sum(r["st"].FuncEvals for r in runs) - ev0
    nsteps = sum(r["st"].NumSteps for r in runs) - n0
    if args.config == 4:
        metric, unit, value = ("scenario-steps/s (accepted EXPREM steps summed over scenarios per second)",
                               "scenario-steps/s", nsteps / total)
        sample = ("%d scenario-steps (scenarios 0-%d of the ensemble, one accepted step each per "
                  "step, after %d warm-up steps)" % (nsteps, len(runs) - 1, args.warmup))
    else:
        metric, unit, value = METRIC, UNIT, evals / total
        sample = ("%d accepted EXPREM steps (%d G evaluations) of the full workload after %d "
                  "warm-up steps from t = 0, Krylov dimensions %s"
                  % (nsteps, evals, args.warmup, [r["st"].CurrentKryDim for r in runs]))
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload(args, probs[0].N if args.config != 4 else ens.N),
        "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port",
                         "sample": sample + "; the oracle's OpenMP Gfunc_parallel form and EXPREM "
                                            "with C-library log/exp, geometry from the oracle's "
                                            "own mesh preprocessing"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "krylov_steps_per_s": nsteps / total,
        "repo_libraries_loaded": repo_libraries(),
    }
    print(json.dumps(line))


def run_ours(args):
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    dist = dist_init()
    lib = capi.load()
    p = make_problem(args)
    N = p.N
    ctx = P.Context(p, max_krylov=p.options.MaxKrylov, gram_schmidt=GS[args.gs])
    h = ctx.h
    tuned = ctx.autotune(p.u0, reps=2)     # packing and block size of the cell kernel
    fp64_peak = C.c_double()
    capi.check(lib.tsr_fp64_peak(C.byref(fp64_peak)), "tsr_fp64_peak")
    opts = p.options
    st = capi.ExpremStats()
    ns = int(p.tspan[0])
    solns = np.zeros(1)   # the timed steps stay before the first saved time
    tspan = p.tspan.copy()
    tspan[0] = 0.0        # no dense output inside the benchmark
    capi.check(lib.tsr_exprem_load(h, capi.ptr(p.u0), 0.0), "tsr_exprem_load")
    t = C.c_double(0.0)

    def advance():
        capi.check(lib.tsr_exprem_advance(h, p.tend, capi.ptr(tspan), capi.ptr(solns),
                                          C.byref(opts), C.byref(st), C.byref(t)),
                   "tsr_exprem_advance")

    # timing events ride in the Arnoldi graphs only while profiling is on:
    # switch it on before the warm-up so that the graphs are captured there
    capi.check(lib.tsr_profile(h, 1), "profile")
    for _ in range(args.warmup):
        advance()
    ev0, steps0, krylov = st.FuncEvals, st.NumSteps, []
    clocks = Clocks()
    clocks.start()
    barrier(dist)
    capi.check(lib.tsr_sync(h), "sync")
    capi.check(lib.tsr_profile(h, 1), "profile")
    launches0 = lib.tsr_kernel_launches()
    capi.check(lib.tsr_mark(h, 0), "mark")
    for _ in range(args.steps):
        advance()
        krylov.append(st.CurrentKryDim)
    capi.check(lib.tsr_mark(h, 1), "mark")
    capi.check(lib.tsr_sync(h), "sync")
    launches = lib.tsr_kernel_launches() - launches0
    barrier(dist)
    clk = clocks.stop()
    ms = C.c_double()
    capi.check(lib.tsr_elapsed_ms(h, 0, 1, C.byref(ms)), "elapsed")
    evals = st.FuncEvals - ev0
    steps = st.NumSteps - steps0
    t_max = allmax(dist, ms.value / 1e3)
    value = allsum(dist, evals) / t_max
    # dominant kernel: the G / Jv evaluation (cell kernel + macro node kernel)
    gms, gcount, gbytes = C.c_double(), C.c_longlong(), C.c_double()
    capi.check(lib.tsr_profile_read(h, 0, C.byref(gms), C.byref(gcount), C.byref(gbytes)), "prof")
    sms, scount, sbytes = C.c_double(), C.c_longlong(), C.c_double()
    capi.check(lib.tsr_profile_read(h, 1, C.byref(sms), C.byref(scount), C.byref(sbytes)), "prof")
    capi.check(lib.tsr_profile(h, 0), "profile")
    hbm_peak, peak_src = measured_peaks()
    g_avg_ms = gms.value / max(gcount.value, 1)
    g_bytes = gbytes.value / max(gcount.value, 1)
    g_gbs = g_bytes / (g_avg_ms * 1e-3) / 1e9
    gs_gbs = sbytes.value / max(sms.value * 1e-3, 1e-30) / 1e9
    # FP64 instructions per G from the instruction counts of the cell
    # kernel (ncu, per unknown)
    fp64_per_unknown = FP64_OPS_PER_UNKNOWN.get(args.n_micro) if args.config == 2 else None
    fp64 = None
    if fp64_per_unknown:
        ach = fp64_per_unknown * N / (g_avg_ms * 1e-3)
        fp64 = {"achieved": ach / 1e9, "peak": fp64_peak.value / 1e9, "unit": "Gop/s",
                "frac": ach / fp64_peak.value, "peak_source": "measured live (DFMA chains)",
                "ops_per_G": fp64_per_unknown * N}

    # e2e: the reference-facing call with u0 in pinned host memory
    u_host = capi.PinnedArray(N)
    capi.check(lib.tsr_exprem_store(h, u_host.a.ctypes.data_as(capi.dp)), "store")
    te = C.c_double(t.value)
    st2 = capi.ExpremStats()
    C.memmove(C.byref(st2), C.byref(st), C.sizeof(st))

    def step_e2e():
        capi.check(lib.tsr_exprem_step(h, C.byref(te), p.tend, capi.ptr(tspan), capi.ptr(solns),
                                       u_host.a.ctypes.data_as(capi.dp), C.byref(opts),
                                       C.byref(st2)), "tsr_exprem_step")

    step_e2e()   # warm (first call after a store: the state is loaded again)
    e0 = st2.FuncEvals
    barrier(dist)
    capi.check(lib.tsr_sync(h), "sync")
    capi.check(lib.tsr_mark(h, 2), "mark")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    capi.check(lib.tsr_mark(h, 3), "mark")
    capi.check(lib.tsr_sync(h), "sync")
    wall_e2e = time.perf_counter() - t0
    barrier(dist)
    ms2 = C.c_double()
    capi.check(lib.tsr_elapsed_ms(h, 2, 3, C.byref(ms2)), "elapsed")
    e2e_t = allmax(dist, max(ms2.value / 1e3, wall_e2e))
    e2e_value = allsum(dist, st2.FuncEvals - e0) / e2e_t
    u_host.free()

    cpu = None
    if RANK == 0 and WORLD == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        u_now = np.empty(N)
        capi.check(lib.tsr_exprem_store(h, capi.ptr(u_now)), "store")
        rate, el, nst, nev = cpu_exprem_rate(p, u_now, te.value, st2, threads, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d accepted EXPREM steps (%d G evaluations) of the full workload by the "
                         "oracle's OpenMP EXPREM (Gfunc_parallel form, C-library log/exp), "
                         "continuing from the GPU's state after its timed steps (%.1f s)"
                         % (nst, nev, el)}
    traffic = G_TRAFFIC_PER_UNKNOWN.get(args.n_micro) if args.config == 2 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": WORLD, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator 20261203, evaluation seed 7)",
        "config": workload(args, N),
        "krylov_steps_per_s": allsum(dist, steps) / t_max,
        "dof_evals_per_s": value * N,
        "krylov_dims": krylov,
        "roofline": {"bound": "hbm", "kernel": "G / Jv evaluation (k_cells + k_macro_nodes)",
                     "achieved": g_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": g_gbs / hbm_peak, "peak_source": peak_src,
                     "traffic": None if traffic is None else traffic * N,
                     "algorithmic_bytes_per_launch": g_bytes, "avg_launch_ms": g_avg_ms,
                     "launches": gcount.value},
        "fp64_roofline": fp64,
        "gram_schmidt": {"achieved_gbs_algorithmic": gs_gbs, "peak": hbm_peak,
                         "frac": gs_gbs / hbm_peak, "ms_total": sms.value,
                         "share_of_step": sms.value / max(ms.value, 1e-30)},
        "g_share_of_step": gms.value / max(ms.value, 1e-30),
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * N,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": int(launches),
        "autotuned": None if tuned is None else dict({"g_ms": tuned[0], "threads": tuned[1],
                                                      "smem_budget": tuned[2]}, **cell_plan(lib, h)),
        "cpu_baseline": cpu,
    }
    if RANK == 0:
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def run_scale_to_end(args):
    """Configs 2/3 from t = 0 towards t_end through device-resident EXPREM
    steps, stopping at t_end or after --to-end-seconds of wall time, with
    what limited every step (tsr_step_diagnostics).  The CPU wall time to the
    same point is an ESTIMATE, labelled as such: the GPU run's G-evaluation
    count divided by the G-evals/s the oracle's OpenMP EXPREM (C-library
    log/exp) reaches on this machine stepping on from the GPU's final state (its
    trajectory is the GPU's: the bitwise oracle takes the same steps)."""
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    if RANK != 0:
        return
    lib = capi.load()
    p = make_problem(args)
    ctx = P.Context(p, max_krylov=p.options.MaxKrylov, gram_schmidt=GS[args.gs])
    h = ctx.h
    ctx.autotune(p.u0, reps=2)
    tspan = p.tspan.copy()
    ns = int(tspan[0])
    solns = np.zeros((ns + 1) * p.N)
    solns[:p.N] = p.u0
    capi.check(lib.tsr_set_calibrated_output(h, 1), "calibrated output")
    capi.check(lib.tsr_exprem_load(h, capi.ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    t = C.c_double(0.0)
    diag = np.zeros(8)
    log = []
    clocks = Clocks()
    clocks.start()
    capi.check(lib.tsr_sync(h), "sync")
    w0 = time.perf_counter()
    while t.value < p.tend and time.perf_counter() - w0 < args.to_end_seconds:
        capi.check(lib.tsr_exprem_advance(h, p.tend, capi.ptr(tspan), capi.ptr(solns), C.byref(p.options),
                                          C.byref(st), C.byref(t)), "tsr_exprem_advance")
        capi.check(lib.tsr_step_diagnostics(h, 0, capi.ptr(diag)), "diagnostics")
        log.append([t.value] + diag.tolist() + [st.FuncEvals])
    capi.check(lib.tsr_sync(h), "sync")
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    L = np.array(log)
    u_end = np.empty(p.N)
    capi.check(lib.tsr_exprem_store(h, capi.ptr(u_end)), "store")
    reached = t.value >= p.tend
    if args.step_log:
        with open(args.step_log, "w") as f:
            f.write("# t dt_proposed dt_taken err krylov_halvings rejects growth_capped krylov_dim clipped func_evals\n")
            for r in log:
                f.write(" ".join("%.9g" % x for x in r) + "\n")
    threads = os.cpu_count() or 1
    cpu_rate, cpu_el, cpu_steps, cpu_evals = cpu_exprem_rate(p, u_end, t.value, st, threads, args.cpu_seconds)
    last = L[-min(len(L), 200):]
    line = {
        "metric": "wall seconds to t_end (device-resident EXPREM steps, calibrated dense output)",
        "value": wall if reached else None, "unit": "s", "n_gpus": 1, "higher_is_better": False,
        "reached_t_end": bool(reached), "t_reached_days": t.value, "t_end_days": p.tend, "wall_s": wall,
        "steps": int(st.NumSteps), "g_evals": int(st.FuncEvals), "dtype": "f64", "data": "synthetic",
        "config": workload(args, p.N),
        "steps_krylov_halved": int(np.sum(L[:, 4] > 0)), "steps_with_rejections": int(np.sum(L[:, 5] > 0)),
        "steps_growth_capped": int(np.sum(L[:, 6] > 0)), "krylov_dim_mean": float(np.mean(L[:, 7])),
        "krylov_dim_max": int(np.max(L[:, 7])),
        "dt_taken_last200_p50": float(np.median(last[:, 2])),
        "dt_taken_last200_p95": float(np.percentile(last[:, 2], 95)),
        "cpu_estimate": {"wall_s_to_same_t": st.FuncEvals / cpu_rate, "unit": "s", "cores": threads,
                         "kind": "port (ESTIMATE: GPU run's G evaluations / CPU G-evals/s)",
                         "cpu_g_evals_per_s": cpu_rate,
                         "sample": "%d accepted EXPREM steps (%d G evaluations) from the GPU's final state, "
                                   "%.1f s" % (cpu_steps, cpu_evals, cpu_el)},
        "clocks": clk,
    }
    line["speedup_vs_cpu_estimate"] = line["cpu_estimate"]["wall_s_to_same_t"] / wall
    print(json.dumps(line))
    ctx.close()


def cpu_ensemble_rate(ens, seconds, threads=None):
    """Scenario-steps per second of the oracle's OpenMP EXPREM (C-library
    log/exp) on scenario 0 alone, stepped from t = 0 for about `seconds`."""
    import oracle
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    threads = threads or os.cpu_count() or 1
    p = P.scenario_problem(ens, 0)
    o = oracle.Oracle(p, nthreads=threads, libm=True)
    u = p.u0.copy()
    st = capi.ExpremStats()
    solns = np.zeros(p.N)
    t, steps = 0.0, 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds and t < p.tend:
        t = o.exprem_step(t, u, p.tspan, solns, p.options, st)
        steps += 1
    el = time.perf_counter() - t0
    o.close()
    return {"value": steps / el, "unit": "scenario-steps/s", "cores": threads, "kind": "port",
            "sample": "%d accepted EXPREM steps of scenario 0 (%d unknowns) from t = 0 by the "
                      "oracle's OpenMP form with C-library log/exp (%.1f s)" % (steps, p.N, el)}


def run_ensemble(args):
    """Config 4: all scenarios advance in lockstep rounds (each scenario one
    accepted step of its own size per round).  value = scenario-steps per
    second over the timed rounds; with --to-end the run continues until every
    scenario reaches t_end and reports the p50/p95 per-scenario wall time."""
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    dist = dist_init()
    lib = capi.load()
    p = make_problem(args)
    N, S = p.N, p.S
    ctx = P.Context(p, max_krylov=p.options.MaxKrylov, gram_schmidt=GS[args.gs])
    h = ctx.h
    tuned = ctx.autotune(p.u0, reps=2)
    stats = (capi.ExpremStats * S)()
    ctx.load(p.u0)
    capi.check(lib.tsr_profile(h, 1), "profile")      # graphs captured with their timing events
    for _ in range(args.warmup):
        ctx.ensemble_advance(stats)
    steps0 = sum(stats[s].NumSteps for s in range(S))
    evals0 = sum(stats[s].FuncEvals for s in range(S))
    clocks = Clocks()
    clocks.start()
    barrier(dist)
    capi.check(lib.tsr_sync(h), "sync")
    capi.check(lib.tsr_profile(h, 1), "profile")
    launches0 = lib.tsr_kernel_launches()
    capi.check(lib.tsr_mark(h, 0), "mark")
    t0 = time.perf_counter()
    round_s = []
    for _ in range(args.steps):
        r0 = time.perf_counter()
        t, status, nrun = ctx.ensemble_advance(stats)
        round_s.append(time.perf_counter() - r0)
    capi.check(lib.tsr_mark(h, 1), "mark")
    capi.check(lib.tsr_sync(h), "sync")
    launches = lib.tsr_kernel_launches() - launches0
    barrier(dist)
    clk = clocks.stop()
    ms = C.c_double()
    capi.check(lib.tsr_elapsed_ms(h, 0, 1, C.byref(ms)), "elapsed")
    steps = sum(stats[s].NumSteps for s in range(S)) - steps0
    evals = sum(stats[s].FuncEvals for s in range(S)) - evals0
    t_max = allmax(dist, ms.value / 1e3)
    value = allsum(dist, steps) / t_max
    gms, gcount, gbytes = C.c_double(), C.c_longlong(), C.c_double()
    capi.check(lib.tsr_profile_read(h, 0, C.byref(gms), C.byref(gcount), C.byref(gbytes)), "prof")
    capi.check(lib.tsr_profile(h, 0), "profile")
    hbm_peak, peak_src = measured_peaks()
    g_avg_ms = gms.value / max(gcount.value, 1)
    g_gbs = gbytes.value / max(gms.value * 1e-3, 1e-30) / 1e9
    # e2e: state from pinned host memory in and out around every round
    u_host = capi.PinnedArray(N)
    capi.check(lib.tsr_exprem_store(h, u_host.a.ctypes.data_as(capi.dp)), "store")
    tq = np.array([stats[s].CurrentTime for s in range(S)])
    e_steps0 = sum(stats[s].NumSteps for s in range(S))
    capi.check(lib.tsr_sync(h), "sync")
    w0 = time.perf_counter()
    for _ in range(args.steps):
        capi.check(lib.tsr_ensemble_load(h, u_host.a.ctypes.data_as(capi.dp), capi.ptr(tq)), "load")
        tq, _, _ = ctx.ensemble_advance(stats)
        capi.check(lib.tsr_exprem_store(h, u_host.a.ctypes.data_as(capi.dp)), "store")
    e_wall = time.perf_counter() - w0
    e2e_value = (sum(stats[s].NumSteps for s in range(S)) - e_steps0) / e_wall
    u_host.free()
    to_end = None
    if args.to_end:
        # restart from t = 0 and run every scenario to t_end
        ctx.load(p.u0)
        st2 = (capi.ExpremStats * S)()
        done_at = [None] * S
        w0 = time.perf_counter()
        rounds = 0
        diag = np.zeros(8)
        lim = np.zeros((S, 4))       # steps with Krylov halvings, rejections, growth cap; dim sum
        while True:
            t_before = [st2[s].NumSteps for s in range(S)]
            t, status, nrun = ctx.ensemble_advance(st2)
            rounds += 1
            for s in range(S):
                if st2[s].NumSteps > t_before[s]:
                    capi.check(lib.tsr_step_diagnostics(h, s, capi.ptr(diag)), "diagnostics")
                    lim[s] += [diag[3] > 0, diag[4] > 0, diag[5] > 0, diag[6]]
            now = time.perf_counter() - w0
            for s in range(S):
                if done_at[s] is None and (t[s] >= p.tend or status[s] != 0):
                    done_at[s] = now
            if nrun == 0 or now > args.to_end_seconds:
                break
        fin = sorted(x for x in done_at if x is not None)
        to_end = {"rounds": rounds, "wall_s": now, "finished": len(fin), "scenarios": S,
                  "stopped_by_time_cap": nrun > 0,
                  "p50_scenario_wall_s": float(np.percentile(fin, 50)) if len(fin) == S else None,
                  "p95_scenario_wall_s": float(np.percentile(fin, 95)) if len(fin) == S else None,
                  "t_reached_p5_p50_p95": [float(np.percentile(t, q)) for q in (5, 50, 95)],
                  "steps_per_scenario": [st2[s].NumSteps for s in range(S)],
                  "failed": int(sum(1 for s in range(S) if status[s] != 0)),
                  "scenario_steps_per_s": sum(st2[s].NumSteps for s in range(S)) / now,
                  "limiters": {"steps": int(sum(st2[s].NumSteps for s in range(S))),
                               "krylov_halved": int(lim[:, 0].sum()), "with_rejections": int(lim[:, 1].sum()),
                               "growth_capped": int(lim[:, 2].sum()),
                               "krylov_dim_mean": float(lim[:, 3].sum() / max(1, sum(st2[s].NumSteps for s in range(S))))}}
    cpu = None
    if RANK == 0 and WORLD == 1 and not args.no_cpu_baseline:
        cpu = cpu_ensemble_rate(p, args.cpu_seconds)
    line = {
        "metric": "scenario-steps/s (accepted EXPREM steps summed over scenarios per second)",
        "value": value, "unit": "scenario-steps/s", "n_gpus": WORLD, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator 20261203, evaluation seed 7)",
        "config": workload(args, N),
        "g_evals_per_s": allsum(dist, evals) / t_max,
        "round_wall_s": {"p50": float(np.percentile(round_s, 50)), "p95": float(np.percentile(round_s, 95))},
        "to_end": to_end,
        "roofline": {"bound": "hbm", "kernel": "G / Jv evaluation (k_cells + k_macro_nodes)",
                     "achieved": g_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": g_gbs / hbm_peak,
                     "peak_source": peak_src, "traffic": None, "avg_launch_ms": g_avg_ms,
                     "launches": gcount.value},
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": "scenario-steps/s", "h2d_bytes_per_step": 8 * N,
                "d2h_bytes_per_step": 8 * N,
                "note": "state reloaded from host each round, so every round re-evaluates G(u)"},
        "gpu_launches": int(launches),
        "autotuned": {"g_ms": tuned[0], "threads": tuned[1], "smem_budget": tuned[2]},
        "cpu_baseline": cpu,
    }
    if RANK == 0:
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def run_to_end_bench(args):
    """Config 1 (21 x 21 macro, 11 x 11 micro, t_end = 1 d): wall seconds
    from t = 0 to t_end through the reference-facing one-step call, on the
    GPU (tsr_exprem_step, u in pinned host memory) and on the host cores
    (the oracle's OpenMP EXPREM with C-library log/exp)."""
    import oracle
    from twoscalerich_gb300 import capi
    from twoscalerich_gb300 import problem as P
    if RANK != 0:
        return
    p = P.config1()
    ctx = P.Context(p, gram_schmidt=GS[args.gs])
    tuned = ctx.autotune(p.u0, reps=5)               # the cell kernel's plan for this size
    for _ in range(args.warmup):                      # warm: one full run
        P.run_to_end(ctx.exprem_step, p)
    clocks = Clocks()
    clocks.start()
    l0 = ctx.lib.tsr_kernel_launches()
    t0 = time.perf_counter()
    runs = []
    for _ in range(args.steps):
        r0 = time.perf_counter()
        u, solns, st, log = P.run_to_end(ctx.exprem_step, p)
        runs.append(time.perf_counter() - r0)
    launches = ctx.lib.tsr_kernel_launches() - l0
    clk = clocks.stop()
    gpu_s = float(np.median(runs))
    threads = os.cpu_count() or 1
    orc = oracle.Oracle(p, nthreads=threads, libm=True)
    c0 = time.perf_counter()
    uc, sc, stc, logc = P.run_to_end(orc.exprem_step, p)
    cpu_s = time.perf_counter() - c0
    line = {
        "metric": "wall seconds to t_end (config 1, EXPREM through the one-step call)",
        "value": gpu_s, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * gpu_s / max(st.NumSteps, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "two-scale Richards, 21x21 macro, 11x11 micro, t_end = 1 d",
                   "orthogonalisation": {"mgs": "modified Gram-Schmidt", "cgs2": "classical Gram-Schmidt twice"}[args.gs],
                   "unknowns": p.N, "accepted_steps": st.NumSteps, "g_evals": st.FuncEvals,
                   "inputs_vs_l2": "working set 0.4 GB of vectors and basis; repeated runs"},
        "runs_s": runs,
        "cpu_baseline": {"value": cpu_s, "unit": "s", "cores": threads, "kind": "port",
                         "sample": "one full run to t_end (%d steps) by the oracle's OpenMP EXPREM "
                                   "with C-library log/exp" % stc.NumSteps},
        "speedup_vs_cpu": cpu_s / gpu_s,
        "e2e": {"value": gpu_s, "unit": "s", "h2d_bytes_per_step": 8 * p.N, "d2h_bytes_per_step": 8 * p.N},
        "clocks": clk, "gpu_launches": int(launches),
        "autotuned": dict({"g_ms": tuned[0], "threads": tuned[1], "smem_budget": tuned[2]},
                          **cell_plan(ctx.lib, ctx.h)),
    }
    print(json.dumps(line))


def run_closure_bench(args):
    """Config 5: the learned closure against the plain FP64 method on the
    same 301 x 301 / 21 x 21 mesh.  The network is trained on the GPU from
    plain-run data (configurations 1 and 2, seeds 1001-1002); both runs go
    from t = 0 to the same output times; value = plain wall time / closure
    wall time (higher is better)."""
    from twoscalerich_gb300 import closure
    from twoscalerich_gb300 import problem as P
    if RANK != 0:
        return
    t_all = time.perf_counter()
    msgs = []
    X, Y, desc = closure.training_set(time_limit=args.log_seconds, log=lambda m: msgs.append(m),
                                      t_stop=args.log_until)
    t_data = time.perf_counter() - t_all
    t0 = time.perf_counter()
    model, hist, err = closure.train_model(X, Y, epochs=args.epochs, batch=4096, lr=2e-3, seed=1001)
    t_train = time.perf_counter() - t0
    times = [float(x) for x in args.times.split(",")]
    mk = lambda: P.config2(n_macro=args.n_macro, n_micro=args.n_micro)
    rp, wp, sp, fp = closure.run_plain(mk(), times)
    # indicator: change of a cell's inflow over a step relative to the
    # largest inflow of the field at t = 0 (norm-wise relative flux error)
    from twoscalerich_gb300.capi import TsrError

    thr_ens = args.ens_indicator if args.ens_indicator > 0 else None

    def attempt(**kw):
        try:
            return closure.run_closure(mk(), model, times, thr=args.indicator, qfloor_rel=1.0,
                                       t_switch=args.closure_start, thr_ens=thr_ens, **kw), None
        except TsrError as e:
            return None, str(e)
    res, fail_c = attempt()
    flagged = list(getattr(closure.run_closure, "flagged_per_step", []))
    if res is None:
        print(json.dumps({"metric": "learned-closure speed-up", "value": None, "error": fail_c}))
        return
    rc, wc, sc, fc, frac = res
    resu, fail_u = attempt(params=closure.init_params(7), params2=closure.init_params(8),
                           max_steps=args.ablation_steps)
    ru, wu, su, fu, fracu = resu if resu is not None else ([], None, None, None, None)

    def errs(rec):
        return [{"t": a[0], "water_rel": abs(a[1] - b[1]) / abs(b[1]),
                 "h_max_abs": float(np.max(np.abs(a[2] - b[2]))),
                 "h_rel": float(np.max(np.abs(a[2] - b[2])) / np.max(np.abs(b[2])))}
                for a, b in zip(rec, rp)]
    line = {
        "metric": "learned-closure speed-up over the plain FP64 GPU run (wall time to the last output time)",
        "value": wp / wc, "unit": "x", "n_gpus": 1, "steps": sc, "warmup": 0,
        "ms_per_step": 1e3 * wc / max(sc, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 state, bf16 network", "data": "synthetic",
        "config": {"workload": "learned closure, two-scale Richards", "indicator_kind":
                   "|dkQ| |theta_B(H_c) - theta| <= thr * max|Q(t=0)| per step, after 3 steps of history; "
                   "two-network ensemble: |kQ_a - kQ_b| |theta_B(H_c) - theta| <= thr_ens * max(kQ |..|, max|Q(t=0)|)",
                   "ensemble_indicator": thr_ens, "training_logs_until_d": args.log_until, "macro_nodes":
                   "%dx%d" % (args.n_macro, args.n_macro), "micro_nodes_per_cell":
                   "%dx%d" % (args.n_micro, args.n_micro), "cells": 2 * (args.n_macro - 1) ** 2,
                   "output_times_d": times, "indicator": args.indicator, "closure_start_d": args.closure_start,
                   "network": "two networks 6 -> 4 x 64 SiLU -> 2 (seeds 1001, 2001), bf16 tcgen05 inference, fp32 accumulation"},
        "plain": {"wall_s": wp, "steps": sp, "g_evals": fp, "water": [r[1] for r in rp]},
        "closure": {"wall_s": wc, "steps": sc, "g_evals": fc, "fallback_fraction": frac,
                    "errors": errs(rc), "out_of_range_at_t0": getattr(closure.run_closure, "ood_t0", None),
                    "flagged_per_step_first": flagged[:12], "flagged_total": int(sum(flagged))},
        "ablation_untrained": {"wall_s": wu, "steps": su, "fallback_fraction": fracu, "errors": errs(ru),
                               "note": "untrained networks (seeds 7 and 8), at most %d steps" % args.ablation_steps,
                               "error": fail_u},
        "training": {"samples": int(X.shape[0]), "data_s": t_data, "train_s": t_train,
                     "epochs": args.epochs, "loss": [float(x) for x in hist], "heldout": err,
                     "runs": desc},
    }
    print(json.dumps(line))


# FP64 instructions (DADD + DMUL + DFMA, thread level) per unknown of one
# finite-difference Jv launch of the cell kernel, and its DRAM bytes (read +
# write) per unknown, from the ncu capture summarised in
# profiles/k_cells_jv_141x141_21x21.md (version 9, the current cell kernel:
# 1,027.5 M instructions and 530.3 MB for 17,307,081 unknowns of the
# 141x141 / 21x21 case); both depend on the micro template (21x21 nodes),
# not on the macro size, and are scaled by the unknowns.
FP64_OPS_PER_UNKNOWN = {21: 59.37}
G_TRAFFIC_PER_UNKNOWN = {21: 30.64}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-macro", type=int, default=201)
    ap.add_argument("--n-micro", type=int, default=21)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--max-krylov", type=int, default=None)
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3, 4, 5],
                    help="1: 21x21 x 11x11 to t_end; 2: 201x201 x 21x21 plain method; "
                         "3: 151x151 batched uneven cells; "
                         "4: 64-scenario ensemble of 51x51 x 15x15; 5: learned closure, 301x301")
    ap.add_argument("--times", default="1e-4,2.5e-4,5e-4", help="config 5 output times [d]")
    ap.add_argument("--indicator", type=float, default=1e-3)
    ap.add_argument("--closure-start", type=float, default=0.0,
                    help="config 5: plain method up to this time [d], then the closure")
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--ens-indicator", type=float, default=0.05,
                    help="config 5: threshold of the two-network disagreement indicator (0: one network)")
    ap.add_argument("--log-until", type=float, default=None,
                    help="config 5: training runs logged up to this time [d] (within --log-seconds)")
    ap.add_argument("--ablation-steps", type=int, default=600,
                    help="config 5: step cap of the untrained-network ablation run")
    ap.add_argument("--log-seconds", type=float, default=45.0)
    ap.add_argument("--scenarios", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="minimum seconds of CPU work in the CPU baseline sample")
    ap.add_argument("--gs", default="mgs", choices=sorted(GS),
                    help="Arnoldi orthogonalisation: modified Gram-Schmidt (the reference's) or classical twice")
    ap.add_argument("--to-end", action="store_true",
                    help="config 4: also run every scenario to t_end (p50/p95 wall time); "
                         "configs 2-3: run to t_end instead of the timed steps")
    ap.add_argument("--to-end-seconds", type=float, default=600.0,
                    help="configs 2-4: wall-time cap of the run to t_end")
    ap.add_argument("--step-log", default=None,
                    help="configs 2-3 with --to-end: write the per-step limiter record to this file")
    args = ap.parse_args()
    if args.config == 3 and args.n_macro == 201:
        args.n_macro = 151
    if args.config == 5 and args.n_macro == 201:
        args.n_macro = 301
    if args.config == 4:
        if args.n_macro == 201:
            args.n_macro = 51
        if args.n_micro == 21:
            args.n_micro = 15
    if args.max_krylov is None:
        args.max_krylov = 30 if args.config in (3, 4) else 40
    if args.impl == "reference":
        run_reference(args)
    elif args.config == 4:
        run_ensemble(args)
    elif args.config == 5:
        run_closure_bench(args)
    elif args.config == 1:
        run_to_end_bench(args)
    elif args.to_end:
        run_scale_to_end(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
