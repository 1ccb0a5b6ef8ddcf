#!/usr/bin/env python
"""Band-structure throughput on GB300: k-points/s for silicon with the Cohen-Bergstresser local form
factors (V3, V8, V11 = -0.21, 0.04, 0.08 Ry, a = 5.43 A), plane-wave basis of 137 vectors (10 shells),
the lowest 16 bands at the 2000 k-points of the path L-G-X-W-K-U-L-W-X-K-G.

One step = one solve of the whole 2000-point batch. Reported:
  value        mixed-precision path (FP32 reduction + FP64 Rayleigh-Ritz), inputs resident in HBM,
               whose max eigenvalue error against the plain FP64 path is checked in the same run
               (<= 1e-6 eV, reported as mixed_max_err_ev)
  fp64         the plain FP64 drop-in path on the same batch
  e2e          the same metric through the C ABI uepm_solve with pinned host buffers (k in, E out)
  roofline     the dominant kernel of the headline path, timed with CUDA events on its stream
  cpu_baseline the oracle (CPU restatement of the reference path) on this host's cores
  cpu_cli_as_shipped  the same on one thread with gradients on, as the reference CLI runs it

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-points/s, Si nb=16 basis 137 (FP64 vs mixed @1e-6 eV); serve p50/p99 ms"
WORKLOAD = "Si Cohen-Bergstresser local EPM, basis 137 (10 shells), 16 bands, 2000 k on LGXWKULWXKG"
NB = 16
SHELLS = 10
NPOINTS = 2000
PATH = "LGXWKULWXKG"
PARAM_FILE = os.path.join(ROOT, "params", "si-cohen-bergstresser.yaml")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def emit(d):
    print(json.dumps(d), flush=True)


# ------------------------------------------------------------------------------------------------
def workload_inputs(world: int = 1, rank: int = 0):
    """The workload of one GPU: with N ranks the path is sampled at N x 2000 points and each rank
    solves its contiguous block (ultimateepm_gb300.partition), so per-GPU work stays fixed."""
    from ultimateepm_gb300 import Materials, SymmetryPoints, generate_basis_vectors
    from ultimateepm_gb300.partition import shard_range

    mats = Materials()
    mats.load_material_parameters(PARAM_FILE)
    si = mats.materials["Si"]
    G = generate_basis_vectors(SHELLS)
    k, _ = SymmetryPoints().GeneratePoints(list(PATH), NPOINTS * world)
    a, b = shard_range(len(k), rank, world)
    return si, G, np.ascontiguousarray(k[a:b])


# The timed CPU baseline is the oracle built with the reference's Release numerics flags
# (CMakeLists.txt:47-55: -O3 -ffast-math, OpenMP; -march=native left out, see oracle/Makefile); the
# strict parity build (no fast-math, no FMA contraction) is reported beside it.
CPU_FLAGS = "-O3 -ffast-math -fopenmp (the reference's Release flags, without -march=native)"


def cpu_time_oracle(nthreads: int, budget_s: float, fast: bool = True):
    """Times the oracle on the workload; whole 2000-point passes until budget_s elapsed."""
    from oracle import oracle as O

    O.build()
    mat = O.load_materials(PARAM_FILE)["Si"]
    G = O.generate_basis(SHELLS)
    k, _ = O.generate_path(PATH, NPOINTS)
    O.band_structure(mat, G, k[:64], NB, nthreads=nthreads, fast=fast)  # warm-up (thread pool, caches)
    done, t0 = 0, time.perf_counter()
    while True:
        O.band_structure(mat, G, k, NB, nthreads=nthreads, fast=fast)
        done += len(k)
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def cpu_time_cli_as_shipped(budget_s: float):
    """The reference CLI as shipped runs BandStructure::Compute_parallel on one thread with
    gradients on: apps/EmpiricalPseudoPotentialMain.cpp:75,122,174 call Compute_parallel(nrThreads),
    whose first parameter is the gradient flag (BandStructure.h:58). The oracle timed that way on
    growing prefixes of the path until budget_s elapsed."""
    from oracle import oracle as O

    O.build()
    mat = O.load_materials(PARAM_FILE)["Si"]
    G = O.generate_basis(SHELLS)
    k, _ = O.generate_path(PATH, NPOINTS)
    O.band_structure(mat, G, k[:4], NB, grad=True, nthreads=1, fast=True)  # warm-up
    done, m, t0 = 0, 8, time.perf_counter()
    while True:
        O.band_structure(mat, G, k[:m], NB, grad=True, nthreads=1, fast=True)
        done += m
        dt = time.perf_counter() - t0
        if dt >= budget_s or m >= len(k):
            break
        m = min(2 * m, len(k))
    return {"value": done / dt, "unit": "k-points/s", "cores": 1, "kind": "port", "flags": CPU_FLAGS,
            "sample": f"{done} path k-points, {dt:.1f} s, FP64 eigenvalues and gradients, one thread"}


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------------------------------
def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from ultimateepm_gb300 import _native as N
    from ultimateepm_gb300 import api

    L = N.load()
    si, G, k = workload_inputs(ws, rank)
    nk = len(k)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    dk = torch.from_numpy(k).cuda()
    dE = torch.zeros((nk, NB), dtype=torch.float64, device="cuda")
    dst = torch.zeros(nk, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    real_h = api._Context(si, G, False, False).real

    def timed(prec):
        ctx = api._Context(si, G, False, False, prec)
        call = lambda: N.check(L.uepm_solve_device(ctx.h, C.c_void_p(dk.data_ptr()), nk, NB, N.UEPM_WANT_VALUES,
                                                    C.c_void_p(dE.data_ptr()), None, None,
                                                    C.c_void_p(dst.data_ptr()), sp))
        for _ in range(args.warmup):
            call()
        barrier()
        N.check(L.uepm_ctx_set_profiling(ctx.h, 1))
        launches0 = L.uepm_kernel_launches()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            call()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        barrier()
        launches = L.uepm_kernel_launches() - launches0
        ms = (C.c_double * N.KERNEL_KINDS)()
        cnt = (C.c_uint64 * N.KERNEL_KINDS)()
        N.check(L.uepm_ctx_read_profile(ctx.h, ms, cnt, N.KERNEL_KINDS))
        prof = {L.uepm_kernel_name(q).decode(): (ms[q], int(cnt[q])) for q in range(N.KERNEL_KINDS) if cnt[q]}
        assert not dst.any().item(), "a k-point reported a non-zero status"
        E = dE.cpu().numpy().copy()
        ctx.close()
        return times, prof, launches, E

    clocks = Clocks(local)
    clocks.start()
    t_mixed, prof_mixed, launches_mixed, E_mixed = timed(N.UEPM_PREC_MIXED)
    t_fp64, prof_fp64, launches_fp64, E_fp64 = timed(N.UEPM_PREC_FP64)
    clk = clocks.stop()

    def max_over_ranks(x):
        if ws == 1:
            return x
        import torch.distributed as dist

        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    ms_mixed = max_over_ranks(sum(t_mixed) / len(t_mixed))
    ms_fp64 = max_over_ranks(sum(t_fp64) / len(t_fp64))
    err = float(np.abs(E_mixed - E_fp64).max())

    # end to end through the public C ABI with pinned host buffers: k in, E and status out
    ctx = api._Context(si, G, False, False, N.UEPM_PREC_MIXED)
    hk = torch.from_numpy(k).pin_memory()
    hE = torch.zeros((nk, NB), dtype=torch.float64).pin_memory()
    hs = torch.zeros(nk, dtype=torch.int32).pin_memory()
    dpp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    e2e_call = lambda: N.check(L.uepm_solve(ctx.h, dpp(hk), nk, NB, N.UEPM_WANT_VALUES, dpp(hE), None, None,
                                            C.cast(C.c_void_p(hs.data_ptr()), C.POINTER(C.c_int32))))
    for _ in range(args.warmup):
        e2e_call()
    barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_call()
        e2e_times.append(time.perf_counter() - t0)
    barrier()
    e2e_s = max_over_ranks(sum(e2e_times) / len(e2e_times))
    ctx.close()

    if rank != 0:
        return
    # roofline of the dominant kernel of each path. Algorithmic flops per k-point; a complex
    # multiply-add is 8 real flops, a real one 2 (H(k) of this workload is exactly real, so the
    # real-symmetric kernels run: 4/3 n^3 for the reduction instead of 16/3 n^3).
    n, m = len(G), min(len(G), NB + 4)
    f = 2.0 if real_h else 8.0
    flops_per_k = {
        "tridiag_fp64": f * (2.0 / 3.0) * n ** 3,
        "tridiag_fp32": f * (2.0 / 3.0) * n ** 3,
        "refine_project": f * n * n * m + f * n * m * (m + 1),  # Y = H X, then S and A (upper halves)
        "backtransform": f * n * n * NB,
    }
    pipe_of = {"tridiag_fp32": "fp32", "backtransform": "fp32"}
    # DRAM bytes per launch of the reduction on this 2000-matrix workload: dram__bytes_read.sum +
    # dram__bytes_write.sum from one ncu capture of the same kernels (ncu cannot run inside a bench).
    # The mixed solve runs its 2000 k-points as two concurrent halves (two streams); the profile
    # counts the pair as one launch, timed from the first start to the last end, and its traffic is
    # the sum of the halves'.
    # Each figure belongs to the kernel named beside it and holds until that kernel changes: the
    # mixed path's k_tridiag_reg_local (profiles/k_tridiag_si137_2000k.md) and the FP64 path's
    # k_tridiag<double> (profiles/launches_si137_2000k.md); re-capture them whenever either is edited.
    traffic = {"tridiag_fp32": 83.66e6, "tridiag_fp64": 9.108e9}
    traffic_kernel = {"tridiag_fp32": "k_tridiag_reg_local (register-resident FP32 reduction, n = 137)",
                      "tridiag_fp64": "k_tridiag<double> (persistent global-memory FP64 reduction, n = 137)"}
    peak64 = C.c_double()
    peak32 = C.c_double()
    N.check(L.uepm_measure_peak(N.UEPM_PREC_FP64, C.byref(peak64)))
    N.check(L.uepm_measure_peak(N.UEPM_PREC_MIXED, C.byref(peak32)))

    def roof(prof, fp64_path):
        timed = {q: v for q, v in prof.items() if q in flops_per_k}
        dom = max(timed, key=lambda q: timed[q][0])
        ms = timed[dom][0] / max(timed[dom][1], 1)
        pipe = "fp64" if fp64_path else pipe_of.get(dom, "fp64")
        peak = peak64.value if pipe == "fp64" else peak32.value
        ach = flops_per_k[dom] * nk / (ms * 1e-3) / 1e12
        tb = traffic.get(dom) if nk == NPOINTS else None
        return {"bound": f"{pipe}_pipe", "kernel": dom, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "frac": ach / peak, "traffic": tb, "traffic_unit": "bytes per launch (ncu)", "kernel_ms": ms,
                "traffic_measured_on": traffic_kernel.get(dom),
                "peak_source": "measured in-run (pure-FMA kernel, uepm_measure_peak)"}

    roof_mixed = roof(prof_mixed, False)
    roof_fp64 = roof(prof_fp64, True)
    # the same achieved rate against the measured dense bf16 tensor peak, for reference (the
    # reduction's arithmetic is FP32 / FP64 on the SIMT pipes, so this fraction is not its bound)
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        for rf in (roof_mixed, roof_fp64):
            rf["frac_of_measured_bf16_tensor_peak"] = rf["achieved"] / float(mp["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        pass

    cores = os.cpu_count() or 1
    cpu_v, cpu_done, cpu_dt = cpu_time_oracle(cores, args.cpu_budget)
    cpu_s, cpu_s_done, cpu_s_dt = cpu_time_oracle(cores, min(args.cpu_budget, 5.0), fast=False)
    value = nk * ws / (ms_mixed * 1e-3)
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "k-points/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32+fp64",
        "data": "synthetic (deterministic k-path; no dataset)",
        "config": {"workload": WORKLOAD, "k_points_per_gpu": nk, "bands": NB, "basis": n,
                   "precision": "mixed: FP32 reduction + FP64 Rayleigh-Ritz", "l2": "flushed (256 MB write) "
                   "between timed steps", "parallelism": f"k-partition x{ws} (contiguous blocks of "
                   f"{NPOINTS * ws} path points, no collective)"},
        "mixed_max_err_ev": err,
        "fp64": {"value": nk * ws / (ms_fp64 * 1e-3), "ms_per_step": ms_fp64, "dtype": "f64",
                 "roofline": roof_fp64,
                 "kernels_ms": {q: v[0] / max(v[1], 1) for q, v in prof_fp64.items()},
                 "gpu_launches": launches_fp64},
        "real_symmetric_kernels": real_h,
        "peaks_tflops": {"fp64": peak64.value, "fp32": peak32.value},
        "mixed_speedup_vs_fp64": ms_fp64 / ms_mixed,
        "e2e": {"value": nk * ws / e2e_s, "unit": "k-points/s", "h2d_bytes_per_step": int(hk.numel() * 8),
                "d2h_bytes_per_step": int(hE.numel() * 8 + hs.numel() * 4), "entry_point": "uepm_solve"},
        "roofline": roof_mixed,
        "kernels_ms": {q: v[0] / max(v[1], 1) for q, v in prof_mixed.items()},
        "kernels_ms_note": "per solve; the mixed solve runs its 2000 k-points as two halves on two streams, "
                           "and each kernel's time spans the first half's start to the second half's end",
        "gpu_launches": launches_mixed,
        "cpu_baseline": {"value": cpu_v, "unit": "k-points/s", "cores": cores, "kind": "port", "flags": CPU_FLAGS,
                         "sample": f"{cpu_done} k-points ({cpu_done // nk} passes over the 2000-point path), "
                                   f"{cpu_dt:.1f} s, FP64 eigenvalues only"},
        "cpu_baseline_strict": {"value": cpu_s, "unit": "k-points/s", "cores": cores, "kind": "port",
                                "flags": "-O3 -fno-fast-math -ffp-contract=off (the parity build)",
                                "sample": f"{cpu_s_done} k-points, {cpu_s_dt:.1f} s"},
        "cpu_cli_as_shipped": cpu_time_cli_as_shipped(min(args.cpu_budget, 3.0)) if ws == 1 else None,
        "clocks": clk,
    }
    if ws == 1 and not args.no_extras:
        out["uneven_batch"] = run_uneven_batch(args)
        out["serve"] = run_serve()
        out["dielectric"] = run_dielectric(cpu_budget=min(args.cpu_budget, 5.0))
        out["configs_2_3"] = run_configs()
    emit(out)


def run_uneven_batch(args, steps: int = 1, warmup: int = 0, total_k: int = 2000000, seed: int = 20261203):
    """The uneven mixed-material batch of config 4: 8 contexts (orders 89..458, real and complex, SOC on
    for four), total_k = 2 000 000 first-zone k-points split by seeded multinomial proportions, 16
    bands, mixed precision, run as one uepm_batch (per-context streams). A separate 16 384-k batch of
    the same contexts warms them up (workspaces, tuning); the 2M batch is then timed once (its first
    run: eager; later runs replay a CUDA graph). Returns k-points/s over the whole batch."""
    import torch

    from ultimateepm_gb300 import _native as N
    from ultimateepm_gb300.serve import MIXED_SET, make_contexts, sample_bz

    L = N.load()
    rng = np.random.default_rng(seed)
    ctxs = make_contexts(N.UEPM_PREC_MIXED)
    orders = [int(c.n) for c in ctxs]
    props = rng.dirichlet(np.ones(len(ctxs)))
    counts = rng.multinomial(total_k, props)
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    # warm-up batch: the same contexts, 16 384 k in the same proportions
    wb, wbufs = C.c_void_p(), []
    N.check(L.uepm_batch_create(C.byref(wb)))
    for ctx, nk in zip(ctxs, rng.multinomial(16384, props)):
        if nk:
            t = (torch.from_numpy(sample_bz(int(nk), rng)).cuda(), torch.zeros((int(nk), NB), dtype=torch.float64,
                 device="cuda"), torch.zeros(int(nk), dtype=torch.int32, device="cuda"))
            wbufs.append(t)
            N.check(L.uepm_batch_add(wb, ctx.h, C.c_void_p(t[0].data_ptr()), int(nk), NB, N.UEPM_WANT_VALUES,
                                     C.c_void_p(t[1].data_ptr()), None, None, C.c_void_p(t[2].data_ptr())))
    N.check(L.uepm_batch_run(wb, sp))
    torch.cuda.synchronize()
    L.uepm_batch_destroy(wb)
    del wbufs
    bufs = []
    b = C.c_void_p()
    N.check(L.uepm_batch_create(C.byref(b)))
    try:
        for ctx, nk in zip(ctxs, counts):
            if nk == 0:
                continue
            dk = torch.from_numpy(sample_bz(int(nk), rng)).cuda()
            dE = torch.zeros((int(nk), NB), dtype=torch.float64, device="cuda")
            ds = torch.zeros(int(nk), dtype=torch.int32, device="cuda")
            bufs.append((dk, dE, ds))
            N.check(L.uepm_batch_add(b, ctx.h, C.c_void_p(dk.data_ptr()), int(nk), NB, N.UEPM_WANT_VALUES,
                                     C.c_void_p(dE.data_ptr()), None, None, C.c_void_p(ds.data_ptr())))
        for _ in range(warmup):
            N.check(L.uepm_batch_run(b, sp))
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(steps):
            N.check(L.uepm_batch_run(b, sp))
        e.record(s)
        e.synchronize()
        ms = a.elapsed_time(e) / steps
        assert not any(ds.any().item() for _, _, ds in bufs), "a k-point reported a non-zero status"
        kpr = int(L.uepm_batch_kernels_per_run(b))
    finally:
        L.uepm_batch_destroy(b)
        for c in ctxs:
            c.close()
    return {"value": total_k / (ms * 1e-3), "unit": "k-points/s", "ms_per_step": ms, "steps": steps,
            "workload": f"{total_k} seeded first-zone k-points over 8 (material, cutoff, SOC) groups, 16 bands, "
                        "mixed precision, one uepm_batch (per-context streams; timed once, eager)",
            "groups": [{"material": m, "shells": sh, "soc": so, "order": o, "k_points": int(nk)}
                       for (m, sh, so), o, nk in zip(MIXED_SET, orders, counts)],
            "kernels_per_step": kpr, "graph": steps > 1}


def run_serve(seed: int = 20261203, kmax: int = 50000):
    """Serving (config 5): seeded Poisson arrivals, each request for a random group of the mixed-material
    set, log-uniform 1..50 000 k-points, 8..16 bands and finite-difference group velocities (7 solves
    per k-point), mixed precision, 4 slots, 16 GB arena. Rates 100, 300, 1000 and 5000 req/s (16
    requests each), and 1 req/s (12 requests) as a reference load. Per rate: p50 / p99 latency, the
    offered and served work (k-point solves / s), and whether the offered work exceeds what the GPU
    serves, i.e. the queue grows without bound at that rate."""
    from ultimateepm_gb300 import _native as N
    from ultimateepm_gb300.serve import Server, make_contexts, poisson_requests, run_load

    ctxs = make_contexts(N.UEPM_PREC_MIXED)
    srv = Server(ctxs, hbm_budget=16 << 30, slots=4, max_chunk=1024)
    sweep = []
    try:
        run_load(srv, poisson_requests(4, 50.0, seed + 7, len(ctxs), 1, 64), seed=seed + 7)  # warm-up
        for q, (rate, nreq) in enumerate(((1.0, 12), (100.0, 16), (300.0, 16), (1000.0, 16), (5000.0, 16))):
            reqs = poisson_requests(nreq, rate, seed + 11 + q, len(ctxs), 1, kmax)
            r = run_load(srv, reqs, seed=seed + 11 + q)
            span = reqs[-1][0] if len(reqs) > 1 else 0.0
            work = 7.0 * sum(nk for _, _, nk, _ in reqs)  # k-point solves (7 per k with velocities)
            offered = work / span if span > 0 else None
            served = 7.0 * r["k_points_per_s"] if r["k_points_per_s"] else None
            sweep.append({"rate_req_per_s": rate, "requests": nreq, "offered_req_per_s": r["offered_req_per_s"],
                          "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
                          "offered_solves_per_s": offered, "served_solves_per_s": served,
                          "k_points_per_s": r["k_points_per_s"], "drain_s": r["wall_s"] - span,
                          "queue_grows": bool(offered and served and offered > served),
                          "requests_with_nonzero_status": r["requests_with_nonzero_status"]})
    finally:
        srv.close()
        for c in ctxs:
            c.close()
    first = next((x["rate_req_per_s"] for x in sweep if x["queue_grows"]), None)
    ref = sweep[0]
    return {"p50_ms": ref["p50_ms"], "p99_ms": ref["p99_ms"], "rate_req_per_s": ref["rate_req_per_s"],
            "k_per_request": f"log-uniform 1..{kmax}", "bands": "8..16",
            "velocities": "central differences, h = 1e-4 (reduced units), 7 solves per k-point", "precision": "mixed",
            "slots": 4, "hbm_budget_gb": 16, "sweep": sweep, "first_rate_queue_grows": first,
            "capacity_req_per_s": (max(x["served_solves_per_s"] or 0 for x in sweep)
                                   / (7.0 * (1 + kmax) / max(np.log(1 + kmax), 1.0))) if sweep else None}


def run_dielectric(nk: int = 8000, ne: int = 1001, seed: int = 20261203, cpu_budget: float = 5.0):
    """The dielectric function from the band states (DielectricFunction::compute_dielectric_function
    for one q): Si Cohen-Bergstresser, basis 137, 16 bands (4 valence x 12 conduction pairs), nk
    seeded first-zone k-points, q = (0.01, 0, 0), ne energies over 0..10 eV, eta = 0.05, FP64 band
    states with vectors at k and k + q. Reports k-points/s of the whole call (host k-points in, the
    [ne] sums out), the sums kernel alone on resident states (CUDA events), and the oracle on a
    bounded sample of the same workload."""
    import torch

    from oracle import oracle as O
    from ultimateepm_gb300 import _native as N
    from ultimateepm_gb300 import api
    from ultimateepm_gb300.dielectric import DielectricFunction

    L = N.load()
    mats = api.Materials()
    mats.load_material_parameters(PARAM_FILE)
    si = mats.materials["Si"]
    G = api.generate_basis_vectors(SHELLS)
    k = O.sample_first_bz(nk, seed)
    q = np.array([0.01, 0.0, 0.0])
    en = np.linspace(0.0, 10.0, ne)
    eta = 0.05
    df = DielectricFunction(si, G, NB)
    df.m_kpoints = k
    df.set_qpoints([q])
    df.set_energies(en)
    df.set_nb_kpoints(nk)
    df.compute_dielectric_function(eta)  # warm-up (builds, allocations)
    times = []
    for _ in range(3):
        df.m_dielectric_function_real = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        df.compute_dielectric_function(eta)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    call_s = min(times)
    # the sums kernel alone, on resident states of the first 2000 k-points
    m = 2000
    ctx = api._Context(si, G, False, False, N.UEPM_PREC_FP64)
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    dev = "cuda"
    p = lambda t: C.c_void_p(t.data_ptr())
    dk = torch.from_numpy(k[:m]).to(dev)
    dkq = dk + torch.from_numpy(q).to(dev)[None, :]
    Ek = torch.zeros((m, NB), dtype=torch.float64, device=dev)
    Ekq = torch.zeros_like(Ek)
    Xk = torch.zeros((m, NB, len(G), 2), dtype=torch.float64, device=dev)
    Xkq = torch.zeros_like(Xk)
    st = torch.zeros(m, dtype=torch.int32, device=dev)
    want = N.UEPM_WANT_VALUES | N.UEPM_WANT_VECTORS
    N.check(L.uepm_solve_device(ctx.h, p(dk), m, NB, want, p(Ek), p(Xk), None, p(st), sp))
    N.check(L.uepm_solve_device(ctx.h, p(dkq), m, NB, want, p(Ekq), p(Xkq), None, p(st), sp))
    den = torch.from_numpy(en).to(dev)
    sums = torch.zeros(ne, dtype=torch.float64, device=dev)
    call = lambda: N.check(L.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), m, NB, len(G), 4, p(den), ne, eta,
                                                          None, p(sums), sp))
    for _ in range(3):
        call()
    kt = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        call()
        b.record(s)
        b.synchronize()
        kt.append(a.elapsed_time(b))
    kernel_ms = min(kt)
    ctx.close()
    pairs = 4 * (NB - 4)
    # the oracle (eigenstates on all host cores, the pair sums in numpy) on a bounded sample
    mat = O.load_materials(PARAM_FILE)["Si"]
    Go = O.generate_basis(SHELLS)
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget and done < nk:
        O.dielectric_sums(mat, Go, k[done:done + 64], q, NB, en, eta)
        done += 64
    cpu_dt = time.perf_counter() - t0
    return {
        "value": nk / call_s, "unit": "k-points/s", "ms_per_call": call_s * 1e3,
        "workload": f"Si Cohen-Bergstresser basis {len(G)}, {NB} bands ({pairs} valence-conduction pairs), {nk} seeded "
                    f"first-zone k, q = (0.01, 0, 0), {ne} energies 0..10 eV, eta = {eta}, FP64 band states",
        "sums_kernel": {"ms_per_2000_k": kernel_ms, "pair_energy_terms_per_s": 2000 * pairs * ne / (kernel_ms * 1e-3)},
        "cpu_baseline": {"value": done / cpu_dt, "unit": "k-points/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"{done} k-points, {cpu_dt:.1f} s (oracle eigenstates on all cores, numpy pair sums)"},
    }


def run_configs(seed: int = 20261203):
    """The precision configurations at their stated sizes, each with FP64 and mixed throughput and the
    mixed path's per-band max error against the FP64 path:
      config 2: 500 000 seeded first-zone k, 12 bands, for Si with the nonlocal d-channel (basis 137,
                real), InP with square d-wells (basis 113, complex) and Ge with the gaussian d-well
                (basis 181, real); FP64 and mixed over all 500 000 k;
      config 3: Ge with nonlocal wells and spin-orbit (12 shells, basis 181 per spin, order 362),
                nb = 8 doubled to 16 as BandStructure::Initialize does with SOC (8 Kramers pairs),
                1 000 000 seeded first-zone k with the mixed path; the FP64 path on the first 4000 of
                them, for the ratio and the per-band error.
    One timed solve each (CUDA events) after a warm-up solve on 2000 of the same k-points."""
    import torch

    from ultimateepm_gb300 import _native as N
    from ultimateepm_gb300 import api
    from ultimateepm_gb300.serve import sample_bz

    L = N.load()
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())

    def solve_timed(ctx, dk, nb):
        nk = dk.shape[0]
        dE = torch.zeros((nk, nb), dtype=torch.float64, device="cuda")
        st = torch.zeros(nk, dtype=torch.int32, device="cuda")
        N.check(L.uepm_solve_device(ctx.h, p(dk), min(nk, 2000), nb, N.UEPM_WANT_VALUES, p(dE), None, None, p(st), sp))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        N.check(L.uepm_solve_device(ctx.h, p(dk), nk, nb, N.UEPM_WANT_VALUES, p(dE), None, None, p(st), sp))
        b.record(s)
        b.synchronize()
        assert not st.any().item(), "a k-point reported a non-zero status"
        return dE, a.elapsed_time(b)

    rng = np.random.default_rng(seed)
    out = {}
    for name, yaml, sym, shells, nl, soc, nb, nk, nk64 in (
            ("config_2", "si-nonlocal-d.yaml", "Si", 10, True, False, 12, 500000, 500000),
            ("config_2_inp", "materials.yaml", "InP", 9, True, False, 12, 500000, 500000),
            ("config_2_ge", "materials.yaml", "Ge", 12, True, False, 12, 500000, 500000),
            ("config_3", "materials.yaml", "Ge", 12, True, True, 8, 1000000, 4000)):
        mats = api.Materials()
        mats.load_material_parameters(os.path.join(ROOT, "params", yaml))
        m = mats.materials[sym]
        G = api.generate_basis_vectors(shells)
        nbt = nb * (2 if soc else 1)  # BandStructure::Initialize doubles nb with SOC
        dk = torch.from_numpy(sample_bz(nk, rng)).cuda()
        res = {}
        for prec, tag, kk in ((N.UEPM_PREC_FP64, "fp64", dk[:nk64].contiguous()), (N.UEPM_PREC_MIXED, "mixed", dk)):
            ctx = api._Context(m, G, nl, soc, prec)
            E, ms = solve_timed(ctx, kk, nbt)
            res[tag] = (E, ms, kk.shape[0], ctx.n)
            ctx.close()
        n64 = res["fp64"][2]
        err = (res["mixed"][0][:n64] - res["fp64"][0]).abs().amax(dim=0).cpu().numpy()
        tc_block = None
        if soc:
            # the mixed solve's kernels on 2000 of the k-points, CUDA events per kernel (a separate,
            # profiled solve: the timed one above runs without events), with the tensor-core kernels'
            # work: the reduction's panel updates (tcgen05 kind::tf32) and Y = H X (kind::f16 on BF16
            # slices: 36 slice pairs x 2 x 128 x N x K per 128-row tile)
            ctx = api._Context(m, G, nl, soc, N.UEPM_PREC_MIXED)
            # one stream, so that each kernel's events time that kernel alone (the timed solve above
            # runs its chunks on two streams)
            N.check(L.uepm_ctx_set_tuning(ctx.h, C.byref(N.UepmTuning(streams=1))))
            n, mm = ctx.n, nbt + 4
            kk = dk[:2000].contiguous()
            solve_timed(ctx, kk, nbt)  # warm
            N.check(L.uepm_ctx_set_profiling(ctx.h, 1))
            dE2 = torch.zeros((2000, nbt), dtype=torch.float64, device="cuda")
            st2 = torch.zeros(2000, dtype=torch.int32, device="cuda")
            N.check(L.uepm_solve_device(ctx.h, p(kk), 2000, nbt, N.UEPM_WANT_VALUES, p(dE2), None, None, p(st2), sp))
            torch.cuda.synchronize()
            kms = (C.c_double * N.KERNEL_KINDS)()
            kcnt = (C.c_uint64 * N.KERNEL_KINDS)()
            N.check(L.uepm_ctx_read_profile(ctx.h, kms, kcnt, N.KERNEL_KINDS))
            prof = {L.uepm_kernel_name(q).decode(): kms[q] for q in range(N.KERNEL_KINDS) if kcnt[q]}
            ctx.close()
            mpad = (mm + 3) // 4 * 4
            ncol = (2 * mpad + 15) // 16 * 16
            kdim = 32 * ((n + 15) // 16)
            bf16_flop = 36 * 2 * 128 * ncol * kdim * ((n + 127) // 128) * 2000
            rp_ms = prof.get("refine_project", float("nan"))
            tc_block = {
                "kernels_ms_per_2000_k": {q: round(v, 3) for q, v in prof.items()},
                "tensor_core_kernels": ["k_tridiag_blocked (panel updates, tcgen05.mma kind::tf32, hi/lo splits)",
                                        "k_refine_y_tc (Y = H X, tcgen05.mma kind::f16 on exact BF16 slices)"],
                "refine_project_bf16_issued_tflops": bf16_flop / (rp_ms * 1e-3) / 1e12,
                "refine_project_note": "refine_project = k_refine_y_tc + the double-single S, A kernel; BF16 "
                                       "flops issued by the slice products over that time",
            }
            try:
                mpk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
                tc_block["refine_project_frac_of_measured_bf16_peak"] = tc_block["refine_project_bf16_issued_tflops"] / float(
                    mpk["bf16_tflops"])
            except (OSError, KeyError, ValueError):
                pass
        fp64_rate = n64 / (res["fp64"][1] * 1e-3)
        mixed_rate = res["mixed"][2] / (res["mixed"][1] * 1e-3)
        out[name] = {
            "workload": f"{sym} ({yaml}, nonlocal{', spin-orbit' if soc else ''}), {shells} shells, order {res['fp64'][3]}, "
                        f"{nbt} bands{' (nb = 8 doubled by SOC)' if soc else ''}, {nk} seeded first-zone k"
                        + (f" (FP64 on the first {n64})" if n64 < nk else ""),
            "k_points": nk, "fp64_k_points": n64,
            "fp64_k_points_per_s": fp64_rate, "mixed_k_points_per_s": mixed_rate,
            "mixed_over_fp64": mixed_rate / fp64_rate,
            "mixed_ms": res["mixed"][1], "fp64_ms": res["fp64"][1],
            "mixed_max_err_ev": float(err.max()), "mixed_max_err_ev_per_band": [float(x) for x in err],
        }
        if tc_block:
            out[name]["profiled"] = tc_block
        del dk, res
        torch.cuda.empty_cache()
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    mat = O.load_materials(PARAM_FILE)["Si"]
    G = O.generate_basis(SHELLS)
    k, _ = O.generate_path(PATH, NPOINTS)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.band_structure(mat, G, k[:256], NB, nthreads=cores, fast=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.band_structure(mat, G, k, NB, nthreads=cores, fast=True)
        times.append(time.perf_counter() - t0)
    s = sum(times) / len(times)
    v = len(k) / s
    emit({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "k-points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (deterministic k-path; no dataset)",
        "config": {"workload": WORKLOAD, "k_points_per_gpu": len(k), "bands": NB, "basis": len(G)},
        "cpu_baseline": {"value": v, "unit": "k-points/s", "cores": cores, "kind": "port", "flags": CPU_FLAGS,
                         "sample": f"{len(k)} k-points per step (the whole path), FP64 eigenvalues only"},
        "e2e": {"value": v, "unit": "k-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of oracle timing for cpu_baseline")
    p.add_argument("--no-extras", action="store_true", help="skip the uneven-batch and serving sub-measurements")
    args = p.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
