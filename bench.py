#!/usr/bin/env python3
"""Benchmark: FP64 eigenvectors/s of the robust level-3 inverse iteration.

Workload (the plain large configuration): one real upper-Hessenberg H of
order n = 10000 from the seeded real-spectrum generator, all 10000 eigenvalues
as shifts with relative 1e-12 noise, tlsz = 160.  One step = one complete
solve (tile sweep, reconciliation, back-transform, normalisation, convergence
check) of all shifts.

* value: eigenvectors/s with H, the shifts and the output block resident in
  HBM (hsr_inverse_iteration_device), timed with CUDA events on the launching
  stream.  H (800 MB) is larger than L2, so no flush is needed between steps.
* e2e: the same metric through the drop-in C entry point
  tiled_inverse_iteration with pinned host buffers: H and the shifts copied
  in, the eigenvectors and shifts copied out, every step (the library moves
  the page-locked blocks by SM copies through their mapped pointers).
* roofline: the dominant kernel (the crossover/update GEMM) against the FP64
  DFMA peak measured in the same run; traffic from the committed ncu capture.
* cpu_baseline: the C restatement of the reference (oracle port, OpenMP over
  shift tiles, OpenBLAS dgemm) on all host cores over a bounded sample of the
  shifts.
``--impl reference`` times that CPU implementation alone on the same config.
Under torchrun every rank solves its own replica (weak scaling, no collective
on the data path); rank 0 prints one JSON line with the max over ranks.
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
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "FP64 eigenvectors/s at n=10k"
UNIT = "eigenvectors/s"
# DRAM bytes per algorithmic FMA of k_gemm, from one ncu capture of this
# workload (n=10000, S=10000, tlsz=160; the launch over the 8080 rows above
# tile 51: 1342.60 MB of dram__bytes_read and 1237.79 MB of
# dram__bytes_write for 8080*319*10000 FMAs; the launch over 7920 rows gives
# the same ratio within 0.1%).  The traffic is the read and write of R and
# X over the rows above, so it grows with rows x shifts as the FMAs do, and
# the ratio gives each launch's traffic.
GEMM_DRAM_BYTES_PER_FMA = (1342.602752e6 + 1237.791744e6) / (8080 * 319 * 10000)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--order", type=int, default=10000, help="n, the order of H")
    ap.add_argument("--nrhs", type=int, default=0, help="0 = all n eigenvalues")
    ap.add_argument("--tlsz", type=int, default=160,
                    help="row tile size (160: fastest of 128..320 on GB300 at n=10k)")
    ap.add_argument("--rhs-tlsz", type=int, default=64)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-sample", type=int, default=0, help="shifts in the CPU sample (0 = 64 per core)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "batched", "served", "stress", "hessenberg", "complex", "dense"],
                    help="plain: n=10k solve (default); batched: 4096 mixed problems in one graph; "
                         "served: a Poisson request trace through the request loop; complex: n=10k with "
                         "n/2 complex-conjugate shifts; dense: reduce + solve + back-transform of a dense matrix")
    ap.add_argument("--problems", type=int, default=4096, help="batched: number of problems")
    ap.add_argument("--requests", type=int, default=20000, help="served: number of requests")
    ap.add_argument("--rate", type=float, default=160.0, help="served: arrivals per second")
    ap.add_argument("--saturate", type=int, default=4000,
                    help="served: the first this many requests arriving at once (capacity)")
    ap.add_argument("--pool", type=int, default=256, help="served: distinct matrices generated on the device")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="served: HBM budget")
    ap.add_argument("--batch-tlsz", type=int, default=0, help="batched/served tile size (0: autotune)")
    ap.add_argument("--stress-order", type=int, default=5000, help="stress: n of the robustness-stress problem")
    ap.add_argument("--only-plain", action="store_true",
                    help="default run: skip the batched and served sub-measurements")
    return ap.parse_args()


# ------------------------------------------------------------------ inputs
def workload(n: int, seed: int):
    """(H, shifts), generated once per host and cached in the temp dir."""
    from hsrq3in_gb300 import generators as G
    d = os.path.join(tempfile.gettempdir(), "hsrq3in_bench")
    os.makedirs(d, exist_ok=True)
    f = os.path.join(d, "real_n%d_s%d_v1.npz" % (n, seed))
    if os.path.exists(f):
        z = np.load(f)
        return np.asfortranarray(z["H"]), z["wr"]
    H, lam = G.real_spectrum(n, seed)
    wr = G.perturbed_shifts(lam, seed + 1)
    tmp = f + ".%d.tmp.npz" % os.getpid()
    np.savez(tmp, H=H, wr=wr)
    os.replace(tmp, f)
    return H, wr


def stress_workload(n: int, seed: int):
    """Robustness-stress problem (H, eigenvalues), cached like workload()."""
    from hsrq3in_gb300 import generators as G
    d = os.path.join(tempfile.gettempdir(), "hsrq3in_bench")
    os.makedirs(d, exist_ok=True)
    f = os.path.join(d, "stress_n%d_s%d_v1.npz" % (n, seed))
    if os.path.exists(f):
        z = np.load(f)
        return np.asfortranarray(z["H"]), z["lam"]
    H, lam = G.stress(n, seed)
    tmp = f + ".%d.tmp.npz" % os.getpid()
    np.savez(tmp, H=H, lam=lam)
    os.replace(tmp, f)
    return H, lam


def _gen_one(args):
    """(H, shifts) of one mixed-size problem; runs in a spawned worker."""
    n, seed, lo, hi = args
    from hsrq3in_gb300 import generators as G
    H, lam = G.real_spectrum(n, seed)
    rng = np.random.default_rng(seed + 7)
    wr = G.shift_subset(G.perturbed_shifts(lam, seed + 3), rng, lo, hi)
    return H, wr


def mixed_problems(count: int, nlo: int, nhi: int, flo: float, fhi: float, seed: int):
    """count problems, n log-uniform in [nlo, nhi], a random fraction U[flo, fhi]
    of their eigenvalues as shifts; generated in a spawn process pool (before
    any GPU work)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(np.log(nlo), np.log(nhi), count))).astype(int)
    jobs = [(int(n), seed * 100003 + i, flo, fhi) for i, n in enumerate(ns)]
    order = np.argsort(-ns)                      # big ones first for balance
    out = [None] * count
    # One BLAS thread per worker: workers x BLAS threads would oversubscribe
    # the cores (measured 60x slower).  Spawned workers read the environment.
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    try:
        with cf.ProcessPoolExecutor(max_workers=os.cpu_count() or 1, mp_context=mp.get_context("spawn")) as ex:
            futs = {ex.submit(_gen_one, jobs[i]): i for i in order}
            for f in cf.as_completed(futs):
                out[futs[f]] = f.result()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return out


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
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
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        load = [x for x in sm if mx and x > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU (port)
def cpu_sample(H, wr, tlsz, rhs_tlsz, sample, steps, warmup):
    """Time the oracle port (reference arithmetic, -O3) on `sample` shifts."""
    from oracle import pyoracle as O
    cores = os.cpu_count() or 1
    O.set_threads(cores, variant="ref_fast")
    w = np.ascontiguousarray(wr[:sample])
    times = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        O.oracle_inverse_iteration(H, w, tlsz, rhs_tlsz, variant="ref_fast")
        dt = time.perf_counter() - t0
        if it >= warmup:
            times.append(dt)
    t = statistics.mean(times)
    return sample / t, t, cores


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, H, wr, rank, world):
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    lib = hsr.load(build_if_missing=True)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n, S = H.shape[0], wr.shape[0]
    ldh = n + (n & 1)
    dHt = torch.zeros((n, ldh), dtype=torch.float64, device=dev)   # row j = column j of H
    dHt[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr0 = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    dwr = dwr0.clone()
    dX = torch.empty((S, ldh), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    opt = _lib.Options(0, 0, -1, 0.0)

    def step():
        dwr.copy_(dwr0)
        rc = lib.hsr_inverse_iteration_device(n, dHt.data_ptr(), ldh, S, dwr.data_ptr(), args.tlsz,
                                              dX.data_ptr(), ldh, C.byref(opt), C.c_void_p(stream.cuda_stream),
                                              None, None)
        if rc < 0:
            raise RuntimeError("device call failed: %d" % rc)
        return rc

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    dfma, dmma = hsr.fp64_peak(200.0)          # after warm-up: clocks ramped
    lib.hsr_set_kernel_timing(1)
    ncls = len(_lib.KERNEL_CLASSES)
    kms = np.zeros(ncls)
    kl = np.zeros(ncls, dtype=np.int64)
    gemm_fma = 0.0
    launches = 0
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        with torch.cuda.stream(stream):
            ev0.record(stream)
            rcs = []
            for _ in range(args.steps):
                rcs.append(step())
                ms = (C.c_double * ncls)()
                ln = (C.c_long * ncls)()
                fm = C.c_double()
                lib.hsr_last_kernel_times(ms, ln, C.byref(fm))
                kms += np.array(ms[:])
                kl += np.array(ln[:])
                gemm_fma += fm.value
                launches += lib.hsr_last_launch_count()
            ev1.record(stream)
        torch.cuda.synchronize()
    lib.hsr_set_kernel_timing(0)
    t_ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    ms_per_step = t_ms / args.steps
    value = world * S / (ms_per_step / 1e3)

    # result sanity: the library's device residuals on 256 sampled columns,
    # finiteness of the whole block
    cols = torch.from_numpy(np.linspace(0, S - 1, 256).astype(np.int64)).to(dev)
    res = hsr.residuals_device(dHt, dwr[cols].contiguous(), dX[cols].contiguous()).cpu().numpy()
    finite = bool(torch.isfinite(dX[:, :n]).all().item())

    gemm_ms = kms[3]
    achieved = 2.0 * gemm_fma / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    peak = dfma / 1e3
    roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": (GEMM_DRAM_BYTES_PER_FMA * gemm_fma / max(kl[3], 1)) if GEMM_DRAM_BYTES_PER_FMA else None,
            "traffic_note": "DRAM bytes per launch: bytes per FMA from an ncu capture of this workload (n=10000, tlsz=160) times this run's FMAs per launch",
            "kernel": "k_gemm (crossover propagation + tile update, DFMA; the launches over the rows above "
                      "the next diagonal tile, which share the GPU with that tile's GEMM and diagonal solve)",
            "peak_source": "FP64 DFMA stream measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
            "algorithmic_flops_per_launch": 2.0 * gemm_fma / max(kl[3], 1),
            "avg_launch_ms": gemm_ms / max(kl[3], 1)}
    whole = 2.0 * n * n * S / (ms_per_step * 1e-3) / 1e12
    out = dict(value=value, ms_per_step=ms_per_step, roofline=roof, clocks=clk.summary(),
               gpu_launches=int(launches), fp64_peak_gflops={"dfma": dfma, "dmma": dmma},
               kernel_ms_per_step={k: float(v) / args.steps for k, v in zip(_lib.KERNEL_CLASSES, kms)},
               whole_solve_tflops_2n2S=whole, whole_solve_frac=whole / peak,
               check={"max_residual_256cols": float(np.max(res)), "residual_bound_10n_eps": 10 * n * 2.0 ** -52,
                      "finite": finite,
                      "rc": rcs[-1] if rcs else None})

    # e2e through the drop-in C entry point with pinned host buffers
    if not args.no_e2e:
        Hp = torch.from_numpy(np.asfortranarray(H).ravel(order="F")).pin_memory()
        Xp = torch.empty(n * S, dtype=torch.float64).pin_memory()
        w0 = np.ascontiguousarray(wr)
        wp = torch.empty(S, dtype=torch.float64).pin_memory()
        lib.tiled_inverse_iteration.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                C.c_int, C.c_int, C.c_void_p, C.c_int]

        def e2e_step():
            wp.numpy()[:] = w0
            lib.tiled_inverse_iteration(n, Hp.data_ptr(), n, S, wp.data_ptr(), args.tlsz, args.rhs_tlsz,
                                        Xp.data_ptr(), n)
            if lib.hsr_last_status() < 0:
                raise RuntimeError("drop-in call failed")
        e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / args.steps
        if world > 1:
            import torch.distributed as dist
            tt = torch.tensor([te], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        lib.hsr_set_kernel_timing(1)
        e2e_step()
        torch.cuda.synchronize()
        ms8 = (C.c_double * len(_lib.KERNEL_CLASSES))()
        lib.hsr_last_kernel_times(ms8, None, None)
        lib.hsr_set_kernel_timing(0)
        out["e2e"] = {"value": world * S / te, "unit": UNIT, "h2d_bytes_per_step": 8 * (n * n + S),
                      "kernel_ms_one_step": {k: round(ms8[i], 2) for i, k in enumerate(_lib.KERNEL_CLASSES)},
                      "d2h_bytes_per_step": 8 * (n * S + S), "ms_per_step": te * 1e3,
                      "api": "tiled_inverse_iteration (C ABI, pinned host buffers)"}
    return out


SMALL_N = 1000
SMALL_STEPS = 50
SMALL_TLSZ = 0          # 0: the plain-path autotuner's choice


def run_plain_small(args, tlsz: int):
    """The plain small workload: one H of order 1000 from the same generator
    (seed 1234), all 1000 eigenvalues with relative 1e-12 noise as shifts.
    Its inputs and workspaces fit in L2, so a 512 MB buffer is written
    between timed steps and every step is timed alone with CUDA events on the
    launching stream.  value: device-resident (hsr_inverse_iteration_device);
    e2e: the drop-in tiled_inverse_iteration with pinned host buffers, each
    step after the same flush; the same-run CPU time of the oracle port on all
    host cores over all 1000 shifts; perturbation counts of the device and of
    the reference arithmetic (oracle "ref", bit-identical to the reference) at
    the same tiling."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    lib = hsr.load(build_if_missing=True)
    n = SMALL_N
    H, wr = workload(n, args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ldh = n + (n & 1)
    dHt = torch.zeros((n, ldh), dtype=torch.float64, device=dev)
    dHt[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr0 = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    dwr = dwr0.clone()
    dX = torch.empty((n, ldh), dtype=torch.float64, device=dev)
    flush = torch.empty(64 << 20, dtype=torch.float64, device=dev)     # 512 MB > L2
    stream = torch.cuda.Stream(device=dev)
    opt = _lib.Options(0, 0, -1, 0.0)
    steps = max(args.steps, SMALL_STEPS)
    # Tile size: the plain-path autotuner on this problem (outside the timed
    # region); its measured alternatives go into the line.
    cands = (48, 64, 96, 128, 160, 200)
    with torch.cuda.stream(stream):
        tuned, tune_ms, tuned_sc, sc_ms, tuned_fused, fused_ms = hsr.autotune_plain(
            dHt, dwr, dX, candidates=cands, stream=stream, detail=True)
    torch.cuda.synchronize()
    if tlsz == 0:
        tlsz = tuned

    def step():
        rc = lib.hsr_inverse_iteration_device(n, dHt.data_ptr(), ldh, n, dwr.data_ptr(), tlsz, dX.data_ptr(), ldh,
                                              C.byref(opt), C.c_void_p(stream.cuda_stream), None, None)
        if rc < 0:
            raise RuntimeError("device call failed: %d" % rc)

    ncls = len(_lib.KERNEL_CLASSES)
    kms = np.zeros(ncls)
    times = []
    launches = 0
    with ClockSampler(0) as clk:
        with torch.cuda.stream(stream):
            for it in range(args.warmup + steps):
                dwr.copy_(dwr0)
                flush.fill_(float(it))
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step()
                e1.record(stream)
                torch.cuda.synchronize()
                if it >= args.warmup:
                    times.append(e0.elapsed_time(e1))
                    launches += lib.hsr_last_launch_count()
            # one more pass with per-kernel-class timing (not part of the value)
            lib.hsr_set_kernel_timing(1)
            dwr.copy_(dwr0)
            flush.fill_(0.0)
            step()
            torch.cuda.synchronize()
            ms = (C.c_double * ncls)()
            lib.hsr_last_kernel_times(ms, None, None)
            kms = np.array(ms[:])
            lib.hsr_set_kernel_timing(0)
    ms_step = float(np.mean(times))
    dfma, _ = hsr.fp64_peak(100.0)
    peak = dfma / 1e3
    whole = 2.0 * n * n * n / (ms_step * 1e-3) / 1e12
    out = {"value": n / (ms_step / 1e3), "unit": UNIT, "ms_per_step": ms_step,
           "ms_min": float(np.min(times)), "steps": steps, "warmup": args.warmup,
           "whole_solve_tflops_2n2S": whole,
           "roofline": {"bound": "fp64", "achieved": whole, "peak": peak, "unit": "TFLOP/s", "frac": whole / peak,
                        "kernel": "whole solve (2 n^2 S algorithmic flops over the solve's wall time; at this "
                                  "order the sequential diagonal chain, not one kernel, sets the time)",
                        "peak_source": "FP64 DFMA stream measured in this run"},
           "kernel_ms_one_step": {k: round(float(v), 3) for k, v in zip(_lib.KERNEL_CLASSES, kms)},
           "autotune": {"candidates": list(cands), "ms": [round(x, 3) for x in tune_ms], "best": tuned,
                        "shifts_per_cta": {"candidates": [8, 16, 32], "ms": [round(x, 3) for x in sc_ms],
                                           "best": tuned_sc},
                        "top_gemm": {"candidates": ["separate launch", "inside the diagonal CTAs"],
                                     "ms": [round(x, 3) for x in fused_ms],
                                     "best": "inside the diagonal CTAs" if tuned_fused else "separate launch"},
                        "api": "hsr_autotune_plain"},
           "gpu_launches_per_step": launches / steps, "clocks": clk.summary()}
    # e2e through the drop-in entry point, pinned host buffers, flush between steps
    Hp = torch.from_numpy(np.asfortranarray(H).ravel(order="F")).pin_memory()
    Xp = torch.empty(n * n, dtype=torch.float64).pin_memory()
    wp = torch.empty(n, dtype=torch.float64).pin_memory()
    w0 = np.ascontiguousarray(wr)
    lib.tiled_inverse_iteration.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                            C.c_int, C.c_int, C.c_void_p, C.c_int]
    te = []
    for it in range(args.warmup + steps):
        wp.numpy()[:] = w0
        flush.fill_(float(it))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lib.tiled_inverse_iteration(n, Hp.data_ptr(), n, n, wp.data_ptr(), tlsz, args.rhs_tlsz, Xp.data_ptr(), n)
        te.append(time.perf_counter() - t0)
        if lib.hsr_last_status() < 0:
            raise RuntimeError("drop-in call failed")
    te = float(np.mean(te[args.warmup:]))
    out["e2e"] = {"value": n / te, "unit": UNIT, "ms_per_step": te * 1e3, "h2d_bytes_per_step": 8 * (n * n + n),
                  "d2h_bytes_per_step": 8 * (n * n + n), "api": "tiled_inverse_iteration (C ABI, pinned host buffers)"}
    info = hsr.inverse_iteration(H, wr, tlsz, args.rhs_tlsz, scaling="double")
    dXc = torch.from_numpy(np.ascontiguousarray(info["vr"].T)).to(dev)
    res = hsr.residuals_device(dHt, torch.from_numpy(info["wr"]).to(dev), dXc).cpu().numpy()
    out["check"] = {"max_residual_all_columns": float(np.max(res)), "residual_bound_10n_eps": 10 * n * 2.0 ** -52,
                    "perturbed_columns_device": int(np.sum(info["perturbed"])), "converged": int(np.sum(info["status"]))}
    if not args.no_cpu_baseline:
        v, t, c = cpu_sample(H, wr, tlsz, args.rhs_tlsz, n, 5, 1)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": c, "kind": "port",
                               "sample": "n=%d, all %d shifts, mean of 5 solves (%.3f s each), tlsz=%d, rhs_tlsz=%d"
                                         % (n, n, t, tlsz, args.rhs_tlsz),
                               "perturbed_columns_reference_arithmetic": reference_perturbations(
                                   H, wr, tlsz, args.rhs_tlsz, args.seed)}
    out["config"] = {"workload": "plain small: n=%d, %d real shifts (eigenvalues, rel. 1e-12 noise), tlsz=%d"
                                 % (n, n, tlsz), "n": n, "nrhs": n, "tlsz": tlsz, "rhs_tlsz": args.rhs_tlsz,
                     "seed": args.seed, "l2": "inputs fit in L2: a 512 MB buffer is written between timed steps"}
    return out


def reference_perturbations(H, wr, tlsz, rhs_tlsz, seed):
    """Columns whose 1x1 solves the reference arithmetic perturbs (the oracle's
    "ref" build, bit-identical to the unmodified reference) at this tiling;
    part of the CPU-baseline leg, computed once per host and cached."""
    from oracle import pyoracle as O
    n, S = H.shape[0], len(wr)
    d = os.path.join(tempfile.gettempdir(), "hsrq3in_bench")
    os.makedirs(d, exist_ok=True)
    f = os.path.join(d, "ref_pert_n%d_S%d_s%d_t%d_r%d_v1.txt" % (n, S, seed, tlsz, rhs_tlsz))
    if os.path.exists(f):
        return int(open(f).read())
    O.set_threads(os.cpu_count() or 1, "ref")
    r = O.oracle_inverse_iteration(H, wr, tlsz, rhs_tlsz, variant="ref")
    cnt = int(np.sum(r["perturbed"]))
    with open(f, "w") as fh:
        fh.write(str(cnt))
    return cnt


def run_batched(args):
    """Config 4: independent problems of mixed order in one graph launch."""
    import torch
    import hsrq3in_gb300 as hsr
    probs = mixed_problems(args.problems, 32, 1024, 0.25, 1.0, args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    tens = []
    for H, wr in probs:
        n = H.shape[0]
        ld = n + (n & 1)
        dH = torch.zeros((n, ld), dtype=torch.float64, device=dev)
        dH[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
        dwr = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
        dvr = torch.empty((len(wr), ld), dtype=torch.float64, device=dev)
        tens.append((dH, dwr, dvr))
    stream = torch.cuda.Stream(device=dev)
    tune = None
    if args.batch_tlsz == 0:
        rng = np.random.default_rng(5)
        sample = [tens[i] for i in rng.choice(len(tens), size=min(512, len(tens)), replace=False)]
        best, ms = hsr.autotune_batch(sample, candidates=(32, 48, 64, 96), stream=stream)
        tune = {"candidates": [32, 48, 64, 96], "ms": ms, "best": best}
    plan = hsr.BatchPlan(tens, tlsz=args.batch_tlsz, stream=stream)
    info = plan.info()
    for _ in range(args.warmup):
        plan.execute()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            plan.execute()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    total_shifts = sum(len(wr) for _, wr in probs)
    flops = sum(2.0 * H.shape[0] ** 2 * len(wr) for H, wr in probs)
    peak = hsr.fp64_peak(200.0)[0] / 1e3
    # Looping the plain device path over a sample of the same problems.
    rng = np.random.default_rng(11)
    idx = rng.choice(len(tens), size=min(256, len(tens)), replace=False)
    tl = info["tlsz"]
    for i in idx[:4]:
        hsr.inverse_iteration_device(tens[i][0], tens[i][1], tens[i][2], tl, stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in idx:
        dH, dwr, dvr = tens[i]
        hsr.inverse_iteration_device(dH, dwr, dvr, tl, stream=stream)
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t0
    loop_rate = sum(len(probs[i][1]) for i in idx) / loop_s
    # spot check: the batch's result for a few problems against their lone solve
    plan.execute()
    torch.cuda.synchronize()
    ok = True
    for i in idx[:8]:
        H, wr = probs[i]
        alone = hsr.inverse_iteration(H, wr, tl, 16)
        got = tens[i][2][:, :H.shape[0]].cpu().numpy().T
        ok = ok and bool(np.array_equal(got, alone["vr"]))
    value = total_shifts / (ms / 1e3)
    cpu = None
    if not args.no_cpu_baseline:
        # The reference looped over the problems (CPU port, all host cores),
        # over a seeded sample of them within a bounded time.
        from oracle import pyoracle as O
        cores = os.cpu_count() or 1
        O.set_threads(cores, variant="ref_fast")
        order = np.random.default_rng(13).permutation(len(probs))
        busy, shifts, cnt = 0.0, 0, 0
        for i in order:
            if busy > 15.0:
                break
            H, wr = probs[i]
            t0 = time.perf_counter()
            O.oracle_inverse_iteration(H, wr, tl, 64, variant="ref_fast")
            busy += time.perf_counter() - t0
            shifts += len(wr)
            cnt += 1
        cpu = {"value": shifts / busy, "unit": "eigenvectors/s", "cores": cores, "kind": "port",
               "sample": "%d of the %d problems (seeded sample), one after another, tlsz %d, rhs_tlsz 64, %.1f s"
                         % (cnt, len(probs), tl, busy)}
    return {"metric": "FP64 eigenvectors/s, batched mixed-size problems", "value": value,
            "unit": "eigenvectors/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "batched: %d problems, n log-uniform [32,1024], shift fraction U[0.25,1], "
                                   "one CUDA-graph launch per step" % len(probs),
                       "problems": len(probs), "total_shifts": total_shifts, "tlsz": tl,
                       "ticks": info["ticks"], "graph_launches": info["launches"], "autotune": tune},
            "solves_per_s": len(probs) / (ms / 1e3),
            "whole_tflops_2n2S": flops / (ms / 1e3) / 1e12, "frac_of_fp64_peak": flops / (ms / 1e3) / 1e12 / peak,
            "plain_loop": {"eigenvectors_per_s": loop_rate, "sample_problems": int(len(idx)),
                           "speedup_batched_over_loop": value / loop_rate},
            "check": {"bitwise_equal_to_lone_solve_8_problems": ok},
            "cpu_baseline": cpu,
            "clocks": clk.summary()}


def device_pool(count: int, nlo: int, nhi: int, seed: int):
    """count distinct matrices of the real-spectrum generator, n log-uniform in
    [nlo, nhi], generated on the GPU: T (jittered-grid diagonal, N(0,1) above)
    drawn per matrix, A = P T P with P the Householder reflector mapping e1 to
    a random unit vector, and A reduced to Hessenberg form by the library's
    own hsr_hessenberg_device.  Returns [(H host Fortran array, eigenvalues)]
    and the generation time in seconds."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import generators as G
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(np.log(nlo), np.log(nhi), count))).astype(int)
    t0 = time.perf_counter()
    out = []
    for i, n in enumerate(ns):
        n = int(n)
        r = np.random.default_rng(seed * 1000003 + i)
        lam = G.jittered_eigenvalues(n, r)
        g = torch.Generator(device=dev)
        g.manual_seed(int(seed * 1000003 + i))
        Tt = torch.triu(torch.randn((n, n), dtype=torch.float64, device=dev, generator=g), 1).T.contiguous()
        Tt.diagonal().copy_(torch.from_numpy(lam).to(dev))       # Tt[c, r] = T[r, c]
        q = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
        q /= torch.linalg.norm(q)
        w = -q
        w[0] += 1.0
        w /= torch.linalg.norm(w)
        T = Tt.T
        Tw = T @ w
        wT = Tt @ w
        c = torch.dot(w, Tw)
        A = T - 2.0 * torch.outer(w, wT) - 2.0 * torch.outer(Tw, w) + 4.0 * c * torch.outer(w, w)
        ld = n + (n & 1)
        dA = torch.zeros((n, ld), dtype=torch.float64, device=dev)
        dA[:, :n] = A.T
        del A, T, Tt
        hsr.hessenberg_device(dA)
        keep = torch.tril(torch.ones((n, n), dtype=torch.bool, device=dev), diagonal=1)   # rows r <= c+1
        Ht = torch.where(keep, dA[:, :n], torch.zeros((), dtype=torch.float64, device=dev))
        out.append((np.asfortranarray(Ht.T.cpu().numpy()), lam))
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def served_trace(args, base, nreq, rate, seed):
    """Requests with Poisson arrivals at `rate` per second (rate 0: all at
    t=0).  Request i draws, from its own seed (seed, i), one of the generated
    matrices and a random 10-100% subset of its eigenvalues as shifts, with
    relative 1e-12 noise."""
    rng = np.random.default_rng(seed)
    if rate > 0:
        arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
        arrivals -= arrivals[0]
    else:
        arrivals = np.zeros(nreq)
    reqs = []
    for i in range(nreq):
        r = np.random.default_rng([seed, i])
        j = int(r.integers(len(base)))
        H, lam = base[j]
        n = H.shape[0]
        m = max(1, int(round(n * r.uniform(0.1, 1.0))))
        wr = np.sort(r.choice(lam, size=m, replace=False))
        wr = wr * (1.0 + 1e-12 * r.standard_normal(m))
        reqs.append((j, n, wr, float(arrivals[i])))
    return reqs


SHARED_OUTPUT_ABOVE = 2000   # requests; beyond this, outputs on one matrix share a host buffer


def replay_served(base, reqs, tl, budget_gb):
    """Replay a trace through the request loop; pinned host buffers.  Traces
    longer than SHARED_OUTPUT_ABOVE requests give all requests on one matrix
    the same output buffer (n x n per matrix), which bounds the pinned host
    memory; their results are then not kept."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    lib = hsr.load()
    Hp = [torch.from_numpy(np.asfortranarray(H).ravel(order="F")).pin_memory() for H, _ in base]
    total = sum(len(wr) for _, _, wr, _ in reqs)
    shared = len(reqs) > SHARED_OUTPUT_ABOVE
    if shared:
        outs_j = [torch.empty(H.shape[0] * H.shape[0], dtype=torch.float64).pin_memory() for H, _ in base]
    else:
        outs = torch.empty(sum(n * len(wr) for _, n, wr, _ in reqs), dtype=torch.float64).pin_memory()
    wrs = torch.empty(total, dtype=torch.float64).pin_memory()
    arr = (_lib.Request * len(reqs))()
    o = w = 0
    for i, (j, n, wr, t) in enumerate(reqs):
        wrs.numpy()[w:w + len(wr)] = wr
        optr = outs_j[j].data_ptr() if shared else outs.data_ptr() + 8 * o
        arr[i] = _lib.Request(n, Hp[j].data_ptr(), n, len(wr), wrs.data_ptr() + 8 * w, optr, n, t)
        o += n * len(wr)
        w += len(wr)
    srv = hsr.Server(hbm_budget_bytes=budget_gb * 1e9, tlsz=tl)
    lat = (C.c_double * len(reqs))()
    st = (C.c_int * len(reqs))()
    stats = _lib.ServerStats()
    rc = lib.hsr_server_replay(srv._h, len(reqs), arr, lat, st, C.byref(stats))
    srv.close()
    if rc < 0:
        raise RuntimeError("server replay failed: %d" % rc)
    lat = np.array(lat[:])
    return {"requests": len(reqs), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "eigenvectors_per_s": total / stats.wall_s, "wall_s": stats.wall_s, "ticks": stats.ticks,
            "launches": stats.launches, "max_active": stats.max_active, "peak_pool_gb": stats.peak_bytes / 1e9,
            "tflops_2n2S": stats.flops / stats.wall_s / 1e12,
            "phase_ms": {k: round(stats.phase_ms[i], 2) for i, k in enumerate(_lib.SERVER_PHASES)}}


def plain_served(base, reqs, tl, limit_s=12.0):
    """The plain path, one request at a time in arrival order, through the
    drop-in entry point; stops after limit_s."""
    import hsrq3in_gb300 as hsr
    t0 = time.perf_counter()
    lat, shifts, k = [], 0, 0
    for (j, n, wr, t) in reqs:
        now = time.perf_counter() - t0
        if now > limit_s:
            break
        if now < t:
            time.sleep(t - now)
        hsr.inverse_iteration(base[j][0], wr, tl, 64)
        lat.append(time.perf_counter() - t0 - t)
        shifts += len(wr)
        k += 1
    wall = time.perf_counter() - t0
    return {"requests": k, "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "eigenvectors_per_s": shifts / wall}


def cpu_served(base, reqs, tl, limit_s=20.0):
    """The CPU baseline of the served trace: the oracle port (reference
    arithmetic, all host cores) solving one request at a time in arrival
    order on the same trace, latency including queueing, over the requests it
    reaches in limit_s seconds of its own service time."""
    from oracle import pyoracle as O
    cores = os.cpu_count() or 1
    O.set_threads(cores, variant="ref_fast")
    clock = 0.0
    lat, shifts, busy = [], 0, 0.0
    for (j, n, wr, t) in reqs:
        if busy > limit_s:
            break
        start = max(clock, t)
        t0 = time.perf_counter()
        O.oracle_inverse_iteration(base[j][0], wr, tl, 64, variant="ref_fast")
        dt = time.perf_counter() - t0
        busy += dt
        clock = start + dt
        lat.append(clock - t)
        shifts += len(wr)
    return {"requests": len(lat), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "eigenvectors_per_s": shifts / busy, "cores": cores, "kind": "port",
            "sample": "the first %d requests of the trace in arrival order (%.1f s of service time)"
                      % (len(lat), busy)}


def run_served(args):
    """The served workload: a Poisson trace of `requests` requests through
    the request loop (latency at the configured rate) and the first
    `saturate` of them arriving at once (capacity); each against the plain
    device path run per request and the CPU port per request."""
    base, gen_s = device_pool(args.pool, 64, 4096, args.seed + 1)
    tl = args.batch_tlsz or 64
    with ClockSampler(0) as clk:
        paced = served_trace(args, base, args.requests, args.rate, args.seed + 2)
        r_paced = replay_served(base, paced, tl, args.budget_gb)
        burst = [(j, n, wr, 0.0) for (j, n, wr, _) in paced[:args.saturate]]
        r_burst = replay_served(base, burst, tl, args.budget_gb)
    p_paced = plain_served(base, paced, tl)
    p_burst = plain_served(base, burst, tl)
    out = {"paced": {"rate_per_s": args.rate, "server": r_paced, "plain_per_request": p_paced},
           "saturated": {"server": r_burst, "plain_per_request": p_burst,
                         "speedup_server_over_plain": r_burst["eigenvectors_per_s"] / p_burst["eigenvectors_per_s"]},
           "config": "%d requests (Poisson, %.0f/s), each seeded per request: n log-uniform [64,4096] through one "
                     "of %d matrices generated on the device (hsr_hessenberg_device, %.1f s), a U[0.1,1] fraction "
                     "of its eigenvalues with rel. 1e-12 noise; HBM budget %.0f GB, tlsz %d; capacity from the first "
                     "%d requests arriving at once%s" % (
                         args.requests, args.rate, len(base), gen_s, args.budget_gb, tl, len(burst),
                         "; outputs on one matrix share a host buffer" if args.requests > SHARED_OUTPUT_ABOVE
                         else ""),
           "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        out["paced"]["cpu_baseline_per_request"] = cpu_served(base, paced, tl)
    return out


def run_stress(args):
    """Config 3: the robustness-stress problem (n = 5000, 50 clusters of width
    1e-13, strictly-upper columns scaled by 10^U[0,150], shifts equal to the
    eigenvalues), device-resident, all n shifts: eigenvectors/s, and the
    checks -- finiteness, device residuals of every column, perturbation and
    scaling statistics from the extended entry point."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    n = args.stress_order
    H, lam = stress_workload(n, args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ld = n + (n & 1)
    dHt = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dHt[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr0 = torch.from_numpy(np.ascontiguousarray(lam)).to(dev)
    dwr = dwr0.clone()
    dX = torch.empty((n, ld), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            dwr.copy_(dwr0)
            hsr.inverse_iteration_device(dHt, dwr, dX, args.tlsz, stream=stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(stream)
            rcs = []
            for _ in range(args.steps):
                dwr.copy_(dwr0)
                rcs.append(hsr.inverse_iteration_device(dHt, dwr, dX, args.tlsz, stream=stream))
            e1.record(stream)
            torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # Device residual validation of every column (hsr_residuals_device),
    # timed: about n^2/2 FMAs per column over the Hessenberg part.
    with torch.cuda.stream(stream):
        hsr.residuals_device(dHt, dwr, dX, stream=stream)
        r0 = torch.cuda.Event(enable_timing=True)
        r1 = torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        res_d = hsr.residuals_device(dHt, dwr, dX, stream=stream)
        r1.record(stream)
        torch.cuda.synchronize()
    res_ms = r0.elapsed_time(r1)
    res = res_d.cpu().numpy()
    finite = bool(torch.isfinite(dX[:, :n]).all().item())
    info = hsr.inverse_iteration(H, lam, args.tlsz, args.rhs_tlsz)
    scale = info["scale"]
    return {"value": n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "whole_tflops_2n2S": 2.0 * n * n * n / (ms / 1e3) / 1e12,
            "check": {"finite": finite, "max_residual_all_columns": float(np.max(res)),
                      "residual_bound_10n_eps": 10 * n * 2.0 ** -52, "rc": rcs[-1] if rcs else None,
                      "perturbed_columns": int(np.sum(info["perturbed"])),
                      "rescaled_columns": int(np.sum(scale != 0.0)),
                      "min_scale_exponent": float(np.min(scale)),
                      "converged_columns": int(np.sum(info["status"]))},
            "residual_validation": {"columns": n, "ms": res_ms,
                                    "tflops": 2.0 * (n * (n + 1) / 2.0 + n) * n / (res_ms / 1e3) / 1e12,
                                    "api": "hsr_residuals_device"},
            "config": {"workload": "stress: n=%d, 50 clusters of width 1e-13, strictly-upper columns scaled by "
                                   "10^U[0,150], shifts = eigenvalues, tlsz=%d" % (n, args.tlsz),
                       "n": n, "nrhs": n, "tlsz": args.tlsz, "seed": args.seed},
            "clocks": clk.summary()}


def complex_workload(n: int, seed: int):
    """Complex-spectrum problem (H, eigenvalues with positive imaginary part),
    cached like workload()."""
    from hsrq3in_gb300 import generators as G
    d = os.path.join(tempfile.gettempdir(), "hsrq3in_bench")
    os.makedirs(d, exist_ok=True)
    f = os.path.join(d, "cplx_n%d_s%d_v1.npz" % (n, seed))
    if os.path.exists(f):
        z = np.load(f)
        return np.asfortranarray(z["H"]), z["pairs"]
    H, pairs, _ = G.complex_spectrum(n, seed)
    tmp = f + ".%d.tmp.npz" % os.getpid()
    np.savez(tmp, H=H, pairs=pairs)
    os.replace(tmp, f)
    return H, pairs


def run_complex(args):
    """Complex-conjugate shifts: H of order n with n/2 conjugate pairs (2x2
    blocks a +- ib, a on a jittered grid in [-1,1], b in [0.1,1], N(0,1) above
    the blocks), every pair's eigenvalue with positive imaginary part as a
    shift.  Each pair gives two eigenvectors (mu and its conjugate), stored as
    two real columns, so eigenvectors/s counts columns.  value: device-resident
    (hsr_inverse_iteration_cplx_device); e2e: hsr_inverse_iteration_cplx_ex with
    pinned host buffers; roofline of the complex GEMM launches; residuals of
    128 sampled pairs; the oracle port's complex path on the host cores."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    lib = hsr.load(build_if_missing=True)
    n = args.order
    H, pairs = complex_workload(n, args.seed)
    npairs = pairs.size
    S = 2 * npairs
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ld = n + (n & 1)
    dHt = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dHt[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr = torch.from_numpy(np.ascontiguousarray(pairs.real)).to(dev)
    dwi = torch.from_numpy(np.ascontiguousarray(pairs.imag)).to(dev)
    dX = torch.empty((S, ld), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    opt = _lib.Options(0, 0, -1, 0.0)

    def step():
        rc = lib.hsr_inverse_iteration_cplx_device(n, dHt.data_ptr(), ld, npairs, dwr.data_ptr(), dwi.data_ptr(),
                                                   args.tlsz, dX.data_ptr(), ld, C.byref(opt),
                                                   C.c_void_p(stream.cuda_stream), None, None)
        if rc < 0:
            raise RuntimeError("complex device call failed: %d" % rc)
        return rc

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    dfma, _ = hsr.fp64_peak(200.0)
    lib.hsr_set_kernel_timing(1)
    ncls = len(_lib.KERNEL_CLASSES)
    kms = np.zeros(ncls)
    kl = np.zeros(ncls, dtype=np.int64)
    gemm_fma = 0.0
    launches = 0
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    rcs = []
    with ClockSampler(0) as clk:
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.steps):
                rcs.append(step())
                ms = (C.c_double * ncls)()
                ln = (C.c_long * ncls)()
                fm = C.c_double()
                lib.hsr_last_kernel_times(ms, ln, C.byref(fm))
                kms += np.array(ms[:])
                kl += np.array(ln[:])
                gemm_fma += fm.value
                launches += lib.hsr_last_launch_count()
            e1.record(stream)
        torch.cuda.synchronize()
    lib.hsr_set_kernel_timing(0)
    ms_step = e0.elapsed_time(e1) / args.steps
    finite = bool(torch.isfinite(dX[:, :n]).all().item())
    # residuals ||H x - mu x|| / (||H||_F ||x||) of 128 sampled pairs (torch, FP64)
    idx = np.linspace(0, npairs - 1, 128).astype(np.int64)
    Xr = dX[2 * idx, :n].T
    Xi = dX[2 * idx + 1, :n].T
    Hm = dHt[:, :n].T
    a = dwr[idx][None, :]
    b = dwi[idx][None, :]
    Rr = Hm @ Xr - (a * Xr - b * Xi)
    Ri = Hm @ Xi - (a * Xi + b * Xr)
    num = torch.sqrt((Rr * Rr + Ri * Ri).sum(0))
    den = torch.linalg.norm(Hm) * torch.sqrt((Xr * Xr + Xi * Xi).sum(0))
    res = (num / den).cpu().numpy()
    gemm_ms = kms[3]
    achieved = 2.0 * gemm_fma / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    peak = dfma / 1e3
    out = {"value": S / (ms_step / 1e3), "unit": UNIT, "ms_per_step": ms_step,
           "pairs_per_s": npairs / (ms_step / 1e3),
           "whole_tflops_2n2S": 2.0 * n * n * S / (ms_step / 1e3) / 1e12,
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": (achieved / peak) if achieved else None,
                        "kernel": "k_gemm_c (the real GEMM over H with the complex epilogue; launches over the "
                                  "rows above the next diagonal tile)",
                        "peak_source": "FP64 DFMA stream measured in this run",
                        "avg_launch_ms": gemm_ms / max(kl[3], 1)},
           "kernel_ms_per_step": {k: float(v) / args.steps for k, v in zip(_lib.KERNEL_CLASSES, kms)},
           "gpu_launches": int(launches), "clocks": clk.summary(),
           "check": {"finite": finite, "max_residual_128_pairs": float(np.max(res)),
                     "residual_bound_10n_eps": 10 * n * 2.0 ** -52, "rc": rcs[-1] if rcs else None},
           "config": {"workload": "complex: n=%d, %d conjugate pairs (2 eigenvectors each), tlsz=%d"
                                  % (n, npairs, args.tlsz),
                      "n": n, "pairs": npairs, "tlsz": args.tlsz, "seed": args.seed,
                      "generator": "T quasi-triangular, 2x2 blocks a+-ib (a jittered grid in [-1,1], b in "
                                   "[0.1,1]), N(0,1) above the blocks; H = hess(Q T Q^T)",
                      "l2": "inputs larger than L2 (H is %.0f MB); no flush" % (8 * n * n / 1e6)}}
    if not args.no_e2e:
        Hp = torch.from_numpy(np.asfortranarray(H).ravel(order="F")).pin_memory()
        Xp = torch.empty(n * S, dtype=torch.float64).pin_memory()
        wrh = np.ascontiguousarray(pairs.real)
        wih = np.ascontiguousarray(pairs.imag)

        def e2e_step():
            rc = lib.hsr_inverse_iteration_cplx_ex(n, Hp.data_ptr(), n, npairs, wrh.ctypes.data, wih.ctypes.data,
                                                   args.tlsz, args.rhs_tlsz, Xp.data_ptr(), n, C.byref(opt), None)
            if rc < 0:
                raise RuntimeError("complex host call failed: %d" % rc)
        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        te = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": S / te, "unit": UNIT, "ms_per_step": te * 1e3,
                      "h2d_bytes_per_step": 8 * (n * n + 2 * npairs), "d2h_bytes_per_step": 8 * n * S,
                      "api": "hsr_inverse_iteration_cplx_ex (C ABI, pinned host buffers)"}
    if not args.no_cpu_baseline:
        from oracle import pyoracle as O
        cores = os.cpu_count() or 1
        O.set_threads(cores, variant="ref_fast")
        sample = min(npairs, args.cpu_sample or 32 * cores)
        t0 = time.perf_counter()
        O.oracle_inverse_iteration_cplx(H, pairs.real[:sample], pairs.imag[:sample], args.tlsz, args.rhs_tlsz,
                                        variant="ref_fast")
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 2 * sample / tc, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "n=%d, first %d of %d pairs, one solve (%.1f s), tlsz=%d; the oracle's "
                                         "complex path (the reference has no complex driver)"
                                         % (n, sample, npairs, tc, args.tlsz)}
    return out


def run_dense(args):
    """Dense input end to end on the device: A = P H0 P (P a random
    Householder reflector, so A is dense with H0's known spectrum), reduced to
    Hessenberg form (hsr_hessenberg_device), all n eigenvectors of H computed
    (hsr_inverse_iteration_device, shifts = eigenvalues with rel. 1e-12
    noise), and back-transformed to eigenvectors of A (hsr_hessenberg_apply_q_
    device).  Each phase timed with CUDA events on the launching stream;
    residuals ||A x - lambda x|| / (||A||_F ||x||) of 64 sampled columns."""
    import torch
    import hsrq3in_gb300 as hsr
    n = args.order
    H0, wr = workload(n, args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ld = n + (n & 1)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 5)
    w = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
    w /= torch.linalg.norm(w)
    Ht = torch.from_numpy(np.ascontiguousarray(H0.T)).to(dev)       # Ht[c, r] = H0[r, c]
    # A = P H0 P with P = I - 2 w w^T; At = A^T in the same row-per-column layout
    Hw = Ht.T @ w
    wH = Ht @ w                                                      # (w^T H0)^T
    c = torch.dot(w, Hw)
    A = Ht.T - 2.0 * torch.outer(w, wH) - 2.0 * torch.outer(Hw, w) + 4.0 * c * torch.outer(w, w)
    A0 = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    A0[:, :n] = A.T
    del A, Hw, wH
    dA = torch.empty_like(A0)
    dH = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dwr0 = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    dwr = dwr0.clone()
    dX = torch.empty((n, ld), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    keep = torch.tril(torch.ones((n, n), dtype=torch.bool, device=dev), diagonal=1)   # rows r <= c+1 of column c
    phases = {"reduce": [], "solve": [], "back_transform": [], "total": []}
    with torch.cuda.stream(stream):
        for it in range(args.warmup + args.steps):
            dA.copy_(A0)
            dwr.copy_(dwr0)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            tau = hsr.hessenberg_device(dA, stream=stream)
            ev[1].record(stream)
            dH[:, :n] = torch.where(keep, dA[:, :n], torch.zeros((), dtype=torch.float64, device=dev))
            hsr.inverse_iteration_device(dH, dwr, dX, args.tlsz, stream=stream)
            ev[2].record(stream)
            hsr.hessenberg_apply_q_device(dA, tau, dX, stream=stream)
            ev[3].record(stream)
            torch.cuda.synchronize()
            if it >= args.warmup:
                phases["reduce"].append(ev[0].elapsed_time(ev[1]))
                phases["solve"].append(ev[1].elapsed_time(ev[2]))
                phases["back_transform"].append(ev[2].elapsed_time(ev[3]))
                phases["total"].append(ev[0].elapsed_time(ev[3]))
    ms = {k: float(np.mean(v)) for k, v in phases.items()}
    idx = torch.from_numpy(np.linspace(0, n - 1, 64).astype(np.int64)).to(dev)
    X = dX[idx, :n].T
    lam = dwr[idx]
    Am = A0[:, :n].T
    res = (torch.linalg.norm(Am @ X - X * lam[None, :], dim=0) /
           (torch.linalg.norm(Am) * torch.linalg.norm(X, dim=0))).cpu().numpy()
    return {"value": n / (ms["total"] / 1e3), "unit": UNIT, "ms_per_step": ms["total"], "phase_ms": ms,
            "tflops_reduce": 10.0 / 3.0 * n ** 3 / (ms["reduce"] / 1e3) / 1e12,
            "tflops_back_transform": 2.0 * n ** 3 / (ms["back_transform"] / 1e3) / 1e12,
            "check": {"max_residual_64_cols": float(np.max(res)), "residual_bound_10n_eps": 10 * n * 2.0 ** -52,
                      "finite": bool(torch.isfinite(dX[:, :n]).all().item())},
            "config": {"workload": "dense: n=%d, A = P H P (P a random Householder reflector), all %d eigenvectors, "
                                   "tlsz=%d" % (n, n, args.tlsz), "n": n, "tlsz": args.tlsz, "seed": args.seed}}


def run_hessenberg(args, host_baseline=True):
    """The input step on the GPU: reduction of a dense n x n matrix to
    upper-Hessenberg form (hsr_hessenberg_device), 10/3 n^3 flops, against
    LAPACK dgehrd (scipy's OpenBLAS, its default of all host cores) at
    min(n, 4096)."""
    import torch
    import hsrq3in_gb300 as hsr
    n = args.order
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed)
    A0 = torch.randn((n, n), dtype=torch.float64, device=dev, generator=g)
    dA = torch.empty_like(A0)
    stream = torch.cuda.Stream(device=dev)
    times = []
    with torch.cuda.stream(stream):
        for it in range(args.warmup + args.steps):
            dA.copy_(A0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tau = hsr.hessenberg_device(dA, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if it >= args.warmup:
                times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    flops = 10.0 / 3.0 * n ** 3
    finite = bool(torch.isfinite(dA).all().item())
    out = {"n": n, "ms": ms, "tflops": flops / (ms / 1e3) / 1e12, "finite": finite, "tau_sample": float(tau[0].item())}
    if not host_baseline:
        return out
    from scipy.linalg import lapack
    nh = min(n, 4096)
    Ah = np.asfortranarray(np.random.default_rng(args.seed).standard_normal((nh, nh)))
    t0 = time.perf_counter()
    lapack.dgehrd(Ah)
    th = time.perf_counter() - t0
    out["host_dgehrd"] = {"n": nh, "s": th, "gflops": 10.0 / 3.0 * nh ** 3 / th / 1e9,
                          "cores": os.cpu_count(), "library": "scipy LAPACK dgehrd (OpenBLAS)"}
    return out


def main():
    args = parse()
    if args.workload == "hessenberg":
        hh = run_hessenberg(args)
        line = {"metric": "Hessenberg reduction time (dense n x n, FP64)", "value": hh["ms"], "unit": "ms",
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": hh["ms"],
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded N(0,1) matrix)", "config": {"workload": "hessenberg: n=%d" % hh["n"]},
                "hessenberg": hh}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "stress":
        st = run_stress(args)
        line = {"metric": "FP64 eigenvectors/s, robustness stress", "value": st["value"], "unit": UNIT,
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": st["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator)", "config": st["config"], "stress": st}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "batched":
        print(json.dumps(run_batched(args)), flush=True)
        return
    if args.workload == "dense":
        de = run_dense(args)
        line = {"metric": "FP64 eigenvectors/s of a dense matrix (reduce + solve + back-transform)",
                "value": de["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": de["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded generator)", "config": de["config"], "dense": de}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "complex":
        cx = run_complex(args)
        line = {"metric": "FP64 eigenvectors/s, complex-conjugate shifts", "value": cx["value"], "unit": UNIT,
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": cx["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator)", "config": cx["config"]}
        for k in ("e2e", "roofline", "clocks", "gpu_launches", "cpu_baseline", "check"):
            if k in cx:
                line[k] = cx[k]
        line["complex"] = {k: cx[k] for k in ("pairs_per_s", "whole_tflops_2n2S", "kernel_ms_per_step")}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "served":
        sv = run_served(args)
        line = {"metric": "served eigenvectors/s with p50/p99 latency",
                "value": sv["saturated"]["server"]["eigenvectors_per_s"], "unit": "eigenvectors/s",
                "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                "config": {"workload": "served: " + sv["config"]}, "served": sv}
        print(json.dumps(line), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if (args.impl == "gb300" and torch.cuda.is_available()) else "gloo"
        dist.init_process_group(backend=backend)
    n = args.order
    S = args.nrhs or n
    sample = args.cpu_sample or S
    config = {"workload": "plain large: n=%d, %d real shifts (eigenvalues, rel. 1e-12 noise), tlsz=%d"
                          % (n, S, args.tlsz),
              "n": n, "nrhs": S, "tlsz": args.tlsz, "rhs_tlsz": args.rhs_tlsz, "seed": args.seed,
              "generator": "T upper triangular, diag jittered-uniform in [-1,1] (gap>=1e-4), strictly-upper "
                           "N(0,1); H = hess(Q T Q^T), Q^T e1 uniform on the sphere",
              "l2": "inputs larger than L2 (H is %.0f MB); no flush" % (8 * n * n / 1e6),
              "parallelism": "replicas" if args.gpus > 1 else "1 gpu"}

    if args.impl == "reference":
        if rank != 0:
            return
        H, wr = workload(n, args.seed)
        v, t, c = cpu_sample(H, wr[:S], args.tlsz, args.rhs_tlsz, sample, args.steps, args.warmup)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)", "config": config,
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": c, "kind": "port",
                                 "sample": "n=%d, %d of %d shifts per step (one whole solve), tlsz=%d, "
                                           "rhs_tlsz=%d; the C restatement of the reference (reference sources "
                                           "are not on this host)" % (n, sample, S, args.tlsz, args.rhs_tlsz)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    H, wr = workload(n, args.seed)
    wr = wr[:S]
    g = run_gpu(args, H, wr, rank, world)
    line = {"metric": METRIC, "value": g["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": g["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": config}
    for k in ("e2e", "roofline", "clocks", "gpu_launches", "fp64_peak_gflops", "kernel_ms_per_step",
              "whole_solve_tflops_2n2S", "whole_solve_frac", "check"):
        if k in g:
            line[k] = g[k]
    if rank == 0 and world == 1 and n == 10000:
        # perturbed columns of the device at this tiling (host call, outside the timed region)
        import hsrq3in_gb300 as hsr
        info = hsr.inverse_iteration(H, wr, args.tlsz, args.rhs_tlsz, scaling="double")
        line["check"]["perturbed_columns_device"] = int(np.sum(info["perturbed"]))
        line["check"]["converged"] = int(np.sum(info["status"]))
        del info
    if rank == 0 and world == 1 and not args.only_plain:
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup = min(args.steps, 5), min(args.warmup, 3)
        line["plain_small"] = run_plain_small(args, SMALL_TLSZ)
        b = run_batched(args)
        line["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "solves_per_s", "whole_tflops_2n2S",
                                              "frac_of_fp64_peak", "plain_loop", "check", "cpu_baseline")}
        line["batched"]["config"] = b["config"]
        sv = run_served(args)
        line["served"] = sv
        line["stress"] = run_stress(sub)
        cx = run_complex(sub)
        line["complex"] = {k: cx[k] for k in ("value", "unit", "ms_per_step", "pairs_per_s", "whole_tflops_2n2S",
                                              "roofline", "e2e", "cpu_baseline", "check", "config", "clocks")
                           if k in cx}
        line["complex"]["steps"], line["complex"]["warmup"] = sub.steps, sub.warmup
        hh = run_hessenberg(sub, host_baseline=False)     # the host LAPACK comparison: --workload hessenberg
        hh["steps"], hh["warmup"] = sub.steps, sub.warmup
        line["hessenberg"] = hh
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, t, c = cpu_sample(H, wr, args.tlsz, args.rhs_tlsz, sample, 1, 0)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": c, "kind": "port",
                                "sample": "n=%d, %d of %d shifts, one solve (%.1f s), tlsz=%d, rhs_tlsz=%d"
                                          % (n, sample, S, t, args.tlsz, args.rhs_tlsz)}
        if sample == S:
            line["cpu_baseline"]["perturbed_columns_reference_arithmetic"] = reference_perturbations(
                H, wr, args.tlsz, args.rhs_tlsz, args.seed)
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
