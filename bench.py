#!/usr/bin/env python3
"""Benchmark of the tiled-Cholesky hot path on GB300.

Workload (one step): FP64 tiled Cholesky of an N x N SPD matrix, tile NB, followed by the solve
of nrhs right-hand sides — N=32768, NB=512, nrhs=1 by default; A = (M+M^T)/2 + N*I with
M ~ U[-0.5, 0.5) from seed 42 (counter-based generator), b ~ N(0,1) from seed 42.

Metric: effective TFLOP/s = (N^3/3) / (factor + solve time), higher is better.
  value  — inputs resident in HBM; per-step CUDA events around factor + solve; the 4.4 GB
           restore of A between steps is outside the events and flushes the 129 MB L2.
  e2e    — the same step through the C ABI with host buffers: pinned H2D of A and b, factor,
           solve, D2H of the factor and x, all inside the events.
  roofline — the persistent flowgraph executor (potrf_dag_f64_kernel) timed alone with events,
           against the measured cuBLAS FP64 GEMM rate of this GPU.
  cpu_baseline — the CPU restatement of the flowgraph with OpenBLAS tile kernels on all host
           cores, on a bounded sample (N=16384).

--impl reference times that CPU restatement (the reference's own PaRSEC build is not available)
on the same metric and the same workload (N=32768 every step, about 27 s per step on 16 cores).
Under torchrun every rank runs an independent replica ("replicas only": the tiled factorisation
of one matrix runs on one GPU; its tiles are not split across GPUs).
"""
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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--N", type=int, default=32768)
    p.add_argument("--NB", type=int, default=512)
    p.add_argument("--nrhs", type=int, default=1)
    p.add_argument("--cpu-N", type=int, default=16384, help="bounded CPU sample size")
    p.add_argument("--fp64-update", choices=["tensor", "fma"], default="tensor",
                   help="trailing updates of the FP64 factor: tensor-core emulation (exact digit-plane "
                        "products, FP64 accumulation) or FP64 FMA block GEMMs")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision configuration")
    p.add_argument("--no-batched", action="store_true", help="skip the batched configuration")
    p.add_argument("--only-main", action="store_true",
                   help="the headline step alone (no e2e, secondary configurations or CPU baseline), e.g. for a "
                        "launch-list capture")
    p.add_argument("--profile-case", choices=["dag", "emu", "mixed", "batched", "refine", "batched_mixed"], default=None,
                   help="run one small case of one kernel (N=8192) for an ncu capture; prints no JSON")
    p.add_argument("--profile-N", type=int, default=8192, help="matrix order of --profile-case dag/mixed")
    return p.parse_args()


def flops_factor(N):
    return N ** 3 / 3.0


class ClockSampler:
    """nvidia-smi clocks/throttle sampling in the background during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
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
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------------------------
def cpu_run(N, NB, reps, nthreads=0):
    """CPU restatement of the flowgraph (oracle) with OpenBLAS tile kernels; returns seconds per rep."""
    import numpy as np
    import oracle
    ok = oracle.load_openblas()
    base = oracle.uniform_sym_tiles(N, NB, 42)
    times = []
    for _ in range(reps):
        t = base.copy()
        t0 = time.perf_counter()
        st, _, _ = oracle.potrf_tiled(t, N, NB, nthreads=nthreads, use_blas=ok)
        b = np.random.default_rng(42).standard_normal(N)
        oracle.potrs_tiled(t, N, NB, b)
        times.append(time.perf_counter() - t0)
        assert st == 0
    return times, ok


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def main_config(args, ws):
    """The workload of a step, the same dictionary in both arms."""
    N, NB, nrhs = args.N, args.NB, args.nrhs
    return {"workload": "potrf+potrs FP64 N=%d NB=%d nrhs=%d" % (N, NB, nrhs), "N": N, "NB": NB,
            "nrhs": nrhs, "generator": "(M+M^T)/2 + N*I, M~U[-0.5,0.5) seed 42",
            "l2": "inputs 4.4 GB > L2; A restored (4.4 GB copy) between timed steps",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args, ws, rank):
    """The reference's CPU potrf (restated flowgraph, OpenBLAS tile kernels, all host cores) on the
    workload of the other arm: every step factorises and solves the full N x N system."""
    if rank != 0:
        return
    N = args.N
    NB = args.NB
    times, blas = cpu_run(N, NB, args.warmup + args.steps)
    t = times[args.warmup:]
    sec = sum(t) / len(t)
    val = flops_factor(N) / sec / 1e12
    cores = cpu_cores()
    line = {
        "impl": "reference", "metric": "cholesky_solve_tflops", "value": val, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": main_config(args, ws),
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": "the whole N=%d NB=%d factor+solve every step, %s tile kernels, %d threads" %
                                   (N, NB, "OpenBLAS" if blas else "plain-loop", cores)},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure_fp64_gemm_peak(dev):
    """cuBLAS FP64 GEMM rate on this GPU (the FP64 counterpart of the driver's bf16 peak)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def run_ours(args, ws, rank, local):
    import ctypes

    import numpy as np
    import torch

    import ttg_gb300 as gbx

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    N, NB, nrhs = args.N, args.NB, args.nrhs
    numel = gbx.tiled_numel(N, NB)
    A0 = torch.empty(numel, dtype=torch.float64, device=dev)
    T = torch.empty_like(A0)
    gbx.gen_uniform_sym(A0, N, NB, seed=42)
    b_host = torch.from_numpy(np.random.default_rng(42).standard_normal((nrhs, N)))
    b0 = b_host.to(dev)
    X = torch.empty_like(b0)
    tensor_update = args.fp64_update == "tensor"
    assert gbx.lib().gbx_set_fp64_update(1 if tensor_update else 0) == 0
    work = torch.empty(gbx.potrf_workspace_bytes(N, NB), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    launches_per_step = 3  # potrf_dag_f64_kernel, then the two persistent solve sweeps (forward, backward)

    def step(events):
        e0, e1, e2 = events
        e0.record()
        gbx.call("gbx_dpotrf_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(work.data_ptr()),
                 work.numel(), sp)
        e1.record()
        gbx.call("gbx_dpotrs_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), nrhs, ctypes.c_void_p(X.data_ptr()), N, sp)
        e2.record()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.warmup + args.steps)]
    for i in range(args.warmup):
        T.copy_(A0)
        X.copy_(b0)
        step(ev[i])
    torch.cuda.synchronize()
    st = gbx.potrf_status(work)
    assert st == 0, st
    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    step_ms, dag_ms = [], []
    for i in range(args.warmup, args.warmup + args.steps):
        T.copy_(A0)  # restore A (4.4 GB): also flushes L2 between timed steps
        X.copy_(b0)
        step(ev[i])
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    for i in range(args.warmup, args.warmup + args.steps):
        e0, e1, e2 = ev[i]
        step_ms.append(e0.elapsed_time(e2))
        dag_ms.append(e0.elapsed_time(e1))
    assert gbx.potrf_status(work) == 0
    ms = max_over_ranks(ws, sum(step_ms) / len(step_ms))
    value = flops_factor(N) / (ms * 1e-3) / 1e12 * ws
    # the same step from host buffers, next to the timed region (after the FMA-form step, the FP64
    # GEMM rate and the backward-error check it measured ~840 ms against ~615 ms run right after the
    # device-resident steps or alone)
    e2e = None if args.no_e2e else run_e2e(gbx, A0, b0, N, NB, nrhs, work, dev, reps=max(1, min(args.steps, 2)))

    # solution quality of the last step (backward error through a matvec with the lower tiles)
    berr = backward_error(gbx, A0, T, X, b0, N, NB, dev)

    line = {
        "metric": "cholesky_solve_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": main_config(args, ws),
        "fp64_update": FP64_UPDATE_NOTE[args.fp64_update],
        "backward_error": berr,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk,
    }

    peak = measure_fp64_gemm_peak(dev)
    bf16_peak, bf16_src = measured_bf16_peak()
    dag_s = statistics.mean(dag_ms) * 1e-3
    achieved = flops_factor(N) / dag_s / 1e12
    if tensor_update:
        line["roofline"] = tensor_roofline(N, NB, dag_s, bf16_peak, bf16_src)
        line["roofline"]["fp64_equivalent"] = {"tflops": achieved, "fp64_gemm_peak": peak,
                                               "ratio": achieved / peak}
        if not args.only_main:  # the same step with FP64 FMA block GEMMs (the former form), once
            line["fma_update"] = run_fma_step(gbx, A0, T, X, b0, N, NB, nrhs, sp, peak)
            assert gbx.lib().gbx_set_fp64_update(1) == 0
    else:
        # DRAM traffic of one launch: ncu capture at N=16384 NB=512 (45.007 GB read + 44.713 GB
        # written), scaled to this N by the number of block tasks (~N^3); N=32768 is too large to capture
        traffic = (45.007e9 + 44.713e9) * (N / 16384.0) ** 3 if NB == 512 else None
        line["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at "
                                              "N=16384 NB=512, scaled by block tasks (N^3)",
                            "kernel": "potrf_dag_f64_kernel<false>",
                            "peak_source": "cuBLAS FP64 GEMM 4096^3 measured in this run (no FP64 entry in the "
                                           "measured-peaks file)"}

    if e2e is not None:
        line["e2e"] = e2e

    if not args.no_mixed:
        del T, A0
        torch.cuda.empty_cache()
        line["mixed"] = run_mixed(gbx, dev)
    if not args.no_batched:
        torch.cuda.empty_cache()
        line["batched"] = run_batched(gbx, dev, reps=max(3, args.steps), cpu=rank == 0 and not args.no_cpu)
    if not args.no_batched:
        torch.cuda.empty_cache()
        line["batched_mixed"] = run_batched_mixed(gbx, dev, cpu=rank == 0 and not args.no_cpu)
    if not args.only_main:
        line["config_small"] = run_config1(gbx, dev, cpu=rank == 0 and not args.no_cpu)
        line["ttg_flowgraph"] = run_ttg_flowgraph(gbx, dev)
        line["potri"] = run_potri(gbx, dev, cpu=rank == 0 and not args.no_cpu)

    if rank == 0 and not args.no_cpu:
        times, blas = cpu_run(args.cpu_N, NB, 2)
        sec = min(times)
        line["cpu_baseline"] = {"value": flops_factor(args.cpu_N) / sec / 1e12, "unit": "TFLOP/s",
                                "cores": cpu_cores(), "kind": "port",
                                "sample": "N=%d NB=%d factor+solve, best of 2, %s tile kernels" %
                                          (args.cpu_N, NB, "OpenBLAS" if blas else "plain-loop")}
    add_roofline_fractions(line, peak, bf16_peak)
    line["peaks"]["bf16_source"] = bf16_src
    if rank == 0:
        print(json.dumps(line), flush=True)


FP64_UPDATE_NOTE = {
    "tensor": "tensor-core emulation: each 128-block of L as 7 bf16 digit planes (8-bit digits, power-of-two "
              "row scales), the 28 plane products of the leading digit groups exact in FP32 on tcgen05, "
              "composed exactly and subtracted from C with one FP64 add; POTRF/TRSM in FP64",
    "fma": "FP64 FMA block GEMMs",
}

# tensor-core work of one emulated GEMM or SYRK task (128 x 128 output, k = 128): two passes of 64
# columns, each 28 plane pairs x 2 chunks x 4 MMAs of 128 x 64 x 16
EMU_TASK_FLOPS = 2 * 28 * 2 * 4 * (2 * 128 * 64 * 16)


def tensor_roofline(N, NB, seconds, bf16_peak, bf16_src):
    """Roofline of the emulated executor: the tensor-core flops its GEMM/SYRK tasks issue per launch
    (EMU_TASK_FLOPS each) over the launch time, against the measured dense bf16 rate. DRAM traffic:
    ncu capture of one launch at N=16384 (EMU_TRAFFIC_16384), scaled by the number of update tasks."""
    ntb = -(-N // 128)
    updates = ntb * (ntb - 1) // 2 + ntb * (ntb - 1) * (ntb - 2) // 6
    flops = updates * EMU_TASK_FLOPS
    achieved = flops / seconds / 1e12
    ntb16 = 128
    upd16 = ntb16 * (ntb16 - 1) // 2 + ntb16 * (ntb16 - 1) * (ntb16 - 2) // 6
    traffic = EMU_TRAFFIC_16384 * updates / upd16 if EMU_TRAFFIC_16384 else None
    return {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": achieved / bf16_peak, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at N=16384 NB=512, "
                              "scaled by the number of update tasks",
            "kernel": "potrf_dag_f64_kernel<true>", "peak_source": bf16_src + " (of measured)",
            "flops_per_launch": flops, "update_tasks": updates}


# bytes per launch (read + write) at N=16384 NB=512: ncu dram__bytes_read.sum 48.017 GB +
# dram__bytes_write.sum 48.069 GB (bench.py --profile-case emu --profile-N 16384, second launch)
EMU_TRAFFIC_16384 = 48.017276160e9 + 48.069112064e9


def run_fma_step(gbx, A0, T, X, b0, N, NB, nrhs, sp, fp64_peak):
    """One factor + solve step of the same system with the FP64 FMA update form (after the timed region)."""
    import ctypes

    import torch
    assert gbx.lib().gbx_set_fp64_update(0) == 0
    work = torch.empty(gbx.potrf_workspace_bytes(N, NB), dtype=torch.uint8, device=T.device)
    T.copy_(A0)
    X.copy_(b0)
    e0, e1, e2 = _events() + (torch.cuda.Event(enable_timing=True),)
    e0.record()
    gbx.call("gbx_dpotrf_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(work.data_ptr()),
             work.numel(), sp)
    e1.record()
    gbx.call("gbx_dpotrs_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), nrhs, ctypes.c_void_p(X.data_ptr()), N, sp)
    e2.record()
    e2.synchronize()
    assert gbx.potrf_status(work) == 0
    ms, dag = e0.elapsed_time(e2), e0.elapsed_time(e1)
    return {"ms_per_step": ms, "tflops": flops_factor(N) / (ms * 1e-3) / 1e12,
            "factor_ms": dag, "factor_frac_of_fp64_peak": flops_factor(N) / (dag * 1e-3) / 1e12 / fp64_peak,
            "kernel": "potrf_dag_f64_kernel<false>"}


def measured_bf16_peak():
    """Dense bf16 tensor-core rate from MEASURED_PEAKS.json (burst), else the fallback figure."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst)"
    except (OSError, ValueError, KeyError, TypeError):
        return 1900.0, "fallback 1.9 PFLOP/s bf16"


def measured_hbm_peak():
    """Copy bandwidth (GB/s) from MEASURED_PEAKS.json, else the fallback figure."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError, TypeError):
        return 6800.0


def add_roofline_fractions(line, fp64_peak, bf16_peak):
    """Adds `frac_of_peak` beside every `tflops` of the secondary configurations: FP64 results against
    the FP64 GEMM rate measured in the run, bf16/fp16 results against the dense bf16 tensor-core
    rate, fp8 against twice it (the nominal fp8:bf16 ratio; no fp8 rate is measured). FP32 results
    (CUDA cores) get none."""
    peaks = {"fp64": fp64_peak, "plain_fp64": fp64_peak, "plain_fp64_per_matrix": fp64_peak, "gpu": fp64_peak,
             "bf16": bf16_peak, "fp16": bf16_peak, "fp8": 2.0 * bf16_peak}
    for sec in ("mixed", "batched", "batched_mixed", "config_small", "potri"):
        part = line.get(sec)
        if not isinstance(part, dict):
            continue
        for key, res in part.items():
            if not isinstance(res, dict) or not isinstance(res.get("tflops"), (int, float)):
                continue
            if key == "tuned":  # the tuner's choice: the peak of its precision
                key = res.get("prec", res.get("mode"))
            if key in peaks:
                res["frac_of_peak"] = res["tflops"] / peaks[key]
    line["peaks"] = {"fp64_tflops": fp64_peak, "bf16_tflops": bf16_peak,
                     "fp8_tflops": 2.0 * bf16_peak, "note": "fp8 = twice the bf16 rate (nominal ratio)"}
    return line


def backward_error(gbx, A0, T, X, b0, N, NB, dev):
    """||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) for the first rhs, with A from its lower tiles."""
    import torch
    nt = gbx.ntiles(N, NB)
    tv = A0.view(-1, NB, NB)
    x = X[0]
    r = b0[0].clone()
    rowsum = torch.zeros(N, dtype=torch.float64, device=dev)
    for n in range(nt):
        for m in range(n, nt):
            s = n * nt - n * (n - 1) // 2 + (m - n)
            blk = tv[s].T  # (rows of tile m) x (cols of tile n)
            rm, rn = min(NB, N - m * NB), min(NB, N - n * NB)
            blk = blk[:rm, :rn]
            if m == n:
                full = torch.tril(blk) + torch.tril(blk, -1).T
                r[m * NB:m * NB + rm] -= full @ x[n * NB:n * NB + rn]
                rowsum[m * NB:m * NB + rm] += full.abs().sum(1)
            else:
                r[m * NB:m * NB + rm] -= blk @ x[n * NB:n * NB + rn]
                r[n * NB:n * NB + rn] -= blk.T @ x[m * NB:m * NB + rm]
                rowsum[m * NB:m * NB + rm] += blk.abs().sum(1)
                rowsum[n * NB:n * NB + rn] += blk.abs().sum(0)
    return (r.abs().max() / (rowsum.max() * x.abs().max() + b0[0].abs().max())).item()


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_mixed(gbx, dev, N=32768, NB=512, nrhs=8, kappa=1e6):
    """Mixed-precision factor + FP64 refinement (tensor-core bf16/fp16 factorisation, CG in FP64) of
    A = H diag(lam) H^T (4 Householder reflectors, kappa = 1e6), 8 right-hand sides, against the
    plain FP64 GPU path (factor + solve) of the same system."""
    import ctypes

    import numpy as np
    import torch

    from ttg_gb300 import workloads
    A = workloads.householder_tiles(N, NB, 4, kappa, 42, dev)
    B = torch.from_numpy(workloads.rhs(N, nrhs, 42)).to(dev)
    out = {"config": {"workload": "potrf+refine N=%d NB=%d nrhs=%d, H diag(lam) H^T, 4 reflectors, kappa=%g"
                                  % (N, NB, nrhs, kappa), "N": N, "NB": NB, "nrhs": nrhs, "kappa": kappa,
                      "tolerance": 1e-14}}
    # plain FP64 GPU path: the reference of the speed-up and of the forward error
    T = A.clone()
    X64 = B.clone()
    work = torch.empty(gbx.potrf_workspace_bytes(N, NB), dtype=torch.uint8, device=dev)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    e0, e1 = _events()
    torch.cuda.synchronize()
    e0.record()
    gbx.call("gbx_dpotrf_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(work.data_ptr()), work.numel(), sp)
    gbx.call("gbx_dpotrs_tiled", N, NB, ctypes.c_void_p(T.data_ptr()), nrhs, ctypes.c_void_p(X64.data_ptr()), N, sp)
    e1.record()
    e1.synchronize()
    assert gbx.potrf_status(work) == 0
    plain_ms = e0.elapsed_time(e1)
    del T, work
    torch.cuda.empty_cache()
    out["plain_fp64"] = {"ms": plain_ms, "tflops": N ** 3 / 3 / (plain_ms * 1e-3) / 1e12}
    for prec in ("bf16", "fp16"):
        W = torch.empty(A.numel(), dtype=torch.float32, device=dev)
        X, info, st = gbx.dposv_mixed(A, N, NB, B, prec=prec, tol=1e-14, maxiter=300, W=W)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        X, info, st = gbx.dposv_mixed(A, N, NB, B, prec=prec, tol=1e-14, maxiter=300, W=W)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        fe = ((X - X64).abs().max() / X64.abs().max()).item()
        # after the timed region: the residual again, from plain FP64 products over the tiles
        be64 = max(gbx.backward_error_fp64(A, N, NB, B, X))
        out[prec] = {"ms": ms, "tflops": N ** 3 / 3 / (ms * 1e-3) / 1e12, "speedup_vs_plain_fp64": plain_ms / ms,
                     "status": st, "iterations": info["iterations"], "factor_retries": info["factor_retries"],
                     "shift": info["shift"], "backward_error": info["backward_error"],
                     "backward_error_fp64_check": be64,
                     "forward_error_vs_fp64": fe, "cond_estimate_diag_tiles": info["cond_estimate"]}
        del W
        torch.cuda.empty_cache()
    return out


def run_batched(gbx, dev, count=4096, reps=3, cpu=True):
    """4096 SPD systems, sizes uniform over 32*{1..16}, (M+M^T)/2 + n I, 1 right-hand side each:
    one persistent launch per solve, captured in a CUDA graph; FP64, FP32 + 2 FP64 refinement steps,
    and the configuration the batched autotuner picks (precision split, queue order, CTA count)."""
    import numpy as np
    import torch

    from ttg_gb300 import autotune
    rng = np.random.default_rng(42)
    sizes = 32 * rng.integers(1, 17, size=count)
    rhs = [rng.standard_normal((1, int(n))) for n in sizes]
    b = gbx.Batch(None, rhs, dev, sizes=sizes, seed=42)
    out = {"config": {"workload": "%d SPD systems, n uniform in 32*{1..16}, 1 rhs, one persistent launch in a CUDA graph"
                                  % count, "count": count, "flops": b.flops}}
    stream = torch.cuda.Stream()
    fp64_peak = measure_fp64_gemm_peak(dev)
    fp32_peak = 2.0 * 128 * torch.cuda.get_device_properties(0).multi_processor_count * 2.07e9  # FFMA issue rate
    hbm = measured_hbm_peak() * 1e9
    n2 = float(np.sum(sizes.astype(np.float64) ** 2))

    def measure(mode, refine, ctas):
        b.reset()
        b.solve(mode=mode, refine=refine, ctas=ctas)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            b.solve(mode=mode, refine=refine, stream=stream, ctas=ctas)
        times = []
        for _ in range(reps + 1):
            b.reset()
            torch.cuda.synchronize()
            e0, e1 = _events()
            with torch.cuda.stream(stream):  # replay() launches on the current stream
                e0.record()
                g.replay()
                e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ms = sum(times[1:]) / reps
        # solution quality on a sample of the systems (checked on the host)
        xs = b.solutions()
        An = b.A0.cpu().numpy()
        worst = 0.0
        offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
        for k in range(0, count, 97):
            n = int(sizes[k])
            Ak = An[offs[k]:offs[k] + n * n].reshape(n, n).T
            r = rhs[k][0] - Ak @ xs[k][0]
            worst = max(worst, np.abs(r).max() / (np.abs(Ak).sum(1).max() * np.abs(xs[k][0]).max()
                                                  + np.abs(rhs[k][0]).max()))
        # size-mix roofline: FP64 mode, the factorisation at the FP64 rate (compute-bound for every
        # n >= 32) plus one read and one write of each matrix (16 n^2 B); FP32 mode, the factorisation
        # at the FP32 FFMA rate plus the HBM bytes (A read 8 n^2, factor written 4 n^2, per refinement
        # step A read again and the factor read twice: 16 n^2)
        if mode == "fp64":
            t_roof = b.flops / (fp64_peak * 1e12) + 16.0 * n2 / hbm
        else:
            t_roof = b.flops / fp32_peak + (12.0 + 16.0 * refine) * n2 / hbm
        return {"ms": ms, "matrices_per_s": count / (ms * 1e-3), "tflops": b.flops / (ms * 1e-3) / 1e12,
                "refine_steps": refine, "ctas": ctas, "info_nonzero": int((b.info != 0).sum().item()),
                "backward_error_sampled": worst, "size_mix_roofline_ms": t_roof * 1e3,
                "frac_of_size_mix_roofline": t_roof * 1e3 / ms}

    out["fp64"] = measure("fp64", 0, 0)
    out["fp32"] = measure("fp32", 2, 0)
    best = autotune.tune_batched(b, rhs, tol=1e-14, use_cache=False)  # leaves its queue order set
    out["tuned"] = measure(best["mode"], best["refine"], best["ctas"])
    out["tuned"].update(mode=best["mode"], schedule=best["schedule"], candidates=len(best["candidates"]))
    if cpu:
        # CPU counterpart: LAPACK dpotrf + dpotrs per matrix (OpenBLAS, one thread per matrix), all
        # host cores over the matrices, largest first; the whole batch (not a sample)
        import oracle
        blas = oracle.load_openblas()
        A_cpu = b.A0.cpu().numpy().copy()
        B0 = np.concatenate([r.ravel() for r in rhs])
        oracle.dposv_batched(sizes[:64], A_cpu[:int(np.sum(sizes[:64].astype(np.int64) ** 2))].copy(),
                             B0[:int(np.sum(sizes[:64]))].copy(), use_blas=blas)  # warm-up
        B_cpu = B0.copy()
        t0 = time.perf_counter()
        info = oracle.dposv_batched(sizes, A_cpu, B_cpu, nrhs=1, nthreads=cpu_cores(), use_blas=blas)
        sec = time.perf_counter() - t0
        assert not info.any()
        out["cpu_baseline"] = {"value": count / sec, "unit": "matrices/s", "tflops": b.flops / sec / 1e12,
                               "cores": cpu_cores(), "kind": "port",
                               "sample": "the whole batch, FP64 dpotrf+dpotrs per matrix (%s), one matrix per thread"
                                         % ("OpenBLAS" if blas else "plain loops")}
    return out


def run_batched_mixed(gbx, dev, cpu=True, count=256, nrhs=4, kappa=1e4, NB=512, cpu_sample=16):
    """Batched mixed precision: 256 SPD systems, n uniform in 128*{4..32}, H diag(lam) H^T with 2
    reflectors (matrix k: seed 42 + k), kappa = 1e4, 4 right-hand sides each; one tensor-core
    factorisation launch for the whole batch (fp16, bf16 and fp8-e4m3 operands) + batched FP64 PCG
    to backward error 1e-14. Against the
    plain FP64 GPU path run matrix by matrix (gbx_dpotrf_tiled + gbx_dpotrs_tiled)."""
    import ctypes

    import numpy as np
    import torch

    from ttg_gb300 import workloads
    sizes = workloads.batch_sizes(count, 4, 32, 128, seed=42)
    A, B = workloads.householder_batch(sizes, NB, 2, kappa, 42, dev, nrhs=nrhs)
    flops = float(np.sum(sizes.astype(np.float64) ** 3) / 3)
    out = {"config": {"workload": "%d SPD systems, n uniform in 128*{4..32}, H diag(lam) H^T (2 reflectors), "
                                  "kappa=%g, %d rhs each, NB=%d" % (count, kappa, nrhs, NB),
                      "count": count, "nrhs": nrhs, "kappa": kappa, "NB": NB, "flops": flops, "tolerance": 1e-14}}
    offs, total = gbx.batched_tile_offsets(sizes, NB)
    # plain FP64 GPU path, one matrix at a time
    T = torch.empty_like(A)
    X64 = B.clone()
    work = torch.empty(gbx.potrf_workspace_bytes(int(sizes.max()), NB), dtype=torch.uint8, device=dev)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    T.copy_(A)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    vo = 0
    for k, n in enumerate(sizes):
        n = int(n)
        tk = ctypes.c_void_p(T.data_ptr() + int(offs[k]) * 8)
        gbx.call("gbx_dpotrf_tiled", n, NB, tk, ctypes.c_void_p(work.data_ptr()), work.numel(), sp)
        gbx.call("gbx_dpotrs_tiled", n, NB, tk, nrhs, ctypes.c_void_p(X64.data_ptr() + vo * 8), n, sp)
        vo += n * nrhs
    e1.record()
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    del T, work
    torch.cuda.empty_cache()
    out["plain_fp64_per_matrix"] = {"ms": plain_ms, "tflops": flops / (plain_ms * 1e-3) / 1e12}
    bf16_peak, _ = measured_bf16_peak()
    hbm = measured_hbm_peak()
    from ttg_gb300 import autotune
    tiles = {NB: A}

    def measure(prec, nb, sched):
        # the whole solve (factorisation with its retry loop, CG to 1e-14 with device-side
        # coefficients and convergence tests) captured once in a CUDA graph, replayed
        if nb not in tiles:
            tiles[nb] = autotune.retile(A, sizes, NB, nb)
        At = tiles[nb]
        W = torch.empty(At.numel(), dtype=torch.float32, device=dev)
        solver = gbx.MixedBatchedSolver(sizes, nb, nrhs, prec=prec, device=dev, sched=sched)
        ms, infos, st, X = autotune.time_mixed_graph(solver, At, B, W, 1e-14, 300, reps=2)
        del solver, W
        it = [i["iterations"] for i in infos]
        be = [i["backward_error"] for i in infos]
        fe = ((X - X64).abs().max() / X64.abs().max()).item()
        # after the timed region: every matrix's residual again, from plain FP64 products
        offs_nb, _ = gbx.batched_tile_offsets(sizes, nb)
        be64, vo = 0.0, 0
        for k, n in enumerate(sizes):
            n = int(n)
            nt = (n + nb - 1) // nb
            Ak = At[int(offs_nb[k]):int(offs_nb[k]) + nt * (nt + 1) // 2 * nb * nb]
            Bk, Xk = B[vo:vo + n * nrhs].view(nrhs, n), X[vo:vo + n * nrhs].view(nrhs, n)
            be64 = max(be64, max(gbx.backward_error_fp64(Ak, n, nb, Bk, Xk)))
            vo += n * nrhs
        # size-mix roofline: per matrix, its factorisation at the tensor-core rate plus the HBM
        # bytes of the refinement (one pass over A writing W and the split: 10 n^2 B; the factor's
        # W read and written: 4 n^2; start-up sweeps and product: 12 n^2; each iteration one product
        # over the split A and two sweeps over W: 8 n^2; the final check: 4 n^2)
        peak_tc = (2.0 if prec == "fp8" else 1.0) * bf16_peak * 1e12
        t_roof = sum((float(n) ** 3 / 3) / peak_tc + (30.0 + 8.0 * i["iterations"]) * float(n) ** 2 / (hbm * 1e9)
                     for n, i in zip(sizes, infos))
        return {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "matrices_per_s": count / (ms * 1e-3),
                "NB": nb, "sched": sched, "cuda_graph": True, "size_mix_roofline_ms": t_roof * 1e3,
                "frac_of_size_mix_roofline": t_roof * 1e3 / ms,
                "speedup_vs_plain_fp64": plain_ms / ms, "status": st, "iterations_max": int(max(it)),
                "iterations_mean": float(np.mean(it)), "factor_retries": int(sum(i["factor_retries"] for i in infos)),
                "fp64_diag_tiles": int(sum(i["fp64_diag_tiles"] for i in infos)),
                "shift_max": float(max(i["shift"] for i in infos)),
                "backward_error_max": float(max(be)), "backward_error_fp64_check_max": be64,
                "forward_error_vs_fp64": fe}

    # the configuration the tuner picks (tile size, operand precision, CTA schedule of the queue),
    # then each operand precision at the configuration's tile size (fp8 is the one the workload names)
    best = autotune.tune_mixed_batched(A, sizes, NB, B, nrhs, tol=1e-14, use_cache=False)
    out["tuned"] = measure(best["prec"], best["NB"], best["sched"])
    out["tuned"].update(prec=best["prec"], tuner_candidates=[
        {k: c[k] for k in ("prec", "NB", "sched", "ms", "ok")} for c in best["candidates"]])
    for prec in ("fp8", "fp16", "bf16"):
        out[prec] = measure(prec, NB, 0)
    if cpu:
        # CPU counterpart: LAPACK dpotrf + dpotrs per matrix (OpenBLAS, one matrix per thread) on a
        # bounded sample: the first `cpu_sample` matrices of the batch
        import oracle
        blas = oracle.load_openblas()
        ss = sizes[:cpu_sample]
        An = A[:int(offs[cpu_sample])].cpu().numpy() if cpu_sample < count else A.cpu().numpy()
        dense = []
        for k, n in enumerate(ss):
            n = int(n)
            nt = (n + NB - 1) // NB
            L = oracle.tiles_to_lower(An[int(offs[k]):int(offs[k]) + nt * (nt + 1) // 2 * NB * NB], n, NB)
            dense.append(np.ascontiguousarray((L + np.tril(L, -1).T).T).ravel())
        Ac = np.concatenate(dense)
        Bc = B[:int(np.sum(ss) * nrhs)].cpu().numpy().copy()
        t0 = time.perf_counter()
        info = oracle.dposv_batched(ss, Ac, Bc, nrhs=nrhs, nthreads=cpu_cores(), use_blas=blas)
        sec = time.perf_counter() - t0
        assert not info.any()
        sflops = float(np.sum(ss.astype(np.float64) ** 3) / 3)
        out["cpu_baseline"] = {"value": sflops / sec / 1e12, "unit": "TFLOP/s", "cores": cpu_cores(), "kind": "port",
                               "sample": "first %d matrices of the batch, FP64 dpotrf+dpotrs per matrix (%s), one "
                                         "matrix per thread" % (cpu_sample, "OpenBLAS" if blas else "plain loops")}
    return out


def _dense_from_tiles(t, N, NB):
    """Full symmetric matrix on the device from lower tiles (torch slicing, one tile at a time)."""
    import torch
    NT = (N + NB - 1) // NB
    D = torch.zeros(N, N, dtype=torch.float64, device=t.device)
    tl = NB * NB
    for n in range(NT):
        for m in range(n, NT):
            slot = n * NT - n * (n - 1) // 2 + (m - n)
            mb, nb = min(NB, N - m * NB), min(NB, N - n * NB)
            blk = t[slot * tl:(slot + 1) * tl].view(NB, NB).T[:mb, :nb]  # column-major tile
            if m == n:
                blk = torch.tril(blk)
            D[m * NB:m * NB + mb, n * NB:n * NB + nb] = blk
    return D + torch.tril(D, -1).T


def run_potri(gbx, dev, N=8192, NB=512, reps=3, cpu=True):
    """Inverse from the factor (the reference's POTRI chain, TRTRI + LAUUM), FP64, N=8192 NB=512:
    device time of gbx_dpotri_tiled and the residual ||A X v - v|| / ||v|| for a random v."""
    import numpy as np
    import torch
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=dev)
    gbx.gen_uniform_sym(A, N, NB, seed=42)
    L = A.clone()
    gbx.potrf_tiled(L, N, NB)
    T = torch.empty_like(L)
    times = []
    for i in range(reps + 1):
        T.copy_(L)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        gbx.potri_tiled(T, N, NB)
        e1.record()
        e1.synchronize()
        if i:
            times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    flops = N * ((2.0 / 3) + N * ((1.0 / 3) * N + 1)) + N * ((1.0 / 6) + N * ((1.0 / 3) * N - 0.5))  # FLOPS_DPOTRI
    Ad, Xd = _dense_from_tiles(A, N, NB), _dense_from_tiles(T, N, NB)
    v = torch.randn(N, dtype=torch.float64, device=dev)
    res = ((Ad @ (Xd @ v) - v).norm() / v.norm()).item()
    out = {"config": {"workload": "potri FP64 N=%d NB=%d from the factor of (M+M^T)/2 + N*I seed 42" % (N, NB),
                      "N": N, "NB": NB, "flops": flops},
           "gpu": {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "residual_AXv_minus_v": res}}
    if cpu:
        import oracle
        n_s = 1024  # bounded CPU sample: the restated tile algorithm in plain loops, one thread
        t = oracle.uniform_sym_tiles(n_s, 128, 42)
        oracle.potrf_tiled(t, n_s, 128, nthreads=0, use_blas=oracle.load_openblas())
        t0 = time.perf_counter()
        oracle.potri_tiled(t, n_s, 128)
        sec = time.perf_counter() - t0
        fs = n_s * ((2.0 / 3) + n_s * ((1.0 / 3) * n_s + 1)) + n_s * ((1.0 / 6) + n_s * ((1.0 / 3) * n_s - 0.5))
        out["cpu_baseline"] = {"value": fs / sec / 1e12, "unit": "TFLOP/s", "cores": 1, "kind": "port",
                               "sample": "N=%d NB=128, the oracle's plain-loop tile TRTRI + LAUUM, one thread" % n_s}
    return out


def run_config1(gbx, dev, cpu=True, reps=5):
    """The reference's own CPU-runnable case, N=2048 NB=128 (FP64 factor only): the GPU executor and the
    CPU restatement of the flowgraph on all host cores, both with the same seeded matrix."""
    import numpy as np
    import torch
    N, NB = 2048, 128
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=dev)
    gbx.gen_uniform_sym(A, N, NB, seed=42)
    T = A.clone()
    work = None
    times = []
    for i in range(reps + 1):
        T.copy_(A)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        work = gbx.potrf_tiled(T, N, NB, workspace=work, check=False)
        e1.record()
        e1.synchronize()
        if i:
            times.append(e0.elapsed_time(e1))
    assert gbx.potrf_status(work) == 0
    ms = statistics.median(times)
    out = {"config": {"workload": "potrf FP64 N=%d NB=%d, (M+M^T)/2 + N*I seed 42" % (N, NB), "N": N, "NB": NB},
           "gpu": {"ms": ms, "tflops": flops_factor(N) / (ms * 1e-3) / 1e12, "reps": reps}}
    if cpu:
        import oracle
        blas = oracle.load_openblas()
        ct, cg = [], []
        for i in range(reps + 1):
            t0 = time.perf_counter()
            base = oracle.uniform_sym_tiles(N, NB, 42)
            t1 = time.perf_counter()
            st, _, _ = oracle.potrf_tiled(base, N, NB, nthreads=cpu_cores(), use_blas=blas)
            t2 = time.perf_counter()
            assert st == 0
            if i:
                ct.append(t2 - t1)
                cg.append(t2 - t0)
        sec = statistics.median(ct)
        out["cpu_baseline"] = {"value": flops_factor(N) / sec / 1e12, "unit": "TFLOP/s", "ms": sec * 1e3,
                               "ms_with_generation": statistics.median(cg) * 1e3, "cores": cpu_cores(),
                               "kind": "port", "sample": "the whole N=%d factorisation, median of %d, %s tile kernels"
                                                         % (N, reps, "OpenBLAS" if blas else "plain-loop")}
        # the CPU and GPU factors of the same matrix agree
        L = torch.from_numpy(base.reshape(-1)).to(dev)
        out["max_abs_diff_gpu_vs_cpu"] = (L - T).abs().max().item()
    return out


def run_ttg_flowgraph(gbx, dev, N=16384, NB=512, iters=2, chain_tasks=20000):
    """The drop-in path: the potrf flowgraph on the TTG API (make_tt device tasks calling the tile
    kernels, ttg_gb300/potrf/testing_dpotrf, the reference driver's timed region: generation on the
    device, factorisation, write-back of the factor) at N=16384 NB=512 and its GF/s as the driver
    prints them; beside it the whole-flowgraph executor (gbx_dpotrf_tiled) on the same matrix, and
    the per-device-task overhead of the runtime (ttg_gb300/potrf/chain_dev, a chain of device tasks
    as in the reference's task benchmark)."""
    import re

    import torch

    from ttg_gb300 import build as gb
    out = {"config": {"workload": "potrf FP64 N=%d NB=%d through the TTG flowgraph (device tasks), PLASMA "
                                  "generator seed 3872" % (N, NB), "N": N, "NB": NB}}
    drv = gb.build_driver()

    def flowgraph(n, extra):
        r = subprocess.run([drv, "-N", str(n), "-t", str(NB), "-n", str(iters), "-x"] + extra, capture_output=True,
                           text=True, timeout=1200)
        g = [float(x) for x in re.findall(r"([0-9.eE+-]+) GF/s", r.stdout)]
        t = [float(x) for x in re.findall(r"Execution Time \(milliseconds\) : ([0-9.eE+-]+)", r.stdout)]
        return {"rc": r.returncode, "N": n, "gflops_per_iter": g, "ms_per_iter": t, "tflops": max(g) / 1e3 if g else None}

    # one launch per device task (grid kernels, host continuations), and the device task queue
    # (the tasks' tile kernels recorded, one persistent launch per batch)
    out["flowgraph"] = flowgraph(N, [])
    out["flowgraph_device_queue"] = flowgraph(N, ["-q"])
    out["flowgraph_N4096"] = flowgraph(4096, [])
    out["flowgraph_N4096_device_queue"] = flowgraph(4096, ["-q"])
    gfs = out["flowgraph"]["gflops_per_iter"]
    # the same factorisation by the persistent executor, device time: with FP64 FMA updates (the
    # flowgraph's tile bodies are FP64 FMA kernels too), and with the tensor-core updates
    t = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=dev)
    gbx.plgsy(t, N, NB, N, 3872)
    mode0 = gbx.lib().gbx_get_fp64_update()
    for key, mode in (("executor", 0), ("executor_tensor_updates", 1)):
        assert gbx.lib().gbx_set_fp64_update(mode) == 0
        work = gbx.potrf_tiled(t.clone(), N, NB)
        T = t.clone()
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        gbx.potrf_tiled(T, N, NB, workspace=work, check=False)
        e1.record()
        e1.synchronize()
        exe_ms = e0.elapsed_time(e1)
        out[key] = {"ms": exe_ms, "tflops": flops_factor(N) / (exe_ms * 1e-3) / 1e12}
        del T, work
    gbx.lib().gbx_set_fp64_update(mode0)
    if gfs:
        out["flowgraph_vs_executor"] = out["flowgraph"]["tflops"] / out["executor"]["tflops"]
    del t
    chain = gb.build_chain()
    out["chain"] = {}
    for flows in (0, 1):
        for mode, extra in (("", []), ("_device_queue", ["-q"])):
            r = subprocess.run([chain, "-f", str(flows), "-n", str(chain_tasks)] + extra, capture_output=True,
                               text=True, timeout=600)
            m = re.search(r"avg ([0-9.eE+-]+)", r.stdout)
            out["chain"]["flows_%d%s" % (flows, mode)] = {"rc": r.returncode, "tasks": chain_tasks + 1,
                                                          "us_per_task": float(m.group(1)) if m else None}
    return out


def run_e2e(gbx, A0, b0, N, NB, nrhs, work, dev, reps):
    """The step through the C ABI from host buffers: gbx_dposv_tiled_host takes pinned host A and b,
    copies tile columns in while the executor runs, copies each finished column of L back, solves,
    and returns x. Every copy is inside the events."""
    import ctypes

    import torch
    A_host = torch.empty(A0.numel(), dtype=torch.float64, pin_memory=True)
    A_host.copy_(A0)
    b_host = torch.empty(b0.shape, dtype=torch.float64, pin_memory=True)
    b_host.copy_(b0)
    L_host = torch.empty_like(A_host, pin_memory=True)
    x_host = torch.empty_like(b_host, pin_memory=True)
    T = torch.empty_like(A0)
    X = torch.empty_like(b0)
    need = ctypes.c_size_t(0)
    gbx.call("gbx_dposv_tiled_host_bufferSize", N, NB, ctypes.byref(need))
    hwork = torch.empty(need.value, dtype=torch.uint8, device=dev)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    times = []
    for i in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        gbx.call("gbx_dposv_tiled_host", N, NB, ctypes.c_void_p(A_host.data_ptr()), ctypes.c_void_p(L_host.data_ptr()),
                 nrhs, ctypes.c_void_p(b_host.data_ptr()), ctypes.c_void_p(x_host.data_ptr()),
                 ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(hwork.data_ptr()),
                 need.value, sp)
        e1.record()
        e1.synchronize()
        if i > 0:
            times.append(e0.elapsed_time(e1))
    assert gbx.potrf_status(hwork) == 0
    ms = sum(times) / len(times)
    del T, X
    return {"value": flops_factor(N) / (ms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": ms,
            "h2d_bytes_per_step": A_host.numel() * 8 + b_host.numel() * 8,
            "d2h_bytes_per_step": L_host.numel() * 8 + x_host.numel() * 8, "steps": reps,
            "api": "gbx_dposv_tiled_host (C ABI): pinned host A, b in; L, x out; copies overlapped with the "
                   "factorisation"}


def profile_case(case, N=8192):
    """One small case of one kernel (inputs larger than L2, a few GB at most), for ncu captures."""
    import torch

    import ttg_gb300 as gbx
    from ttg_gb300 import workloads
    dev = torch.device("cuda:0")
    NB = 512
    if case == "batched_mixed":  # the 256-system batched mixed solve (fp16) of the benchmark, once
        sizes = workloads.batch_sizes(256, 4, 32, 128, seed=42)
        A, B = workloads.householder_batch(sizes, NB, 2, 1e4, 42, dev, nrhs=4)
        X, infos, st = gbx.dposv_mixed_batched(A, sizes, NB, B, 4, prec="fp16", tol=1e-14)
        assert st == 0
    elif case == "refine":  # the refinement of a kappa = 1e6 fp16 solve: sweeps and double-float products
        A = workloads.householder_tiles(N, NB, 4, 1e6, 42, dev)
        B = torch.from_numpy(workloads.rhs(N, 8, 42)).to(dev)
        X, info, st = gbx.dposv_mixed(A, N, NB, B, prec="fp16", tol=1e-14)
        assert st == 0, info
    elif case in ("dag", "emu", "mixed"):
        assert gbx.lib().gbx_set_fp64_update(1 if case == "emu" else 0) == 0
        A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=dev)
        gbx.gen_uniform_sym(A, N, NB, seed=42)
        for _ in range(2):  # the second launch is the captured one (-s 1 -c 1), or both (-c 2)
            if case in ("dag", "emu"):
                gbx.potrf_tiled(A.clone(), N, NB)
            else:
                W, work, st, cond = gbx.potrf_mixed(A, N, NB, prec="bf16")
                assert st == 0
    else:
        import numpy as np
        rng = np.random.default_rng(42)
        sizes = 32 * rng.integers(1, 17, size=1024)
        b = gbx.Batch(None, [np.ones((1, int(n))) for n in sizes], dev, sizes=sizes, seed=42)
        for _ in range(2):
            b.reset()
            b.solve(mode="fp64")
    torch.cuda.synchronize()
    print("profile case %s done" % case)


def main():
    args = parse()
    if args.only_main:
        args.no_e2e = args.no_mixed = args.no_batched = args.no_cpu = True
    if args.profile_case:
        profile_case(args.profile_case, args.profile_N)
        return
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
