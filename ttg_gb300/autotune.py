"""Autotuners of the batched solvers.

tune_batched (small systems, gbx_dposv_batched_ex): for one batch (its size mix) it times every
candidate of
  * precision split: FP64, or FP32 factor + 1 or 2 FP64 refinement steps,
  * CTA schedule: queue order largest-first (longest processing time), natural, or
    interleaved large/small; and the number of CTAs (1 or 2 per SM for FP32, 1 per SM for FP64),
keeps the candidates whose sampled backward error meets the tolerance, and returns the fastest.

tune_mixed_batched (tiled systems, gbx_dposv_mixed_batched): times every tile size (256, 512),
tensor-core operand precision (fp16, bf16, fp8-e4m3) and CTA schedule of the factorisation queue
(0: trailing updates before each panel's TRSMs, 1: TRSMs first) of the mixed solve on the batch,
each as the replay of a captured CUDA graph of the whole solve, keeps the candidates with which
every matrix met the tolerance, and returns the fastest. The tiles of the other tile sizes are
made on the device by `retile`.

Choices are cached per (GPU, size histogram, nrhs, tolerance) in a JSON file next to this module.
"""
import hashlib
import json
import os

import numpy as np

_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_autotune_cache.json")


def _orders(sizes):
    lpt = np.argsort(-sizes, kind="stable")
    nat = np.arange(len(sizes))
    inter = np.empty_like(lpt)
    inter[0::2] = lpt[: (len(lpt) + 1) // 2]
    inter[1::2] = lpt[(len(lpt) + 1) // 2:][::-1]
    return {"lpt": lpt, "natural": nat, "interleave": inter}


def _key(batch, tol):
    import torch
    hist = np.bincount(np.asarray(batch.sizes), minlength=1).tobytes()
    h = hashlib.sha1(hist).hexdigest()[:16]
    return "%s|%s|%d|%g" % (torch.cuda.get_device_name(), h, batch.nrhs, tol)


def _time(batch, mode, refine, ctas, reps):
    import torch
    times = []
    for _ in range(reps + 1):
        batch.reset()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        batch.solve(mode=mode, refine=refine, ctas=ctas)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.mean(times[1:]))


def _berr(batch, mats_fn, rhs, sample):
    xs = batch.solutions()
    worst = 0.0
    for k in sample:
        A = mats_fn(k)
        x, b = xs[k][0], rhs[k][0]
        r = b - A @ x
        worst = max(worst, np.abs(r).max() / (np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(b).max()))
    return worst


def tune_batched(batch, rhs, tol=1e-14, reps=2, use_cache=True, sample_every=97):
    """Returns {"mode", "refine", "schedule", "ctas", "ms", "candidates": [...]} and leaves the batch
    configured with the chosen queue order."""
    import torch
    key = _key(batch, tol)
    cache = {}
    if use_cache and os.path.exists(_CACHE):
        try:
            cache = json.load(open(_CACHE))
        except (OSError, ValueError):
            cache = {}
    orders = _orders(np.asarray(batch.sizes))
    if use_cache and key in cache:
        best = cache[key]
        batch.set_order(orders[best["schedule"]])
        return best
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    A0 = batch.A0.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(np.asarray(batch.sizes, dtype=np.int64) ** 2)])
    mats_fn = lambda k: A0[offs[k]:offs[k + 1]].reshape(int(batch.sizes[k]), int(batch.sizes[k])).T
    sample = list(range(0, batch.batch, sample_every))
    cands = []
    for mode, refine in (("fp64", 0), ("fp32", 1), ("fp32", 2)):
        for sched, order in orders.items():
            for per_sm in ((1,) if mode == "fp64" else (1, 2)):
                batch.set_order(order)
                ms = _time(batch, mode, refine, per_sm * sms, reps)
                be = _berr(batch, mats_fn, rhs, sample)
                cands.append({"mode": mode, "refine": refine, "schedule": sched, "ctas": per_sm * sms, "ms": ms,
                              "backward_error": be, "ok": bool(be <= tol and int(batch.info.abs().sum()) == 0)})
    ok = [c for c in cands if c["ok"]] or cands
    best = dict(min(ok, key=lambda c: c["ms"]))
    best["candidates"] = cands
    batch.set_order(orders[best["schedule"]])
    if use_cache:
        cache[key] = best
        try:
            json.dump(cache, open(_CACHE, "w"), indent=1)
        except OSError:
            pass
    return best


# ---- tiled batches: tile size and operand precision of the mixed solver ----------------------

def _lower_index(n, NB, device):
    """Tile-storage offsets of the lower triangle (i >= j) of an n x n matrix, row-major over (i, j)."""
    import torch
    NT = (n + NB - 1) // NB
    i, j = torch.tril_indices(n, n, device=device)
    ti, tj = i // NB, j // NB
    slot = tj * NT - tj * (tj - 1) // 2 + (ti - tj)
    return slot * NB * NB + (i % NB) + (j % NB) * NB


def retile(A, sizes, NB_from, NB_to):
    """The concatenated tile-major lower matrices of a batch (ttg_gb300.batched_tile_offsets layout)
    re-laid for another tile size, on A's device: the lower triangle is moved, everything else
    (strict upper parts of diagonal tiles, padding) is zero."""
    import torch
    from . import batched_tile_offsets
    if NB_from == NB_to:
        return A
    off1, _ = batched_tile_offsets(sizes, NB_from)
    off2, total2 = batched_tile_offsets(sizes, NB_to)
    out = torch.zeros(total2, dtype=A.dtype, device=A.device)
    for k, n in enumerate(sizes):
        n = int(n)
        src = _lower_index(n, NB_from, A.device) + int(off1[k])
        dst = _lower_index(n, NB_to, A.device) + int(off2[k])
        out[dst] = A[src]
    return out


def select_mixed(run, candidates, tol):
    """Runs `run(prec, NB, sched)` for every candidate (it returns a dict with "ms", "status" and
    "backward_error_max"), and returns the fastest candidate with status 0 and backward error
    within tol, with every result under "candidates". Raises if none qualifies."""
    results = []
    for prec, nb, sched in candidates:
        r = dict(run(prec, nb, sched))
        r.update(prec=prec, NB=nb, sched=sched)
        r["ok"] = bool(r["status"] == 0 and r["backward_error_max"] <= tol)
        results.append(r)
    ok = [r for r in results if r["ok"]]
    if not ok:
        raise RuntimeError("no candidate of the mixed solver met the tolerance %g" % tol)
    best = dict(min(ok, key=lambda r: r["ms"]))
    best["candidates"] = results
    return best


def time_mixed_graph(solver, A, B, W, tol, maxiter, reps):
    """Captures one solve of `solver` (a ttg_gb300.MixedBatchedSolver) in a CUDA graph, replays it
    1 + reps times (the first is a warm-up) and returns (mean ms of the timed replays, infos,
    status, X of the last replay)."""
    import torch
    X = torch.empty_like(B)
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
        solver.run(A, B, X, W, tol=tol, maxiter=maxiter, stream=side)
    times = []
    for _ in range(1 + reps):
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            g.replay()
            e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    infos, st = solver.result()
    del g
    return float(np.mean(times[1:])), infos, st, X


def tune_mixed_batched(A, sizes, NB, B, nrhs, tol=1e-14, precs=("fp16", "bf16", "fp8"), NBs=(256, 512),
                       scheds=(0, 1), maxiter=300, reps=1, use_cache=True):
    """Tile size, operand precision and CTA schedule for the batched mixed solve on this batch (A:
    its tiles at tile size NB on the device, B: its right-hand sides). Returns {"prec", "NB",
    "sched", "ms", ..., "candidates": [...]}; the solution of the chosen candidate is not kept."""
    import torch
    from . import MixedBatchedSolver
    sizes = np.asarray(sizes)
    hist = np.bincount(sizes.astype(np.int64), minlength=1).tobytes()
    key = "mixed|%s|%s|%d|%g" % (torch.cuda.get_device_name(), hashlib.sha1(hist).hexdigest()[:16], nrhs, tol)
    cache = {}
    if use_cache and os.path.exists(_CACHE):
        try:
            cache = json.load(open(_CACHE))
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        return cache[key]
    tiles = {NB: A}

    def run(prec, nb, sched):
        if nb not in tiles:
            tiles[nb] = retile(A, sizes, NB, nb)
        At = tiles[nb]
        W = torch.empty(At.numel(), dtype=torch.float32, device=At.device)
        solver = MixedBatchedSolver(sizes, nb, nrhs, prec=prec, device=At.device, sched=sched)
        ms, infos, st, _ = time_mixed_graph(solver, At, B, W, tol, maxiter, reps)
        return {"ms": ms, "status": int(st),
                "backward_error_max": float(max(i["backward_error"] for i in infos)),
                "iterations_max": int(max(i["iterations"] for i in infos)),
                "factor_retries": int(sum(i["factor_retries"] for i in infos))}

    best = select_mixed(run, [(p, nb, sc) for nb in NBs for p in precs for sc in scheds], tol)
    if use_cache:
        cache[key] = best
        try:
            json.dump(cache, open(_CACHE, "w"), indent=1)
        except OSError:
            pass
    return best
