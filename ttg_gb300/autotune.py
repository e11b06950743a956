"""Autotuner of the batched persistent solver (gbx_dposv_batched_ex).

For one batch (its size mix) it times every candidate of
  * precision split: FP64, or FP32 factor + 1 or 2 FP64 refinement steps,
  * CTA schedule: queue order largest-first (longest processing time), natural, or
    interleaved large/small; and the number of CTAs (1 or 2 per SM for FP32, 1 per SM for FP64),
keeps the candidates whose sampled backward error meets the tolerance, and returns the fastest.
The choice is cached per (GPU, size histogram, nrhs, tolerance) in a JSON file next to this module.
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
