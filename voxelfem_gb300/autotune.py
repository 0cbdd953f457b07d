"""Autotuner of the layer-by-layer evaluator's execution shape.

The evaluator solves one masked problem per build height (LayerByLayer.hh:223-296). How fast a
run is depends on choices that leave its numbers unchanged:
- the number of concurrent solver slots;
- the launch form of the FP32 fine Gauss-Seidel sweep ("lines": four launches of colour pairs
  on whole z-lines per CTA; "colours": eight colour launches; "planes": two launches, one
  thread-block cluster per x-plane; "staged", the line pairs with each CTA's neighbourhood in
  shared memory, is measured 3x slower and left out of the default candidates). This is the fine
  level's tile shape.
It also depends on one numerical choice, the smoothing sweeps per V-cycle: more sweeps cost more
per iteration and save iterations.

``tune_layer_by_layer`` times every candidate on a sample of the heights (every
``sample_increment``-th height, after one warm-up run that captures the solve graphs) and
records the fastest in a JSON cache keyed by grid shape, coarsening count, precision,
initial-guess method and GPU name. ``LayerByLayerEvaluator.run(..., tuned=True)`` reads it back
through ``lookup``. The cache shipped with the package (``tuning_cache.json``) holds entries
measured on GB300; a run of the tuner adds or replaces its own entry.
"""
import itertools
import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "tuning_cache.json")

DEFAULT_CANDIDATES = {"slots": (4, 8, 12), "sweepForm": ("lines", "colours", "planes"),
                      "mgSmoothingIterations": (1, 2, 3)}


def _device_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def key(sim, solver, init_method, device=None):
    ne = [int(v) for v in sim.NbElementsPerDimension]
    prec = getattr(solver, "_prec", "fp64")
    dev = device or _device_name()
    return "lbl|%s|c%d|%s|%s|%s" % ("x".join(str(v) for v in ne), int(solver.numLevels - 1), prec,
                                     init_method, dev)


def load(path=None):
    path = path or CACHE
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def lookup(sim, solver, init_method, path=None):
    """The cached best configuration for this evaluation, or None."""
    return load(path).get(key(sim, solver, init_method))


def tune_layer_by_layer(sim, solver, init_method="zero", tol=1e-8, maxIter=500, sample_increment=8,
                        candidates=None, path=None, write=True):
    """Time the candidate configurations on every ``sample_increment``-th height and cache the
    fastest. Returns the cache entry (best configuration, its time and every candidate's)."""
    import torch

    from . import pyVoxelFEM as pv

    cand = dict(DEFAULT_CANDIDATES)
    if candidates:
        cand.update(candidates)
    results = []
    ref = None
    for slots, form, sweeps in itertools.product(cand["slots"], cand["sweepForm"], cand["mgSmoothingIterations"]):
        ev = pv.LayerByLayerEvaluator(sim)
        ev.selectInitMethod(init_method)
        kw = dict(layerIncrement=sample_increment, maxIter=maxIter, tol=tol, mgIterations=1,
                  mgSmoothingIterations=sweeps, slots=slots, sweepForm=form)
        ev.run(solver, True, **kw)  # warm-up: slot set-up and graph capture
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev.run(solver, True, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if ref is None:
            ref = ev.compliances.copy()
        err = float(max(abs(a - b) / abs(b) for a, b in zip(ev.compliances, ref)))
        results.append({"slots": slots, "sweepForm": form, "mgSmoothingIterations": sweeps, "seconds": dt,
                        "iterations": int(ev.iterations.sum()), "max_rel_diff": err})
        ev._release()
    best = min(results, key=lambda r: r["seconds"])
    entry = {"slots": best["slots"], "sweepForm": best["sweepForm"],
             "mgSmoothingIterations": best["mgSmoothingIterations"], "seconds": best["seconds"],
             "heights_sampled": len(range(int(sim.NbElementsPerDimension[1]), 0, -sample_increment)),
             "tol": tol, "candidates": results}
    if write:
        path = path or CACHE
        data = load(path)
        data[key(sim, solver, init_method)] = entry
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return entry
