"""Autotuner of the z-sweep depth of the interior kernels.

Each interior block sweeps a chunk of z planes.  Long chunks amortise the
pipeline prologue (the first planes of every ring are loaded before any
compute); short chunks create more blocks, which small grids need to fill the
GPU.  The best depth depends on the grid shape and on what else shares the
GPU (a batch), so it is measured: every candidate depth is timed on the real
simulations with CUDA events on the launching stream, then the simulations
are reset to their initial state.  Results are cached in a JSON file keyed by
the shape class (interior extents rounded up to 32, storage precision, batch
size), so later runs with the same shapes skip the measurement.
"""
import hashlib
import json
import os

import numpy as np

from . import gpu

CANDIDATES = (8, 16, 32, 64, 128, 0)  # 0 = the library's automatic choice
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _shape_key(sims, store):
    shapes = sorted((s.dims.nx // 32, s.dims.ny // 32, s.dims.nz // 32) if s.dims is not None else (0, 0, 0)
                    for s in sims)
    h = hashlib.sha1(json.dumps(shapes).encode()).hexdigest()[:16]
    return "%s-%s-n%d" % (store, h, len(sims))


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time(runner, stream, steps):
    import torch
    st = torch.cuda.ExternalStream(stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    runner(steps)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def tune(sims, store="fp32", warmup=2, steps=6, cache=DEFAULT_CACHE, candidates=CANDIDATES, batch=None):
    """Pick the z-sweep depth for `sims` (one simulation, or the members of a
    batch when len(sims) > 1), apply it to every member and return
    {"zchunk": depth, "ms_per_step": {depth: ms}}.

    The members are stepped while timing and reset afterwards, so call this
    after set-up and before the production run.
    """
    key = _shape_key(sims, store)
    db = _load(cache) if cache else {}
    if key in db:
        z = db[key]["zchunk"]
        for s in sims:
            s.set_zchunk(z)
        return db[key]
    times = {}
    for z in candidates:
        for s in sims:
            s.set_zchunk(z)
        if len(sims) == 1:
            s = sims[0]
            it = [1]

            def runner(n, s=s, it=it):
                s.run(it[0], it[0] + n - 1)
                it[0] += n

            runner(warmup)
            s.sync()
            times[z] = _time(runner, s.stream(), steps)
        else:
            b = gpu.Batch(sims)
            b.run(warmup)
            b.sync()
            times[z] = _time(b.run, b.stream(), steps)
            b.close()
        for s in sims:
            s.reset()
    best = min(times, key=times.get)
    for s in sims:
        s.set_zchunk(best)
    rec = {"zchunk": best, "ms_per_step": {str(k): float(v) for k, v in times.items()}}
    if cache:
        db = _load(cache)
        db[key] = rec
        _save(cache, db)
    return rec
