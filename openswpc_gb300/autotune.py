"""Autotuner of the tile shapes and z-sweep depths of the interior kernels.

Each interior block sweeps a chunk of z planes of a tile of 32 columns by 8
or 16 rows (velocity also 12).  Taller tiles read fewer halo rows per point but run fewer
blocks per SM.  Long chunks amortise the
pipeline prologue (the first planes of every ring are loaded before any
compute); short chunks create more blocks, which small grids need to fill the
GPU, and keep neighbouring blocks on the same planes so that they share halo
rows in L2.  The stress and velocity kernels weigh these differently, so each
gets its own depth.  The best depths depend on the grid shape and on what
else shares the GPU (a batch), so they are measured: every candidate depth is
timed on the real simulations with CUDA events on the launching stream, then
the simulations are reset to their initial state.  Results are cached in a JSON file keyed by
the shape class (interior extents rounded up to 32, storage precision, batch
size), so later runs with the same shapes skip the measurement.
"""
import hashlib
import json
import os

import numpy as np

from . import gpu

CANDIDATES = (8, 16, 32, 64, 128, 0)  # 0 = the library's automatic choice
TILE_ROWS = (8, 16)  # rows of the 32-column stress tiles
TILE_ROWS_VEL = (8, 12, 16)  # and of the velocity tiles
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


def tune(sims, store="fp32", warmup=8, steps=8, cache=DEFAULT_CACHE, candidates=CANDIDATES, batch=None,
         rows=TILE_ROWS, rows_vel=TILE_ROWS_VEL):
    """Pick the tile shapes and z-sweep depths of the stress and velocity
    kernels for `sims` (one simulation, or the members of a batch when
    len(sims) > 1), apply them to every member and return {"tiles": [stress
    rows, velocity rows], "zchunk": stress depth, "zchunk_vel": velocity
    depth, "ms_per_step": {"rows/depth": ms}, "ms_per_step_vel": {...}}
    (depth 0 = the library's automatic choice).

    The stress kernel's (rows, depth) pairs are swept first with the
    velocity kernel at 8 rows and its automatic depth, then the velocity
    kernel's pairs with the stress kernel fixed at its best.  The warm-up
    builds the CUDA graph of the step (8 steps), so the timed steps replay it
    as a production run does.  The members are stepped while timing and
    reset afterwards, so call this after set-up and before the production
    run.
    """
    key = _shape_key(sims, store) + "-tiles12"
    db = _load(cache) if cache else {}
    if key in db and "tiles" in db[key]:
        r = db[key]
        for s in sims:
            s.set_tiles(*r["tiles"])
            s.set_zchunks(r["zchunk"], r["zchunk_vel"])
        return r

    def measure(rs, ks, rv, kv):
        for s in sims:
            s.set_tiles(rs, rv)
            s.set_zchunks(ks, kv)
        if len(sims) == 1:
            s = sims[0]
            it = [1]

            def runner(n, s=s, it=it):
                s.run(it[0], it[0] + n - 1)
                it[0] += n

            runner(warmup)
            s.sync()
            ms = _time(runner, s.stream(), steps)
        else:
            b = gpu.Batch(sims)
            b.run(warmup)
            b.sync()
            ms = _time(b.run, b.stream(), steps)
            b.close()
        for s in sims:
            s.reset()
        return ms

    t_s = {(r, z): measure(r, z, 8, 0) for r in rows for z in candidates}
    best_s = min(t_s, key=t_s.get)
    t_v = {(r, z): measure(best_s[0], best_s[1], r, z) for r in rows_vel for z in candidates}
    best_v = min(t_v, key=t_v.get)
    for s in sims:
        s.set_tiles(best_s[0], best_v[0])
        s.set_zchunks(best_s[1], best_v[1])
    rec = {"tiles": [best_s[0], best_v[0]], "zchunk": best_s[1], "zchunk_vel": best_v[1],
           "ms_per_step": {"%d/%d" % k: float(v) for k, v in t_s.items()},
           "ms_per_step_vel": {"%d/%d" % k: float(v) for k, v in t_v.items()}}
    if cache:
        db = _load(cache)
        db[key] = rec
        _save(cache, db)
    return rec
