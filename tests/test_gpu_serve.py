"""Serving form: requests that arrive while others run are admitted by the
device-memory budget and advanced together with them; each result must be
the same as the same input run alone on the plain path (bit for bit: the
batched launches do the same arithmetic per member)."""
import os
import time

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu

SHAPES = [(96, 96, 96, 21), (128, 96, 96, 22), (96, 128, 128, 23), (128, 128, 96, 24), (96, 96, 128, 25)]
NT = 120


@pytest.fixture(scope="module")
def infs(tmp_path_factory):
    out = []
    for nx, ny, nz, seed in SHAPES:
        d = tmp_path_factory.mktemp("s%d" % seed)
        out.append(configs.write_layered(str(d), nx, ny, nz, seed, nt=NT, n_station=8, src_depth_max=4.0))
    return out


def _alone(inf):
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    w = s.waveforms()
    s.close()
    return w


@pytest.mark.gpu
def test_results_alone_equal_results_in_the_mix(infs):
    alone = [_alone(f) for f in infs]
    need = sorted(gpu.Request(f).device_bytes for f in infs)
    budget = need[-1] + need[-2] + need[0] // 2  # room for two at a time
    with gpu.Server(hbm_budget=budget, quantum=16, prep_threads=2) as srv:
        ids = [srv.submit(infs[0]), srv.submit(infs[1])]
        time.sleep(0.05)
        ids += [srv.submit(f) for f in infs[2:]]
        for rid in ids:
            assert srv.wait(rid, 120.0) == gpu.REQ_DONE
        st = srv.stats()
        assert st["done"] == len(infs) and st["failed"] == 0
        assert 0 < st["peak_bytes"] <= budget
        assert st["bytes_granted"] == 0
        times = [srv.times(rid) for rid in ids]
        for rid, w in zip(ids, alone):
            got = srv.result(rid)
            assert np.abs(w).max() > 0
            assert np.array_equal(got, w)
            srv.release(rid)
    for t in times:
        assert t["submitted"] <= t["admitted"] <= t["started"] <= t["finished"]
    # at least one pair of requests shared the GPU
    overlap = any(a["started"] < b["finished"] and b["started"] < a["finished"]
                  for q, a in enumerate(times) for b in times[q + 1:])
    assert overlap


@pytest.mark.gpu
def test_failed_request_does_not_block_the_line(infs, tmp_path):
    with gpu.Server(quantum=32, prep_threads=2) as srv:
        bad = srv.submit(os.path.join(str(tmp_path), "missing.inf"))
        good = srv.submit(infs[0])
        with pytest.raises(gpu.SwpcError):
            srv.wait(bad, 60.0)
        assert srv.state(bad) < 0 and srv.error(bad)
        assert srv.wait(good, 120.0) == gpu.REQ_DONE
        assert srv.result(good).shape[0] == 8
