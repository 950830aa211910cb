"""The batched form: several simulations of different shapes advanced by
fused launches must give exactly the results of running each one alone, and
each must match the CPU oracle (relative L2 <= 1e-5)."""
import os

import numpy as np
import pytest

from openswpc_gb300 import autotune, configs, gpu
from oracle import pyoracle
from tests.helpers import misfit

SHAPES = [(96, 128, 96, 11), (128, 96, 128, 12), (96, 96, 160, 13)]
NT = 120


@pytest.fixture(scope="module")
def infs(tmp_path_factory):
    out = []
    for nx, ny, nz, seed in SHAPES:
        d = tmp_path_factory.mktemp("b%d" % seed)
        out.append(configs.write_layered(str(d), nx, ny, nz, seed, nt=NT, n_station=8,
                                         src_depth_max=4.0))
    return out


def _alone(inf):
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    w = s.waveforms()
    s.close()
    return w


@pytest.mark.gpu
def test_batch_equals_members_alone(infs):
    alone = [_alone(f) for f in infs]
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    b = gpu.Batch(sims)
    b.run(NT)
    b.sync()
    for s, w in zip(sims, alone):
        got = s.waveforms()
        assert np.abs(w).max() > 0
        assert np.array_equal(got, w)
    assert b.launch_count() > 0
    b.close()
    for s in sims:
        s.close()


@pytest.mark.gpu
def test_batch_member_matches_oracle(infs):
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    b = gpu.Batch(sims)
    b.run(NT)
    b.sync()
    for f, s in zip(infs, sims):
        o = pyoracle.Oracle(f, "fp32")
        o.run(NT)
        assert misfit(s.waveforms(), o.waveforms()) < 1e-5
    b.close()


@pytest.mark.gpu
def test_reset_and_autotune_leave_results_unchanged(infs, tmp_path):
    alone = [_alone(f) for f in infs]
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    rec = autotune.tune(sims, cache=str(tmp_path / "tune.json"), steps=3, candidates=(8, 0))
    assert rec["zchunk"] in (8, 0) and rec["zchunk_vel"] in (8, 0)
    b = gpu.Batch(sims)
    b.run(NT)
    b.sync()
    for s, w in zip(sims, alone):
        assert np.array_equal(s.waveforms(), w)
    # a second tuning call is served from the cache
    rec2 = autotune.tune(sims, cache=str(tmp_path / "tune.json"), steps=3, candidates=(8, 0))
    assert (rec2["zchunk"], rec2["zchunk_vel"]) == (rec["zchunk"], rec["zchunk_vel"])
    if rec["zchunk"] and rec["zchunk_vel"]:
        assert sims[0].zchunks() == (rec["zchunk"], rec["zchunk_vel"])
    b.close()
