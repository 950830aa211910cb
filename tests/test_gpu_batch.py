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
@pytest.mark.parametrize("persistent", [True, False])
def test_batch_equals_members_alone(infs, persistent):
    """Both forms of the batch -- one persistent fused launch per step over a
    work queue, and one launch per phase -- give each member's traces bit
    for bit as the member run alone."""
    alone = [_alone(f) for f in infs]
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    b = gpu.Batch(sims, persistent=persistent)
    if persistent:
        assert b.item_count() > 3 * len(sims)
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
    assert rec["tiles"][0] in (8, 16) and rec["tiles"][1] in (8, 12, 16) and len(rec["ms_per_step"]) == 4
    assert len(rec["ms_per_step_vel"]) == 6
    assert sims[0].tiles() == tuple(rec["tiles"])
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


@pytest.mark.gpu
def test_persistent_batch_in_pieces_and_graph(infs):
    """The persistent form replayed through its graph (8 steps per replay)
    and stepped in odd pieces, members continuing from their own steps, gives
    the traces of the members alone."""
    alone = [_alone(f) for f in infs]
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    sims[0].run(1, 5)  # the first member starts ahead
    b = gpu.Batch(sims, persistent=True)
    b.run(3)
    b.run(NT - 13)  # members at steps NT - 5 and NT - 10
    b.sync()
    b.close()
    sims[0].run(NT - 4, NT)
    sims[1].run(NT - 9, NT)
    sims[2].run(NT - 9, NT)
    for s, w in zip(sims, alone):
        s.sync()
        assert np.array_equal(s.waveforms(), w)
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [(16, 16), (8, 12)])
def test_batch_with_other_tiles_equals_alone(infs, rows):
    """Members with 16-row stress and 16- or 12-row velocity tiles, advanced
    by the phase launches, give the traces of the members alone (8-row
    tiles); the persistent form refuses other than 8-row tiles."""
    alone = [_alone(f) for f in infs]
    sims = [gpu.Simulation.from_inf(f) for f in infs]
    for s in sims:
        s.set_tiles(*rows)
    b = gpu.Batch(sims)
    with pytest.raises(gpu.SwpcError):
        b.set_persistent(True)
    b.run(NT)
    b.sync()
    for s, w in zip(sims, alone):
        assert np.array_equal(s.waveforms(), w)
    b.close()
    for s in sims:
        s.close()
