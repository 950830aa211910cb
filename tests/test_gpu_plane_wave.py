"""Plane-wave mode (pw_mode, m_source.f90:316-466 with the ghost
extrapolation of m_absorb_p.f90): the analytic P or S plane-wave initial
condition, run through the time loop; receiver traces against the oracle
(relative L2 <= 1e-5)."""
import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit

NT = 300


@pytest.mark.gpu
@pytest.mark.parametrize("ps", ["p", "s"])
def test_plane_wave_matches_oracle(tmp_path, ps):
    inf = configs.write_plane_wave(str(tmp_path), ps=ps, nt=NT)
    o = pyoracle.Oracle(inf, "fp32")
    o.run(NT)
    ref = o.waveforms()
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    got = s.waveforms()
    s.close()
    assert np.abs(ref).max() > 0
    m = misfit(got, ref)
    print("plane wave %s: misfit %.3e" % (ps, m))
    assert m <= 1e-5


def test_plane_wave_host_setup(tmp_path):
    """No source grid; fcut = v / pw_zlen at the centre column; M0 = 1/UC."""
    inf = configs.write_plane_wave(str(tmp_path), ps="s", nt=10)
    h = gpu.host_check(inf)
    o = pyoracle.Oracle(inf, "fp32")
    assert h["nsrc"] == 0
    assert abs(h["fcut"] - o.fcut) < 1e-6 * o.fcut
    assert h["M0"] == np.float32(o.M0)


@pytest.mark.gpu
def test_plane_wave_batched_equals_alone(tmp_path):
    inf = configs.write_plane_wave(str(tmp_path), ps="s", nt=120)
    a = gpu.Simulation.from_inf(inf)
    a.run(1, 120)
    a.sync()
    alone = a.waveforms()
    a.close()
    sims = [gpu.Simulation.from_inf(inf), gpu.Simulation.from_inf(inf)]
    b = gpu.Batch(sims)
    b.run(120)
    b.sync()
    for q in sims:
        assert np.array_equal(q.waveforms(), alone)
    b.close()
    for q in sims:
        q.close()
