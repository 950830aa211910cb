"""Parity of the drop-in path (input.inf -> host set-up -> GPU) with the
oracle over the options of the time loop: the Cerjan sponge instead of the
PML, every receiver output (velocity, displacement, stress, strain) with
decimation, body-force sources, and every source time function.
Tolerance: relative L2 <= 1e-5 per output kind."""
import os

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit

NT = 160
KINDS = [gpu.SWPC_WAV_V, gpu.SWPC_WAV_U, gpu.SWPC_WAV_STRESS, gpu.SWPC_WAV_STRAIN]


def _compare(inf, kinds=(gpu.SWPC_WAV_V,)):
    o = pyoracle.Oracle(inf, "fp32")
    o.run(NT)
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    out = {}
    for k in kinds:
        ref = o.waveforms({1: 0, 2: 1, 4: 2, 8: 3}[k])
        got = s.waveforms(k)
        assert np.abs(ref).max() > 0, k
        out[k] = misfit(got, ref)
    s.close()
    return out


def _shallow(d, **over):
    inf = configs.write_plain_small(str(d), nt=NT, **over)
    return inf


@pytest.mark.gpu
def test_cerjan_sponge(tmp_path):
    m = _compare(_shallow(tmp_path, abc_type="cerjan"))
    print("cerjan: %s" % m)
    assert max(m.values()) <= 1e-5


@pytest.mark.gpu
def test_every_receiver_output_with_decimation(tmp_path):
    inf = _shallow(tmp_path, sw_wav_u=True, sw_wav_stress=True, sw_wav_strain=True, ntdec_w=3)
    m = _compare(inf, kinds=KINDS)
    print("receiver outputs: %s" % m)
    assert max(m.values()) <= 1e-5


@pytest.mark.gpu
def test_body_force_source(tmp_path):
    inf = _shallow(tmp_path, bf_mode=True, stf_format="xy")
    with open(os.path.join(str(tmp_path), "source.dat"), "w") as f:
        f.write("  1.0 -2.0 6.0 0.0 1.0 3.0e15 -1.0e15 2.0e15\n")
    m = _compare(inf)
    print("body force: %s" % m)
    assert max(m.values()) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("stf", ["boxcar", "triangle", "herrmann", "cosine", "texp"])
def test_source_time_functions(tmp_path, stf):
    m = _compare(_shallow(tmp_path, stftype=stf))
    assert max(m.values()) <= 1e-5, (stf, m)


@pytest.mark.gpu
def test_point_force_matches_analytic_whole_space(tmp_path):
    """The drop-in path against the complete analytic solution of a point
    force in a uniform whole space (the same case the oracle is pinned on):
    Vz 8 km along x (S) and along z (P) within 5 % after one common scale,
    the two scales equal to 1.5 %."""
    from tests.helpers import point_force_fit, write_point_force_case
    inf = write_point_force_case(tmp_path)
    s = gpu.Simulation.from_inf(inf)
    s.run(1, 300)
    s.sync()
    w = s.waveforms()
    s.close()
    (a_s, r_s), (a_p, r_p) = point_force_fit(w, 0.02, [np.array([8.0, 0, 0]), np.array([0, 0, 8.0])])
    print("point force (GPU): S residual %.3f, P residual %.3f, scale ratio %.4f" % (r_s, r_p, a_s / a_p))
    assert r_s < 0.05 and r_p < 0.05
    assert abs(a_s / a_p - 1) < 0.015
