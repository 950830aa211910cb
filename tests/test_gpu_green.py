"""Reciprocal Green's-function mode (green_mode, m_green.f90): a unit body
force at a station, displacement gradients (and displacement) recorded at
the points of a list file.  The GPU traces must match the oracle's
(relative L2 <= 1e-5), the batched form must reproduce the single run bit for
bit, and the SAC export must carry the reference's names, headers and the
sign flip of a vertical force."""
import os

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit

NT = 160


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = tmp_path_factory.mktemp("green")
    inf = configs.write_green(str(d), nt=NT, cmp="z", bforce=True, title="grn")
    o = pyoracle.Oracle(inf, "fp32")
    o.run(NT)
    return inf, o.green()


@pytest.mark.gpu
def test_green_traces_match_oracle(case):
    inf, ref = case
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    got = s.green()
    s.close()
    assert got.shape == ref.shape == (24, 9, NT // 2)
    assert np.abs(ref).max() > 0
    m6 = misfit(got[:, :6], ref[:, :6])
    m3 = misfit(got[:, 6:], ref[:, 6:])
    print("green mode: misfit strain %.3e, displacement %.3e" % (m6, m3))
    assert m6 <= 1e-5 and m3 <= 1e-5


@pytest.mark.gpu
def test_green_batched_equals_alone(case):
    inf, _ = case
    a = gpu.Simulation.from_inf(inf)
    a.run(1, NT)
    a.sync()
    alone = a.green()
    a.close()
    s = [gpu.Simulation.from_inf(inf), gpu.Simulation.from_inf(inf)]
    b = gpu.Batch(s)
    b.run(NT)
    b.sync()
    for q in s:
        assert np.array_equal(q.green(), alone)
    b.close()
    for q in s:
        q.close()


@pytest.mark.gpu
def test_green_sac_export(case, tmp_path):
    inf, _ = case
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    g = s.green()
    s.write_green(str(tmp_path))
    s.close()
    d = tmp_path / "green" / "G01"
    files = sorted(os.listdir(str(d)))
    assert len(files) == 24 * 9
    fn = "grn__00001003__G01__z__mzz__.sac"
    assert fn in files
    b = open(str(d / fn), "rb").read()
    fh = np.frombuffer(b[:280], np.float32)
    ih = np.frombuffer(b[280:420], np.int32)
    kh = b[440:632]
    data = np.frombuffer(b[632:], np.float32)
    assert ih[9] == NT // 2 and ih[16] == 7
    assert kh[0:8].decode().strip() == "G01"
    assert kh[8:24].decode().strip() == "00001003"
    assert kh[160:168].decode().strip() == "G_Vz_mzz"
    assert fh[58] == 0.0  # cmpinc of a vertical force
    assert np.array_equal(data, -g[3, 2])  # the vertical force is positive upward
    ux = np.frombuffer(open(str(d / "grn__00001003__G01__z__fx___.sac"), "rb").read()[632:], np.float32)
    assert np.array_equal(ux, -g[3, 6])
