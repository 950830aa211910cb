"""All fifteen snapshots of m_snap.f90 (xy/yz/xz/fs/ob sections x velocity,
displacement, divergence-rotation) against the oracle on identical inputs,
and their native .snp files through the host layer.

Tolerance: relative L2 <= 1e-5 per snapshot over all frames (the waveform
bar); the displacement sums are FP64 on the GPU and FP32 in the oracle, as
in the reference."""
import os
import struct

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit, sim_from_oracle

NT = 41
ALL = {"%s_%s_sw" % (s, k): True for s in ("xy", "yz", "xz", "fs", "ob") for k in ("v", "u", "ps")}
KEYS = dict(ALL, ntdec_s=20, idec=2, jdec=2, kdec=2, z0_xy=5.0, x0_yz=3.0, y0_xz=-2.0, title="snp")


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = tmp_path_factory.mktemp("snaps")
    inf = configs.write_plain_small(str(d), nt=NT, **KEYS)
    with open(str(d / "source.dat"), "w") as f:  # shallow source: every section sees waves by it = 41
        f.write("  0.0 0.0 3.0 0.0 1.0 1.0e16 30.0 60.0 90.0\n")
    o = pyoracle.Oracle(inf, "fp32")
    o.run(NT)
    return inf, o


def _fix(sec):
    # k0 = ceil((5 - (-1.5)) / 0.5) = 13, i0 = ceil((3 + 32) / 0.5) = 70, j0 = ceil((-2 + 32) / 0.5) = 60
    return {gpu.SEC_XY: 13, gpu.SEC_YZ: 70, gpu.SEC_XZ: 60}.get(sec, 1)


@pytest.mark.gpu
def test_every_snapshot_matches_oracle(case):
    inf, o = case
    s = sim_from_oracle(o)
    for sec in range(5):
        for kind in range(3):
            s.add_snapshot(sec, kind, _fix(sec), 2, 2, 20)
    s.run(1, NT)
    s.sync()
    checked = 0
    for sec in range(5):
        for kind in range(3):
            q = s.query_section(sec, kind)
            assert q["nframes"] == 3
            got = np.stack([s.section(sec, kind, f) for f in range(3)])
            ref = o.snap(sec, kind, q["n1"], q["n2"])
            assert ref.shape == got.shape, (sec, kind, ref.shape, got.shape)
            assert np.abs(ref[1:]).max() > 0, (sec, kind)
            m = misfit(got, ref)
            assert m <= 1e-5, (sec, kind, m)
            checked += 1
    assert checked == 15
    s.close()


@pytest.mark.gpu
def test_snp_files_of_every_section(case, tmp_path):
    inf, o = case
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    yz = np.stack([s.section(gpu.SEC_YZ, gpu.SNAPK_PS, f) for f in range(3)])
    fs = np.stack([s.section(gpu.SEC_FS, gpu.SNAPK_V, f) for f in range(3)])
    s.write_snp(str(tmp_path))
    s.close()
    names = sorted(os.listdir(str(tmp_path)))
    assert len([n for n in names if n.endswith(".snp")]) == 15

    def header(fn):
        b = open(str(tmp_path / fn), "rb").read()
        h = struct.unpack_from("<8s8si80si2s2sii4ffiiii6f", b, 0)
        return h, np.frombuffer(b[struct.calcsize("<8s8si80si2s2sii4ffiiii6f"):], np.float32)

    h, rest = header("snp.3d.yz.ps.snp")
    assert h[5] == b"yz" and h[6] == b"ps" and (h[7], h[8]) == (64, 32)
    assert h[9] == np.float32(-32.0) + np.float32(0.5) * np.float32(0.5)   # y of pixel 1: j = 2 - 1 = 1
    assert h[10] == np.float32(-1.5) + np.float32(0.5) * np.float32(0.5)   # z of pixel 1: k = 1
    assert h[11] == np.float32(1.0) and h[12] == np.float32(1.0)
    assert (h[14], h[15], h[16], h[17]) == (10, 10, 3, 4)
    n2 = 64 * 32
    assert rest.size == 3 * n2 + 3 * 4 * n2
    assert np.array_equal(rest[3 * n2:].reshape(3, 4, 32, 64), yz)

    h, rest = header("snp.3d.fs.v.snp")
    assert h[5] == b"fs" and h[6] == b"v3" and (h[7], h[8]) == (64, 64) and (h[16], h[17]) == (6, 3)
    n2 = 64 * 64
    assert rest.size == 4 * n2 + 3 * 3 * n2
    assert 2.6 < rest[:n2].min() and rest[:n2].max() < 3.0  # density just below the free surface
    assert np.array_equal(rest[4 * n2:].reshape(3, 3, 64, 64), fs)
