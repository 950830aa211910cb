"""Output files of the drop-in path: SAC traces (m_sac.f90 layout), native
.snp xy snapshots (header version 6 of m_snap.f90) and the swpc_3d_gpu
command, which reads input.inf and writes both."""
import os
import struct
import subprocess

import numpy as np
import pytest

from openswpc_gb300 import build, configs, gpu

NT = 60


def _inputs(d):
    return configs.write_plain_small(str(d), nt=NT, xy_v_sw=True, z0_xy=0.25, ntdec_s=20, title="outs")


def read_sac(fn):
    b = open(fn, "rb").read()
    fh = np.frombuffer(b[:280], np.float32)
    ih = np.frombuffer(b[280:420], np.int32)
    kh = b[440:632]
    data = np.frombuffer(b[632:], np.float32)
    return fh, ih, kh, data


def read_snp(fn):
    b = open(fn, "rb").read()
    o = 0

    def take(fmt):
        nonlocal o
        v = struct.unpack_from("<" + fmt, b, o)
        o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    h = {}
    h["bin"], h["code"] = take("8s"), take("8s")
    h["ver"] = take("i")
    h["title"] = take("80s")
    h["exedate"] = take("i")
    h["coord"], h["type"] = take("2s"), take("2s")
    h["ns1"], h["ns2"] = take("i"), take("i")
    h["x1"], h["y1"], h["dxs"], h["dys"] = take("4f")
    h["dts"] = take("f")
    h["na1"], h["na2"], h["nmed"], h["nsnp"] = take("4i")
    h["clon"], h["clat"], h["phi"], _, _, _ = take("6f")
    rest = np.frombuffer(b[o:], np.float32)
    return h, rest


@pytest.mark.gpu
def test_sac_and_snp_files(tmp_path):
    inf = _inputs(tmp_path)
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    w = s.waveforms()
    q = s.query()
    frames = [s.snapshot(gpu.SWPC_SNAP_XY_V, f) for f in range(q["nframes"])]
    out = tmp_path / "out"
    s.write_sac(str(out))
    s.write_snp(str(out))
    s.close()

    # SAC: one file per station and component, data = the fetched traces
    fh, ih, kh, data = read_sac(str(out / "wav" / "outs.3d.ST01.Vx.sac"))
    assert ih[6] == 6 and ih[9] == NT and ih[15] == 1
    assert abs(fh[0] - 0.02) < 1e-7
    assert kh[0:8].decode().strip() == "ST01"
    assert kh[160:168].decode().strip() == "Vx"
    assert np.array_equal(data, w[0, 0])
    _, _, _, dz = read_sac(str(out / "wav" / "outs.3d.ST16.Vz.sac"))
    assert np.array_equal(dz, w[15, 2])

    # .snp: header, 4 medium planes, then 3 planes per frame
    h, rest = read_snp(str(out / "outs.3d.xy.v.snp"))
    assert h["bin"] == b"STREAMIO" and h["code"] == b"SWPC_3D " and h["ver"] == 6
    assert h["title"].decode().strip() == "outs"
    assert h["coord"] == b"xy" and h["type"] == b"v3"
    assert (h["ns1"], h["ns2"]) == (128, 128)
    assert h["x1"] == np.float32(-32.0) + np.float32(0.5) * np.float32(0.5)
    assert h["dxs"] == np.float32(0.5) and h["dys"] == np.float32(0.5)
    assert h["dts"] == np.float32(0.02) * np.float32(20)
    assert (h["na1"], h["na2"], h["nmed"], h["nsnp"]) == (20, 20, 6, 3)
    n2 = 128 * 128
    assert rest.size == 4 * n2 + len(frames) * 3 * n2
    assert len(frames) == (NT - 1) // 20 + 1
    rho = rest[:n2]
    assert 2.6 < rho.min() and rho.max() < 3.0  # upper layer density at z0 = 0.25 km
    assert np.all(rest[3 * n2:4 * n2] == np.float32(-0.0) * 1000)  # flat topography at depth 0
    for f, fr in enumerate(frames):
        got = rest[(4 + 3 * f) * n2:(7 + 3 * f) * n2]
        assert np.array_equal(got, fr.ravel())


@pytest.mark.gpu
def test_command_line_driver(tmp_path):
    """swpc_3d_gpu -i input.inf -o odir writes the same traces as the API."""
    build.build()
    inf = _inputs(tmp_path)
    r = subprocess.run([build.DRIVER, "-i", inf, "-o", str(tmp_path / "cli")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    w = s.waveforms()
    s.close()
    _, _, _, d = read_sac(str(tmp_path / "cli" / "wav" / "outs.3d.ST07.Vy.sac"))
    assert np.array_equal(d, w[6, 1])
    assert os.path.getsize(str(tmp_path / "cli" / "outs.3d.xy.v.snp")) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["csf", "tar_st", "tar_node"])
def test_csf_and_tar_trace_formats(tmp_path, fmt):
    """wav_format = csf / tar_st / tar_node hold the same SAC images as the
    per-trace files (m_wav.f90:707-779)."""
    import tarfile
    inf = configs.write_plain_small(str(tmp_path), nt=NT, title="outs", wav_format=fmt)
    s = gpu.Simulation.from_inf(inf)
    s.run(1, NT)
    s.sync()
    w = s.waveforms()
    s.write_sac(str(tmp_path / "o"))
    s.close()
    one = 632 + 4 * NT
    if fmt == "csf":
        b = open(str(tmp_path / "o" / "wav" / "outs__00000__.csf"), "rb").read()
        assert b[:4] == b"CSFD"
        ntr, npts = struct.unpack_from("<2i", b, 4)
        assert (ntr, npts) == (16 * 3, NT) and len(b) == 12 + ntr * one
        for st, c in ((0, 0), (5, 2), (15, 1)):
            o = 12 + (3 * st + c) * one
            assert np.array_equal(np.frombuffer(b[o + 632:o + one], np.float32), w[st, c])
            assert b[o + 440:o + 448].decode().strip() == "ST%02d" % (st + 1)
        return
    fn = "outs.3d.ST03.sac.tar" if fmt == "tar_st" else "outs.3d.000000.sac.tar"
    path = str(tmp_path / "o" / "wav" / fn)
    raw = open(path, "rb").read()
    assert len(raw) % 512 == 0 and raw[-1024:] == b"\0" * 1024
    with tarfile.open(path) as t:
        names = t.getnames()
        assert "outs.ST03.3d.Vz.sac" in names
        assert len(names) == (3 if fmt == "tar_st" else 48)
        img = t.extractfile("outs.ST03.3d.Vz.sac").read()
        m = t.getmember("outs.ST03.3d.Vz.sac")
        assert m.size == one and m.mode == 0o644 and m.uname == "root"
    assert np.array_equal(np.frombuffer(img[632:], np.float32), w[2, 2])
