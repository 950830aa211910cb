"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point of include/swpc_gpu.h, the host set-up (input.inf parsing,
medium post-processing, sources, stations) agrees with the oracle, and bad
inputs fail with an error code instead of exiting."""
import os
import re

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "swpc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(swpc_(?:gpu|host|batch|serve)_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = gpu.lib()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(gpu.EXPORTS)


def test_required_bytes_of_the_large_workload():
    d = gpu.make_dims(1024, 1024, 512, 4000, 0.25, 0.25, 0.25, 0.01)
    b = gpu.required_bytes(d)
    # 14 halo fields + 18 interior memory variables + 18 shell ADE arrays
    assert 65e9 < b < 80e9, b


def test_host_setup_matches_oracle(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=50)
    h = gpu.host_check(inf)
    o = pyoracle.Oracle(inf, "fp32")
    assert (h["nx"], h["ny"], h["nz"], h["nt"], h["na"]) == (o.nx, o.ny, o.nz, o.nt, o.na)
    assert abs(h["M0"] - o.M0) / o.M0 < 1e-6
    assert abs(h["fcut"] - o.fcut) < 1e-6
    assert np.allclose(h["ts"], o.medium("ts"), rtol=1e-6)
    src = [tuple(int(v) for v in s.split(",")) for s in h["src"].split(";")]
    assert src == [tuple(r) for r in o.sources()[0]]
    sta = [tuple(int(v) for v in s.split(",")) for s in h["sta"].split(";")]
    assert sta == [tuple(r) for r in o.stations()]


def test_two_phase_load_needs_no_gpu(tmp_path):
    """swpc_host_load runs the whole host set-up without a device and knows
    the device bytes the simulation will take before it is created."""
    inf = configs.write_plain_small(str(tmp_path), nt=50)
    r = gpu.Request(inf)
    d = r.dims
    h = gpu.host_check(inf)
    assert (d.nx, d.ny, d.nz, d.nt, d.na) == (h["nx"], h["ny"], h["nz"], h["nt"], h["na"])
    assert abs(d.M0 - h["M0"]) <= 1e-9 * h["M0"]
    assert r.device_bytes == gpu.required_bytes(d)
    r.close()
    with pytest.raises(gpu.SwpcError):
        gpu.Request(os.path.join(str(tmp_path), "missing.inf"))


def test_host_medium_matches_oracle(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=5, nx=64, ny=64, nz=48, xbeg=-16.0, ybeg=-16.0)
    o = pyoracle.Oracle(inf, "fp64")
    # raw two-layer model over the halo grid, as m_vmodel_lhm builds it
    nx, ny, nz = 64, 64, 48
    z = -1.5 + (np.arange(-2, nz + 4) - 0.5) * 0.5
    shape = (ny + 6, nx + 6, nz + 6)
    rho = np.empty(shape, np.float32); lam = np.empty(shape, np.float32); mu = np.empty(shape, np.float32)
    qp = np.empty(shape, np.float32); qs = np.empty(shape, np.float32)
    for k, zk in enumerate(z):
        if zk < 0:
            r, vp, vs, a, b = 0.001, 0, 0, 10, 10
        elif zk < 4:
            r, vp, vs, a, b = 2.7, 5.5, 3.2, 200, 100
        else:
            r, vp, vs, a, b = 2.9, 6.5, 3.7, 600, 300
        rho[..., k] = r; mu[..., k] = r * vs * vs; lam[..., k] = r * (vp * vp - 2 * vs * vs)
        qp[..., k] = a; qs[..., k] = b
    taup, taus, maps, ts = gpu.host_medium(nx, ny, nz, 20, 0.05, 5.0, 1.0, rho, lam, mu, qp, qs)
    for name, arr in (("rho", rho), ("lam", lam), ("mu", mu), ("taup", taup), ("taus", taus)):
        ref = o.medium(name)
        err = np.max(np.abs(arr - ref)) / np.max(np.abs(ref))
        assert err < 2e-6, (name, err)
    for q, name in enumerate(("kfs", "kob", "kfs_top", "kfs_bot", "kob_top", "kob_bot")):
        ref = o.medium(name)
        assert np.array_equal(maps[q][2:-2, 2:-2], ref[2:-2, 2:-2]), name


def test_readini_semantics(tmp_path):
    d = str(tmp_path)
    inf = configs.write_plain_small(d, nt=7)
    txt = open(inf).read()
    # comments and a later duplicate must not win; inline comments are ignored
    txt = txt.replace("  nt               = 7\n", "# nt = 99\n  nt  =  11   !! steps\n  nt = 12\n")
    open(inf, "w").write(txt)
    assert gpu.host_check(inf)["nt"] == 11


def test_strict_mode_rejects_missing_keys(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=7)
    txt = open(inf).read().replace("strict_mode      = .false.", "strict_mode      = .true.")
    txt = txt.replace("  ntdec_r          = 50\n", "")
    open(inf, "w").write(txt)
    with pytest.raises(gpu.SwpcError):
        gpu.host_check(inf)


def test_bad_inputs_fail_with_error_codes(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=7)
    txt = open(inf).read().replace("abc_type         = 'pml'", "abc_type         = 'sponge'")
    open(inf, "w").write(txt)
    with pytest.raises(gpu.SwpcError):
        gpu.host_check(inf)
    with pytest.raises(gpu.SwpcError):
        gpu.host_check(os.path.join(str(tmp_path), "does_not_exist.inf"))
    # a source in the grid sleeve but below the model space (zend = 30.5 km)
    # trips the reference's assertion (m_source.f90:277-281) ...
    inf2 = configs.write_plain_small(os.path.join(str(tmp_path), "b"), nt=7)
    with open(os.path.join(os.path.dirname(inf2), "source.dat"), "w") as f:
        f.write("0.0 0.0 30.8 0.0 1.0 1.0e16 0 45 90\n")
    with pytest.raises(gpu.SwpcError):
        gpu.host_check(inf2)
    # ... while one far outside the grid is dropped, as the reference drops
    # source grids outside the node (m_source.f90:200-218)
    with open(os.path.join(os.path.dirname(inf2), "source.dat"), "w") as f:
        f.write("0.0 0.0 500.0 0.0 1.0 1.0e16 0 45 90\n")
    assert gpu.host_check(inf2)["nsrc"] == 0


def test_create_rejects_bad_dims():
    d = gpu.make_dims(30, 30, 30, 10, 0.5, 0.5, 0.5, 0.02, na=20)
    assert gpu.required_bytes(d) < 0  # na leaves no interior
    d = gpu.make_dims(64, 64, 64, 10, 0.5, 0.5, 0.5, 0.02, na=10)
    d.nm = 2
    assert gpu.required_bytes(d) < 0  # nm must be 3


def test_green_mode_host_setup(tmp_path):
    """green_mode: no regular source grid, one body-force pseudo source at
    the station, no station recording (m_source.f90:84-91, m_wav.f90:76-82)."""
    inf = configs.write_green(str(tmp_path), nt=20)
    h = gpu.host_check(inf)
    assert h["nsrc"] == 1 and h["nst"] == 0
    assert h["M0"] == 1.0 and h["fcut"] == 0.0
