"""Parity pinned to the reference's own run: example/input.inf and its log
example/example.out (tests/golden/example_384.json, made by
tests/golden/make_example_pin.py from the reference's example directory).

The log holds the run banner of report__setup (src/swpc_3d/m_report.f90:71-88)
and, every ntdec_r = 50 steps, max |V| at the ocean bottom * UC * M0
(report__progress, m_report.f90:120-181, through kernel__vmax,
m_kernel.f90:350-374), both to 3 significant figures (F15.3 and ES9.2).

* CPU: the host set-up's banner numbers (c, r, vmin, vmax, fmax) equal the
  log's; the CPU oracle's progress triples over the whole 1000-step run
  (mixed precision, the reference's default MP = DP build; stored in the
  fixture by make_example_pin.py --oracle) print as the log's.
* GPU: swpc_3d_gpu -i input.inf prints the same banner numbers and the same
  20 progress lines as the log.

The log was written by version 25.01; the reference source is 25.05.2.  Its
memory estimate (13.292 GiB) is not what 25.05.2's memory_size_3d
(src/shared/m_fdtool.f90:137-187) computes for this run (11.925 GiB), so the
memory line is checked against the 25.05.2 formula instead.
"""
import json
import math
import os
import re
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_example_pin import write_case  # noqa: E402

with open(os.path.join(HERE, "golden", "example_384.json")) as _f:
    FX = json.load(_f)


def es92(v):
    """Fortran ES9.2 as the progress line prints it (3 significant figures)."""
    return "%.2E" % v


def mem_estimate(nx, ny, nz, na, nm, npx, npy):
    """memory_size_3d of src/shared/m_fdtool.f90:137-187 (version 25.05.2)."""
    nxp, nyp = math.ceil(nx / npx), math.ceil(ny / npy)
    rn_com = (nxp + 6) * npx * (nyp + 6) * npy * (nz + 6)
    rn_int = (nx - 2 * na) * (ny - 2 * na) * (nz - na)
    rn_abc = nx * ny * nz - (nx - 2 * nxp) * (ny - 2 * nyp) * (nz - na)
    return ((5 * 4 + 3 * 8 + 6 * 8) * rn_com + 6 * nm * 4 * rn_int + 18 * 4 * rn_abc) / 1024.0 ** 3


def check_banner(b):
    ref = FX["banner"]
    for k in ("c", "r", "vmin", "vmax", "fmax"):
        assert "%.3f" % b[k] == "%.3f" % ref[k], (k, b[k], ref[k])
    assert list(b["nproc"]) == ref["nproc"]
    nx, ny, nz = ref["grid"]
    m = mem_estimate(nx, ny, nz, 20, 3, *ref["nproc"])
    assert abs(b["mem_total_gib"] - m) <= 1e-3 * m, (b["mem_total_gib"], m)


def test_host_banner_matches_reference_log(tmp_path):
    from openswpc_gb300 import gpu
    inf = write_case(FX, str(tmp_path))
    s = gpu.host_check(inf)
    assert (s["nx"], s["ny"], s["nz"], s["nt"]) == (384, 384, 384, 1000)
    check_banner(s["banner"])


def test_oracle_progress_matches_reference_log():
    """The oracle (mixed precision) over all 1000 steps of the example prints
    every progress triple of the log to its 3 significant figures."""
    if "oracle_mixed" not in FX:
        pytest.skip("fixture made without --oracle")
    got = FX["oracle_mixed"]
    ref = FX["progress"]
    assert [int(r[0]) for r in got] == [int(r[0]) for r in ref]
    for g, r in zip(got, ref):
        assert [es92(v) for v in g[1:]] == r[1:], (g, r)


def parse_run(text):
    banner = {}
    pats = {"c": r"Stability\s+Condition c\s*:\s*(\S+)", "r": r"Wavelength Condition r\s*:\s*(\S+)",
            "vmin": r"Minimum velocity\s*:\s*(\S+)", "vmax": r"Maximum velocity\s*:\s*(\S+)",
            "fmax": r"Maximum frequency\s*:\s*(\S+)", "mem_total_gib": r"Total Memory Size\s*:\s*(\S+)"}
    for k, p in pats.items():
        banner[k] = float(re.search(p, text).group(1))
    m = re.search(r"MPI Partitioning\s*:\s*(\d+)\s*x\s*(\d+)", text)
    banner["nproc"] = [int(m.group(1)), int(m.group(2))]
    prog = [[int(m.group(1)), m.group(2), m.group(3), m.group(4)]
            for m in re.finditer(r"it=(\d+),.*\(\s*(\S+)\s+(\S+)\s+(\S+)\s*\)", text)]
    return banner, prog


@pytest.mark.gpu
def test_gpu_example_run_matches_reference_log(tmp_path):
    """The reference's example, run as shipped through the drop-in command
    (swpc_3d_gpu -i input.inf, FP32 on the GPU): banner numbers and all 20
    progress lines (max |V| at the ocean bottom every 50 steps) equal the
    reference's log to the 3 significant figures it prints."""
    from openswpc_gb300 import build
    build.build()
    inf = write_case(FX, str(tmp_path))
    r = subprocess.run([build.DRIVER, "-i", inf], cwd=str(tmp_path), stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    print(r.stderr)
    banner, prog = parse_run(r.stderr)
    check_banner(banner)
    ref = FX["progress"]
    assert [p[0] for p in prog] == [q[0] for q in ref]
    bad = [(p, q) for p, q in zip(prog, ref) if p[1:] != q[1:]]
    assert not bad, bad
    # the receivers of stloc.xy were written as SAC files
    wav = os.path.join(str(tmp_path), "out", "wav")
    assert len([f for f in os.listdir(wav) if f.endswith(".sac")]) == 9
