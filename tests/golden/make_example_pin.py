"""Build tests/golden/example_384.json: the reference's own example run as a
known answer for the parity tests (test infrastructure only).

The reference ships one run log, example/example.out, written by swpc_3d for
example/input.inf (384^3 grid, dx = 0.5 km, dt = 0.02 s, nt = 1000, layered
'lhm' model of example/lhm.dat, an isotropic source of example/source.dat at
2 km depth, the 19 stations of example/stloc.xy, 20-cell PML, 2 x 2 MPI
ranks).  Its banner (src/swpc_3d/m_report.f90:71-88) and the max |V| at the
ocean bottom every 50 steps (report__progress, m_report.f90:120-181, through
kernel__vmax, m_kernel.f90:350-374) are printed to 3 significant figures.

This script reads those files from a checkout of the reference and writes a
compact fixture: the input.inf keys (comment-free key/value text), the rows
of the three data files it names, the banner numbers and the progress
triples.  With --oracle it also runs the CPU oracle (mixed precision, the
reference's default MP = DP build) over the whole example and stores the
oracle's own progress triples, so that a CPU test can hold the oracle to the
reference's log without rerunning it (the run takes minutes on 8 cores).

Usage:  python tests/golden/make_example_pin.py [--ref DIR] [--oracle]
"""
import argparse
import json
import os
import re
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "example_384.json")


def data_rows(path):
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if s and not s.startswith("#"):
                rows.append(s)
    return rows


def inf_keys(path):
    """key = value pairs of input.inf without comments (m_readini.f90:29-166
    reads the first value after '=' and ignores text after '!!')."""
    keys = []
    with open(path) as f:
        for line in f:
            s = line.split("!!")[0].strip()
            m = re.match(r"^([A-Za-z_][A-Za-z0-9_%]*)\s*=\s*(.+)$", s)
            if m:
                keys.append([m.group(1), m.group(2).strip()])
    return keys


def parse_log(path):
    banner, prog = {}, []
    pats = {
        "mem_total_gib": r"Total Memory Size\s*:\s*([0-9.Ee+-]+)",
        "mem_node_gib": r"Node Memory Size\s*:\s*([0-9.Ee+-]+)",
        "c": r"Stability\s+Condition c\s*:\s*([0-9.Ee+-]+)",
        "r": r"Wavelength Condition r\s*:\s*([0-9.Ee+-]+)",
        "vmin": r"Minimum velocity\s*:\s*([0-9.Ee+-]+)",
        "vmax": r"Maximum velocity\s*:\s*([0-9.Ee+-]+)",
        "fmax": r"Maximum frequency\s*:\s*([0-9.Ee+-]+)",
    }
    with open(path) as f:
        text = f.read()
    for k, p in pats.items():
        m = re.search(p, text)
        banner[k] = float(m.group(1))
    m = re.search(r"Grid Size\s*:\s*(\d+)\s*x\s*(\d+)\s*x\s*(\d+)", text)
    banner["grid"] = [int(m.group(i)) for i in (1, 2, 3)]
    m = re.search(r"MPI Partitioning\s*:\s*(\d+)\s*x\s*(\d+)", text)
    banner["nproc"] = [int(m.group(1)), int(m.group(2))]
    m = re.search(r"version\s+(\S+)", text)
    banner["version"] = m.group(1)
    for m in re.finditer(r"it=(\d+),.*\(\s*([0-9.Ee+-]+)\s+([0-9.Ee+-]+)\s+([0-9.Ee+-]+)\s*\)", text):
        prog.append([int(m.group(1)), m.group(2), m.group(3), m.group(4)])
    return banner, prog


def write_case(fx, d):
    """Write the example's input.inf and data files into directory d with
    the file keys pointing at the local copies; returns the input.inf path."""
    names = {"fn_lhm": "lhm.dat", "fn_stf": "source.dat", "fn_stloc": "stloc.xy"}
    with open(os.path.join(d, "input.inf"), "w") as f:
        for k, v in fx["inf"]:
            if k in names:
                v = "'%s'" % names[k]
            elif k == "odir":
                v = "'./out'"
            f.write("%s = %s\n" % (k, v))
    for fn, rows in fx["files"].items():
        with open(os.path.join(d, fn), "w") as f:
            f.write("\n".join(rows) + "\n")
    return os.path.join(d, "input.inf")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference", help="checkout of the reference")
    ap.add_argument("--oracle", action="store_true", help="also run the CPU oracle over the example")
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    ex = os.path.join(a.ref, "example")
    banner, prog = parse_log(os.path.join(ex, "example.out"))
    fx = {
        "source": "example/input.inf, lhm.dat, source.dat, stloc.xy and example.out of the reference",
        "inf": inf_keys(os.path.join(ex, "input.inf")),
        "files": {"lhm.dat": data_rows(os.path.join(ex, "lhm.dat")),
                  "source.dat": data_rows(os.path.join(ex, "source.dat")),
                  "stloc.xy": data_rows(os.path.join(ex, "stloc.xy"))},
        "banner": banner,
        "progress": prog,
    }
    if os.path.exists(OUT):
        with open(OUT) as f:
            old = json.load(f)
        if "oracle_mixed" in old:
            fx["oracle_mixed"] = old["oracle_mixed"]
    if a.oracle:
        from oracle import pyoracle
        with tempfile.TemporaryDirectory() as d:
            inf = write_case(fx, d)
            o = pyoracle.Oracle(inf, "mixed", a.threads)
            o.run(o.nt)
            # report__progress prints max |V| * UC * M0 (m_report.f90:157)
            sc = o.UC * o.M0
            fx["oracle_mixed"] = [[int(r[0]), float(r[1]) * sc, float(r[2]) * sc, float(r[3]) * sc]
                                  for r in o.vmax_log()]
            o.close()
    with open(OUT, "w") as f:
        json.dump(fx, f, indent=1)
    print(OUT, len(prog), "progress lines", "(with oracle)" if "oracle_mixed" in fx else "")


if __name__ == "__main__":
    main()
