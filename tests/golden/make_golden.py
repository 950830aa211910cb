"""Regenerate the golden receiver traces under tests/golden/ with the CPU
oracle (test infrastructure; the product never reads these files except
through the tests).

plain_small_nt200.npz: the small plain configuration (128 x 128 x 64,
dx = 0.5 km, dt = 0.02 s, two-layer viscoelastic medium, free surface,
20-cell PML, one double couple at 10 km depth, 16 surface receivers), seed
20261203, 200 time steps, receiver velocity traces from the oracle built in
fp32 (the reference rebuilt with MP = SP), mixed (the reference default
MP = DP) and fp64.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from openswpc_gb300 import configs  # noqa: E402
from oracle import pyoracle  # noqa: E402

NT = 200
SEED = 20261203


def write_inputs(d):
    return configs.write_plain_small(d, seed=SEED, nt=NT)


def main():
    with tempfile.TemporaryDirectory() as d:
        inf = write_inputs(d)
        out = {}
        for mode in ("fp32", "mixed", "fp64"):
            o = pyoracle.Oracle(inf, mode)
            o.run(NT)
            out[mode] = o.waveforms().astype(np.float32 if mode == "fp32" else np.float64)
            out["stations"] = o.stations()
    path = os.path.join(HERE, "plain_small_nt200.npz")
    np.savez_compressed(path, nt=NT, seed=SEED, **out)
    print(path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
