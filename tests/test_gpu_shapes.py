"""Parity on grids whose sizes are not multiples of the kernels' tiles, with
absorbing layers of other widths: interior tiles end part-way in x, y and z,
the PML boxes have odd widths, and the z chunks do not divide the depth.

For each shape, all nine wavefields after 40 steps (GPU fed with the
oracle's own arrays) and the receiver traces of the drop-in path
(input.inf -> host set-up -> GPU) after 160 steps against the fp32 oracle:
relative L2 <= 1e-5."""
import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit, sim_from_oracle

TOL = 1e-5
NT = 160
# (nx, ny, nz, na, abc_type)
SHAPES = [(101, 77, 53, 12, "pml"), (67, 130, 41, 8, "pml"), (90, 70, 45, 10, "cerjan")]


def _inf(d, nx, ny, nz, na, abc):
    return configs.write_plain_small(str(d), nt=NT, nx=nx, ny=ny, nz=nz, na=na, abc_type=abc,
                                     xbeg=-nx * 0.25, ybeg=-ny * 0.25)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%dx%d_na%d_%s" % s for s in SHAPES])
def test_odd_shapes_match_oracle(tmp_path, shape):
    inf = _inf(tmp_path, *shape)
    o = pyoracle.Oracle(inf, "fp32")
    s = sim_from_oracle(o, abc=shape[4])
    o.run(40)
    s.run(1, 40)
    s.sync()
    worst = max(misfit(s.field(n), o.field(n)) for n in pyoracle.FIELDS)
    s.close()
    o.run(NT - 40)
    ref = o.waveforms()
    d = gpu.Simulation.from_inf(inf)
    d.run(1, NT)
    d.sync()
    w = d.waveforms()
    d.close()
    assert np.abs(ref).max() > 0
    mw = misfit(w, ref)
    print("%s: fields after 40 steps %.2e, traces after %d steps %.2e" % (shape, worst, NT, mw))
    assert worst <= TOL and mw <= TOL
