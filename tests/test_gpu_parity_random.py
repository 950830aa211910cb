"""Parity on the large single-source workload's medium, at a size the CPU
oracle runs in seconds.

The 1024 x 1024 x 512 workload's medium (a 1-D gradient Vp 5 -> 7 km/s with
Vs = Vp/1.73, rho = 1.74 Vp^0.25, times a seeded 5 % exponential von Karman
field applied per point, src/swpc_3d/m_vmodel_lhm_rmed.f90:187-206) varies at
every grid point, so the harmonic mean of mu and the buoyancy of every cell
enter the stencils, not only those at layer interfaces.  Here the same
generator builds a 192 x 192 x 128 grid at the workload's spacing
(dx = 0.25 km, dt = 0.01 s), with the source depth scaled from 15 km of a
128 km deep model to 3.75 km of a 32 km deep one, 64 surface receivers on an
8 x 8 lattice and 600 steps.  The GPU path and the fp32 oracle (the
reference rebuilt with MP = SP) get identical inputs; the receiver misfit
must be <= 1e-5 relative L2, and the misfit against the fp64 oracle is
stated.
"""
import numpy as np
import pytest

from openswpc_gb300 import configs
from oracle import pyoracle
from tests.helpers import misfit, sim_from_oracle

TOL = 1e-5
NX, NY, NZ, DX, DT, NT = 192, 192, 128, 0.25, 0.01, 600
SEED = 20261203


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("random_medium"))
    return configs.write_random_medium_case(d, nx=NX, ny=NY, nz=NZ, dx=DX, dt=DT, nt=NT, seed=SEED)


@pytest.mark.gpu
def test_random_medium_waveforms_match_oracle(case):
    inf, med = case
    o = pyoracle.Oracle(inf, "fp32", medium=med)
    assert o.nst == 64
    s = sim_from_oracle(o, ntdec_r=o.ntdec_r)
    o.run(NT)
    s.run(1, NT)
    s.sync()
    w, w32 = s.waveforms(), o.waveforms()
    vmax_gpu = s.vmax()
    s.close()
    o.close()
    o64 = pyoracle.Oracle(inf, "fp64", medium=med)
    o64.run(NT)
    w64 = o64.waveforms()
    o64.close()
    m32, m64 = misfit(w, w32), misfit(w, w64)
    print("random medium 192x192x128, %d steps: misfit vs fp32 oracle %.3e, vs fp64 oracle %.3e (fp32 oracle vs "
          "fp64 oracle %.3e)" % (NT, m32, m64, misfit(w32, w64)))
    # every receiver saw the P and S arrivals
    assert np.all(np.abs(w32).max(axis=2) > 0)
    assert m32 <= TOL, m32
    assert m64 <= TOL, m64
    assert np.all(np.isfinite(vmax_gpu)) and vmax_gpu.max() > 0
