"""PML kernels: one and two shell points per thread evaluate the same
expressions in the same order, so the wavefields agree bit for bit, both
when the shell runs as one general launch (small grid) and when it runs in
the per-axis launch classes (a shell of at least 4 M points)."""
import numpy as np
import pytest

from openswpc_gb300 import configs, gpu


def _sim(n, pml_points, nt=30):
    nx, ny, nz = n
    dx, dt = 0.25, 0.01
    d = gpu.make_dims(nx, ny, nz, nt, dx, dx, dx, dt, na=20, xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=-3 * dx,
                      fcut=1.0, M0=1e16, UC=1e-15, pml_points=pml_points)
    s = gpu.Simulation(d)
    bg, xi, kxi0 = configs.gradient_random_fields(nx, ny, nz, dx, -3 * dx, seed=3)
    s.build_medium_rmed(bg, xi, kxi0)
    # sources next to two opposite corners of the shell, so that every
    # launch class sees signal within a few steps
    s.set_sources(np.array([[24, 26, 12], [nx - 23, ny - 25, nz - 22]], np.int32), np.array([[0.0, 0.1]] * 2),
                  mo=np.array([0.5, 0.5]), mij=np.array([[0.3, -0.5, 0.2, 0.6, -0.4, 0.7]] * 2), stftype="kupper")
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(96, 80, 64), (288, 288, 144)])
@pytest.mark.parametrize("other", [2, 0])
def test_two_points_per_thread_equal_one(n, other):
    a, b = _sim(n, 1), _sim(n, other)
    a.run(1, 30)
    b.run(1, 30)
    for name in gpu.FIELDS:
        fa, fb = a.field(name), b.field(name)
        assert np.abs(fa).max() > 0, name
        assert np.array_equal(fa, fb), name
    a.close()
    b.close()
