"""PML shell: its launches of its own with one and two shell points per
thread, and the sweep of the shell inside the TMA tile kernels, evaluate the
same expressions in the same order, so the wavefields agree bit for bit, both
when the shell launches run as one general launch (small grid) and when they
run in the per-axis launch classes (a shell of at least 4 M points)."""
import numpy as np
import pytest

from openswpc_gb300 import configs, gpu


def _same(fa, fb, name):
    """Bit-equal fields, or an assertion naming where they differ."""
    if np.array_equal(fa, fb):
        return
    bad = np.argwhere(fa != fb)
    raise AssertionError("%s: %d points differ, first (j, i, k) %s, last %s, max |diff| %g"
                         % (name, len(bad), tuple(bad[0]), tuple(bad[-1]), np.abs(fa - fb).max()))


def _sim(n, pml_points, nt=30, fused=False, store="fp32", na=20):
    nx, ny, nz = n
    dx, dt = 0.25, 0.01
    d = gpu.make_dims(nx, ny, nz, nt, dx, dx, dx, dt, na=na, xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=-3 * dx,
                      fcut=1.0, M0=1e16, UC=1e-15, pml_points=pml_points, pml_fused=fused, store=store)
    s = gpu.Simulation(d)
    assert s.pml_fused == fused
    bg, xi, kxi0 = configs.gradient_random_fields(nx, ny, nz, dx, -3 * dx, seed=3)
    s.build_medium_rmed(bg, xi, kxi0)
    # sources next to two opposite corners of the shell, so that every
    # launch class sees signal within a few steps
    s.set_sources(np.array([[na + 4, na + 6, 12], [nx - na - 3, ny - na - 5, nz - na - 2]], np.int32),
                  np.array([[0.0, 0.1]] * 2),
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


@pytest.mark.gpu
@pytest.mark.parametrize("n,store,na,rows", [((96, 80, 64), "fp32", 20, (8, 8)), ((100, 84, 70), "fp32", 13, (8, 8)),
                                             ((288, 288, 144), "fp32", 20, (8, 8)), ((100, 84, 70), "fp16", 20, (8, 8)),
                                             ((100, 84, 70), "fp32", 20, (16, 12)), ((96, 80, 64), "fp32", 20, (16, 16))])
def test_shell_in_tile_kernels_equals_shell_launches(n, store, na, rows):
    """The tile kernels' sweep of the shell (x origin left of the grid, edge
    tiles loading from x < 0, odd interior widths, the z layer below the
    interior, every tile shape) against the shell's own launches, every
    wavefield bit for bit."""
    a, b = _sim(n, 0, fused=False, store=store, na=na), _sim(n, 0, fused=True, store=store, na=na)
    b.set_tiles(*rows)
    a.run(1, 30)
    b.run(1, 30)
    for name in gpu.FIELDS:
        fa, fb = a.field(name), b.field(name)
        assert np.abs(fa).max() > 0, name
        _same(fa, fb, name)
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("persistent", [False, True])
def test_shell_in_tile_kernels_batched(persistent):
    """Batched members whose tile kernels sweep the shell against the same
    simulations run alone with the shell's own launches."""
    sizes = [(96, 80, 64), (100, 84, 70), (64, 96, 72)]
    alone = [_sim(n, 0, fused=False) for n in sizes]
    members = [_sim(n, 0, fused=True) for n in sizes]
    for s in alone:
        s.run(1, 30)
    b = gpu.Batch(members, persistent=persistent)
    b.run(30)
    b.sync()
    for s, m in zip(alone, members):
        for name in gpu.FIELDS:
            _same(s.field(name), m.field(name), name)
    b.close()
    for s in alone + members:
        s.close()
