"""The staggered-grid operators of the stress update, pinned on polynomials
(m_kernel.f90:142-344, coefficients m_kernel.f90:43-54).

Where isign = sign(1, max((k-kfs_top)(kfs_bot-k), (k-kob_top)(kob_bot-k)))
is -1 (m_kernel.f90:188-196) the derivatives are fourth order (9/8, -1/24),
exact on cubics.  Inside the free-surface / ocean-bottom band, edges
included (sign(1,0) = +1), they are second order (1, 0): exact on
quadratics, off by f'''/24 on a cubic.  After one step from a polynomial
velocity field (S = R = 0, no source active), every stress component is a
per-cell constant times one derivative, so stress / expected derivative
must be the same at every checked cell.

The polynomial values are dyadic rationals held exactly in FP32, so the
FP64 oracle must be exact to rounding; the FP32 oracle and the GPU to a
few ulps.  The oracle runs on the CPU; the GPU kernels are reached through
the C ABI (set_field, run, fetch_field)."""
import os

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle

# f(u) = 1/4 + u/2 - 3u^2/8 + u^3/4 with u = (n - c)/8: at half-integer n,
# 2^14 f is an integer below 2^24, so FP32 holds it exactly
A = (0.25, 0.5, -0.375, 0.25)
SCALE = 2.0 ** -30


def _f(n, c):
    u = (n - c) / 8.0
    return A[0] + A[1] * u + A[2] * u * u + A[3] * u ** 3


def _df(n, c):  # d f / d n
    u = (n - c) / 8.0
    return (A[1] + 2 * A[2] * u + 3 * A[3] * u * u) / 8.0


def _d2nd(n, c):  # second-order staggered difference f(n+1/2) - f(n-1/2)
    return _f(n + 0.5, c) - _f(n - 0.5, c)


# (velocity, axis, field offset, stress, derivative offset): a field staggered
# along the axis (offset 1/2) feeds a normal stress at the cell centre, an
# unstaggered one a shear stress at the half point
CASES = [
    ("Vx", "x", 0.5, "Sxx", 0.0),
    ("Vy", "y", 0.5, "Syy", 0.0),
    ("Vz", "z", 0.5, "Szz", 0.0),
    ("Vx", "y", 0.0, "Sxy", 0.5),
    ("Vy", "z", 0.0, "Syz", 0.5),
    ("Vz", "x", 0.0, "Sxz", 0.5),
]
AX = {"x": 1, "y": 0, "z": 2}  # axis of the (ny, nx, nz) arrays


def _halo_field(nx, ny, nz, axis, off, c=None):
    """(ny+6, nx+6, nz+6) array of f along one axis (Fortran index n = -2..N+3),
    centred at index c (the middle of the axis by default)."""
    shape = (ny + 6, nx + 6, nz + 6)
    N = {"x": nx, "y": ny, "z": nz}[axis]
    c = float(N // 2) if c is None else float(c)
    n = np.arange(-2, N + 4, dtype=np.float64)
    v = (_f(n + off, c) * SCALE).astype(np.float32)
    assert np.array_equal(v.astype(np.float64), _f(n + off, c) * SCALE)  # exact in FP32
    sh = [1, 1, 1]
    sh[AX[axis]] = N + 6
    return np.broadcast_to(v.reshape(sh), shape).copy(), c


def _isign(o):
    """isign over the physical cells, (ny, nx, nz), from the oracle's band maps."""
    m = {n: o.medium(n)[3:-3, 3:-3, None] for n in ("kfs_top", "kfs_bot", "kob_top", "kob_bot")}
    k = np.arange(1, o.nz + 1)[None, None, :]
    a = (k - m["kfs_top"]) * (m["kfs_bot"] - k)
    b = (k - m["kob_top"]) * (m["kob_bot"] - k)
    return np.where(np.maximum(a, b) >= 0, 1, -1)


def _expected(shape, axis, doff, c, isign):
    N = shape[AX[axis]]
    n = np.arange(1, N + 1, dtype=np.float64) + doff
    d4, d2 = _df(n, c), _d2nd(n, c)
    sh = [1, 1, 1]
    sh[AX[axis]] = N
    d4 = np.broadcast_to(d4.reshape(sh), shape)
    d2 = np.broadcast_to(d2.reshape(sh), shape)
    return np.where(isign > 0, d2, d4), d4


def _uniform(d):
    inf = configs.write_uniform(str(d), nx=64, ny=64, nz=64, nt=4)
    with open(os.path.join(str(d), "source.dat"), "w") as f:  # starts long after step 1
        f.write("  0.0 0.0 0.0 50.0 1.0 1.0e16 0 0 0 0 0 1\n")
    return inf


def _interior_mask(o, shape, kmax=None):
    """Cells of the interior update box, two cells in from its x/y edges."""
    ny, nx, nz = shape
    na = o.na
    m = np.zeros(shape, bool)
    m[na + 2:ny - na - 2, na + 2:nx - na - 2, :(kmax or nz - na - 2)] = True
    return m


def _ratio_spread(S, D, mask):
    r = S[mask] / D[mask]
    ref = np.median(r)
    assert ref != 0
    return np.abs(r / ref - 1).max(), ref


def _run_oracle(inf, mode, vname, halo):
    o = pyoracle.Oracle(inf, mode)
    o.set_field(vname, halo)
    o.run(1)
    return o


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-11), ("fp32", 1e-5)])
@pytest.mark.parametrize("case", CASES, ids=[c[3] + "_d" + c[1] for c in CASES])
def test_fourth_order_exact_on_cubics(tmp_path, mode, tol, case):
    vname, axis, off, sname, doff = case
    inf = _uniform(tmp_path)
    o0 = pyoracle.Oracle(inf, mode)
    halo, c = _halo_field(o0.nx, o0.ny, o0.nz, axis, off)
    isign = _isign(o0)
    o0.close()
    o = _run_oracle(inf, mode, vname, halo)
    S = o.field(sname)
    shape = S.shape
    D, D4 = _expected(shape, axis, doff, c, isign)
    mask = _interior_mask(o, shape) & (isign < 0)
    mask[:, :, :6] = False
    assert mask.sum() > 1000
    spread, _ = _ratio_spread(S, D, mask)
    assert spread < tol, (sname, axis, spread)
    # a second-order operator would be visibly off on this cubic
    spread2, _ = _ratio_spread(S, np.broadcast_to(_expected(shape, axis, doff, c, np.ones_like(isign))[0], shape), mask)
    assert spread2 > 100 * tol
    o.close()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-11), ("fp32", 1e-5)])
def test_free_surface_band_is_second_order(tmp_path, mode, tol):
    """Two-layer model with air on top: the band around kfs is second order
    (isign = +1, edges included), the cells below it fourth order."""
    inf = configs.write_plain_small(str(tmp_path), nt=4)
    o0 = pyoracle.Oracle(inf, mode)
    halo, c = _halo_field(o0.nx, o0.ny, o0.nz, "z", 0.5, c=6)  # f' small at the band
    isign = _isign(o0)
    mu = o0.medium("mu")[3:-3, 3:-3, 3:-3]
    o0.close()
    o = _run_oracle(inf, mode, "Vz", halo)
    S = o.field("Szz")
    D, D4 = _expected(S.shape, "z", 0.0, c, isign)
    # solid cells of the top layer (z < 4 km: k <= 10), far from the source
    mask = _interior_mask(o, S.shape, kmax=10) & (mu > 0)
    band = mask & (isign > 0)
    deep = mask & (isign < 0)
    assert band.sum() > 1000 and deep.sum() > 1000
    spread, _ = _ratio_spread(S, D, mask)
    assert spread < tol, spread
    spread4, _ = _ratio_spread(S, D4, mask)  # fourth order everywhere would not fit
    assert spread4 > 20 * tol
    o.close()


def _gpu_stress(inf, vname, halo, sname):
    s = gpu.Simulation.from_inf(inf)
    s.set_field(vname, halo)
    s.run(1, 1)
    s.sync()
    S = s.field(sname)
    s.close()
    return S


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[3] + "_d" + c[1] for c in CASES])
def test_gpu_fourth_order_exact_on_cubics(tmp_path, case):
    vname, axis, off, sname, doff = case
    inf = _uniform(tmp_path)
    o = pyoracle.Oracle(inf, "fp32")
    halo, c = _halo_field(o.nx, o.ny, o.nz, axis, off)
    isign = _isign(o)
    o.set_field(vname, halo)
    o.run(1)
    ref = o.field(sname)
    S = _gpu_stress(inf, vname, halo, sname)
    D, _ = _expected(S.shape, axis, doff, c, isign)
    mask = _interior_mask(o, S.shape) & (isign < 0)
    mask[:, :, :6] = False
    spread, _ = _ratio_spread(S, D, mask)
    assert spread < 1e-5, (sname, axis, spread)
    # and the whole field (PML shell included) equals the oracle's
    err = np.linalg.norm(S - ref) / np.linalg.norm(ref)
    assert err < 1e-6, err
    o.close()


@pytest.mark.gpu
def test_gpu_free_surface_band_is_second_order(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=4)
    o = pyoracle.Oracle(inf, "fp32")
    halo, c = _halo_field(o.nx, o.ny, o.nz, "z", 0.5, c=6)
    isign = _isign(o)
    mu = o.medium("mu")[3:-3, 3:-3, 3:-3]
    S = _gpu_stress(inf, "Vz", halo, "Szz")
    D, D4 = _expected(S.shape, "z", 0.0, c, isign)
    mask = _interior_mask(o, S.shape, kmax=10) & (mu > 0)
    spread, _ = _ratio_spread(S, D, mask)
    assert spread < 1e-5, spread
    spread4, _ = _ratio_spread(S, D4, mask)
    assert spread4 > 2e-4
    o.close()
