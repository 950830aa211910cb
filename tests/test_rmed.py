"""Host restatement of the random-medium cell rule (configs.rmed_apply) on
the CPU: every cell of a small grid against a scalar, cell-by-cell reading of
src/swpc_3d/m_vmodel_lhm_rmed.f90:161-212 with vcheck
(src/shared/m_fdtool.f90:15-48), in single precision, with the velocity
window narrowed so that vcheck clips both ways; and the periodic wrap of the
field (src/shared/m_rdrmed.f90:73-134)."""
import numpy as np

from openswpc_gb300 import configs

f32 = np.float32


def scalar_cell(bg, xi, k, i, j, kxi0, vmin, vmax, rhomin):
    nzc, nyc, nxc = xi.shape
    r0, vp0, vs0 = f32(bg[0][k + 2]), f32(bg[1][k + 2]), f32(bg[2][k + 2])
    if k < kxi0:
        rho, vp, vs = r0, vp0, vs0
    else:
        x = f32(xi[(k - 1) % nzc, (j - 1) % nyc, (i - 1) % nxc])
        rho = r0 * (f32(1) + f32(0.8) * x)
        vp = vp0 * (f32(1) + x)
        vs = vs0 * (f32(1) + x)
        if vp0 > 0 and vs0 > 0:
            gamma = vp / vs
            if gamma < f32(np.finfo(np.float32).eps):
                gamma = f32(np.sqrt(3.0))
            if vp > vmax or vs > vmax:
                xi2 = (f32(1) + x) * vmax / vp - f32(1)
                vp = vmax
                vs = vmax / gamma
                rho = rho * (f32(1) + f32(0.8) * xi2) / (f32(1) + f32(0.8) * x)
            if vp < vmin or vs < vmin:
                vs = vmin
                vp = vmin * gamma
            if rho < rhomin:
                rho = rhomin
    return rho, rho * vp * vp - f32(2) * rho * vs * vs, rho * vs * vs, vp, vs


def test_rmed_cells_match_scalar_rule():
    nx, ny, nz, dx = 24, 20, 16, 0.5
    bg, xi, kxi0 = configs.gradient_random_fields(nx, ny, nz, dx, -3 * dx, seed=5, eps=0.1)
    # a field smaller than the grid, so that the wrap is exercised
    xi = np.ascontiguousarray(xi[:7, :9, :11])
    vmin, vmax, rhomin = f32(3.2), f32(6.3), f32(2.5)
    rho, lam, mu, qp, qs = configs.rmed_apply(bg, xi, nx, ny, nz, kxi0, vmin=vmin, vmax=vmax, rhomin=rhomin)
    clipped = 0
    for j in range(-2, ny + 4):
        for i in range(-2, nx + 4):
            for k in range(-2, nz + 4):
                r, _, m, vp, vs = scalar_cell(bg, xi, k, i, j, kxi0, vmin, vmax, rhomin)
                q = (j + 2, i + 2, k + 2)
                assert rho[q] == r and mu[q] == f32(f32(r * vs) * vs), (k, i, j)
                lam_ref = r * (f32(vp * vp) - f32(f32(f32(2) * vs) * vs))
                assert lam[q] == lam_ref, (k, i, j)
                clipped += k >= kxi0 and (vs == vmin or vp == vmax)
                assert qp[q] == bg[3][k + 2] and qs[q] == bg[4][k + 2]
    assert clipped > 100
