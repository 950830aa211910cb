"""Device-side medium set-up of a layered model with a random perturbation
(swpc_gpu_build_medium_rmed) against the host set-up of the same cells.

The host path builds every cell of the halo grid with
configs.rmed_apply (the rule of src/swpc_3d/m_vmodel_lhm_rmed.f90:161-212,
vcheck of src/shared/m_fdtool.f90:15-48) and post-processes it with
swpc_host_medium (m_medium.f90:124-394 in FP64) before uploading five full
arrays; the device path receives only the background column and the
periodic field.  The medium fields, the six surface maps, the relaxation
times and the receiver traces of a run must be identical bit for bit.
"""
import numpy as np
import pytest

from openswpc_gb300 import configs, gpu

NX, NY, NZ, DX, DT, NT = 112, 96, 80, 0.25, 0.01, 120


def _sim(nt=NT):
    d = gpu.make_dims(NX, NY, NZ, nt, DX, DX, DX, DT, na=20, xbeg=-NX * DX / 2, ybeg=-NY * DX / 2, zbeg=-3 * DX,
                      fcut=1.0, M0=1e16, UC=1e-15, ntdec_r=20)
    return gpu.Simulation(d)


def _finish(s, maps):
    kfs = maps[0]
    src = np.array([[NX // 2, NY // 2, 30]], np.int32)
    s.set_sources(src, np.array([[0.0, 1.0]]), mo=np.array([1.0]),
                  mij=np.array([[0.3, -0.5, 0.2, 0.6, -0.4, 0.7]]), stftype="kupper")
    ii = np.array([30, 50, 70, 85])
    jj = np.array([30, 45, 60, 70])
    kk = kfs[jj + 2, ii + 2] + 1
    s.set_receivers(np.stack([ii, jj, kk], 1).astype(np.int32), ntdec_w=1, flags=gpu.SWPC_WAV_V)


@pytest.mark.gpu
@pytest.mark.parametrize("clip", [False, True])
def test_device_rmed_medium_equals_host_setup(clip):
    bg, xi, kxi0 = configs.gradient_random_fields(NX, NY, NZ, DX, -3 * DX, seed=11, eps=0.08)
    # a narrowed velocity window makes vcheck clip both ways
    lim = dict(vmin=3.3, vmax=6.4, rhomin=2.6) if clip else dict(vmin=0.0, vmax=float("inf"), rhomin=1.0)
    raw = configs.rmed_apply(bg, xi, NX, NY, NZ, kxi0, **lim)
    if clip:
        sol = raw[2][:, :, kxi0 + 2:] > 0
        vs = np.sqrt(raw[2][:, :, kxi0 + 2:] / raw[0][:, :, kxi0 + 2:])[sol]
        assert vs.min() >= 3.3 * (1 - 1e-6) and (vs > 6.4 * 0.999).sum() == 0
    rho, lam, mu = [np.ascontiguousarray(a) for a in raw[:3]]
    taup, taus, maps_h, ts_h = gpu.host_medium(NX, NY, NZ, 20, 0.05, 5.0, 1.0, rho, lam, mu,
                                               np.ascontiguousarray(raw[3]), np.ascontiguousarray(raw[4]))
    a = _sim()
    a.upload_medium(rho, lam, mu, taup, taus, *maps_h, ts_h)
    b = _sim()
    maps_d, ts_d = b.build_medium_rmed(bg, xi, kxi0, fq_min=0.05, fq_max=5.0, fq_ref=1.0, **lim)
    assert np.array_equal(ts_d, ts_h)
    for m_h, m_d in zip(maps_h, maps_d):
        assert np.array_equal(np.asarray(m_h).reshape(m_d.shape), m_d)
    for name in gpu.MEDIUM_FIELDS:
        fa, fb = a.field(name), b.field(name)
        assert np.array_equal(fa, fb), (name, np.abs(fa - fb).max())
    _finish(a, maps_h)
    _finish(b, maps_d)
    a.run(1, NT)
    b.run(1, NT)
    wa, wb = a.waveforms(), b.waveforms()
    assert np.abs(wa).max() > 0
    assert np.array_equal(wa, wb)
    a.close()
    b.close()
