"""Shared helpers of the test suite: build a GPU simulation from exactly the
arrays the CPU oracle prepared, and the misfit measure used throughout."""
import numpy as np

from openswpc_gb300 import gpu


def misfit(a, b):
    """Relative L2 misfit ||a - b|| / ||b|| over all samples."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def sim_from_oracle(o, store="fp32", nt=None, abc=None, ntdec_r=0, snapshot=None, variant=0):
    """GPU simulation fed with the oracle's medium, surface maps, relaxation
    times, sources and stations (so both sides see identical inputs)."""
    nt = o.nt if nt is None else nt
    na = o.na
    dims = gpu.make_dims(o.nx, o.ny, o.nz, nt, o.dx, o.dy, o.dz, o.dt, na=na,
                         abc=abc or "pml", store=store, xbeg=o.xbeg, ybeg=o.ybeg, zbeg=o.zbeg, tbeg=o.tbeg,
                         fcut=o.fcut, M0=o.M0, UC=o.UC, ntdec_r=ntdec_r, variant=variant)
    s = gpu.Simulation(dims)
    med = [o.medium(n) for n in ("rho", "lam", "mu", "taup", "taus")]
    maps = [o.medium(n) for n in ("kfs", "kob", "kfs_top", "kfs_bot", "kob_top", "kob_bot")]
    ts = o.medium("ts").astype(np.float64)
    s.upload_medium(*med, *maps, ts)
    ijk, vals = o.sources()
    if len(ijk):
        if o.bf_mode:
            s.set_sources(ijk, vals[:, 10:12], fxyz=vals[:, 7:10], stftype=o.stf(), bf_mode=True)
        else:
            s.set_sources(ijk, vals[:, 10:12], mo=vals[:, 0], mij=vals[:, 1:7], stftype=o.stf())
    if o.nst:
        s.set_receivers(o.stations(), ntdec_w=o.ntdec_w, flags=gpu.SWPC_WAV_V)
    if snapshot:
        s.set_snapshot(*snapshot)
    return s


def kupper(t, T):
    """Kupper wavelet of duration T, unit integral: 3 pi / (4 T) sin^3(pi t / T)."""
    t = np.asarray(t, np.float64)
    return np.where((t >= 0) & (t <= T), 3 * np.pi / (4 * T) * np.sin(np.pi * t / T) ** 3, 0.0)


def point_force_velocity(t, xr, fdir, rho, vp, vs, T):
    """Particle velocity (3, len(t)) at offset xr from a point force
    fdir * kupper(t, T) in a homogeneous elastic whole space: the complete
    solution of Aki & Richards (2002, eq. 4.23) -- near field, far P and far S
    terms -- differentiated in time."""
    t = np.asarray(t, np.float64)
    r = float(np.linalg.norm(xr))
    g = np.asarray(xr, np.float64) / r
    tau = np.linspace(r / vp, r / vs, 2001)
    dtau = tau[1] - tau[0]
    near = np.array([np.sum(tau * kupper(tt - tau, T)) * dtau for tt in t])
    u = np.zeros((3, len(t)))
    for i in range(3):
        for j in range(3):
            if fdir[j] == 0:
                continue
            gij, dij = g[i] * g[j], float(i == j)
            u[i] += fdir[j] / (4 * np.pi * rho) * ((3 * gij - dij) / r ** 3 * near
                                                  + gij / (vp * vp * r) * kupper(t - r / vp, T)
                                                  - (gij - dij) / (vs * vs * r) * kupper(t - r / vs, T))
    return np.gradient(u, t[1] - t[0], axis=1)


def write_point_force_case(d, nt=300, T=2.0):
    """Uniform whole space (Vp 6, Vs 3.5 km/s, rho 2.8, Q 1e6), 96^3 cells of
    0.5 km, dt 0.02 s; a vertical unit-direction force with a Kupper pulse of
    T s at the centre; receivers 8 km away along x (pure S plus near field in
    Vz) and along z (pure P plus near field in Vz)."""
    import os
    from openswpc_gb300 import configs
    inf = configs.write_uniform(str(d), nx=96, ny=96, nz=96, nt=nt, dx=0.5, dt=0.02, vp=6.0, vs=3.5, rho=2.8,
                                stations=[("8.0", "0.0", "0.0", "S"), ("0.0", "0.0", "8.0", "P")], bf=(0, 0, 1))
    with open(os.path.join(str(d), "source.dat"), "w") as f:
        f.write("  0.0 0.0 0.0 0.0 %g 0 0 1.0e15\n" % T)
    return inf


def point_force_fit(w, dt, offsets, T=2.0):
    """Best-fit scale and relative residual of each receiver's Vz trace
    against the analytic velocity, samples at t = (i + 1/2) dt (velocity
    lives at half steps)."""
    out = []
    t = (np.arange(w.shape[2]) + 0.5) * dt
    for q, xr in enumerate(offsets):
        v = point_force_velocity(t, xr, (0.0, 0.0, 1.0), 2.8, 6.0, 3.5, T)[2]
        ww = np.asarray(w[q, 2], np.float64)
        a = float(np.dot(ww, v) / np.dot(v, v))
        out.append((a, float(np.linalg.norm(ww - a * v) / np.linalg.norm(ww))))
    return out
