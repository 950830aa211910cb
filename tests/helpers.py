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
