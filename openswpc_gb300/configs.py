"""Synthetic swpc_3d inputs with the shapes of the benchmark workloads.

Every generator writes the same file set the reference reads -- an
``input.inf`` (key = value, src/shared/m_readini.f90), a layered-model table
(``fn_lhm``, src/swpc_3d/m_vmodel_lhm.f90:78-89), a source-grid file
(``fn_stf``, src/swpc_3d/m_source.f90:468-700) and an ``xy`` station file
(src/swpc_3d/m_wav.f90:141-271) -- so the same directory can be handed to
the GPU driver, to the Python front end or to the CPU oracle.  All random
choices come from ``numpy.random.default_rng(seed)``.
"""
import os
import numpy as np

DEFAULT_SEED = 20261203


def _fmt(v):
    if isinstance(v, bool):
        return ".true." if v else ".false."
    if isinstance(v, str):
        return "'%s'" % v
    if isinstance(v, float):
        return repr(v)
    return str(v)


def write_inf(path, keys):
    with open(path, "w") as f:
        f.write("!! swpc_3d input file (synthetic workload)\n")
        for k, v in keys.items():
            f.write("  %-16s = %s\n" % (k, _fmt(v)))


def write_lhm(path, rows):
    with open(path, "w") as f:
        f.write("# depth  rho(g/cm^3)  vp(km/s)  vs(km/s)  Qp  Qs\n")
        for r in rows:
            f.write("  " + "  ".join("%.6g" % x for x in r) + "\n")


def base_keys(**kw):
    keys = dict(
        title="swpc", odir="./out", ntdec_r=50, strict_mode=False,
        nproc_x=1, nproc_y=1, nx=128, ny=128, nz=64, nt=1000,
        dx=0.5, dy=0.5, dz=0.5, dt=0.02, vcut=0.0,
        xbeg=-32.0, ybeg=-32.0, zbeg=-1.5, tbeg=0.0,
        clon=139.7604, clat=35.7182, phi=0.0,
        fq_min=0.05, fq_max=5.0, fq_ref=1.0,
        snp_format="native", xy_v_sw=False, z0_xy=0.25, ntdec_s=100, idec=1, jdec=1, kdec=1,
        sw_wav_v=True, sw_wav_u=False, sw_wav_stress=False, sw_wav_strain=False,
        ntdec_w=1, st_format="xy", fn_stloc="stations.xy", wav_format="sac", ntdec_w_prg=0,
        stf_format="xym0dc", stftype="kupper", fn_stf="source.dat", sdep_fit="asis",
        bf_mode=False, pw_mode=False, green_mode=False,
        abc_type="pml", na=20, stabilize_pml=False,
        vmodel_type="lhm", is_ocean=False, topo_flatten=False, munk_profile=False, earth_flattening=False,
        fn_lhm="lhm.dat", stopwatch_mode=False, benchmark_mode=False,
    )
    keys.update(kw)
    # Fortran-style component keys (xy_v%sw) cannot be Python identifiers
    out = {}
    for k, v in keys.items():
        if k.endswith("_sw"):
            k = k[:-3] + "%sw"
        out[k] = v
    return out


def double_couple(rng):
    strike = float(rng.uniform(0.0, 360.0))
    dip = float(rng.uniform(0.0, 90.0))
    rake = float(rng.uniform(-180.0, 180.0))
    return strike, dip, rake


def write_plain_small(d, seed=DEFAULT_SEED, nt=1000, **over):
    """Plain method, small, CPU-runnable: 128x128x64, dx = 0.5 km, dt = 0.02 s,
    two-layer viscoelastic medium, free surface, 20-point PML, one double
    couple at 10 km depth, 16 surface receivers on a 4x4 lattice."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    strike, dip, rake = double_couple(rng)
    keys = base_keys(nt=nt, **over)
    write_inf(os.path.join(d, "input.inf"), keys)
    write_lhm(os.path.join(d, "lhm.dat"), [(0, 2.7, 5.5, 3.2, 200, 100), (4, 2.9, 6.5, 3.7, 600, 300)])
    with open(os.path.join(d, "source.dat"), "w") as f:
        f.write("# x y z tbeg trise mo strike dip rake\n")
        f.write("  0.0 0.0 10.0 0.0 1.0 1.0e16 %.4f %.4f %.4f\n" % (strike, dip, rake))
    with open(os.path.join(d, "stations.xy"), "w") as f:
        f.write("# x y z name zsw\n")
        n = 0
        for y in (-12.0, -4.0, 4.0, 12.0):
            for x in (-12.0, -4.0, 4.0, 12.0):
                n += 1
                f.write("  %.3f %.3f 0.0 ST%02d fsb\n" % (x, y, n))
    return os.path.join(d, "input.inf")


def write_layered(d, nx, ny, nz, seed, nt=1500, dx=0.5, dt=0.02, n_station=8, body_force=None,
                  src_depth_max=None, **over):
    """One member of the batched many-instance workload: a seeded 3-5 layer
    medium (Vp 4.5-7.5 km/s sorted with depth, Vs = Vp/1.73,
    rho = 1.74 Vp^0.25, Qp = 600, Qs = 300), a single force or a double
    couple, and receivers at the free surface.  `src_depth_max` (km) caps the
    source depth, so that short runs record the direct waves."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    nlay = int(rng.integers(3, 6))
    zmax = nz * dx
    depths = np.sort(rng.uniform(0.0, 0.7 * zmax, nlay))
    depths[0] = 0.0
    vps = np.sort(rng.uniform(4.5, 7.5, nlay))
    rows = [(float(z), float(1.74 * vp ** 0.25), float(vp), float(vp / 1.73), 600.0, 300.0) for z, vp in zip(depths, vps)]
    if body_force is None:
        body_force = bool(rng.integers(0, 2))
    xbeg, ybeg = -nx * dx / 2, -ny * dx / 2
    keys = base_keys(nx=nx, ny=ny, nz=nz, nt=nt, dx=dx, dy=dx, dz=dx, dt=dt, xbeg=xbeg, ybeg=ybeg,
                     zbeg=-3 * dx, bf_mode=body_force, stf_format="xy" if body_force else "xym0dc", **over)
    write_inf(os.path.join(d, "input.inf"), keys)
    write_lhm(os.path.join(d, "lhm.dat"), rows)
    margin = (keys["na"] + 4) * dx
    sx = float(rng.uniform(xbeg + margin, -xbeg - margin))
    sy = float(rng.uniform(ybeg + margin, -ybeg - margin))
    zlim = zmax - (keys["na"] + 6) * dx
    if src_depth_max is not None:
        zlim = min(zlim, src_depth_max)
    sz = float(rng.uniform(3 * dx, zlim))
    with open(os.path.join(d, "source.dat"), "w") as f:
        if body_force:
            v = rng.normal(size=3)
            v /= np.linalg.norm(v)
            f.write("  %.4f %.4f %.4f 0.0 1.0 %.6e %.6e %.6e\n" % (sx, sy, sz, v[0] * 1e15, v[1] * 1e15, v[2] * 1e15))
        else:
            s, dp, r = double_couple(rng)
            f.write("  %.4f %.4f %.4f 0.0 1.0 1.0e16 %.4f %.4f %.4f\n" % (sx, sy, sz, s, dp, r))
    with open(os.path.join(d, "stations.xy"), "w") as f:
        for n in range(n_station):
            x = float(rng.uniform(xbeg + margin, -xbeg - margin))
            y = float(rng.uniform(ybeg + margin, -ybeg - margin))
            f.write("  %.4f %.4f 0.0 R%03d fsb\n" % (x, y, n))
    return os.path.join(d, "input.inf")


def write_green(d, nx=96, ny=96, nz=64, nt=200, cmp="z", bforce=True, n_points=24, seed=7, **over):
    """Reciprocal Green's-function run (green_mode): a unit body force in
    direction `cmp` at the free-surface station G01, strain (and, with
    bforce, displacement) recorded at `n_points` seeded grid points of the
    list file green.lst (x y z id)."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    keys = base_keys(nx=nx, ny=ny, nz=nz, nt=nt, xbeg=-nx * 0.25, ybeg=-ny * 0.25, green_mode=True,
                     green_stnm="G01", green_cmp=cmp, green_trise=1.0, green_bforce=bforce, fn_glst="green.lst",
                     green_fmt="xyz", sw_wav_v=False, ntdec_w=2, **over)
    write_inf(os.path.join(d, "input.inf"), keys)
    write_lhm(os.path.join(d, "lhm.dat"), [(0, 2.7, 5.5, 3.2, 200, 100), (4, 2.9, 6.5, 3.7, 600, 300)])
    with open(os.path.join(d, "stations.xy"), "w") as f:
        f.write("  1.000 -2.000 0.0 G01 fsb\n  5.000 5.000 0.0 G02 fsb\n")
    with open(os.path.join(d, "green.lst"), "w") as f:
        f.write("# x y z id\n")
        for q in range(n_points):
            x, y = rng.uniform(-8, 8, 2)
            z = rng.uniform(1.0, 9.0)
            f.write("  %.3f %.3f %.3f %d\n" % (x, y, z, 1000 + q))
    return os.path.join(d, "input.inf")


def write_plane_wave(d, nx=96, ny=96, nz=64, nt=200, ps="p", strike=30.0, dip=20.0, rake=0.0, **over):
    """Plane-wave mode (pw_mode): a P or S plane wave of Kupper shape
    (pw_zlen = 6 km) whose front starts at 20 km depth, incident with the
    given strike/dip(/rake), in the two-layer medium of the small plain
    configuration; 9 surface receivers."""
    os.makedirs(d, exist_ok=True)
    keys = base_keys(nx=nx, ny=ny, nz=nz, nt=nt, xbeg=-nx * 0.25, ybeg=-ny * 0.25, pw_mode=True, pw_ztop=20.0,
                     pw_zlen=6.0, pw_ps=ps, pw_strike=strike, pw_dip=dip, pw_rake=rake, **over)
    write_inf(os.path.join(d, "input.inf"), keys)
    write_lhm(os.path.join(d, "lhm.dat"), [(0, 2.7, 5.5, 3.2, 200, 100), (4, 2.9, 6.5, 3.7, 600, 300)])
    with open(os.path.join(d, "stations.xy"), "w") as f:
        n = 0
        for y in (-6.0, 0.0, 6.0):
            for x in (-6.0, 0.0, 6.0):
                n += 1
                f.write("  %.3f %.3f 0.0 P%02d fsb\n" % (x, y, n))
    return os.path.join(d, "input.inf")


def write_uniform(d, nx=64, ny=64, nz=64, nt=100, dx=0.5, dt=0.02, vp=6.0, vs=3.5, rho=2.8, q=1e6,
                  source="0.0 0.0 0.0", stations=(("0.0", "0.0", "0.0", "C"),), bf=None, **over):
    """Uniform whole-space medium (no air layer), used by the analytic and
    reciprocity tests."""
    os.makedirs(d, exist_ok=True)
    keys = base_keys(nx=nx, ny=ny, nz=nz, nt=nt, dx=dx, dy=dx, dz=dx, dt=dt,
                     xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=-nz * dx / 2,
                     vmodel_type="uni", vp0=vp, vs0=vs, rho0=rho, qp0=q, qs0=q, topo0=-1e9, **over)
    if bf is not None:
        keys["bf_mode"] = True
        keys["stf_format"] = "xy"
    write_inf(os.path.join(d, "input.inf"), keys)
    with open(os.path.join(d, "source.dat"), "w") as f:
        if bf is not None:
            f.write("  %s 0.0 1.0 %g %g %g\n" % (source, bf[0], bf[1], bf[2]))
        else:
            f.write("  %s 0.0 1.0 1.0e16 0 0 0 0 0 1\n" % source)
    with open(os.path.join(d, "stations.xy"), "w") as f:
        for x, y, z, nm in stations:
            f.write("  %s %s %s %s dep\n" % (x, y, z, nm))
    return os.path.join(d, "input.inf")


def von_karman_field(nxc, nyc, nzc, dx, seed=DEFAULT_SEED, a=5.0, eps=0.05):
    """Exponential von Karman perturbation (correlation length ``a`` km, rms
    ``eps``) on an nxc x nyc x nzc lattice of spacing dx, by the spectral
    method (white noise -> FFT -> sqrt(PSDF) -> IFFT -> de-mean -> rescale).
    Returns float32 (nzc, nyc, nxc), x fastest -- the layout of one k plane
    after another, as src/shared/m_rdrmed.f90:73-134 reads a field."""
    rng = np.random.default_rng(seed)
    nc = (nxc, nyc, nzc)
    kx = np.fft.fftfreq(nc[0], d=dx) * 2 * np.pi
    ky = np.fft.fftfreq(nc[1], d=dx) * 2 * np.pi
    kz = np.fft.rfftfreq(nc[2], d=dx) * 2 * np.pi
    K2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2 + kz[None, None, :] ** 2
    psdf = 8 * np.pi * eps ** 2 * a ** 3 / (1 + K2 * a * a) ** 2  # exponential ACF
    w = rng.standard_normal(nc)
    f = np.fft.irfftn(np.fft.rfftn(w) * np.sqrt(psdf), s=nc, axes=(0, 1, 2))
    f -= f.mean()
    f *= eps / f.std()
    return np.ascontiguousarray(f.astype(np.float32).transpose(2, 1, 0))


def gradient_random_fields(nx, ny, nz, dx, zbeg, seed=DEFAULT_SEED, a=5.0, eps=0.05, qp=600.0, qs=300.0):
    """The large single-source workload's medium as a background column and a
    perturbation field: a 1-D gradient Vp = 5 -> 7 km/s over depth,
    Vs = Vp/1.73, rho = 1.74 Vp^0.25 (air above z = 0) and a periodic
    exponential von Karman field on a lattice of at most 256 cells per axis
    (src/shared/m_rdrmed.f90 wraps its field the same way), which keeps
    set-up memory bounded for very large grids.

    Returns bg (5, nz+6) float32 -- rho0, vp0, vs0, qp, qs at k = -2 .. nz+3 --
    the field xi (nzc, nyc, nxc) and kxi0, the first 1-based k of the solid
    (the perturbation applies from there down)."""
    nc = [min(n, 256) for n in (nx, ny, nz)]
    xi = von_karman_field(nc[0], nc[1], nc[2], dx, seed=seed, a=a, eps=eps)
    k = np.arange(-2, nz + 4)
    z = (zbeg + (k - 0.5) * dx).astype(np.float32)
    zmax = zbeg + nz * dx
    vp0 = (5.0 + 2.0 * np.clip(z, 0, None) / zmax).astype(np.float32)
    vs0 = vp0 / np.float32(1.73)
    rho0 = np.float32(1.74) * vp0 ** np.float32(0.25)
    air = z < 0
    bg = np.stack([np.where(air, np.float32(0.001), rho0), np.where(air, np.float32(0), vp0),
                   np.where(air, np.float32(0), vs0), np.where(air, np.float32(10), np.float32(qp)),
                   np.where(air, np.float32(10), np.float32(qs))]).astype(np.float32)
    kxi0 = int(k[np.argmax(~air)])
    return bg, xi, kxi0


def rmed_apply(bg, xi, nx, ny, nz, kxi0, vmin=0.0, vmax=np.inf, rhomin=1.0):
    """Every cell of the halo grid from the background column and the
    periodic perturbation, as vmodel_lhm_rmed builds it
    (src/swpc_3d/m_vmodel_lhm_rmed.f90:161-212): below the topography
    rho = rho0 (1 + 0.8 xi), vp = vp0 (1 + xi), vs = vs0 (1 + xi), held inside
    [vmin, vmax] and above rhomin by vcheck (src/shared/m_fdtool.f90:15-48);
    air and water keep the column.  Single precision in the reference's
    order.  Returns rho, lam, mu, qp, qs as float32 (ny+6, nx+6, nz+6) (the
    Fortran (k, i, j) halo layout)."""
    f32 = np.float32
    nzc, nyc, nxc = xi.shape
    r0, vp0, vs0, qp0, qs0 = [np.asarray(c, np.float32) for c in bg]
    ii = (np.arange(-2, nx + 4) - 1) % nxc
    jj = (np.arange(-2, ny + 4) - 1) % nyc
    kk = (np.arange(-2, nz + 4) - 1) % nzc
    solid = (np.arange(-2, nz + 4) >= kxi0)[None, :]
    check = solid & ((vp0 > 0) & (vs0 > 0))[None, :]
    vmin, vmax, rhomin = f32(vmin), f32(vmax), f32(rhomin)
    shape = (ny + 6, nx + 6, nz + 6)
    rho = np.empty(shape, np.float32)
    lam = np.empty(shape, np.float32)
    mu = np.empty(shape, np.float32)
    xk = xi[kk]  # (nz+6, nyc, nxc)
    with np.errstate(divide="ignore", invalid="ignore"):
        for jo, j in enumerate(jj):
            x = xk[:, j, :][:, ii].T  # (nx+6, nz+6)
            one = f32(1) + x
            r = np.where(solid, r0[None, :] * (f32(1) + f32(0.8) * x), r0[None, :])
            vp = np.where(solid, vp0[None, :] * one, vp0[None, :])
            vs = np.where(solid, vs0[None, :] * one, vs0[None, :])
            gamma = vp / vs
            gamma = np.where(gamma < f32(1.1920928955078125e-07), f32(np.sqrt(3.0)), gamma)
            over = check & ((vp > vmax) | (vs > vmax))
            if over.any():
                xi2 = (one * vmax) / vp - f32(1)
                r = np.where(over, r * (f32(1) + f32(0.8) * xi2) / (f32(1) + f32(0.8) * x), r)
                vp = np.where(over, vmax, vp)
                vs = np.where(over, vmax / gamma, vs)
            under = check & ((vp < vmin) | (vs < vmin))
            if under.any():
                vs = np.where(under, vmin, vs)
                vp = np.where(under, vmin * gamma, vp)
            r = np.where(check & (r < rhomin), rhomin, r)
            rho[jo] = r
            mu[jo] = r * vs * vs
            lam[jo] = r * (vp * vp - f32(2) * vs * vs)
    qpv = np.broadcast_to(qp0[None, None, :], shape)
    qsv = np.broadcast_to(qs0[None, None, :], shape)
    return rho, lam, mu, qpv, qsv


def gradient_random_medium(nx, ny, nz, dx, zbeg, seed=DEFAULT_SEED, a=5.0, eps=0.05, na=20, qp=600.0, qs=300.0):
    """Large single-source workload medium over the halo grid, Fortran (k,i,j)
    order flattened as (ny+6, nx+6, nz+6): the background column and the
    perturbation of gradient_random_fields applied per point by rmed_apply.

    Returns float32 arrays rho, lam, mu, qp, qs of shape (ny+6, nx+6, nz+6)."""
    bg, xi, kxi0 = gradient_random_fields(nx, ny, nz, dx, zbeg, seed=seed, a=a, eps=eps, qp=qp, qs=qs)
    return rmed_apply(bg, xi, nx, ny, nz, kxi0)


def write_random_medium_case(d, nx=192, ny=192, nz=128, dx=0.25, dt=0.01, nt=600, seed=DEFAULT_SEED,
                             src_depth=3.75, n_side=8):
    """The large single-source workload's medium at a size the CPU oracle runs
    in seconds: the gradient + von Karman medium of gradient_random_medium at
    the workload's spacing (dx = 0.25 km, dt = 0.01 s), one double couple
    (mechanism from the seed, Kupper 1 s) at src_depth km -- 15 km of a
    128 km deep model scaled to 3.75 km of a 32 km deep one -- and
    n_side x n_side receivers on the free surface.  Returns the input.inf
    path and the raw medium (rho, lam, mu, qp, qs stacked over the halo
    grid) that the oracle and the GPU path both take."""
    zbeg = -3 * dx
    inf = write_plain_small(d, seed=seed, nt=nt, nx=nx, ny=ny, nz=nz, dx=dx, dy=dx, dz=dx, dt=dt,
                            xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=zbeg, ntdec_r=50)
    rng = np.random.default_rng(seed + 1)
    strike, dip, rake = double_couple(rng)
    with open(os.path.join(d, "source.dat"), "w") as f:
        f.write("# x y z tbeg trise mo strike dip rake\n")
        f.write("  0.0 0.0 %.4f 0.0 1.0 1.0e16 %.4f %.4f %.4f\n" % (src_depth, strike, dip, rake))
    half = 0.5 * min(nx, ny) * dx - (20 + 6) * dx
    with open(os.path.join(d, "stations.xy"), "w") as f:
        n = 0
        for y in np.linspace(-half, half, n_side):
            for x in np.linspace(-half, half, n_side):
                n += 1
                f.write("  %.3f %.3f 0.0 R%03d fsb\n" % (x, y, n))
    med = np.stack(gradient_random_medium(nx, ny, nz, dx, zbeg, seed=seed))
    return inf, med
