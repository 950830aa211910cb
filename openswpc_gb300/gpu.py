"""ctypes binding of include/swpc_gpu.h -- the Python mirror of the host
side of swpc_3d's time loop.

The reference's driver (src/swpc_3d/main.f90) sets up the grid, medium,
sources and stations on the host, then calls the step routines nt times and
finally writes waveforms and snapshots.  ``Simulation`` exposes exactly those
stages over the C ABI; ``Simulation.from_inf`` runs the whole host set-up
chain from an ``input.inf`` file.  There is no CPU fallback: if the CUDA
library cannot be loaded, every call raises.
"""
import ctypes
import os
import numpy as np

from . import build as _build

SWPC_WAV_V, SWPC_WAV_U, SWPC_WAV_STRESS, SWPC_WAV_STRAIN = 1, 2, 4, 8
SWPC_SNAP_XY_V, SWPC_SNAP_XY_U = 1, 2
SEC_XY, SEC_YZ, SEC_XZ, SEC_FS, SEC_OB = range(5)
SNAPK_V, SNAPK_U, SNAPK_PS = range(3)
STORE = {"fp32": 0, "fp16": 1, "bf16": 2}
STF = {"boxcar": 0, "triangle": 1, "herrmann": 2, "kupper": 3, "cosine": 4, "scosine": 4, "texp": 5}
FIELDS = ["Vx", "Vy", "Vz", "Sxx", "Syy", "Szz", "Syz", "Sxz", "Sxy"]
MEDIUM_FIELDS = ["rho", "lam", "mu", "taup", "taus"]  # fetch_field codes 9..13
STATIC_FIELD_MAX = 4 * 1024 * 1024  # SWPC_STATIC_FIELD_MAX of include/swpc_gpu.h


class SwpcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("swpc_gpu error %d: %s" % (code, msg))
        self.code = code


class Dims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nt", ctypes.c_int),
                ("na", ctypes.c_int), ("nm", ctypes.c_int), ("abc_type", ctypes.c_int), ("store", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("xbeg", ctypes.c_double), ("ybeg", ctypes.c_double), ("zbeg", ctypes.c_double),
                ("tbeg", ctypes.c_double), ("fcut", ctypes.c_double), ("M0", ctypes.c_double),
                ("UC", ctypes.c_double), ("ntdec_r", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


_lib = None

# every entry point declared in include/swpc_gpu.h
EXPORTS = [
    "swpc_gpu_create", "swpc_gpu_required_bytes", "swpc_gpu_upload_medium", "swpc_gpu_set_sources",
    "swpc_gpu_set_receivers", "swpc_gpu_set_snapshot", "swpc_gpu_step", "swpc_gpu_run", "swpc_gpu_sync",
    "swpc_gpu_fetch_waveforms", "swpc_gpu_fetch_snapshot", "swpc_gpu_query", "swpc_gpu_vmax",
    "swpc_gpu_fetch_field", "swpc_gpu_profile", "swpc_gpu_profile_read", "swpc_gpu_stream",
    "swpc_gpu_launch_count", "swpc_gpu_destroy", "swpc_gpu_last_error", "swpc_host_prepare",
    "swpc_host_write_sac", "swpc_host_write_snp", "swpc_host_nt", "swpc_host_medium",
    "swpc_host_check", "swpc_gpu_fetch_field_static", "swpc_gpu_reset", "swpc_gpu_get_dims", "swpc_gpu_set_zchunk", "swpc_gpu_set_zchunks", "swpc_gpu_get_zchunks",
    "swpc_gpu_get_zchunk", "swpc_batch_create", "swpc_batch_run", "swpc_batch_sync", "swpc_batch_stream",
    "swpc_batch_launch_count", "swpc_batch_destroy", "swpc_host_load", "swpc_host_request_bytes", "swpc_gpu_selftest_wait",
    "swpc_gpu_add_snapshot", "swpc_gpu_query_snapshot", "swpc_gpu_fetch_section", "swpc_gpu_set_green",
    "swpc_gpu_fetch_green", "swpc_host_write_green", "swpc_gpu_set_field", "swpc_gpu_set_plane_wave",
    "swpc_gpu_upload_medium_column",
    "swpc_host_request_dims", "swpc_host_materialize", "swpc_host_request_free", "swpc_serve_create",
    "swpc_serve_submit", "swpc_serve_state", "swpc_serve_wait", "swpc_serve_result", "swpc_serve_error",
    "swpc_serve_times", "swpc_serve_release", "swpc_serve_drain", "swpc_serve_stats", "swpc_serve_destroy",
    "swpc_gpu_profile_read_pml", "swpc_host_banner", "swpc_host_ntdec_r",
    "swpc_batch_set_persistent", "swpc_batch_item_count", "swpc_gpu_build_medium_rmed",
    "swpc_gpu_set_tiles", "swpc_gpu_get_tiles", "swpc_gpu_pml_fused",
]


class ServeConfig(ctypes.Structure):
    """swpc_serve_config of include/swpc_gpu.h."""
    _fields_ = [("hbm_budget", ctypes.c_double), ("max_active", ctypes.c_int), ("quantum", ctypes.c_int),
                ("prep_threads", ctypes.c_int), ("write_sac", ctypes.c_int), ("reserved", ctypes.c_int * 8)]


REQ_QUEUED, REQ_LOADING, REQ_WAITING, REQ_RUNNING, REQ_DONE = range(5)


def lib(build=True):
    """Load libswpc_gb300.so (building it first when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise SwpcError(-2, "CUDA library %s is missing; run openswpc_gb300.build.build()" % _build.LIB)
    L = ctypes.CDLL(_build.LIB)
    vp, i, d, fp, ip, dp = (ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p)
    L.swpc_gpu_create.argtypes = [ctypes.POINTER(Dims), ctypes.POINTER(vp)]
    L.swpc_gpu_required_bytes.argtypes = [ctypes.POINTER(Dims)]
    L.swpc_gpu_required_bytes.restype = ctypes.c_longlong
    L.swpc_gpu_upload_medium.argtypes = [vp] + [fp] * 5 + [ip] * 6 + [dp]
    L.swpc_gpu_set_sources.argtypes = [vp, i, ip, dp, dp, dp, dp, i, i]
    L.swpc_gpu_set_receivers.argtypes = [vp, i, ip, i, i]
    L.swpc_gpu_set_snapshot.argtypes = [vp, i, i, i, i, i]
    L.swpc_gpu_step.argtypes = [vp, i]
    L.swpc_gpu_run.argtypes = [vp, i, i]
    L.swpc_gpu_sync.argtypes = [vp]
    L.swpc_gpu_fetch_waveforms.argtypes = [vp, i, fp]
    L.swpc_gpu_fetch_snapshot.argtypes = [vp, i, i, fp]
    L.swpc_gpu_query.argtypes = [vp, ip, ip, ip, ip, ip]
    L.swpc_gpu_vmax.argtypes = [vp, fp]
    L.swpc_gpu_fetch_field.argtypes = [vp, i, dp]
    L.swpc_gpu_fetch_field_static.argtypes = [vp, i, dp]
    L.swpc_gpu_profile.argtypes = [vp, i]
    L.swpc_gpu_profile_read.argtypes = [vp, dp, ip]
    L.swpc_gpu_profile_read_pml.argtypes = [vp, dp, ip, ip, ip]
    L.swpc_gpu_stream.argtypes = [vp]
    L.swpc_gpu_stream.restype = vp
    L.swpc_gpu_launch_count.argtypes = [vp]
    L.swpc_gpu_launch_count.restype = ctypes.c_longlong
    L.swpc_gpu_destroy.argtypes = [vp]
    L.swpc_gpu_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.swpc_host_prepare.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    L.swpc_host_write_sac.argtypes = [vp, ctypes.c_char_p]
    L.swpc_host_write_snp.argtypes = [vp, ctypes.c_char_p]
    L.swpc_host_nt.argtypes = [vp]
    L.swpc_host_ntdec_r.argtypes = [vp]
    L.swpc_host_banner.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.swpc_host_check.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
    L.swpc_host_medium.argtypes = [i, i, i, i, d, d, d] + [fp] * 5 + [ip] * 6 + [dp]
    L.swpc_gpu_reset.argtypes = [vp]
    L.swpc_gpu_get_dims.argtypes = [vp, ctypes.POINTER(Dims)]
    L.swpc_gpu_set_zchunk.argtypes = [vp, i]
    L.swpc_gpu_get_zchunk.argtypes = [vp]
    L.swpc_gpu_set_zchunks.argtypes = [vp, i, i]
    L.swpc_gpu_set_tiles.argtypes = [vp, i, i]
    L.swpc_gpu_get_tiles.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.swpc_gpu_pml_fused.argtypes = [vp]
    L.swpc_gpu_get_zchunks.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.swpc_batch_create.argtypes = [ctypes.c_void_p, i, ctypes.POINTER(vp)]
    L.swpc_batch_run.argtypes = [vp, i]
    L.swpc_batch_sync.argtypes = [vp]
    L.swpc_batch_set_persistent.argtypes = [vp, i]
    L.swpc_batch_item_count.argtypes = [vp]
    L.swpc_batch_stream.argtypes = [vp]
    L.swpc_batch_stream.restype = vp
    L.swpc_batch_launch_count.argtypes = [vp]
    L.swpc_batch_launch_count.restype = ctypes.c_longlong
    L.swpc_batch_destroy.argtypes = [vp]
    L.swpc_gpu_selftest_wait.argtypes = [dp]
    L.swpc_gpu_add_snapshot.argtypes = [vp, i, i, i, i, i, i]
    L.swpc_gpu_query_snapshot.argtypes = [vp, i, i, ip, ip, ip]
    L.swpc_gpu_fetch_section.argtypes = [vp, i, i, i, fp]
    L.swpc_gpu_set_green.argtypes = [vp, i, ip, i, i]
    L.swpc_gpu_fetch_green.argtypes = [vp, fp, ip, ip, ip]
    L.swpc_host_write_green.argtypes = [vp, ctypes.c_char_p]
    L.swpc_gpu_set_field.argtypes = [vp, i, fp]
    L.swpc_gpu_set_plane_wave.argtypes = [vp, i]
    L.swpc_gpu_upload_medium_column.argtypes = [vp] + [fp] * 5 + [ip] * 6 + [dp]
    L.swpc_gpu_build_medium_rmed.argtypes = [vp, fp, fp, i, i, i, i, d, d, d, d, d, d, ip, dp]
    L.swpc_host_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    L.swpc_host_request_bytes.argtypes = [vp]
    L.swpc_host_request_bytes.restype = ctypes.c_longlong
    L.swpc_host_request_dims.argtypes = [vp, ctypes.POINTER(Dims)]
    L.swpc_host_materialize.argtypes = [vp, ctypes.POINTER(vp)]
    L.swpc_host_request_free.argtypes = [vp]
    L.swpc_serve_create.argtypes = [ctypes.POINTER(ServeConfig), ctypes.POINTER(vp)]
    L.swpc_serve_submit.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]
    L.swpc_serve_state.argtypes = [vp, ctypes.c_longlong]
    L.swpc_serve_wait.argtypes = [vp, ctypes.c_longlong, d]
    L.swpc_serve_result.argtypes = [vp, ctypes.c_longlong, i, fp, ctypes.c_size_t, ip, ip]
    L.swpc_serve_error.argtypes = [vp, ctypes.c_longlong, ctypes.c_char_p, ctypes.c_size_t]
    L.swpc_serve_times.argtypes = [vp, ctypes.c_longlong, dp]
    L.swpc_serve_release.argtypes = [vp, ctypes.c_longlong]
    L.swpc_serve_drain.argtypes = [vp]
    L.swpc_serve_stats.argtypes = [vp, dp]
    L.swpc_serve_destroy.argtypes = [vp]
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(2048)
    lib().swpc_gpu_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def _ck(rc):
    if rc != 0:
        raise SwpcError(rc, last_error())
    return rc


def _ptr(a):
    return a.ctypes.data if a is not None else None


def make_dims(nx, ny, nz, nt, dx, dy, dz, dt, na=20, abc="pml", store="fp32", xbeg=0.0, ybeg=0.0, zbeg=0.0,
              tbeg=0.0, fcut=1.0, M0=1.0, UC=1e-15, ntdec_r=0, variant=0, concurrent=None, pml_points=0,
              pml_fused=None):
    """swpc_dims for swpc_gpu_create.  variant 0 selects the TMA-fed interior
    kernels, 1 the shared-memory sweep without TMA (kept for comparison);
    pml_fused (with variant 0): True makes the tile kernels sweep the PML
    shell too (interior kernels over the tiles inside the interior,
    shell-tile kernels over the rest); False or None (the library default)
    runs the shell in launches of its own, where the next two options apply;
    concurrent runs the PML shell kernels beside the interior kernels on a
    second stream (True/False; None lets the library choose by grid size);
    pml_points: shell points per thread of the PML kernels (2, or 0/1 for
    the library default of one)."""
    d = Dims()
    d.nx, d.ny, d.nz, d.nt, d.na, d.nm = nx, ny, nz, nt, na, 3
    d.abc_type = 0 if abc == "pml" else 1
    d.store = STORE[store]
    d.dx, d.dy, d.dz, d.dt = dx, dy, dz, dt
    d.xbeg, d.ybeg, d.zbeg, d.tbeg = xbeg, ybeg, zbeg, tbeg
    d.fcut, d.M0, d.UC, d.ntdec_r = fcut, M0, UC, ntdec_r
    d.reserved[0] = int(variant)
    d.reserved[1] = 0 if concurrent is None else (2 if concurrent else 1)
    d.reserved[2] = int(pml_points)
    d.reserved[3] = 0 if pml_fused is None else (2 if pml_fused else 1)
    return d


def host_medium(nx, ny, nz, na, fq_min, fq_max, fq_ref, rho, lam, mu, qp, qs):
    """Medium post-processing of medium__setup in FP64 (swpc_host_medium).
    Arrays are Fortran (k,i,j) halo arrays shaped (ny+6, nx+6, nz+6); rho,
    lam, mu are modified in place and (taup, taus, maps..., ts) returned."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (rho, lam, mu, qp, qs)]
    for a, b in zip(arrs[:3], (rho, lam, mu)):
        if a is not b:
            raise ValueError("rho, lam, mu must be contiguous float32 arrays (modified in place)")
    maps = [np.zeros((ny + 6, nx + 6), np.int32) for _ in range(6)]
    ts = np.zeros(3, np.float64)
    _ck(lib().swpc_host_medium(nx, ny, nz, na, fq_min, fq_max, fq_ref, *[_ptr(a) for a in arrs],
                               *[_ptr(m) for m in maps], _ptr(ts)))
    return arrs[3], arrs[4], maps, ts


def host_check(inf_path):
    """Host set-up summary of an input.inf without a GPU (swpc_host_check)."""
    import json
    buf = ctypes.create_string_buffer(1 << 20)
    rc = lib().swpc_host_check(os.fsencode(os.path.abspath(inf_path)), buf, 1 << 20)
    if rc < 0:
        raise SwpcError(rc, last_error())
    return json.loads(buf.value.decode())


def required_bytes(dims):
    return int(lib().swpc_gpu_required_bytes(ctypes.byref(dims)))


class Simulation:
    """One swpc_3d simulation resident on the current CUDA device."""

    def __init__(self, dims=None, handle=None):
        self._h = ctypes.c_void_p()
        if handle is not None:
            self._h = handle
            dims = Dims()
            _ck(lib().swpc_gpu_get_dims(self._h, ctypes.byref(dims)))
        else:
            _ck(lib().swpc_gpu_create(ctypes.byref(dims), ctypes.byref(self._h)))
        self.dims = dims
        self._keep = []

    @classmethod
    def from_inf(cls, inf_path):
        h = ctypes.c_void_p()
        _ck(lib().swpc_host_prepare(os.fsencode(os.path.abspath(inf_path)), ctypes.byref(h)))
        return cls(handle=h)

    @property
    def handle(self):
        return self._h

    def upload_medium(self, rho, lam, mu, taup, taus, kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot, ts):
        f = [np.ascontiguousarray(a, np.float32) for a in (rho, lam, mu, taup, taus)]
        m = [np.ascontiguousarray(a, np.int32) for a in (kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot)]
        t = np.ascontiguousarray(ts, np.float64)
        _ck(lib().swpc_gpu_upload_medium(self._h, *[_ptr(a) for a in f], *[_ptr(a) for a in m], _ptr(t)))

    def build_medium_rmed(self, bg, xi, kxi0, vmin=0.0, vmax=float("inf"), rhomin=1.0, fq_min=0.05, fq_max=5.0,
                          fq_ref=1.0):
        """Medium of a layered model with a periodic random perturbation,
        built on the device (swpc_gpu_build_medium_rmed): bg (5, nz+6)
        background column, xi (nzc, nyc, nxc) field.  Returns the six
        surface maps ((ny+6, nx+6) int32 each: kfs, kob, kfs_top, kfs_bot,
        kob_top, kob_bot) and the relaxation times."""
        d = self.dims
        bg = np.ascontiguousarray(bg, np.float32)
        xi = np.ascontiguousarray(xi, np.float32)
        if d is None or bg.shape != (5, d.nz + 6) or xi.ndim != 3:
            raise SwpcError(-1, "build_medium_rmed(): bg must be (5, nz+6) and xi 3-D")
        maps = np.zeros((6, d.ny + 6, d.nx + 6), np.int32)
        ts = np.zeros(3, np.float64)
        nzc, nyc, nxc = xi.shape
        _ck(lib().swpc_gpu_build_medium_rmed(self._h, bg.ctypes.data, xi.ctypes.data, nxc, nyc, nzc, int(kxi0),
                                             float(vmin), float(vmax), float(rhomin), float(fq_min), float(fq_max),
                                             float(fq_ref), maps.ctypes.data, ts.ctypes.data))
        return list(maps), ts

    def set_sources(self, ijk, prm, mo=None, mij=None, fxyz=None, stftype="kupper", bf_mode=False):
        ijk = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        n = ijk.shape[0]
        prm = np.ascontiguousarray(prm, np.float64).reshape(n, 2)
        mo = None if mo is None else np.ascontiguousarray(mo, np.float64).reshape(n)
        mij = None if mij is None else np.ascontiguousarray(mij, np.float64).reshape(n, 6)
        fxyz = None if fxyz is None else np.ascontiguousarray(fxyz, np.float64).reshape(n, 3)
        stf = STF[stftype] if isinstance(stftype, str) else int(stftype)
        _ck(lib().swpc_gpu_set_sources(self._h, n, _ptr(ijk), _ptr(mo), _ptr(mij), _ptr(fxyz), _ptr(prm), stf,
                                       int(bool(bf_mode))))

    def set_receivers(self, ijk, ntdec_w=1, flags=SWPC_WAV_V):
        ijk = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        _ck(lib().swpc_gpu_set_receivers(self._h, ijk.shape[0], _ptr(ijk), int(ntdec_w), int(flags)))

    def set_snapshot(self, kinds, k0, idec=1, jdec=1, ntdec_s=10):
        _ck(lib().swpc_gpu_set_snapshot(self._h, int(kinds), int(k0), int(idec), int(jdec), int(ntdec_s)))

    def step(self, it):
        _ck(lib().swpc_gpu_step(self._h, int(it)))

    def run(self, it0, it1):
        _ck(lib().swpc_gpu_run(self._h, int(it0), int(it1)))

    def sync(self):
        _ck(lib().swpc_gpu_sync(self._h))

    def query(self):
        v = np.zeros(5, np.int32)
        _ck(lib().swpc_gpu_query(self._h, *[v[q:].ctypes.data for q in range(5)]))
        return dict(ntw=int(v[0]), nst=int(v[1]), nxs=int(v[2]), nys=int(v[3]), nframes=int(v[4]))

    def waveforms(self, kind=SWPC_WAV_V):
        q = self.query()
        nc = 3 if kind in (SWPC_WAV_V, SWPC_WAV_U) else 6
        out = np.zeros((q["nst"], nc, q["ntw"]), np.float32)
        _ck(lib().swpc_gpu_fetch_waveforms(self._h, int(kind), out.ctypes.data))
        return out

    def add_snapshot(self, section, kind, fix=1, dec1=1, dec2=1, ntdec_s=10):
        _ck(lib().swpc_gpu_add_snapshot(self._h, int(section), int(kind), int(fix), int(dec1), int(dec2), int(ntdec_s)))

    def query_section(self, section, kind):
        v = np.zeros(3, np.int32)
        _ck(lib().swpc_gpu_query_snapshot(self._h, int(section), int(kind), *[v[q:].ctypes.data for q in range(3)]))
        return dict(n1=int(v[0]), n2=int(v[1]), nframes=int(v[2]))

    def section(self, section, kind, frame):
        """Frame `frame` of a snapshot: (nc, n2, n1) float32."""
        q = self.query_section(section, kind)
        nc = 4 if kind == SNAPK_PS else 3
        out = np.zeros((nc, q["n2"], q["n1"]), np.float32)
        _ck(lib().swpc_gpu_fetch_section(self._h, int(section), int(kind), int(frame), out.ctypes.data))
        return out

    def snapshot(self, kind, frame):
        q = self.query()
        out = np.zeros((3, q["nys"], q["nxs"]), np.float32)
        _ck(lib().swpc_gpu_fetch_snapshot(self._h, int(kind), int(frame), out.ctypes.data))
        return out

    def field(self, name):
        d = self.dims
        if d is None:
            raise SwpcError(-1, "field() needs the dims the simulation was created with")
        out = np.zeros((d.ny, d.nx, d.nz), np.float64)
        code = FIELDS.index(name) if name in FIELDS else 9 + MEDIUM_FIELDS.index(name)
        _ck(lib().swpc_gpu_fetch_field(self._h, code, out.ctypes.data))
        return out

    def set_field(self, name, halo):
        """Overwrite a state field from a (ny+6, nx+6, nz+6) halo-grid array
        (Fortran A(k,i,j)): the physical columns including the z halo planes
        are taken, the x/y ghost columns stay zero."""
        d = self.dims
        if d is None:
            raise SwpcError(-1, "set_field() needs the dims the simulation was created with")
        a = np.ascontiguousarray(halo, dtype=np.float32)
        if a.shape != (d.ny + 6, d.nx + 6, d.nz + 6):
            raise SwpcError(-1, "set_field(): expected shape %s" % ((d.ny + 6, d.nx + 6, d.nz + 6),))
        _ck(lib().swpc_gpu_set_field(self._h, FIELDS.index(name), a.ctypes.data))

    def field_static(self, name):
        """field() through the library's fixed scratch array: no device
        allocation, grids up to STATIC_FIELD_MAX points."""
        d = self.dims
        if d is None:
            raise SwpcError(-1, "field_static() needs the dims the simulation was created with")
        if name not in FIELDS:
            raise SwpcError(-1, "field_static() reads the wavefields %s only, not %r" % (", ".join(FIELDS), name))
        out = np.zeros((d.ny, d.nx, d.nz), np.float64)
        _ck(lib().swpc_gpu_fetch_field_static(self._h, FIELDS.index(name), out.ctypes.data))
        return out

    def vmax(self):
        out = np.zeros(3, np.float32)
        _ck(lib().swpc_gpu_vmax(self._h, out.ctypes.data))
        return out

    def profile(self, enable=True):
        _ck(lib().swpc_gpu_profile(self._h, int(enable)))

    def profile_read(self):
        ms = np.zeros(6, np.float64)
        n = np.zeros(6, np.int64)
        _ck(lib().swpc_gpu_profile_read(self._h, ms.ctypes.data, n.ctypes.data))
        return ms, n

    def profile_read_pml(self):
        """PML time by launch class (x only, y only, z only, rest): ms and
        launches as (2, 4) arrays (stress, velocity), the shell points of
        each class and the sum of damped axes over those points."""
        ms = np.zeros(8, np.float64)
        n = np.zeros(8, np.int64)
        pts = np.zeros(4, np.int64)
        ax = np.zeros(4, np.int64)
        _ck(lib().swpc_gpu_profile_read_pml(self._h, ms.ctypes.data, n.ctypes.data, pts.ctypes.data, ax.ctypes.data))
        return ms.reshape(2, 4), n.reshape(2, 4), pts, ax

    def stream(self):
        return lib().swpc_gpu_stream(self._h)

    def launch_count(self):
        return int(lib().swpc_gpu_launch_count(self._h))

    def nt(self):
        return int(lib().swpc_host_nt(self._h))

    def reset(self):
        _ck(lib().swpc_gpu_reset(self._h))

    def set_zchunk(self, kchunk):
        _ck(lib().swpc_gpu_set_zchunk(self._h, int(kchunk)))

    def zchunk(self):
        return int(lib().swpc_gpu_get_zchunk(self._h))

    def set_zchunks(self, kstress, kvel):
        """z-sweep depths of the stress and velocity kernels (0: automatic)."""
        _ck(lib().swpc_gpu_set_zchunks(self._h, int(kstress), int(kvel)))

    def set_tiles(self, rows_stress, rows_vel):
        """Tile rows (8 or 16; 0 = 8) of the interior stress and velocity kernels."""
        _ck(lib().swpc_gpu_set_tiles(self._h, int(rows_stress), int(rows_vel)))

    def tiles(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        _ck(lib().swpc_gpu_get_tiles(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    @property
    def pml_fused(self):
        """True when the tile kernels sweep the PML shell with the interior."""
        rc = lib().swpc_gpu_pml_fused(self._h)
        if rc < 0:
            _ck(rc)
        return rc == 1

    def zchunks(self):
        ks, kv = ctypes.c_int(), ctypes.c_int()
        _ck(lib().swpc_gpu_get_zchunks(self._h, ctypes.byref(ks), ctypes.byref(kv)))
        return ks.value, kv.value

    def write_sac(self, odir=None):
        _ck(lib().swpc_host_write_sac(self._h, os.fsencode(odir) if odir else None))

    def green(self):
        """Green's-function traces (n, ncmp, ntw) float32 (green mode)."""
        n, nc, nw = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ck(lib().swpc_gpu_fetch_green(self._h, None, ctypes.byref(n), ctypes.byref(nc), ctypes.byref(nw)))
        out = np.zeros(n.value * nc.value * nw.value, np.float32)
        _ck(lib().swpc_gpu_fetch_green(self._h, out.ctypes.data, None, None, None))
        return out.reshape(n.value, nc.value, nw.value)

    def set_green(self, ijk, ntdec_w=1, bforce=False):
        ijk = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        _ck(lib().swpc_gpu_set_green(self._h, ijk.shape[0], ijk.ctypes.data, int(ntdec_w), int(bool(bforce))))

    def write_green(self, odir=None):
        _ck(lib().swpc_host_write_green(self._h, os.fsencode(odir) if odir else None))

    def write_snp(self, odir=None):
        _ck(lib().swpc_host_write_snp(self._h, os.fsencode(odir) if odir else None))

    def close(self):
        if self._h:
            lib().swpc_gpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several simulations advanced together by fused launches
    (swpc_batch_*).  The members stay owned by the caller."""

    def __init__(self, sims, persistent=None):
        self.sims = list(sims)
        arr = (ctypes.c_void_p * len(self.sims))(*[s.handle.value for s in self.sims])
        self._h = ctypes.c_void_p()
        _ck(lib().swpc_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(self.sims), ctypes.byref(self._h)))
        if persistent is not None:
            self.set_persistent(persistent)

    def set_persistent(self, on=True):
        """One persistent fused launch per step (True) or one launch per
        phase of the step (False); the results are the same."""
        _ck(lib().swpc_batch_set_persistent(self._h, int(bool(on))))

    def item_count(self):
        return int(lib().swpc_batch_item_count(self._h))

    def run(self, nsteps):
        _ck(lib().swpc_batch_run(self._h, int(nsteps)))

    def sync(self):
        _ck(lib().swpc_batch_sync(self._h))

    def stream(self):
        return lib().swpc_batch_stream(self._h)

    def launch_count(self):
        return int(lib().swpc_batch_launch_count(self._h))

    def close(self):
        if self._h:
            lib().swpc_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Request:
    """Host half of the set-up of one input.inf (swpc_host_load): medium,
    sources and stations in host memory, no device touched."""

    def __init__(self, inf_path):
        self._h = ctypes.c_void_p()
        _ck(lib().swpc_host_load(os.fsencode(os.path.abspath(inf_path)), ctypes.byref(self._h)))

    @property
    def device_bytes(self):
        n = lib().swpc_host_request_bytes(self._h)
        if n < 0:
            raise SwpcError(int(n), last_error())
        return int(n)

    @property
    def dims(self):
        d = Dims()
        _ck(lib().swpc_host_request_dims(self._h, ctypes.byref(d)))
        return d

    def materialize(self):
        """Create the simulation on the current device and upload it."""
        h = ctypes.c_void_p()
        _ck(lib().swpc_host_materialize(self._h, ctypes.byref(h)))
        return Simulation(handle=h)

    def close(self):
        if self._h:
            lib().swpc_host_request_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop with continuous batching (swpc_serve_*): submit input.inf
    paths at any time; admitted requests share fused launches on the GPU."""

    def __init__(self, hbm_budget=0.0, max_active=0, quantum=0, prep_threads=0, write_sac=False):
        cfg = ServeConfig(hbm_budget=float(hbm_budget), max_active=int(max_active), quantum=int(quantum),
                          prep_threads=int(prep_threads), write_sac=int(bool(write_sac)))
        self._h = ctypes.c_void_p()
        _ck(lib().swpc_serve_create(ctypes.byref(cfg), ctypes.byref(self._h)))

    def submit(self, inf_path):
        rid = ctypes.c_longlong()
        _ck(lib().swpc_serve_submit(self._h, os.fsencode(os.path.abspath(inf_path)), ctypes.byref(rid)))
        return int(rid.value)

    def state(self, rid):
        return int(lib().swpc_serve_state(self._h, rid))

    def wait(self, rid, timeout=-1.0):
        st = int(lib().swpc_serve_wait(self._h, rid, float(timeout)))
        if st < 0:
            raise SwpcError(st, self.error(rid))
        return st

    def error(self, rid):
        buf = ctypes.create_string_buffer(2048)
        lib().swpc_serve_error(self._h, rid, buf, 2048)
        return buf.value.decode(errors="replace")

    def result(self, rid, kind=SWPC_WAV_V):
        nst, ntw = ctypes.c_int(), ctypes.c_int()
        _ck(lib().swpc_serve_result(self._h, rid, int(kind), None, 0, ctypes.byref(nst), ctypes.byref(ntw)))
        nc = 3 if kind in (SWPC_WAV_V, SWPC_WAV_U) else 6
        out = np.zeros((nst.value, nc, ntw.value), np.float32)
        _ck(lib().swpc_serve_result(self._h, rid, int(kind), out.ctypes.data, out.size, None, None))
        return out

    def times(self, rid):
        t = np.zeros(4)
        _ck(lib().swpc_serve_times(self._h, rid, t.ctypes.data))
        return dict(submitted=t[0], admitted=t[1], started=t[2], finished=t[3])

    def release(self, rid):
        _ck(lib().swpc_serve_release(self._h, rid))

    def drain(self):
        _ck(lib().swpc_serve_drain(self._h))

    def stats(self):
        st = np.zeros(10)
        _ck(lib().swpc_serve_stats(self._h, st.ctypes.data))
        keys = ("done", "failed", "running", "waiting", "queued", "bytes_granted", "peak_bytes", "quanta",
                "rebuilds", "updates")
        return dict(zip(keys, st.tolist()))

    def close(self):
        if self._h:
            lib().swpc_serve_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
