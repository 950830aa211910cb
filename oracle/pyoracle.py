"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a C++ restatement of OpenSWPC's swpc_3d time loop
(oracle/swpc_oracle.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs load it; the product (openswpc_gb300) never does.
"""
import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "swpc_oracle.cpp")

# -ffp-contract=off and no fast-math keep the restatement's rounding
# deterministic and close to the reference's scalar evaluation order.
CXXFLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c++17"]
# The timed CPU baseline uses the optimisation flags of the reference's
# ubuntu-gfortran build (src/shared/makefile.arch:28: -O2 -ffast-math -fopenmp).
LIB_FAST = os.path.join(BUILD, "liboracle_fast.so")
CXXFLAGS_FAST = ["-O2", "-ffast-math", "-fopenmp", "-fPIC", "-shared", "-std=c++17"]

MODES = {"fp32": 0, "mixed": 1, "fp64": 2}
FIELDS = ["Vx", "Vy", "Vz", "Sxx", "Syy", "Szz", "Syz", "Sxz", "Sxy"]
MEDIA = ["rho", "lam", "mu", "taup", "taus", "kfs", "kob", "kfs_top", "kfs_bot", "kob_top", "kob_bot", "ts"]


def build(force=False, fast=False):
    os.makedirs(BUILD, exist_ok=True)
    out, flags = (LIB_FAST, CXXFLAGS_FAST) if fast else (LIB, CXXFLAGS)
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(SRC):
        tmp = out + ".tmp"
        subprocess.check_call(["g++", *flags, "-o", tmp, SRC])
        os.replace(tmp, out)
    return out


_libs = {}


def use_fast_build():
    """Route every Oracle created afterwards through the -ffast-math build
    (timing only; the parity tests use the deterministic build)."""
    global _fast
    _fast = True


_fast = False


def lib():
    key = "fast" if _fast else "exact"
    if key not in _libs:
        path = build(fast=_fast)
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.oracle_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(vp)]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_run.argtypes = [vp, ctypes.c_int]
        L.oracle_info.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_waveforms.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
        L.oracle_stations.argtypes = [vp, ctypes.c_void_p]
        L.oracle_field.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
        L.oracle_medium.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
        L.oracle_set_field.argtypes = [vp, ctypes.c_int, ctypes.c_void_p]
        L.oracle_coefs.argtypes = [vp, ctypes.c_void_p]
        L.oracle_vmax.argtypes = [vp, ctypes.c_void_p]
        L.oracle_snap_xy_v.argtypes = [vp, ctypes.c_void_p]
        L.oracle_snap.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.oracle_snap.restype = ctypes.c_longlong
        L.oracle_green.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_sources.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_stf.argtypes = [vp]
        L.oracle_momentrate.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_float]
        L.oracle_momentrate.restype = ctypes.c_float
        L.oracle_sdr2moment.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_void_p]
        _libs[key] = L
    return _libs[key]


class Oracle:
    """One oracle simulation built from an input.inf file."""

    def __init__(self, inf_path, mode="fp32", nthreads=0, medium=None):
        L = self._L = lib()
        h = ctypes.c_void_p()
        vm = None
        if medium is not None:
            vm = np.ascontiguousarray(medium, dtype=np.float32)
        rc = L.oracle_create(os.fsencode(inf_path), MODES[mode], int(nthreads),
                             vm.ctypes.data if vm is not None else None, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("oracle: " + L.oracle_last_error().decode())
        self.h = h
        self._keep = vm
        self.refresh()

    def refresh(self):
        ints = np.zeros(16, np.int32)
        reals = np.zeros(16, np.float64)
        self._L.oracle_info(self.h, ints.ctypes.data, reals.ctypes.data)
        (self.nx, self.ny, self.nz, self.nt, self.na, self.nst, self.ntw, self.nt_done,
         self.nxs, self.nys, self.k0_xy, self.nvmax, self.nsnap) = [int(v) for v in ints[:13]]
        self.M0, self.UC, self.fcut = [float(v) for v in reals[:3]]
        self.dx, self.dy, self.dz, self.dt, self.xbeg, self.ybeg, self.zbeg, self.tbeg = [float(v) for v in reals[3:11]]
        self.ntdec_w, self.ntdec_r, self.bf_mode = int(ints[13]), int(ints[14]), bool(ints[15])

    def run(self, n):
        if self._L.oracle_run(self.h, int(n)) != 0:
            raise RuntimeError("oracle: " + self._L.oracle_last_error().decode())
        self.refresh()

    def waveforms(self, kind=0):
        ncmp = 3 if kind in (0, 1) else 6
        out = np.zeros((self.nst, ncmp, self.ntw), np.float32)  # Fortran (ntw,ncmp,nst)
        self._L.oracle_waveforms(self.h, kind, out.ctypes.data)
        return out

    def stations(self):
        out = np.zeros((self.nst, 3), np.int32)
        self._L.oracle_stations(self.h, out.ctypes.data)
        return out

    def field(self, name):
        out = np.zeros((self.ny, self.nx, self.nz), np.float64)  # Fortran (nz,nx,ny)
        if self._L.oracle_field(self.h, FIELDS.index(name), out.ctypes.data) != 0:
            raise RuntimeError(self._L.oracle_last_error().decode())
        return out

    def coefs(self):
        """Zener coefficients c1, c2, d1 (nm), d2 and, with the PML, the
        damping profiles gxc, gxe, gyc, gye, gzc, gze as (n, 4) arrays."""
        nm = 3
        out = np.zeros(4 * nm + 1 + 8 * (self.nx + self.ny + self.nz), np.float64)
        n = self._L.oracle_coefs(self.h, out.ctypes.data)
        if n < 0:
            raise RuntimeError(self._L.oracle_last_error().decode())
        r = {"c1": out[0:nm], "c2": out[nm:2 * nm], "d1": out[2 * nm:3 * nm], "d2": out[3 * nm]}
        q = 3 * nm + 1
        if n > q:
            for name, m in (("gxc", self.nx), ("gxe", self.nx), ("gyc", self.ny), ("gye", self.ny),
                            ("gzc", self.nz), ("gze", self.nz)):
                r[name] = out[q:q + 4 * m].reshape(m, 4)
                q += 4 * m
        return r

    def set_field(self, name, halo):
        """Overwrite a state field from a (ny+6, nx+6, nz+6) halo-grid
        array: the physical columns including the z halo planes are taken,
        the x/y ghost columns are zeroed."""
        a = np.ascontiguousarray(halo, dtype=np.float32)
        assert a.shape == (self.ny + 6, self.nx + 6, self.nz + 6)
        if self._L.oracle_set_field(self.h, FIELDS.index(name), a.ctypes.data) != 0:
            raise RuntimeError(self._L.oracle_last_error().decode())

    def medium(self, name):
        w = MEDIA.index(name)
        if w < 5:
            out = np.zeros((self.ny + 6, self.nx + 6, self.nz + 6), np.float32)
        elif w < 11:
            out = np.zeros((self.ny + 6, self.nx + 6), np.float32)
        else:
            out = np.zeros(3, np.float32)
        if self._L.oracle_medium(self.h, w, out.ctypes.data) != 0:
            raise RuntimeError(self._L.oracle_last_error().decode())
        return out if w < 5 or w == 11 else out.astype(np.int32)

    def vmax_log(self):
        out = np.zeros((self.nvmax, 4), np.float32)
        self._L.oracle_vmax(self.h, out.ctypes.data)
        return out

    def snap(self, section, kind, n1, n2):
        """Stacked frames of one snapshot: (nframes, nc, n2, n1) float32
        (section 0 xy, 1 yz, 2 xz, 3 fs, 4 ob; kind 0 v, 1 u, 2 ps)."""
        n = self._L.oracle_snap(self.h, int(section), int(kind), None)
        if n < 0:
            raise RuntimeError("snapshot not requested")
        out = np.zeros(n, np.float32)
        self._L.oracle_snap(self.h, int(section), int(kind), out.ctypes.data)
        nc = 4 if kind == 2 else 3
        return out.reshape(-1, nc, n2, n1)

    def green(self):
        """Green's-function traces as (ng, ncmp, ntw) float32 (green_mode)."""
        v = np.zeros(3, np.int32)
        if self._L.oracle_green(self.h, v.ctypes.data, None) != 0:
            raise RuntimeError("not in green_mode")
        out = np.zeros(int(v[0]) * int(v[1]) * int(v[2]), np.float32)
        self._L.oracle_green(self.h, v.ctypes.data, out.ctypes.data)
        return out.reshape(int(v[0]), int(v[1]), int(v[2]))

    def snap_xy_v(self):
        out = np.zeros(self.nsnap, np.float32)
        self._L.oracle_snap_xy_v(self.h, out.ctypes.data)
        return out.reshape(-1, 3, self.nys, self.nxs)

    def sources(self):
        n = self._L.oracle_sources(self.h, None, None)
        ijk = np.zeros((n, 3), np.int32)
        vals = np.zeros((n, 12), np.float64)
        self._L.oracle_sources(self.h, ijk.ctypes.data, vals.ctypes.data)
        return ijk, vals

    def stf(self):
        return self._L.oracle_stf(self.h)

    def close(self):
        if self.h:
            self._L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def momentrate(t, stf, ts, tr):
    return lib().oracle_momentrate(t, stf, ts, tr)


def sdr2moment(strike, dip, rake):
    m = np.zeros(6, np.float32)
    lib().oracle_sdr2moment(strike, dip, rake, m.ctypes.data)
    return m  # xx yy zz yz xz xy
