"""Known-answer tests that pin the CPU oracle itself (the reference ships no
tests or golden vectors for this path, so the oracle is checked against
closed forms and physical invariants)."""
import math
import os

import numpy as np
import pytest

from openswpc_gb300 import configs
from oracle import pyoracle
from tests.helpers import misfit


@pytest.mark.parametrize("stf", range(6))
def test_source_time_functions_integrate_to_one(stf):
    # m_fdtool.f90:339-497 are normalised moment-rate functions: integral 1
    tr, dt = 1.0, 1e-4
    t = np.arange(-0.5, 8.0, dt, dtype=np.float64)
    v = np.array([pyoracle.momentrate(float(x), stf, 0.0, tr) for x in t])
    integral = np.trapezoid(v, t) if hasattr(np, "trapezoid") else np.trapz(v, t)
    assert abs(integral - 1.0) < 2e-3, integral
    assert np.all(v >= -1e-6)


def test_kupper_closed_form():
    for t in (0.1, 0.37, 0.5, 0.9):
        ref = 3 * math.pi * math.sin(math.pi * t) ** 3 / 4
        assert abs(pyoracle.momentrate(t, 3, 0.0, 1.0) - ref) < 1e-5


@pytest.mark.parametrize("sdr", [(0, 90, 0), (30, 60, 90), (123.4, 45.6, -78.9), (350, 10, 170)])
def test_double_couple_moment_tensor(sdr):
    m = pyoracle.sdr2moment(*sdr).astype(np.float64)  # xx yy zz yz xz xy
    assert abs(m[0] + m[1] + m[2]) < 1e-5            # no volume change
    norm = math.sqrt((m[0] ** 2 + m[1] ** 2 + m[2] ** 2 + 2 * (m[3] ** 2 + m[4] ** 2 + m[5] ** 2)) / 2)
    assert abs(norm - 1) < 1e-5                        # unit scalar moment
    M = np.array([[m[0], m[5], m[4]], [m[5], m[1], m[3]], [m[4], m[3], m[2]]])
    ev = np.sort(np.linalg.eigvalsh(M))
    assert np.allclose(ev, [-1, 0, 1], atol=1e-5)      # pure double couple


def test_relaxation_and_zeta(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=2)
    o = pyoracle.Oracle(inf, "fp64")
    ts = o.medium("ts").astype(np.float64)
    # log-spaced relaxation times 1/omega over [fq_min, fq_max] (m_fdtool.f90:720-723)
    om = 2 * np.pi * np.array([0.05, 0.5, 5.0])
    assert np.allclose(ts, 1 / om, rtol=1e-6)
    # taup = nm * zeta / Qp: the ratio of taup between the layers is the Q ratio
    tp = o.medium("taup")
    k_upper, k_lower = 3 + 5, 3 + 30  # halo offset 3
    assert abs(tp[64, 64, k_upper] / tp[64, 64, k_lower] - 600 / 200) < 1e-6


def test_surface_detection_and_bands(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=2)
    o = pyoracle.Oracle(inf, "fp32")
    kfs = o.medium("kfs")
    # zbeg = -1.5 km, dz = 0.5 km: cells k = 1..3 are air, the free surface is k = 3
    assert np.all(kfs[3:-3, 3:-3] == 3)
    top, bot = o.medium("kfs_top"), o.medium("kfs_bot")
    assert np.all(top[5:-5, 5:-5] == 1) and np.all(bot[5:-5, 5:-5] == 5)
    # stations 'fsb' sit one cell below the free surface
    assert np.all(o.stations()[:, 2] == 4)


def test_cross_precision_agreement(tmp_path):
    inf = configs.write_plain_small(str(tmp_path), nt=120, nx=64, ny=64, nz=48, xbeg=-16.0, ybeg=-16.0)
    w = {}
    for mode in ("fp32", "mixed", "fp64"):
        o = pyoracle.Oracle(inf, mode)
        o.run(120)
        w[mode] = o.waveforms()
    assert np.abs(w["fp64"]).max() > 0
    assert misfit(w["mixed"], w["fp64"]) < 1e-4
    assert misfit(w["fp32"], w["fp64"]) < 1e-4


def _point_force_run(tmp_path, name, src, rec, force):
    d = os.path.join(str(tmp_path), name)
    inf = configs.write_uniform(d, nx=48, ny=48, nz=48, nt=90, source=src,
                                stations=[(rec[0], rec[1], rec[2], "R")], bf=force, na=10)
    o = pyoracle.Oracle(inf, "fp64")
    o.run(90)
    return o.waveforms()[0]


def test_reciprocity_of_point_forces(tmp_path):
    # G_zx(A <- B) == G_xz(B <- A): Vz at A from an x force at B equals Vx at B
    # from a z force at A (staggered-grid averaging keeps this exact up to
    # the stencil's symmetry)
    A = ("-2.0", "1.0", "-1.0")
    B = ("3.0", "-2.0", "2.0")
    w1 = _point_force_run(tmp_path, "ab", " ".join(B), A, (1e15, 0, 0))  # force x at B, record at A
    w2 = _point_force_run(tmp_path, "ba", " ".join(A), B, (0, 0, 1e15))  # force z at A, record at B
    vz_at_a = -w1[2]  # the recorder reports Vz positive upward
    vx_at_b = w2[0]
    assert np.abs(vx_at_b).max() > 0
    assert misfit(vz_at_a, vx_at_b) < 0.05


def test_p_wave_arrival_time(tmp_path):
    # explosion in a uniform whole space: the P pulse reaches r = 8 km at r / vp
    d = str(tmp_path)
    inf = configs.write_uniform(d, nx=64, ny=64, nz=64, nt=150, dx=0.5, dt=0.02, vp=6.0, vs=3.5,
                                source="0.0 0.0 0.0", stations=[("8.0", "0.0", "0.0", "P")], na=12)
    with open(os.path.join(d, "source.dat"), "w") as f:
        f.write("0.0 0.0 0.0 0.0 1.0 1.0e16 1 1 1 0 0 0\n")
    o = pyoracle.Oracle(inf, "fp64")
    o.run(150)
    vx = o.waveforms()[0, 0]
    t = np.arange(len(vx)) * 0.02
    tpk = t[np.argmax(np.abs(vx))]
    # peak of a Kupper pulse of rise time 1 s radiated at t = 0.5 s (its centre)
    assert abs(tpk - (8.0 / 6.0 + 0.5)) < 0.25, tpk


def test_oracle_reproduces_golden_traces(tmp_path):
    """The oracle is pinned to its committed golden traces
    (tests/golden/make_golden.py): any change of its arithmetic shows here."""
    from tests.golden import make_golden
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "plain_small_nt200.npz"))
    inf = make_golden.write_inputs(str(tmp_path))
    o = pyoracle.Oracle(inf, "fp32")
    assert np.array_equal(o.stations(), g["stations"])
    o.run(int(g["nt"]))
    w = o.waveforms()
    assert np.abs(g["fp32"]).max() > 0
    assert misfit(w, g["fp32"]) < 1e-6
    # the three builds agree to the expected orders
    assert misfit(g["fp32"], g["fp64"]) < 1e-5
    assert misfit(g["mixed"], g["fp64"]) < 1e-6


def _zener_closed_form(nm, fmin, fmax, dt):
    """visco_set_relaxtime (m_fdtool.f90:691-727) and kernel__setup's Zener
    coefficients (m_kernel.f90:58-67), in FP64."""
    wa, wb = 2 * np.pi * fmin, 2 * np.pi * fmax
    ts = 1 / (wa * (wb / wa) ** (np.arange(nm) / (nm - 1)))
    c1 = (2 * ts - dt) / (2 * ts + dt)
    c2 = 2 / (2 * ts + dt) / nm
    d1 = 2 * ts / (2 * ts - dt)
    d2 = np.sum(dt / (2 * ts - dt)) / nm
    return c1, c2, d1, d2


def _damping_closed_form(x, H, xb, xe, na, fcut, dt):
    """damping_profile (m_absorb_p.f90:533-573): ADE-CFS g1..g4, in FP64."""
    R0 = 10 ** (-(np.log10(na) - 1) / np.log10(2.0) - 3.0)
    d0 = -(1 / (2 * H)) * 2 * 6.0 * np.log(R0)
    a0, b0 = np.pi * fcut, 7.0
    xx = np.where(x <= xb + H, (xb + H) - x, np.where(x >= xe - H, x - (xe - H), 0.0))
    r = np.abs(xx / H)
    d, a, b = d0 * r, a0 * (1 - r), 1 + (b0 - 1) * r * r
    den = 1 + dt / 2 * (a + d / b)
    return np.stack([((1 + dt / 2 * a) / b) / den, (-1 / b) / den, (1 - dt / 2 * (a + d / b)) / den, (d / b) / den], 1)


@pytest.mark.parametrize("mode,rtol", [("fp64", 1e-12), ("fp32", 3e-6)])
def test_zener_and_pml_coefficients_closed_form(tmp_path, mode, rtol):
    """The oracle's Zener coefficients and PML damping profiles against the
    closed forms in FP64 (exact in fp64 mode, within single-precision
    rounding in fp32 mode, which evaluates them as the reference does)."""
    inf = configs.write_plain_small(str(tmp_path), nt=2)
    o = pyoracle.Oracle(inf, mode)
    cf = o.coefs()
    c1, c2, d1, d2 = _zener_closed_form(3, 0.05, 5.0, o.dt)
    for name, ref in (("c1", c1), ("c2", c2), ("d1", d1)):
        assert np.allclose(cf[name], ref, rtol=rtol, atol=0), name
    assert abs(cf["d2"] / d2 - 1) < rtol
    for ax, n, beg, h in (("x", o.nx, o.xbeg, o.dx), ("y", o.ny, o.ybeg, o.dy), ("z", o.nz, o.zbeg, o.dz)):
        xc = beg + (np.arange(1, n + 1) - 0.5) * h  # i2x (m_fdtool.f90:639-680)
        H, xe = o.na * h, beg + n * h
        for stag, x in (("c", xc), ("e", xc + h / 2)):
            ref = _damping_closed_form(x, H, beg, xe, o.na, o.fcut, o.dt)
            got = cf["g%s%s" % (ax, stag)]
            assert np.allclose(got, ref, rtol=rtol, atol=rtol * np.abs(ref).max()), (ax, stag)
    # outside the layer d = 0: g1 = 1 (plain derivative) and g4 = 0 (the
    # auxiliary variables get no source and stay zero)
    mid = cf["gxc"][o.nx // 2]
    assert abs(mid[0] - 1) < rtol and mid[3] == 0
    o.close()


def test_point_force_matches_analytic_whole_space(tmp_path):
    """A vertical point force in a uniform whole space against the complete
    analytic solution (near field, far P, far S): the Vz traces 8 km along x
    (S) and along z (P) fit it to a few per cent after one common amplitude
    scale, and the two receivers need the same scale to 1.5 %, so the P/S
    amplitude ratio, radiation pattern and arrival times are right."""
    from tests.helpers import point_force_fit, write_point_force_case
    inf = write_point_force_case(tmp_path)
    o = pyoracle.Oracle(inf, "fp32")
    o.run(o.nt)
    w = o.waveforms()
    (ijk,), _ = o.sources()
    st = o.stations()
    offsets = [((st[q] - ijk) * 0.5).astype(np.float64) for q in range(2)]
    assert np.allclose(offsets[0], [8, 0, 0]) and np.allclose(offsets[1], [0, 0, 8])
    (a_s, r_s), (a_p, r_p) = point_force_fit(w, o.dt, offsets)
    print("point force: S residual %.3f, P residual %.3f, scale ratio %.4f" % (r_s, r_p, a_s / a_p))
    assert r_s < 0.05 and r_p < 0.05
    assert abs(a_s / a_p - 1) < 0.015
