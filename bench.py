#!/usr/bin/env python
"""Benchmark of the GB300 swpc_3d time loop.

Workload (the large single-source configuration): a 1024 x 1024 x 512 grid,
dx = dy = dz = 0.25 km, dt = 0.01 s, nt = 4000, FP32 fields, nm = 3 Zener
bodies over 0.05-5 Hz, 1-D gradient background (Vp 5 -> 7 km/s, Vs = Vp/1.73,
rho = 1.74 Vp^0.25) with a seeded exponential von Karman perturbation
(a = 5 km, 5 % rms), Qp/Qs = 600/300, free surface below 3 air cells, a 20-cell
ADE-CFS PML on the other faces, one moment-tensor source at 15 km depth, 1024
receivers on the free surface and an xy velocity snapshot every 100 steps.
Inputs are synthetic (seeded); the reference names no public data set for
this path.

A step is one time step of the whole grid (stress update, PML, source,
velocity update, PML, receiver and snapshot taps).  The metric is grid-point
updates per second (nx*ny*nz per step).  The working set (~73 GB) is far
larger than L2, so every step streams from HBM; no L2 flush is needed.

`--impl reference` times the reference's CPU path (the C++ restatement in
oracle/, built with the reference's -O2 -ffast-math -fopenmp flags, mixed
precision as the reference's default MP = DP) on all host threads.

Multi-GPU: the plain path does not shard (one domain per GPU); `--gpus N`
under torchrun runs N independent replicas ("replicas only").
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAK_FALLBACK_GBS = 6800.0

WORKLOADS = {
    # name: grid, spacing, dt, nt, receivers, snapshot interval
    "large": dict(nx=1024, ny=1024, nz=512, dx=0.25, dt=0.01, nt=4000, nst=1024, ntdec_s=100),
    "mid": dict(nx=512, ny=512, nz=256, dx=0.5, dt=0.02, nt=3000, nst=256, ntdec_s=100),
    "small": dict(nx=128, ny=128, nz=64, dx=0.5, dt=0.02, nt=1000, nst=16, ntdec_s=100),
    # the profiling case: the large workload's medium model on a grid of about
    # 3.7 GB on the device (its PML shell large enough to run the per-axis
    # launch classes), far larger than L2, so that DRAM counters of one
    # launch mean something
    "profile": dict(nx=384, ny=384, nz=192, dx=0.25, dt=0.01, nt=1000, nst=64, ntdec_s=100),
}

# Algorithmic bytes per grid point and step (FP32 storage, nm = 3): every
# state word read and written once, every medium word read once.
#   viscoelastic interior: (3 V + 6 S + 18 R) x 2 + 5 medium = 59 words
#   PML shell:             (3 V + 6 S + 18 ADE) x 2 + 3 medium = 57 words
B_INT, B_PML = 236, 228
# Per kernel (compulsory traffic of each kernel of the two-kernel schedule):
#   stress interior: V read 3, lam mu taup taus 4, S RMW 12, R RMW 36 -> 55 words
#   velocity interior: S read 6, rho 1, V RMW 6 -> 13 words
KERNEL_BYTES = {"stress_interior": 220, "vel_interior": 52, "stress_pml": 140, "vel_pml": 124}


def byte_model(store):
    """(interior B/pt, PML B/pt, per-kernel B/pt) for a storage precision:
    16-bit storage halves the 18 memory-variable words (36 RMW words,
    144 B -> 72 B per interior point); the PML shell and the medium stay FP32."""
    if store == "fp32":
        return B_INT, B_PML, dict(KERNEL_BYTES)
    kb = dict(KERNEL_BYTES)
    kb["stress_interior"] -= 72
    return B_INT - 72, B_PML, kb


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return PEAK_FALLBACK_GBS, "fallback"


def counts(w):
    nx, ny, nz, na = w["nx"], w["ny"], w["nz"], 20
    n_int = (nx - 2 * na) * (ny - 2 * na) * (nz - na)
    return n_int, nx * ny * nz - n_int


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx.append(float(c[2]))
            except ValueError:
                continue
            for nme, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nme)
        os.unlink(self.f.name)
        if sm:
            out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "samples": len(sm), "reasons": sorted(reasons)}
        return out


def make_medium(w, seed, where="device"):
    """The workload's medium.  where = "device": the background column and
    the periodic perturbation field, from which the library builds and
    post-processes every cell on the GPU (swpc_gpu_build_medium_rmed);
    where = "host": every cell built in numpy and post-processed on the host
    in FP64 (swpc_host_medium), then uploaded as five full arrays.  Both give
    the same medium bit for bit."""
    from openswpc_gb300 import configs, gpu
    nx, ny, nz, dx = w["nx"], w["ny"], w["nz"], w["dx"]
    zbeg = -3 * dx
    bg, xi, kxi0 = configs.gradient_random_fields(nx, ny, nz, dx, zbeg, seed=seed)
    if where == "device":
        return dict(bg=bg, xi=xi, kxi0=kxi0, zbeg=zbeg, where=where)
    rho, lam, mu, qp, qs = configs.rmed_apply(bg, xi, nx, ny, nz, kxi0)
    qp = np.ascontiguousarray(qp)
    qs = np.ascontiguousarray(qs)
    taup, taus, maps, ts = gpu.host_medium(nx, ny, nz, 20, 0.05, 5.0, 1.0, rho, lam, mu, qp, qs)
    return dict(rho=rho, lam=lam, mu=mu, taup=taup, taus=taus, maps=maps, ts=ts, zbeg=zbeg, where=where)


def medium_bytes(med):
    """Host bytes the medium upload reads."""
    if med["where"] == "device":
        return int(med["bg"].nbytes + med["xi"].nbytes)
    return sum(int(med[k].nbytes) for k in ("rho", "lam", "mu", "taup", "taus")) + sum(int(m.nbytes) for m in med["maps"])


def source_and_stations(w, kfs, zbeg, seed):
    rng = np.random.default_rng(seed + 1)
    nx, ny, nz, dx = w["nx"], w["ny"], w["nz"], w["dx"]
    ks = int(np.ceil((min(15.0, 0.6 * nz * dx) - zbeg) / dx))
    src = np.array([[nx // 2, ny // 2, ks]], np.int32)
    s, d, r = [np.deg2rad(v) for v in (rng.uniform(0, 360), rng.uniform(0, 90), rng.uniform(-180, 180))]
    mij = np.array([[-(np.sin(d) * np.cos(r) * np.sin(2 * s) + np.sin(2 * d) * np.sin(r) * np.sin(s) ** 2),
                     np.sin(d) * np.cos(r) * np.sin(2 * s) - np.sin(2 * d) * np.sin(r) * np.cos(s) ** 2,
                     np.sin(2 * d) * np.sin(r),
                     -(np.cos(d) * np.cos(r) * np.sin(s) - np.cos(2 * d) * np.sin(r) * np.cos(s)),
                     -(np.cos(d) * np.cos(r) * np.cos(s) + np.cos(2 * d) * np.sin(r) * np.sin(s)),
                     np.sin(d) * np.cos(r) * np.cos(2 * s) + 0.5 * np.sin(2 * d) * np.sin(r) * np.sin(2 * s)]])
    ii = rng.integers(26, nx - 25, w["nst"])
    jj = rng.integers(26, ny - 25, w["nst"])
    kk = kfs[jj + 2, ii + 2] + 1
    sta = np.stack([ii, jj, kk], 1).astype(np.int32)
    return src, mij, sta


def build_sim(w, med, nt, store="fp32", ntdec_r=100, variant=0, concurrent=None, seed=20261203, pml_points=0,
              pml_fused=None):
    """A simulation of the workload: medium (built on the device or uploaded,
    see make_medium), the moment-tensor source, the receivers and the xy
    velocity snapshot."""
    from openswpc_gb300 import gpu
    dims = gpu.make_dims(w["nx"], w["ny"], w["nz"], nt, w["dx"], w["dx"], w["dx"], w["dt"], na=20, store=store,
                         xbeg=-w["nx"] * w["dx"] / 2, ybeg=-w["ny"] * w["dx"] / 2, zbeg=med["zbeg"], fcut=1.0,
                         M0=1e16, UC=1e-15, ntdec_r=ntdec_r, variant=variant, concurrent=concurrent,
                         pml_points=pml_points, pml_fused=pml_fused)
    sim = gpu.Simulation(dims)
    if med["where"] == "device":
        maps, _ = sim.build_medium_rmed(med["bg"], med["xi"], med["kxi0"], fq_min=0.05, fq_max=5.0, fq_ref=1.0)
    else:
        maps = med["maps"]
        sim.upload_medium(med["rho"], med["lam"], med["mu"], med["taup"], med["taus"], *maps, med["ts"])
    if "sta" not in med:
        med["src"], med["mij"], med["sta"] = source_and_stations(w, maps[0], med["zbeg"], seed)
    sim.set_sources(med["src"], np.array([[0.0, 1.0]]), mo=np.array([1.0]), mij=med["mij"], stftype="kupper")
    sim.set_receivers(med["sta"], ntdec_w=1, flags=gpu.SWPC_WAV_V)
    z0 = int(np.ceil((0.25 - med["zbeg"]) / w["dx"]))
    sim.set_snapshot(gpu.SWPC_SNAP_XY_V, z0, 1, 1, w["ntdec_s"])
    return sim


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:  # host-only runs of the replica logic (tests)
            dist.init_process_group("gloo")
    return world, rank, local


def reduce_max(v, world):
    """Maximum over ranks (the timed region of the slowest replica)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def mem_available():
    """Host memory available now (bytes), from /proc/meminfo."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def oracle_bytes(nx, ny, nz, na=20, mode="mixed"):
    """Host bytes the oracle holds for a grid (mixed precision: V and S in
    FP64, the medium, the 18 shell auxiliaries over the whole grid as the
    reference allocates them, the 18 memory variables over the interior),
    plus the raw medium handed to it."""
    halo = (nx + 6) * (ny + 6) * (nz + 6)
    vs = 9 * (8 if mode != "fp32" else 4)
    n_int = (nx - 2 * na) * (ny - 2 * na) * (nz - na)
    return halo * (vs + 20 + 72 + 20) + 72 * n_int


def write_workload_inputs(d, w, nt, seed):
    """input.inf, source and stations of the large single-source workload for
    the CPU oracle: the grid, spacing and time step of `w`, the bench's
    moment tensor (same draws as source_and_stations) at 15 km, 1024 random
    surface receivers and the xy velocity snapshot every ntdec_s steps."""
    from openswpc_gb300 import configs
    nx, ny, nz, dx = w["nx"], w["ny"], w["nz"], w["dx"]
    inf = configs.write_plain_small(d, nt=nt, nx=nx, ny=ny, nz=nz, dx=dx, dy=dx, dz=dx, dt=w["dt"],
                                    xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=-3 * dx, ntdec_r=100,
                                    xy_v_sw=True, z0_xy=0.25, ntdec_s=w["ntdec_s"])
    rng = np.random.default_rng(seed + 1)
    s, dp, r = rng.uniform(0, 360), rng.uniform(0, 90), rng.uniform(-180, 180)
    with open(os.path.join(d, "source.dat"), "w") as f:
        f.write("  0.0 0.0 %.4f 0.0 1.0 1.0e16 %.6f %.6f %.6f\n" % (min(15.0, 0.6 * nz * dx), s, dp, r))
    ii = rng.integers(26, nx - 25, w["nst"])
    jj = rng.integers(26, ny - 25, w["nst"])
    with open(os.path.join(d, "stations.xy"), "w") as f:
        for q, (i, j) in enumerate(zip(ii, jj)):
            f.write("  %.4f %.4f 0.0 R%04d fsb\n" % (-nx * dx / 2 + (i - 0.5) * dx, -ny * dx / 2 + (j - 0.5) * dx, q))
    return inf


def cpu_sample(steps=8, warmup=2, n=(512, 512, 256), dx=0.5, dt=0.02, mode="mixed", seed=20261203, w=None):
    """The reference's CPU path (oracle restatement, -O2 -ffast-math -fopenmp,
    all host threads).  With `w` the workload itself (its grid, spacing,
    source, receivers and snapshot); otherwise a bounded sample: the same
    medium construction on a smaller grid."""
    from openswpc_gb300 import configs
    from oracle import pyoracle
    pyoracle.use_fast_build()
    if w is not None:
        nx, ny, nz, dx = w["nx"], w["ny"], w["nz"], w["dx"]
    else:
        nx, ny, nz = n
    cores = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        if w is not None:
            inf = write_workload_inputs(d, w, steps + warmup, seed)
        else:
            inf = configs.write_plain_small(d, nt=steps + warmup, nx=nx, ny=ny, nz=nz, dx=dx, dy=dx, dz=dx, dt=dt,
                                            xbeg=-nx * dx / 2, ybeg=-ny * dx / 2, zbeg=-3 * dx, sw_wav_v=False)
        t0 = time.perf_counter()
        rho, lam, mu, qp, qs = configs.gradient_random_medium(nx, ny, nz, dx, -3 * dx, seed=seed)
        vm = np.empty((5,) + rho.shape, np.float32)
        for q, a in enumerate((rho, lam, mu, qp, qs)):
            vm[q] = a
        del rho, lam, mu, qp, qs
        o = pyoracle.Oracle(inf, mode, cores, medium=vm)
        del vm
        t_setup = time.perf_counter() - t0
        o.run(warmup)
        t = time.perf_counter()
        o.run(steps)
        el = time.perf_counter() - t
        o.close()
    if w is not None:
        sample = "the workload itself (%dx%dx%d, its source, %d receivers and xy snapshot), %d timed steps after %d " \
                 "warm-up, %s precision" % (nx, ny, nz, w["nst"], steps, warmup, mode)
    else:
        sample = "%dx%dx%d grid of the same medium model, %d timed steps after %d warm-up, %s precision" \
                 % (nx, ny, nz, steps, warmup, mode)
    return dict(value=nx * ny * nz * steps / el, unit="pt/s", cores=cores, kind="port", sample=sample,
                seconds=el, setup_s=t_setup, same_config=w is not None)


def parity_statement():
    """Receiver misfit of the drop-in path (input.inf -> host set-up -> GPU)
    on the small plain configuration (128x128x64, 200 steps) against the
    committed golden traces of the oracle's fp32 and fp64 builds, so that
    every bench line states its error against both."""
    from openswpc_gb300 import configs, gpu
    g = np.load(os.path.join(ROOT, "tests", "golden", "plain_small_nt200.npz"))
    with tempfile.TemporaryDirectory() as d:
        inf = configs.write_plain_small(d, seed=int(g["seed"]), nt=int(g["nt"]))
        s = gpu.Simulation.from_inf(inf)
        s.run(1, int(g["nt"]))
        s.sync()
        w = s.waveforms()
        s.close()

    def mis(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))

    return {"case": "plain 128x128x64, 200 steps, golden traces of the oracle", "metric": "relative L2 receiver misfit",
            "vs_oracle_fp32": mis(w, g["fp32"]), "vs_oracle_fp64": mis(w, g["fp64"]), "bar": 1e-5}


def arm_config(w, args, world):
    """The workload description both arms print."""
    n_int, n_pml = counts(w)
    gb = (B_INT * n_int + B_PML * n_pml) / 1e9
    return {"workload": "large single source %dx%dx%d" % (w["nx"], w["ny"], w["nz"]),
            "dx_km": w["dx"], "dt_s": w["dt"], "nt": w["nt"], "nm": 3, "na": 20, "receivers": w["nst"],
            "snapshot": "xy_v every %d steps" % w["ntdec_s"], "parallelism": "replicas x%d" % world,
            "store": args.store,
            "l2": "inputs larger than L2: every step streams %.0f GB (model bytes), no flush" % gb}


def run_reference(args, w):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    # the stated grid when the host can hold the oracle's arrays; otherwise a
    # bounded sample of the same medium (and the line says so)
    full = mem_available() > 1.2 * oracle_bytes(w["nx"], w["ny"], w["nz"])
    if full:
        cb = cpu_sample(steps=args.steps, warmup=2, w=w)
    else:
        cb = cpu_sample(steps=args.steps, warmup=args.warmup)
    line = {
        "metric": "grid-pt updates/s", "value": cb["value"], "unit": "pt/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * cb["seconds"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64/f32 (mixed, reference default)", "data": "synthetic",
        # the workload's own config when the oracle ran the stated grid; the
        # sample's description otherwise
        "config": arm_config(w, args, 1) if cb["same_config"] else dict(arm_config(w, args, 1), sample=cb["sample"]),
        "reference_run": {"sample": cb["sample"], "same_grid": cb["same_config"], "oracle_setup_s": cb["setup_s"],
                          "timed_s": cb["seconds"],
                          "what": "C++ restatement of the reference's CPU time loop (oracle/swpc_oracle.cpp), "
                                  "-O2 -ffast-math -fopenmp as the reference's gfortran build, all host threads; "
                                  "the Fortran reference itself needs gfortran, MPI and netcdf-fortran, absent here"},
        "cpu_baseline": {"value": cb["value"], "unit": "pt/s", "cores": cb["cores"], "kind": "port",
                         "sample": cb["sample"]},
        "e2e": {"value": cb["value"], "unit": "pt/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def timed_window(w, steps, warmup):
    """First step of the timed window: the window of `steps` steps holds a
    snapshot frame (it = 1 + m * ntdec_s, m >= 1) near its middle and at
    least `warmup` untimed steps come before it."""
    nts = w["ntdec_s"]
    m = 1
    while 1 + m * nts - steps // 2 - 1 < warmup:
        m += 1
    return 1 + m * nts - steps // 2


def interior_tile_points(w, rows, na=20):
    """Interior points inside the tiles that the interior kernels sweep when
    the tile kernels sweep the shell too (interior_tiles of kernels_tma.cuh):
    whole 32-column tiles of the grid shifted so that the interior starts on
    a tile boundary, whole rows-row tiles from y = 0, the interior's planes."""
    x0 = y0 = na
    nxi, nyi, nzi = w["nx"] - 2 * na, w["ny"] - 2 * na, w["nz"] - na
    tx0 = x0 - 32 * (-(-x0 // 32))
    bxl, byl = (x0 - tx0 + 31) // 32, (y0 + rows - 1) // rows
    bxh, byh = max(bxl, (x0 + nxi - tx0) // 32), max(byl, (y0 + nyi) // rows)
    return (bxh - bxl) * 32 * (byh - byl) * rows * nzi


def shell_bytes(sim):
    """PML shell points and their algorithmic bytes per step in each phase of
    the shell-tile kernels, which take the edge moduli and buoyancies from
    the staged medium tiles instead of the precomputed arrays: per point the
    figures of pml_class_report without those 12 B (and with rho, 4 B, for
    the velocity update), summed over the classes."""
    _, _, pts, ax = sim.profile_read_pml()
    n, a = float(pts.sum()), float(ax.sum())
    return int(n), {"stress": 68.0 * n + 24.0 * a, "vel": 52.0 * n + 24.0 * a}


def pml_class_report(sim, peak):
    """Per launch class of the PML kernels: time per launch and the
    algorithmic bytes of its points.  Per shell point the stress update
    reads V (12 B), lam, mu (8 B) and the three precomputed edge moduli
    (12 B) and rewrites S (48 B); the velocity update reads S (24 B) and the
    three precomputed buoyancies (12 B) and rewrites V (24 B); every damped
    axis adds three auxiliaries read and written (24 B)."""
    ms, n, pts, ax = sim.profile_read_pml()
    names = ["x", "y", "z", "general"]
    out = {}
    for u, (kname, base) in enumerate((("stress_pml", 80), ("vel_pml", 60))):
        tot_b, tot_ms = 0.0, 0.0
        cls = {}
        for q in range(4):
            if n[u, q] == 0:
                continue
            b = base * float(pts[q]) + 24.0 * float(ax[q])
            t = ms[u, q] / n[u, q]
            cls[names[q]] = {"points": int(pts[q]), "bytes_per_point": b / max(pts[q], 1), "ms": t,
                             "GBps": b / (t / 1e3) / 1e9, "frac": b / (t / 1e3) / 1e9 / peak}
            tot_b += b
            tot_ms += t
        out[kname] = {"classes": cls, "bytes": tot_b, "ms": tot_ms,
                      "GBps": tot_b / (tot_ms / 1e3) / 1e9 if tot_ms > 0 else None,
                      "frac": tot_b / (tot_ms / 1e3) / 1e9 / peak if tot_ms > 0 else None}
    return out


def run_gpu(args, w):
    world, rank, local = dist_init()
    from openswpc_gb300 import gpu
    import torch
    torch.cuda.set_device(local)
    gpu.lib()
    peak, peak_kind = peaks()
    seed = 20261203 + 7 * rank
    t_setup = time.time()
    med = make_medium(w, seed, args.medium)
    sim = build_sim(w, med, w["nt"], store=args.store, variant=args.variant, concurrent=args.pml_overlap, seed=seed,
                    pml_points=args.pml_points, pml_fused=args.pml_form == "tiles")
    if args.tiles:
        sim.set_tiles(*[int(v) for v in args.tiles.split(",")])
    if args.zchunks:
        sim.set_zchunks(*[int(v) for v in args.zchunks.split(",")])
    stream = torch.cuda.ExternalStream(sim.stream())
    t_setup = time.time() - t_setup

    # untimed warm-up up to the timed window, which holds a snapshot frame
    it = timed_window(w, args.steps, args.warmup)
    sim.run(1, it - 1)
    sim.sync()
    # timed region: the production path (graph replay), CUDA events on the
    # simulation's stream
    n0 = sim.launch_count()
    clk = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clk.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.run(it, it + args.steps - 1)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(world)
    ms = e0.elapsed_time(e1)
    launches = sim.launch_count() - n0
    frames = [f for f in range(it, it + args.steps) if (f - 1) % w["ntdec_s"] == 0]
    it += args.steps
    # per-kernel pass: the next K steps launched one by one with an event
    # pair around every kernel (outside the headline region)
    sim.profile(True)
    sim.run(it, it + args.steps - 1)
    it += args.steps
    kms, kn = sim.profile_read()
    fused = sim.pml_fused
    pml = pml_class_report(sim, peak)
    shell_pts, shell_b = shell_bytes(sim)
    sim_tiles, sim_z = sim.tiles(), sim.zchunks()
    sim.profile(False)
    sim.sync()
    ms_max = reduce_max(ms, world)
    npt = w["nx"] * w["ny"] * w["nz"]
    value = world * npt * args.steps / (ms_max / 1e3)
    n_int, n_pml = counts(w)
    b_int, b_pml, kbytes = byte_model(args.store)
    step_bytes = b_int * n_int + b_pml * n_pml
    kern = {}
    if fused:
        # the interior kernels sweep the tiles wholly inside the interior, the
        # shell-tile kernels the rest: the shell points (bytes as in the
        # shell launches' accounting, see pml_class_report) and the interior
        # points of the tiles that straddle the interior's edge
        for q, (ph, kb, sb, rows) in enumerate((("stress", "stress_interior", "stress", sim_tiles[0]),
                                                ("vel", "vel_interior", "vel", sim_tiles[1]))):
            n_it = interior_tile_points(w, rows)
            for nm, cls, b in ((ph + "_interior", q, kbytes[kb] * n_it),
                               (ph + "_shell", 2 + q, kbytes[kb] * (n_int - n_it) + shell_b[sb])):
                t = float(kms[cls] / max(kn[cls], 1))
                kern[nm] = {"ms": t, "bytes": b, "GBps": b / (t / 1e3) / 1e9 if t > 0 else None}
                kern[nm]["frac"] = kern[nm]["GBps"] / peak if kern[nm]["GBps"] else None
            kern[ph + "_interior"]["points"] = n_it
            kern[ph + "_shell"].update({"shell_points": shell_pts, "interior_points": n_int - n_it})
        top = "stress_interior"
    else:
        for q, nm in enumerate(["stress_interior", "vel_interior"]):
            t = float(kms[q] / max(kn[q], 1))
            kern[nm] = {"ms": t, "bytes": kbytes[nm] * n_int,
                        "GBps": kbytes[nm] * n_int / (t / 1e3) / 1e9 if t > 0 else None}
            kern[nm]["frac"] = kern[nm]["GBps"] / peak if kern[nm]["GBps"] else None
        kern.update(pml)
        top = "stress_interior"
    tot = sum(kern[k]["ms"] for k in kern)
    for k in kern:
        kern[k]["share"] = kern[k]["ms"] / tot if tot > 0 else None
    achieved = kern[top]["GBps"]
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp) and args.store == "fp32" and w is WORKLOADS["large"]:
        try:
            with open(tp) as f:
                traffic = json.load(f).get(("fused_" if fused else "") + top + "_bytes_per_launch")
        except Exception:
            traffic = None
    sim.close()
    del stream

    # end to end through the C ABI: create + upload from pinned host memory +
    # K steps + waveform read-back + destroy
    e2e = None
    if not args.no_e2e:
        keys = ("bg", "xi") if med["where"] == "device" else ("rho", "lam", "mu", "taup", "taus")
        pin = {}
        for k in keys:
            t = torch.empty(med[k].shape, dtype=torch.float32, pin_memory=True)
            t.numpy()[...] = med[k]
            pin[k] = t
        med_p = dict(med)
        for k in pin:
            med_p[k] = pin[k].numpy()
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim2 = build_sim(w, med_p, args.steps, store=args.store, variant=args.variant, concurrent=args.pml_overlap,
                         seed=seed, pml_points=args.pml_points, pml_fused=args.pml_form == "tiles")
        if args.tiles:
            sim2.set_tiles(*[int(v) for v in args.tiles.split(",")])
        if args.zchunks:
            sim2.set_zchunks(*[int(v) for v in args.zchunks.split(",")])
        sim2.run(1, args.steps)
        wav = sim2.waveforms()
        sim2.close()
        t1 = time.perf_counter()
        e_s = reduce_max(t1 - t0, world)
        h2d = medium_bytes(med)
        what = ("build_medium_rmed (background column + perturbation field from pinned host memory)"
                if med["where"] == "device" else "upload_medium (five halo arrays from pinned host memory)")
        e2e = {"value": world * npt * args.steps / e_s, "unit": "pt/s",
               "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": int(wav.nbytes) // args.steps,
               "job": "create + %s + sources/receivers/snapshot + %d steps + fetch_waveforms + destroy"
                      % (what, args.steps),
               "seconds": e_s}
        del pin, med_p

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cb = cpu_sample()
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    batch = serve = prec = None
    if rank == 0 and world == 1 and not args.no_batch:
        batch = batch_block(args)
        serve = serve_block()
        if args.store == "fp32":
            prec = precision_block(w, med, ms_max / args.steps)

    if rank == 0:
        line = {
            "metric": "grid-pt updates/s", "value": value, "unit": "pt/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": arm_config(w, args, world),
            "kernel_shape": {"tiles": list(sim_tiles), "zchunks": list(sim_z),
                             "pml_shell": "swept by the tile kernels" if fused else
                             "own launches, %s" % ({0: "one point per thread", 1: "one point per thread",
                                                    2: "two points per thread"}[args.pml_points])},
            "timed_window": "it=%d..%d (graph replay; snapshot frame at it=%s)"
                            % (it - 2 * args.steps, it - args.steps - 1, ",".join(map(str, frames))),
            "hbm_fraction_step": {"bytes_per_step": step_bytes, "GBps": step_bytes / (ms_max / args.steps / 1e3) / 1e9,
                                  "peak": peak, "frac": step_bytes / (ms_max / args.steps / 1e3) / 1e9 / peak,
                                  "model": "%d B/interior pt + %d B/PML pt per step" % (b_int, b_pml)},
            "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "traffic": traffic,
                         "algorithmic_bytes_per_launch": kern[top]["bytes"], "peak_source": peak_kind},
            "kernels": kern,
            "kernel_timing": "per-launch CUDA events on the simulation's stream over the %d steps after the "
                             "timed region (launched one by one)" % args.steps,
            "clocks": clocks,
            "gpu_launches": launches,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "parity": parity_statement(),
            "batched": batch,
            "served": serve,
            "precision": prec,
            "setup_s": t_setup,
            "medium_setup": med["where"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def batch_inputs(n, seed, nt, root):
    """The batched many-instance workload: n simulations, each axis drawn
    uniformly from {96, 128, ..., 256}, dt = 0.02 s, seeded 3-5 layer media,
    a 50/50 mix of single forces and double couples, 8 receivers each."""
    from openswpc_gb300 import configs
    rng = np.random.default_rng(seed)
    sizes = rng.choice(np.arange(96, 257, 32), size=(n, 3))
    infs = []
    for q, (nx, ny, nz) in enumerate(sizes):
        d = os.path.join(root, "m%03d" % q)
        infs.append(configs.write_layered(d, int(nx), int(ny), int(nz), seed + q, nt=nt, n_station=8))
    return infs, sizes


def member_bytes(nx, ny, nz, na=20):
    """Model bytes of one time step of a member (236 B per interior point,
    228 B per PML point)."""
    n_int = (nx - 2 * na) * (ny - 2 * na) * (nz - na)
    return B_INT * n_int + B_PML * (nx * ny * nz - n_int)


def batch_measure(nsim, steps, warmup, tune=True, seed=20261203, nt_full=1500, tiles=None, zchunks=None):
    """n simulations of the batched workload advanced together (swpc_batch)
    versus the same simulations one after another on the plain path; both
    timed with CUDA events over `steps` steps and scaled to nt_full steps
    (every step of a run costs the same).  Returns ms per step of each arm,
    solves/s, grid-point updates/s and the HBM fraction of the model bytes."""
    from openswpc_gb300 import autotune, gpu
    import torch
    gpu.lib()
    peak, _ = peaks()
    with tempfile.TemporaryDirectory() as root:
        infs, sizes = batch_inputs(nsim, seed, nt_full, root)
        sims = [gpu.Simulation.from_inf(f) for f in infs]
        pts = [int(np.prod(s)) for s in sizes]
        step_bytes = float(sum(member_bytes(*map(int, s)) for s in sizes))
        rec, t_tune = None, 0.0
        for s in sims:
            if tiles:
                s.set_tiles(*tiles)
            if zchunks:
                s.set_zchunks(*zchunks)
        if tune:
            t0 = time.time()
            rec = autotune.tune(sims)
            t_tune = time.time() - t0
        b = gpu.Batch(sims)
        st = torch.cuda.ExternalStream(b.stream())
        b.run(warmup)
        b.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = b.launch_count()
        e0.record(st)
        b.run(steps)
        e1.record(st)
        e1.synchronize()
        ms_batch = e0.elapsed_time(e1) / steps
        launches = b.launch_count() - n0
        items = b.item_count()
        # the same batch as one persistent fused launch per step (8-row tiles)
        ms_persist = None
        shape = sims[-1].tiles()
        if shape == (8, 8):
            b.set_persistent(True)
            b.run(warmup)
            b.sync()
            e0.record(st)
            b.run(steps)
            e1.record(st)
            e1.synchronize()
            ms_persist = e0.elapsed_time(e1) / steps
        b.close()
        # the same members one after another, each on its own plain path
        ms_seq = 0.0
        for s in sims:
            s.reset()
            s.set_tiles(0, 0)
            s.set_zchunk(0)
            s.run(1, warmup)
            s.sync()
            stq = torch.cuda.ExternalStream(s.stream())
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(stq)
            s.run(warmup + 1, warmup + steps)
            a1.record(stq)
            a1.synchronize()
            ms_seq += a0.elapsed_time(a1) / steps
        for s in sims:
            s.close()
    gbps_b = step_bytes / (ms_batch / 1e3) / 1e9
    gbps_s = step_bytes / (ms_seq / 1e3) / 1e9
    return {"members": nsim, "points_total": int(sum(pts)), "steps": steps, "warmup": warmup,
            "form": "one launch per phase of the time step over all members, graph-replayed",
            "ms_per_step": ms_batch, "sequential_ms_per_step": ms_seq,
            "persistent_ms_per_step": ms_persist, "persistent_items_per_step": items,
            "solves_per_s": nsim / (nt_full * ms_batch / 1e3), "sequential_solves_per_s": nsim / (nt_full * ms_seq / 1e3),
            "speedup_vs_sequential": ms_seq / ms_batch,
            "grid_pt_updates_per_s": sum(pts) / (ms_batch / 1e3),
            "sequential_grid_pt_updates_per_s": sum(pts) / (ms_seq / 1e3),
            "model_bytes_per_step": step_bytes,
            "hbm_frac": gbps_b / peak, "sequential_hbm_frac": gbps_s / peak,
            "gpu_launches": launches, "autotune": rec, "autotune_s": t_tune,
            "nt_full": nt_full}


def batch_block(args):
    """Short batched block of the default run: 16 members of the batched
    workload, 20 steps each arm."""
    try:
        r = batch_measure(16, 20, 3, tune=False)
        r["workload"] = "batched many-instance: 16 simulations, axes in {96..256}, timed 20 steps, solves/s at nt=1500"
        return r
    except Exception as e:  # the headline line is still printed
        return {"error": str(e)}


def run_batch(args):
    """Batched form: solves/s of n simulations advanced together versus the
    same simulations run one after another on the plain path."""
    r = batch_measure(args.nsim, args.steps, args.warmup, tune=not args.no_tune,
                      tiles=[int(v) for v in args.tiles.split(",")] if args.tiles else None,
                      zchunks=[int(v) for v in args.zchunks.split(",")] if args.zchunks else None)
    line = {"metric": "batched solves/s", "value": r["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched many-instance: %d simulations, axes in {96..256}, nt=%d"
                                   % (args.nsim, r["nt_full"]), "points_total": r["points_total"],
                       "zchunk": [r["autotune"]["zchunk"], r["autotune"]["zchunk_vel"]] if r["autotune"] else None,
                       "tiles": r["autotune"]["tiles"] if r["autotune"] else None},
            "gpu_launches": r["gpu_launches"]}
    line.update({k: v for k, v in r.items() if k not in ("gpu_launches",)})
    print(json.dumps(line), flush=True)
    return 0


def serve_inputs(n, seed, nt, root, tail=0.1):
    """Requests of the serving workload: the batched generator, with a
    fraction `tail` of the requests replaced by 512 x 512 x 256 grids."""
    from openswpc_gb300 import configs
    rng = np.random.default_rng(seed)
    sizes = rng.choice(np.arange(96, 257, 32), size=(n, 3))
    big = rng.random(n) < tail
    sizes[big] = (512, 512, 256)
    infs = []
    for q, (nx, ny, nz) in enumerate(sizes):
        d = os.path.join(root, "r%04d" % q)
        infs.append(configs.write_layered(d, int(nx), int(ny), int(nz), seed + q, nt=nt, n_station=8))
    return infs, sizes


def serve_measure(requests, nt, rates, budget_gb, quantum, seed=20261203):
    """Serving form: Poisson arrivals at each rate submitted to the
    continuous-batching server (swpc_serve_*), latency = completion minus
    arrival; then the same requests one after another on the plain path
    (host set-up + run + trace read-back each), which also gives every
    request's result alone for the misfit check."""
    from openswpc_gb300 import gpu
    gpu.lib()
    with tempfile.TemporaryDirectory() as root:
        infs, sizes = serve_inputs(requests, seed, nt, root)
        pts = [int(np.prod(s)) for s in sizes]
        # sequential plain path: each request alone, end to end
        alone = []
        t0 = time.perf_counter()
        for f in infs:
            s = gpu.Simulation.from_inf(f)
            s.run(1, nt)
            s.sync()
            alone.append(s.waveforms())
            s.close()
        t_seq = time.perf_counter() - t0
        per_rate = []
        worst = 0.0
        for lam in rates:
            rng = np.random.default_rng(int(lam * 1000) + 7)
            gaps = rng.exponential(1.0 / lam, size=len(infs))
            with gpu.Server(hbm_budget=budget_gb * 1e9, quantum=quantum, prep_threads=8) as srv:
                ids = []
                tstart = time.perf_counter()
                tnext = tstart
                for f, g in zip(infs, gaps):
                    tnext += g
                    dly = tnext - time.perf_counter()
                    if dly > 0:
                        time.sleep(dly)
                    ids.append(srv.submit(f))
                for rid in ids:
                    srv.wait(rid)
                t_all = time.perf_counter() - tstart
                lat = []
                for rid, w in zip(ids, alone):
                    t = srv.times(rid)
                    lat.append(t["finished"] - t["submitted"])
                    got = srv.result(rid)
                    den = float(np.linalg.norm(w))
                    worst = max(worst, float(np.linalg.norm(got - w)) / den if den > 0 else 0.0)
                    srv.release(rid)
                st = srv.stats()
            lat = np.array(lat)
            per_rate.append({"rate_per_s": lam, "solves_per_s": len(ids) / t_all, "wall_s": t_all,
                             "p50_s": float(np.percentile(lat, 50)), "p95_s": float(np.percentile(lat, 95)),
                             "p99_s": float(np.percentile(lat, 99)), "peak_device_gb": st["peak_bytes"] / 1e9,
                             "quanta": int(st["quanta"]), "batch_rebuilds": int(st["rebuilds"]),
                             "grid_pt_updates_per_s": st["updates"] / t_all})
    best = max(per_rate, key=lambda r: r["solves_per_s"])
    return {"requests": len(infs), "nt": nt, "rates": per_rate, "best_solves_per_s": best["solves_per_s"],
            "sequential_solves_per_s": len(infs) / t_seq, "sequential_wall_s": t_seq,
            "speedup_vs_sequential": best["solves_per_s"] / (len(infs) / t_seq), "misfit_vs_alone_max": worst,
            "points_total": int(sum(pts)), "hbm_budget_gb": budget_gb, "quantum_steps": quantum}


def serve_block():
    """Short serving block of the default run: 24 requests of the serving
    workload (10 % of them 512 x 512 x 256), nt = 300, arriving at 20 per s."""
    try:
        r = serve_measure(24, 300, [20.0], 150.0, 50)
        r["workload"] = "serving: 24 Poisson requests at 20/s, axes in {96..256} with 10% 512x512x256, nt=300"
        return r
    except Exception as e:  # the headline line is still printed
        return {"error": str(e)}


def run_serve(args):
    rates = [float(r) for r in args.rates.split(",")]
    r = serve_measure(args.requests, args.nt, rates, args.budget_gb, args.quantum)
    out = {"metric": "served solves/s and latency", "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "value": r["best_solves_per_s"],
           "config": {"workload": "serving: Poisson arrivals, %d requests per rate, axes in {96..256} with 10%% "
                                  "512x512x256, nt=%d" % (r["requests"], args.nt),
                      "hbm_budget_gb": args.budget_gb, "quantum_steps": args.quantum,
                      "points_total": r["points_total"],
                      "timing": "wall clock from first arrival to last completion, host set-up included"}}
    out.update({k: v for k, v in r.items() if k not in ("points_total", "hbm_budget_gb", "quantum_steps")})
    print(json.dumps(out), flush=True)
    return 0


def precision_block(w, med, ms_fp32, steps=20, warmup=3):
    """Short precision block of the default run: the headline workload with
    FP16 memory variables, timed like the headline (graph replay, CUDA events
    over `steps` steps) against the FP32 step time."""
    try:
        import torch
        sim = build_sim(w, med, w["nt"], store="fp16")
        st = torch.cuda.ExternalStream(sim.stream())
        sim.run(1, warmup)
        sim.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sim.run(warmup + 1, warmup + steps)
        e1.record(st)
        e1.synchronize()
        sim.sync()
        sim.close()
        ms = e0.elapsed_time(e1) / steps
        n_int, n_pml = counts(w)
        b16, bp, _ = byte_model("fp16")
        return {"workload": "large single source, FP16 memory variables", "ms_per_step": ms,
                "updates_per_s": w["nx"] * w["ny"] * w["nz"] / (ms / 1e3), "speedup_vs_fp32": ms_fp32 / ms,
                "bytes_per_step": b16 * n_int + bp * n_pml,
                "misfit": "see the precision workload (bench.py --workload precision)"}
    except Exception as e:
        return {"error": str(e)}


def run_precision(args):
    """Precision form: the large workload's medium generator and source at
    512 x 512 x 256 (dx = 0.5 km), run with FP32, FP16 and BF16 storage of
    the memory variables for --nt steps; reports updates/s (CUDA events over
    the whole run), the byte model per step and the receiver misfit of each
    16-bit form against the FP32 path."""
    from openswpc_gb300 import gpu
    import torch
    gpu.lib()
    w = WORKLOADS["mid"]
    seed = 20261203
    med = make_medium(w, seed, args.medium)
    n_int, n_pml = counts(w)
    npt = w["nx"] * w["ny"] * w["nz"]
    res = {}
    for store in ("fp32", "fp16", "bf16"):
        sim = build_sim(w, med, args.nt, store=store)
        st = torch.cuda.ExternalStream(sim.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sim.run(1, args.nt)
        e1.record(st)
        e1.synchronize()
        sim.sync()
        ms = e0.elapsed_time(e1) / args.nt
        wav = sim.waveforms()
        sim.close()
        b_int, b_pml, _ = byte_model(store)
        res[store] = {"ms_per_step": ms, "updates_per_s": npt / (ms / 1e3),
                      "bytes_per_step": b_int * n_int + b_pml * n_pml, "wav": wav}
    ref = res["fp32"]["wav"]
    den = float(np.linalg.norm(ref))
    forms = {}
    for store, r in res.items():
        forms[store] = {k: v for k, v in r.items() if k != "wav"}
        forms[store]["misfit_vs_fp32"] = float(np.linalg.norm(r["wav"] - ref)) / den if den > 0 else None
        forms[store]["speedup_vs_fp32"] = res["fp32"]["ms_per_step"] / r["ms_per_step"]
    out = {"metric": "grid-pt updates/s by storage precision", "value": forms["fp16"]["updates_per_s"],
           "unit": "pt/s", "n_gpus": 1, "steps": args.nt, "warmup": 0, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "forms": forms,
           "config": {"workload": "precision form 512x512x256, large-workload medium and source, nt=%d" % args.nt,
                      "timing": "CUDA events over the whole run from it=1 (graph replay)"}}
    if not args.no_cpu:
        out["vs_fp64_oracle"] = precision_vs_fp64(args.nt, seed)
    print(json.dumps(out), flush=True)
    return 0


def precision_vs_fp64(nt, seed):
    """Receiver misfit of the three storage forms against the oracle built in
    FP64, on a downscaled copy of the precision workload (256 x 256 x 128 at
    the same spacing, the same medium model, source and receiver rule): the
    FP64 oracle over the full 512 x 512 x 256 grid and nt steps would keep
    the host busy for a quarter of an hour."""
    from oracle import pyoracle
    from openswpc_gb300 import configs
    wq = dict(WORKLOADS["mid"], nx=256, ny=256, nz=128, nst=64)
    med = make_medium(wq, seed, "device")
    wavs = {}
    for store in ("fp32", "fp16", "bf16"):
        sim = build_sim(wq, med, nt, store=store, seed=seed)
        sim.run(1, nt)
        wavs[store] = sim.waveforms()
        sim.close()
    with tempfile.TemporaryDirectory() as d:
        inf = write_workload_inputs(d, wq, nt, seed)
        bg, xi, kxi0 = configs.gradient_random_fields(wq["nx"], wq["ny"], wq["nz"], wq["dx"], -3 * wq["dx"], seed=seed)
        vm = np.stack(configs.rmed_apply(bg, xi, wq["nx"], wq["ny"], wq["nz"], kxi0))
        t0 = time.perf_counter()
        o = pyoracle.Oracle(inf, "fp64", os.cpu_count() or 1, medium=vm)
        o.run(nt)
        ref = o.waveforms()
        sta = o.stations()
        o.close()
        t_or = time.perf_counter() - t0
    assert np.array_equal(sta[:, :2], med["sta"][:, :2]), "oracle and GPU receivers differ"
    den = float(np.linalg.norm(ref))
    return {"grid": "256x256x128, dx=0.5 km, nt=%d" % nt, "oracle": "fp64 build of the oracle", "oracle_s": t_or,
            "misfit": {k: float(np.linalg.norm(w.astype(np.float64) - ref)) / den for k, w in wavs.items()},
            "fp16_vs_fp32": float(np.linalg.norm(wavs["fp16"] - wavs["fp32"]) / np.linalg.norm(wavs["fp32"])),
            "bf16_vs_fp32": float(np.linalg.norm(wavs["bf16"] - wavs["fp32"]) / np.linalg.norm(wavs["fp32"]))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS) + ["batch", "serve", "precision"])
    ap.add_argument("--nsim", type=int, default=64, help="members of the batched workload")
    ap.add_argument("--rates", default="2,10,50", help="serving: Poisson arrival rates [1/s]")
    ap.add_argument("--requests", type=int, default=48, help="serving: requests per rate")
    ap.add_argument("--nt", type=int, default=300, help="serving / precision: time steps per simulation")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: device-memory budget")
    ap.add_argument("--quantum", type=int, default=50, help="serving: steps between scheduling points")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the short batched block of the default run")
    ap.add_argument("--no-tune", action="store_true",
                    help="batch workload: no autotuning (the members take --tiles/--zchunks or the library's choice)")
    ap.add_argument("--tiles", default="", help="rows of the stress and velocity tiles, e.g. 16,8 (default: 8,8)")
    ap.add_argument("--zchunks", default="", help="z-sweep depths of the stress and velocity kernels, e.g. 8,128")
    ap.add_argument("--pml-points", type=int, default=0, choices=[0, 1, 2],
                    help="shell points per thread of the PML kernels (0: library default)")
    ap.add_argument("--medium", default="device", choices=["device", "host"],
                    help="build the random medium on the GPU (default) or on the host and upload it")
    ap.add_argument("--store", default="fp32", choices=["fp32", "fp16", "bf16"])
    ap.add_argument("--variant", type=int, default=0, help="0: TMA-fed interior kernels, 1: plain smem sweep")
    ap.add_argument("--pml-form", choices=["launches", "tiles"], default="launches",
                    help="PML shell in launches of its own, or swept by shell-tile kernels beside the interior ones")
    ap.add_argument("--pml-overlap", type=lambda v: {"auto": None, "on": True, "off": False}[v], default=None,
                    help="auto|on|off: run the PML kernels beside the interior ones")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "precision":
        return run_precision(args)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())
