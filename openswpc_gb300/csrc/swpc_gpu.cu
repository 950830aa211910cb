// swpc_gpu.cu -- C ABI, device memory and launch sequencing of the GB300
// swpc_3d time step.  The kernels are in kernels.cuh.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/swpc_gpu.h"
#include "kernels.cuh"
#include "medium.cuh"
#include "persist.cuh"
#include "sim.hpp"
#include "visco.hpp"

using namespace swpc;

namespace {
thread_local std::string g_err;
}

namespace swpc {
int set_err(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
}  // namespace swpc

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return set_err(SWPC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static inline long long rup(long long v, long long m) { return (v + m - 1) / m * m; }

// ---------------------------------------------------------------------------
// geometry and allocation plan
// ---------------------------------------------------------------------------
static int plan(const swpc_dims* d, Plan& p) {
    if (!d) return set_err(SWPC_E_ARG, "null dims");
    if (d->nm != NM) return set_err(SWPC_E_ARG, "nm must be 3 (compile-time constant NM of m_global.f90:31)");
    if (d->nx < 8 || d->ny < 8 || d->nz < 8) return set_err(SWPC_E_ARG, "grid too small (nx, ny, nz >= 8)");
    if (d->abc_type != SWPC_ABC_PML && d->abc_type != SWPC_ABC_CERJAN) return set_err(SWPC_E_ARG, "abc_type must be PML or Cerjan");
    if (d->na < 0 || (d->abc_type == SWPC_ABC_PML && (d->nx <= 2 * d->na + 2 || d->ny <= 2 * d->na + 2 || d->nz <= d->na + 2)))
        return set_err(SWPC_E_ARG, "absorber thickness na leaves no interior");
    if (!(d->dx > 0 && d->dy > 0 && d->dz > 0 && d->dt > 0)) return set_err(SWPC_E_ARG, "dx, dy, dz, dt must be positive");
    if (d->store < SWPC_STORE_FP32 || d->store > SWPC_STORE_BF16) return set_err(SWPC_E_ARG, "bad store mode");
    if ((long long)d->nx * d->ny * d->nz > (1LL << 36)) return set_err(SWPC_E_ARG, "grid too large");
    p.pml = d->abc_type == SWPC_ABC_PML;
    p.x0 = p.pml ? d->na : 0;
    p.y0 = p.pml ? d->na : 0;
    p.nxi = p.pml ? d->nx - 2 * d->na : d->nx;
    p.nyi = p.pml ? d->ny - 2 * d->na : d->ny;
    p.nzi = p.pml ? d->nz - d->na : d->nz;
    Geo& g = p.g;
    g.nx = d->nx; g.ny = d->ny; g.nz = d->nz; g.na = d->na;
    g.hx = 4 + ((32 - (4 + p.x0) % 32) % 32);
    g.pitch = (int)rup(g.hx + d->nx + 40, 32);
    g.nyp = HYT + d->ny + TBY + 3;
    g.nzp = HZT + d->nz + 3;
    p.rpitch = (int)rup(p.nxi, 32);
    const long long cell = (long long)g.pitch * g.nyp * g.nzp;
    p.nV = 3 * cell; p.nS = 6 * cell; p.nM = 5 * cell;
    p.rbytes = d->store == SWPC_STORE_FP32 ? 4 : 2;
    p.nR = 18LL * p.rpitch * p.nyi * p.nzi;
    // PML shell boxes
    p.nbox = 0;
    p.nade = 0;
    p.nshm = 0;
    long long first = 0;
    if (p.pml) {
        const int na = d->na, nx = d->nx, ny = d->ny, nz = d->nz;
        int bx[5][6] = {{0, 0, 0, na, ny, nz}, {nx - na, 0, 0, na, ny, nz}, {na, 0, 0, nx - 2 * na, na, nz},
                        {na, ny - na, 0, nx - 2 * na, na, nz}, {na, na, nz - na, nx - 2 * na, ny - 2 * na, na}};
        for (int b = 0; b < 5; ++b) {
            if (bx[b][3] <= 0 || bx[b][4] <= 0 || bx[b][5] <= 0) continue;
            PmlBox& B = p.box[p.nbox++];
            B.x0 = bx[b][0]; B.y0 = bx[b][1]; B.z0 = bx[b][2]; B.nx = bx[b][3]; B.ny = bx[b][4]; B.nz = bx[b][5];
            B.pitch = B.nx;  // rows without padding, one array per auxiliary
            const long long vol = (long long)B.nx * B.ny * B.nz;
            if (vol > 0x7fffffffLL) return set_err(SWPC_E_ARG, "a PML box holds more than 2^31 - 1 cells");
            B.qs = (int)vol;
            B.off = p.nade;
            p.nade += 9LL * B.pitch * B.ny * B.nz;
            B.moff = p.nshm;
            p.nshm += 6LL * B.pitch * B.ny * B.nz;
            first += (long long)B.nx * B.ny * B.nz;
        }
    }
    p.npml = first;
    p.bytes = 4 * (p.nV + p.nS + p.nM) + p.rbytes * p.nR + 4 * (2 * p.nade + p.nshm) + 16LL * p.nxi * p.nyi;
    return 0;
}

// ---------------------------------------------------------------------------
// FP64 coefficient set-up
// ---------------------------------------------------------------------------
static void damping_profile(double x, double H, double xb, double xe, double na, double fcut, double dt, float* g) {
    // m_absorb_p.f90:533-573 (FP64 arithmetic, rounded to FP32 storage)
    const double R0 = std::pow(10.0, -(std::log10(na) - 1) / std::log10(2.0) - 3.0);
    const double d0 = -(1.0 / (2.0 * H)) * 2.0 * 6.0 * std::log(R0);
    const double b0 = 7.0, a0 = M_PI * fcut;
    double xx;
    if (x <= xb + H) xx = (xb + H) - x;
    else if (x >= xe - H) xx = x - (xe - H);
    else xx = 0;
    const double r = std::fabs(xx / H);
    const double d = d0 * r, a = a0 * (1 - r), b = 1 + (b0 - 1) * r * r;
    const double h = dt / 2.0, den = 1 + h * (a + d / b);
    g[0] = (float)(((1 + h * a) / b) / den);
    g[1] = (float)((-1.0 / b) / den);
    g[2] = (float)((1 - h * (a + d / b)) / den);
    g[3] = (float)((d / b) / den);
}

static void cerjan_profile(int n, int na, double d, std::vector<float>& c, std::vector<float>& bnd, bool zaxis) {
    // m_absorb_c.f90:55-101: exp(-alpha (1 - x/L)^2) at cell centre and boundary
    const double alpha = 0.09, L = na * d;
    c.assign(n, 1.f); bnd.assign(n, 1.f);
    for (int q = 1; q <= n; ++q) {
        auto e = [&](double x) { double t = 1.0 - x / L; return (float)std::exp(-alpha * t * t); };
        if (q <= na && !zaxis) {
            double xc = (q - 0.5) * d;
            c[q - 1] = e(xc); bnd[q - 1] = e(xc + d / 2);
        } else if (q >= n - na + 1) {
            double xr = n * d - (q - 0.5) * d;
            c[q - 1] = e(xr + d / 2); bnd[q - 1] = e(xr);
        }
    }
}

// ---------------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------------
void Sim::fill_zargs(ZArgs& z, bool shell_view) const {
    // shell_view: the sweep over the whole grid when the tile kernels sweep
    // the shell (interior and shell-tile kernels); otherwise the interior box
    const bool f = shell_view && pml_fused;
    z.g = p.g;
    z.V = V; z.S = S; z.M = M; z.R = R; z.band = band;
    z.x0 = p.x0; z.y0 = p.y0; z.nxi = p.nxi; z.nyi = p.nyi; z.nzi = p.nzi;
    z.kz_end = f ? p.g.nz : p.nzi;
    z.tx0 = f ? p.x0 - 32 * ((p.x0 + 31) / 32) : p.x0;
    z.ty0 = f ? 0 : p.y0;
    z.sx = f ? p.g.nx - z.tx0 : p.nxi;
    z.sy = f ? p.g.ny : p.nyi;
    z.sh = PmlShell{};
    if (f) {
        const PArgs& a = pml_args;
        PmlShell& h = z.sh;
        h.prof = a.prof; h.adeV = a.adeV; h.adeS = a.adeS;
        h.pxc = a.pxc; h.pxe = a.pxe; h.pyc = a.pyc; h.pye = a.pye; h.pzc = a.pzc; h.pze = a.pze;
        for (int q = 0; q < 6; ++q) { h.dlo[q] = shell_dlo[q]; h.dhi[q] = shell_dhi[q]; }
        h.r20x = a.r20x; h.r20y = a.r20y; h.r20z = a.r20z; h.dt = a.dt;
        for (int b = 0; b < 5; ++b) h.box[b] = p.box[b];
    }
    z.kchunk = kchunk; z.kchunk_v = kchunk_v; z.rpitch = p.rpitch;
    z.cer = p.pml ? nullptr : cer;
    for (int q = 0; q < 6; ++q) z.cer_off[q] = cer_off[q];
    z.c = coef;
}

// the PML stress (or velocity) update: one launch per class that has parts
// (timed: an event pair around each launch, timing class 6 + q for the
// stress and 6 + PML_NCLASS + q for the velocity update of class q)
void Sim::launch_pml(bool stress, cudaStream_t st, bool timed) {
    const int base = 6 + (stress ? 0 : PML_NCLASS);
    auto ev = [&](int c) {
        cudaEvent_t a = get_event(), b = get_event();
        cudaEventRecord(a, st);
        return Pending{c, a, b};
    };
    auto done = [&](Pending pe) {
        cudaEventRecord(pe.b, st);
        pending.push_back(pe);
    };
    // one launch of a class: one or two shell points per thread.  By
    // default one: with the shell's edge moduli and buoyancies precomputed,
    // two points per thread are no faster for any class on the
    // 1024x1024x512 grid (stress y 0.320 -> 0.328 ms, z 0.327 -> 0.331 ms,
    // corners 0.129 -> 0.146 ms, velocity y 0.263 -> 0.274 ms)
    auto go = [&](int mask, const PArgs& a) {
        const bool two = pml_np == 2;
        if (two) {
            const unsigned nb = (unsigned)((a.nblocks + 1) / 2);
            switch (mask) {
            case 1: stress ? k_stress_pml2<1><<<nb, PTPB, 0, st>>>(a) : k_vel_pml2<1><<<nb, PTPB, 0, st>>>(a); break;
            case 2: stress ? k_stress_pml2<2><<<nb, PTPB, 0, st>>>(a) : k_vel_pml2<2><<<nb, PTPB, 0, st>>>(a); break;
            case 4: stress ? k_stress_pml2<4><<<nb, PTPB, 0, st>>>(a) : k_vel_pml2<4><<<nb, PTPB, 0, st>>>(a); break;
            default: stress ? k_stress_pml2<7><<<nb, PTPB, 0, st>>>(a) : k_vel_pml2<7><<<nb, PTPB, 0, st>>>(a); break;
            }
            return;
        }
        const unsigned nb = (unsigned)a.nblocks;
        switch (mask) {
        case 1: stress ? k_stress_pml<1><<<nb, PTPB, 0, st>>>(a) : k_vel_pml<1><<<nb, PTPB, 0, st>>>(a); break;
        case 2: stress ? k_stress_pml<2><<<nb, PTPB, 0, st>>>(a) : k_vel_pml<2><<<nb, PTPB, 0, st>>>(a); break;
        case 4: stress ? k_stress_pml<4><<<nb, PTPB, 0, st>>>(a) : k_vel_pml<4><<<nb, PTPB, 0, st>>>(a); break;
        default: stress ? k_stress_pml<7><<<nb, PTPB, 0, st>>>(a) : k_vel_pml<7><<<nb, PTPB, 0, st>>>(a); break;
        }
    };
    if (!pml_split) {
        if (pml_all.nblocks == 0) return;
        Pending pe{};
        if (timed) pe = ev(base + PML_NCLASS - 1);
        go(7, pml_all);
        if (timed) done(pe);
        ++launches;
        return;
    }
    for (int q = 0; q < PML_NCLASS; ++q) {
        const PArgs& a = pml_cls[q];
        if (a.nblocks == 0) continue;
        Pending pe{};
        if (timed) pe = ev(base + q);
        go(PML_CLASS_MASK[q], a);
        if (timed) done(pe);
        ++launches;
    }
}

int Sim::launch_step(bool timed) {
    const dim3 blk(TBX, TBY);
    const dim3 grd((p.nxi + TBX - 1) / TBX, (p.nyi + TBY - 1) / TBY, (p.nzi + kchunk - 1) / kchunk);
    const dim3 grd_v(grd.x, grd.y, (p.nzi + kchunk_v - 1) / kchunk_v);
    // timed: an event pair on the launching stream around each kernel, read
    // back later by drain_events() so the launches are not serialised
    cudaEvent_t e_a[6] = {};
    auto ev0 = [&](int c, cudaStream_t st) {
        if (timed) { e_a[c] = get_event(); cudaEventRecord(e_a[c], st); }
    };
    auto ev1 = [&](int c, cudaStream_t st) {
        if (timed) {
            cudaEvent_t e_b = get_event();
            cudaEventRecord(e_b, st);
            pending.push_back({c, e_a[c], e_b});
        }
    };
    // the PML shell kernels run beside the interior kernels on a second
    // stream (two branches of the captured graph); they touch disjoint points
    // (none when the tile kernels sweep the shell themselves)
    const bool shell = p.pml && !pml_fused;
    const bool two = shell && concurrent;
    cudaStream_t sp = two ? stream2 : stream;
    if (vmax_args.ntdec_r > 0) { k_vmax<<<64, 256, 0, stream>>>(vmax_args); ++launches; }
    if (tap_args.n > 0) {
        ev0(4, stream);
        k_taps<<<(tap_args.n + 127) / 128, 128, 0, stream>>>(tap_args); ++launches;
        ev1(4, stream);
    }
    if (green_args.n) {
        k_green<<<(green_args.n + 127) / 128, 128, 0, stream>>>(green_args); ++launches;
    }
    if (snap_args.n) {
        dim3 sg((snap_args.maxpix + 127) / 128, snap_args.n);
        k_snap<<<sg, 128, 0, stream>>>(snap_args); ++launches;
    }
    ZArgs z;
    fill_zargs(z);
    targs.z = z;
    const dim3 tblk(32, ty_s), tblk_v(32, ty_v);
    // interior kernels over interior_tiles; with the shell swept by the tile
    // kernels, the shell-tile kernels over the rest (timing classes 2 and 3)
    int bxl, bxh, byl, byh;
    interior_tiles(z, ty_s, bxl, bxh, byl, byh);
    const unsigned nlin = (unsigned)((bxh - bxl) * (byh - byl) * ((p.nzi + kchunk - 1) / kchunk));
    interior_tiles(z, ty_v, bxl, bxh, byl, byh);
    const dim3 tgrd_v(bxh - bxl, byh - byl, (p.nzi + kchunk_v - 1) / kchunk_v);
    const unsigned nsh_s = (unsigned)shell_tile_count(z, ty_s, kchunk), nsh_v = (unsigned)shell_tile_count(z, ty_v, kchunk_v);
    if (pw && p.pml) { k_pw_ghost<<<256, 256, 0, stream>>>(V, p.g, 3); ++launches; }
    if (two) {
        cudaEventRecord(ev_fork, stream);
        cudaStreamWaitEvent(stream2, ev_fork, 0);
    }
    if (shell) {
        ev0(2, sp);
        launch_pml(true, sp, timed);
        ev1(2, sp);
        if (two) cudaEventRecord(ev_join, stream2);
    }
    if (nsh_s) {
        ev0(2, stream);
        if (ty_s == 16) {
            if (p.rbytes == 4) k_stress_tma_shell<float, 16><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
            else if (dims.store == SWPC_STORE_FP16) k_stress_tma_shell<__half, 16><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
            else k_stress_tma_shell<__nv_bfloat16, 16><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
        } else {
            if (p.rbytes == 4) k_stress_tma_shell<float><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
            else if (dims.store == SWPC_STORE_FP16) k_stress_tma_shell<__half><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
            else k_stress_tma_shell<__nv_bfloat16><<<nsh_s, tblk, smem_stress_sh, stream>>>(targs);
        }
        ++launches;
        ev1(2, stream);
    }
    ev0(0, stream);
    if (variant == 0 && nlin == 0) {
        // no tile lies wholly inside the interior: the shell-tile kernel did all
    } else if (variant == 0) {
        // 1-D grid, grouped block order
        if (ty_s == 16) {
            if (p.rbytes == 4) k_stress_tma<float, 16><<<nlin, tblk, smem_stress, stream>>>(targs);
            else if (dims.store == SWPC_STORE_FP16) k_stress_tma<__half, 16><<<nlin, tblk, smem_stress, stream>>>(targs);
            else k_stress_tma<__nv_bfloat16, 16><<<nlin, tblk, smem_stress, stream>>>(targs);
        } else {
            if (p.rbytes == 4) k_stress_tma<float><<<nlin, tblk, smem_stress, stream>>>(targs);
            else if (dims.store == SWPC_STORE_FP16) k_stress_tma<__half><<<nlin, tblk, smem_stress, stream>>>(targs);
            else k_stress_tma<__nv_bfloat16><<<nlin, tblk, smem_stress, stream>>>(targs);
        }
    } else {
        if (p.rbytes == 4) k_stress_interior<float><<<grd, blk, 0, stream>>>(z);
        else if (dims.store == SWPC_STORE_FP16) k_stress_interior<__half><<<grd, blk, 0, stream>>>(z);
        else k_stress_interior<__nv_bfloat16><<<grd, blk, 0, stream>>>(z);
    }
    if (variant != 0 || nlin) ++launches;
    ev1(0, stream);
    if (two) cudaStreamWaitEvent(stream, ev_join, 0);
    if (src_args.n > 0 && !bf_mode) {
        ev0(5, stream);
        k_stressglut<<<(src_args.n + 127) / 128, 128, 0, stream>>>(src_args); ++launches;
        ev1(5, stream);
    }
    if (pw && p.pml) { k_pw_ghost<<<256, 256, 0, stream>>>(S, p.g, 6); ++launches; }
    if (two) {
        cudaEventRecord(ev_fork2, stream);
        cudaStreamWaitEvent(stream2, ev_fork2, 0);
    }
    if (shell) {
        ev0(3, sp);
        launch_pml(false, sp, timed);
        ev1(3, sp);
        if (two) cudaEventRecord(ev_join2, stream2);
    }
    if (nsh_v) {
        ev0(3, stream);
        if (ty_v == 16) k_vel_tma_shell<16><<<nsh_v, tblk_v, smem_vel_sh, stream>>>(targs);
        else if (ty_v == 12) k_vel_tma_shell<12><<<nsh_v, tblk_v, smem_vel_sh, stream>>>(targs);
        else k_vel_tma_shell<><<<nsh_v, tblk_v, smem_vel_sh, stream>>>(targs);
        ++launches;
        ev1(3, stream);
    }
    ev0(1, stream);
    if (variant == 0 && tgrd_v.x * tgrd_v.y * tgrd_v.z == 0) {
        // every tile went to the shell-tile kernel
    } else if (variant == 0) {
        if (ty_v == 16) k_vel_tma<16><<<tgrd_v, tblk_v, smem_vel, stream>>>(targs);
        else if (ty_v == 12) k_vel_tma<12><<<tgrd_v, tblk_v, smem_vel, stream>>>(targs);
        else k_vel_tma<><<<tgrd_v, tblk_v, smem_vel, stream>>>(targs);
    } else {
        k_vel_interior<<<grd_v, blk, 0, stream>>>(z);
    }
    if (variant != 0 || tgrd_v.x * tgrd_v.y * tgrd_v.z) ++launches;
    ev1(1, stream);
    if (two) cudaStreamWaitEvent(stream, ev_join2, 0);
    if (src_args.n > 0 && bf_mode) {
        k_bodyforce<<<(src_args.n + 127) / 128, 128, 0, stream>>>(src_args); ++launches;
    }
    k_advance<<<1, 1, 0, stream>>>(d_it); ++launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return 0;
}

cudaEvent_t Sim::get_event() {
    if (!ev_pool.empty()) {
        cudaEvent_t e = ev_pool.back();
        ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

int Sim::drain_events() {
    CK(cudaStreamSynchronize(stream));
    for (auto& q : pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, q.a, q.b) == cudaSuccess) {
            prof_ms[q.cls] += ms;
            prof_n[q.cls] += 1;
        }
        ev_pool.push_back(q.a);
        ev_pool.push_back(q.b);
    }
    pending.clear();
    return 0;
}

int Sim::ensure_graph() {
    if (graph_exec) return 0;
    long long l0 = launches;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int q = 0; q < graph_steps && rc == 0; ++q) rc = launch_step(false);
    cudaGraph_t gr;
    cudaError_t e = cudaStreamEndCapture(stream, &gr);
    if (rc) return rc;
    if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&graph_exec, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    launches_per_graph = launches - l0;
    launches = l0;
    return 0;
}

// ---------------------------------------------------------------------------
// TMA tensor maps over the device groups (cuTensorMapEncodeTiled through the
// runtime's driver entry point, so the library needs no -lcuda)
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)f;
    });
    return fn;
}

int tile_kernel_attributes();

// 4-D map (x, field, y, z) over a row-interleaved group
static int make_map(CUtensorMap* m, void* base, CUtensorMapDataType dt, int es, long long nx, int nf, long long ny,
                    long long nz, int bx, int bf, int by, bool wide = false) {
    // L2 fetch granularity: each FP32 box row is one 128-byte line (a
    // 16-bit row half of one).  The stress kernel's maps promote to 256
    // bytes (wide): its grouped block order keeps the x-neighbour tile,
    // which reads the other half, resident at the same time (1024x1024x512:
    // 15.44 -> 15.39 ms); the velocity kernel's stay at 128 (256: 4.26 ->
    // 4.27 ms; 64: 4.32 ms)
    const CUtensorMapL2promotion promo = bx * es >= 128 ? (wide ? CU_TENSOR_MAP_L2_PROMOTION_L2_256B
                                                               : CU_TENSOR_MAP_L2_PROMOTION_L2_128B)
                                                        : CU_TENSOR_MAP_L2_PROMOTION_NONE;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_err(SWPC_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[4] = {(cuuint64_t)nx, (cuuint64_t)nf, (cuuint64_t)ny, (cuuint64_t)nz};
    cuuint64_t strides[3] = {(cuuint64_t)(nx * es), (cuuint64_t)(nx * nf * es), (cuuint64_t)(nx * nf * ny * es)};
    cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)bf, (cuuint32_t)by, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(m, dt, 4, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    promo, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(SWPC_E_CUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return 0;
}

int Sim::build_tensor_maps() {
    const Geo& g = p.g;
    const CUtensorMapDataType F = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    int rc;
    const int ts_ = ty_s, tv_ = ty_v;
    if ((rc = make_map(&targs.tmV, V, F, 4, g.pitch, 3, g.nyp, g.nzp, 40, 3, ts_ + 4, true))) return rc;
    if ((rc = make_map(&targs.tmS, S, F, 4, g.pitch, 6, g.nyp, g.nzp, 32, 6, ts_, true))) return rc;
    if ((rc = make_map(&targs.tmM, M, F, 4, g.pitch, 5, g.nyp, g.nzp, 36, 4, ts_ + 1, true))) return rc;
    if ((rc = make_map(&targs.tmSh, S, F, 4, g.pitch, 6, g.nyp, g.nzp, 40, 6, tv_ + 4))) return rc;
    if ((rc = make_map(&targs.tmRho, M, F, 4, g.pitch, 5, g.nyp, g.nzp, 36, 1, tv_ + 1))) return rc;
    if ((rc = make_map(&targs.tmVc, V, F, 4, g.pitch, 3, g.nyp, g.nzp, 32, 3, tv_))) return rc;
    const CUtensorMapDataType RTy = dims.store == SWPC_STORE_FP32 ? F
                                    : dims.store == SWPC_STORE_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                    : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if ((rc = make_map(&targs.tmR, R, RTy, p.rbytes, p.rpitch, 18, p.nyi, p.nzi, 32, 18, ts_, true))) return rc;
    targs.err = d_err;
    if (ts_ == 16) smem_stress = p.rbytes == 4 ? sizeof(StressSmem<float, 16>) : sizeof(StressSmem<__half, 16>);
    else smem_stress = p.rbytes == 4 ? sizeof(StressSmem<float>) : sizeof(StressSmem<__half>);
    smem_vel = tv_ == 16 ? sizeof(VelSmem<16>) : tv_ == 12 ? sizeof(VelSmem<12>) : sizeof(VelSmem<>);
    if (ts_ == 16) smem_stress_sh = p.rbytes == 4 ? sizeof(StressSm<float, 16, true>) : sizeof(StressSm<__half, 16, true>);
    else smem_stress_sh = p.rbytes == 4 ? sizeof(StressSm<float, 8, true>) : sizeof(StressSm<__half, 8, true>);
    smem_vel_sh = tv_ == 16 ? sizeof(VelSm<16, true>) : tv_ == 12 ? sizeof(VelSm<12, true>) : sizeof(VelSm<8, true>);
    return tile_kernel_attributes();
}

// Dynamic shared memory of every instantiation of the TMA tile kernels (set
// once per process: the attribute belongs to the kernel)
int tile_kernel_attributes() {
    static std::mutex mu;
    static bool set_on[128] = {};
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return set_err(SWPC_E_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (set_on[dev]) return 0;
    cudaError_t err = cudaSuccess;
    {
        auto set = [&err](const void* f, size_t bytes, bool carve) {
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            // the velocity kernel is sized for several blocks per SM: ask for
            // the largest shared-memory carve-out
            if (e == cudaSuccess && carve)
                e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
            if (e != cudaSuccess && err == cudaSuccess) err = e;
        };
        set((const void*)k_stress_tma<float>, sizeof(StressSmem<float>), false);
        set((const void*)k_stress_tma<__half>, sizeof(StressSmem<__half>), false);
        set((const void*)k_stress_tma<__nv_bfloat16>, sizeof(StressSmem<__nv_bfloat16>), false);
        set((const void*)k_stress_tma<float, 16>, sizeof(StressSmem<float, 16>), false);
        set((const void*)k_stress_tma<__half, 16>, sizeof(StressSmem<__half, 16>), false);
        set((const void*)k_stress_tma<__nv_bfloat16, 16>, sizeof(StressSmem<__nv_bfloat16, 16>), false);
        set((const void*)k_vel_tma<>, sizeof(VelSmem<>), true);
        set((const void*)k_vel_tma<16>, sizeof(VelSmem<16>), true);
        set((const void*)k_vel_tma<12>, sizeof(VelSmem<12>), true);
        set((const void*)k_stress_tma_batch<float>, sizeof(StressSmem<float>), false);
        set((const void*)k_stress_tma_batch<__half>, sizeof(StressSmem<__half>), false);
        set((const void*)k_stress_tma_batch<__nv_bfloat16>, sizeof(StressSmem<__nv_bfloat16>), false);
        set((const void*)k_stress_tma_batch<float, 16>, sizeof(StressSmem<float, 16>), false);
        set((const void*)k_stress_tma_batch<__half, 16>, sizeof(StressSmem<__half, 16>), false);
        set((const void*)k_stress_tma_batch<__nv_bfloat16, 16>, sizeof(StressSmem<__nv_bfloat16, 16>), false);
        set((const void*)k_vel_tma_batch<>, sizeof(VelSmem<>), true);
        set((const void*)k_vel_tma_batch<16>, sizeof(VelSmem<16>), true);
        set((const void*)k_vel_tma_batch<12>, sizeof(VelSmem<12>), true);
        // shell-tile kernels (rings + staged auxiliaries), single and batched
        set((const void*)k_stress_tma_shell<float>, sizeof(StressSm<float, 8, true>), false);
        set((const void*)k_stress_tma_shell<__half>, sizeof(StressSm<__half, 8, true>), false);
        set((const void*)k_stress_tma_shell<__nv_bfloat16>, sizeof(StressSm<__nv_bfloat16, 8, true>), false);
        set((const void*)k_stress_tma_shell<float, 16>, sizeof(StressSm<float, 16, true>), false);
        set((const void*)k_stress_tma_shell<__half, 16>, sizeof(StressSm<__half, 16, true>), false);
        set((const void*)k_stress_tma_shell<__nv_bfloat16, 16>, sizeof(StressSm<__nv_bfloat16, 16, true>), false);
        set((const void*)k_vel_tma_shell<>, sizeof(VelSm<8, true>), true);
        set((const void*)k_vel_tma_shell<16>, sizeof(VelSm<16, true>), true);
        set((const void*)k_vel_tma_shell<12>, sizeof(VelSm<12, true>), true);
        set((const void*)k_stress_tma_batch<float, 8, true>, sizeof(StressSm<float, 8, true>), false);
        set((const void*)k_stress_tma_batch<__half, 8, true>, sizeof(StressSm<__half, 8, true>), false);
        set((const void*)k_stress_tma_batch<__nv_bfloat16, 8, true>, sizeof(StressSm<__nv_bfloat16, 8, true>), false);
        set((const void*)k_stress_tma_batch<float, 16, true>, sizeof(StressSm<float, 16, true>), false);
        set((const void*)k_stress_tma_batch<__half, 16, true>, sizeof(StressSm<__half, 16, true>), false);
        set((const void*)k_stress_tma_batch<__nv_bfloat16, 16, true>, sizeof(StressSm<__nv_bfloat16, 16, true>), false);
        set((const void*)k_vel_tma_batch<8, true>, sizeof(VelSm<8, true>), true);
        set((const void*)k_vel_tma_batch<16, true>, sizeof(VelSm<16, true>), true);
        set((const void*)k_vel_tma_batch<12, true>, sizeof(VelSm<12, true>), true);
    }
    if (err != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(err));
    set_on[dev] = true;
    return 0;
}

int Sim::check_divergence() {
    if (d_err) {
        int e = 0;
        CK(cudaMemcpyAsync(&e, d_err, 4, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (e) return set_err(SWPC_E_TIMEOUT, "a bounded wait on a shared-memory pipeline barrier ran out");
    }
    if (vmax_args.ntdec_r <= 0 || !rep_host.size()) return 0;
    CK(cudaMemcpyAsync(rep_host.data(), vmax_args.rep, rep_host.size() * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    for (size_t q = 0; q < rep_host.size(); ++q) {
        float v;
        std::memcpy(&v, &rep_host[q], 4);
        if (v != v || (double)v * dims.UC > 1e5) {
            char buf[160];
            snprintf(buf, sizeof buf, "numerical divergence detected at it=%d with max amp = %g [(m/s)/moment]",
                     (int)((q / 3 + 1) * vmax_args.ntdec_r), (double)v * dims.UC);
            diverged = true;
            return set_err(SWPC_E_DIVERGED, buf);
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

long long swpc_gpu_required_bytes(const swpc_dims* d) {
    Plan p;
    if (plan(d, p)) return -1;
    return p.bytes;
}

int swpc_gpu_create(const swpc_dims* d, swpc_sim** out) {
    if (!out) return set_err(SWPC_E_ARG, "null output pointer");
    *out = nullptr;
    Sim* s = new Sim();
    int rc = plan(d, s->p);
    if (rc) { delete s; return rc; }
    s->dims = *d;
    rc = s->allocate();
    if (rc) { delete s; return rc; }
    *out = reinterpret_cast<swpc_sim*>(s);
    return 0;
}

int swpc_gpu_destroy(swpc_sim* sim) {
    delete reinterpret_cast<Sim*>(sim);
    return 0;
}

int swpc_gpu_last_error(char* buf, size_t n) {
    if (buf && n) {
        size_t m = std::min(n - 1, g_err.size());
        std::memcpy(buf, g_err.data(), m);
        buf[m] = 0;
    }
    return (int)g_err.size();
}

void* swpc_gpu_stream(swpc_sim* sim) { return sim ? (void*)reinterpret_cast<Sim*>(sim)->stream : nullptr; }

long long swpc_gpu_launch_count(swpc_sim* sim) { return sim ? reinterpret_cast<Sim*>(sim)->launches : -1; }

int swpc_gpu_upload_medium(swpc_sim* sim, const float* rho, const float* lam, const float* mu, const float* taup,
                           const float* taus, const int* kfs, const int* kob, const int* kfs_top, const int* kfs_bot,
                           const int* kob_top, const int* kob_bot, const double* ts) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !rho || !lam || !mu || !taup || !taus || !kob || !kfs_top || !kfs_bot || !kob_top || !kob_bot || !ts)
        return set_err(SWPC_E_ARG, "null argument to swpc_gpu_upload_medium");
    if (!kfs) return set_err(SWPC_E_ARG, "null argument to swpc_gpu_upload_medium");
    return s->upload_medium(rho, lam, mu, taup, taus, kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot, ts, false);
}

int swpc_gpu_upload_medium_column(swpc_sim* sim, const float* rho, const float* lam, const float* mu, const float* taup,
                                  const float* taus, const int* kfs, const int* kob, const int* kfs_top,
                                  const int* kfs_bot, const int* kob_top, const int* kob_bot, const double* ts) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !rho || !lam || !mu || !taup || !taus || !kfs || !kob || !kfs_top || !kfs_bot || !kob_top || !kob_bot || !ts)
        return set_err(SWPC_E_ARG, "null argument to swpc_gpu_upload_medium_column");
    return s->upload_medium(rho, lam, mu, taup, taus, kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot, ts, true);
}

int swpc_gpu_build_medium_rmed(swpc_sim* sim, const float* bg, const float* xi, int nxc, int nyc, int nzc, int kxi0,
                               double vmin, double vmax, double rhomin, double fq_min, double fq_max, double fq_ref,
                               int* maps6, double* ts) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !bg || !xi || !ts || nxc <= 0 || nyc <= 0 || nzc <= 0)
        return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_build_medium_rmed");
    if (!(fq_min > 0 && fq_max > fq_min && fq_ref > 0)) return set_err(SWPC_E_ARG, "need 0 < fq_min < fq_max, fq_ref > 0");
    return s->build_medium_rmed(bg, xi, nxc, nyc, nzc, kxi0, vmin, vmax, rhomin, fq_min, fq_max, fq_ref, maps6, ts);
}

int swpc_gpu_set_sources(swpc_sim* sim, int n, const int* ijk, const double* mo, const double* mij, const double* fxyz,
                         const double* prm, int stftype, int bf_mode) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || n < 0 || (n > 0 && (!ijk || !prm || (bf_mode ? !fxyz : (!mo || !mij)))))
        return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_sources");
    if (stftype < 0 || stftype > 5) return set_err(SWPC_E_ARG, "unknown source time function");
    return s->set_sources(n, ijk, mo, mij, fxyz, prm, stftype, bf_mode != 0);
}

int swpc_gpu_set_receivers(swpc_sim* sim, int n, const int* ijk, int ntdec_w, int flags) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || n < 0 || (n > 0 && !ijk) || ntdec_w <= 0 || (flags & ~15))
        return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_receivers");
    return s->set_receivers(n, ijk, ntdec_w, flags);
}

int swpc_gpu_set_snapshot(swpc_sim* sim, int kinds, int k0, int idec, int jdec, int ntdec_s) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || (kinds & ~3) || idec <= 0 || jdec <= 0 || ntdec_s <= 0) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_snapshot");
    if (kinds && (k0 < 1 || k0 > s->dims.nz)) return set_err(SWPC_E_ARG, "snapshot plane k0 outside 1..nz");
    int rc = 0;
    if (kinds & SWPC_SNAP_XY_V) rc = s->add_snapshot(SWPC_SEC_XY, SWPC_SNAPK_V, k0, idec, jdec, ntdec_s);
    if (!rc && (kinds & SWPC_SNAP_XY_U)) rc = s->add_snapshot(SWPC_SEC_XY, SWPC_SNAPK_U, k0, idec, jdec, ntdec_s);
    return rc;
}

int swpc_gpu_add_snapshot(swpc_sim* sim, int section, int kind, int fix, int dec1, int dec2, int ntdec_s) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || section < SWPC_SEC_XY || section > SWPC_SEC_OB || kind < SWPC_SNAPK_V || kind > SWPC_SNAPK_PS ||
        dec1 <= 0 || dec2 <= 0 || ntdec_s <= 0)
        return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_add_snapshot");
    const int lim = section == SWPC_SEC_XY ? s->dims.nz : section == SWPC_SEC_YZ ? s->dims.nx
                  : section == SWPC_SEC_XZ ? s->dims.ny : 1;
    if (section >= SWPC_SEC_FS) fix = 1;  // the surface maps choose k per column
    if (fix < 1 || fix > lim) return set_err(SWPC_E_ARG, "snapshot section index outside the grid");
    return s->add_snapshot(section, kind, fix, dec1, dec2, ntdec_s);
}

int swpc_gpu_set_field(swpc_sim* sim, int which, const float* field) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !field || which < 0 || which > 8) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_field");
    const Geo& g = s->p.g;
    const size_t n = (size_t)(g.nz + 6) * (g.nx + 6) * (g.ny + 6);
    float* stage = nullptr;
    CK(cudaMallocAsync(&stage, n * 4, s->stream));
    CK(cudaMemcpyAsync(stage, field, n * 4, cudaMemcpyHostToDevice, s->stream));
    const dim3 tg((g.nz + 6 + 31) / 32, (g.nx + 6 + 31) / 32, g.ny + 6), tb(32, 8);
    if (which < 3) k_scatter_t<<<tg, tb, 0, s->stream>>>(stage, s->V, g, 3, which, 1);
    else k_scatter_t<<<tg, tb, 0, s->stream>>>(stage, s->S, g, 6, which - 3, 1);
    ++s->launches;
    CK(cudaFreeAsync(stage, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

int swpc_gpu_set_plane_wave(swpc_sim* sim, int on) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    if (on && !s->p.pml) return set_err(SWPC_E_ARG, "plane-wave mode needs the PML absorber");
    s->pw = on != 0;
    if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
    return 0;
}

int swpc_gpu_set_green(swpc_sim* sim, int n, const int* ijk, int ntdec_w, int bforce) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || n < 0 || (n > 0 && !ijk) || ntdec_w <= 0) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_green");
    return s->set_green(n, ijk, ntdec_w, bforce);
}

int swpc_gpu_fetch_green(swpc_sim* sim, float* out, int* n, int* ncmp, int* ntw) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    const GreenArgs& a = s->green_args;
    if (!a.n) return set_err(SWPC_E_STATE, "no Green's-function points were set");
    if (n) *n = a.n;
    if (ncmp) *ncmp = a.ncmp;
    if (ntw) *ntw = a.ntw;
    if (!out) return 0;
    CK(cudaMemcpyAsync(out, a.gf, (size_t)a.ntw * a.ncmp * a.n * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return s->check_divergence();
}

int swpc_gpu_query_snapshot(swpc_sim* sim, int section, int kind, int* n1, int* n2, int* nframes) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    const SnapPlane* P = s->find_plane(section, kind);
    if (!P) return set_err(SWPC_E_STATE, "that snapshot was not requested");
    if (n1) *n1 = P->n1;
    if (n2) *n2 = P->n2;
    if (nframes) *nframes = s->nframes_done();
    return 0;
}

int swpc_gpu_fetch_section(swpc_sim* sim, int section, int kind, int frame, float* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument");
    const SnapPlane* P = s->find_plane(section, kind);
    if (!P) return set_err(SWPC_E_STATE, "that snapshot was not requested");
    if (frame < 0 || frame >= s->snap_args.maxframes) return set_err(SWPC_E_ARG, "frame out of range");
    const size_t n = (size_t)P->n1 * P->n2 * P->nc;
    CK(cudaMemcpyAsync(out, P->frames + frame * n, n * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

int swpc_gpu_step(swpc_sim* sim, int it) { return swpc_gpu_run(sim, it, it); }

int swpc_gpu_run(swpc_sim* sim, int it0, int it1) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    if (!s->medium_ready) return set_err(SWPC_E_STATE, "upload the medium before stepping");
    if (s->diverged) return set_err(SWPC_E_DIVERGED, "simulation has diverged");
    if (it1 < it0) return 0;
    k_set_it<<<1, 1, 0, s->stream>>>(s->d_it, it0);
    ++s->launches;
    int n = it1 - it0 + 1, rc = 0;
    if (s->profiling) {
        for (int q = 0; q < n && rc == 0; ++q) rc = s->launch_step(true);
    } else {
        if (n >= s->graph_steps) {
            rc = s->ensure_graph();
            while (rc == 0 && n >= s->graph_steps) {
                cudaError_t e = cudaGraphLaunch(s->graph_exec, s->stream);
                if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
                s->launches += s->launches_per_graph;
                n -= s->graph_steps;
            }
        }
        for (int q = 0; q < n && rc == 0; ++q) rc = s->launch_step(false);
    }
    s->it_done = it1;
    return rc;
}

int swpc_gpu_sync(swpc_sim* sim) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    CK(cudaStreamSynchronize(s->stream));
    return s->check_divergence();
}

int swpc_gpu_query(swpc_sim* sim, int* ntw, int* nst, int* nxs, int* nys, int* nframes) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    if (ntw) *ntw = s->tap_args.ntw;
    if (nst) *nst = s->tap_args.n;
    const SnapPlane* P = s->find_plane(SWPC_SEC_XY, SWPC_SNAPK_V);
    if (!P) P = s->find_plane(SWPC_SEC_XY, SWPC_SNAPK_U);
    if (nxs) *nxs = P ? P->n1 : 0;
    if (nys) *nys = P ? P->n2 : 0;
    if (nframes) *nframes = P ? s->nframes_done() : 0;
    return 0;
}

int swpc_gpu_fetch_waveforms(swpc_sim* sim, int kind, float* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument");
    const TapArgs& t = s->tap_args;
    float* src = nullptr;
    int nc = 3;
    switch (kind) {
    case SWPC_WAV_V: src = t.wav_v; break;
    case SWPC_WAV_U: src = t.wav_u; break;
    case SWPC_WAV_STRESS: src = t.wav_s; nc = 6; break;
    case SWPC_WAV_STRAIN: src = t.wav_e; nc = 6; break;
    default: return set_err(SWPC_E_ARG, "kind must be one SWPC_WAV_* bit");
    }
    if (!src || !(t.flags & kind)) return set_err(SWPC_E_STATE, "that waveform kind was not requested");
    CK(cudaMemcpyAsync(out, src, (size_t)t.ntw * nc * t.n * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return s->check_divergence();
}

int swpc_gpu_fetch_snapshot(swpc_sim* sim, int kind, int frame, float* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument");
    if (kind != SWPC_SNAP_XY_V && kind != SWPC_SNAP_XY_U) return set_err(SWPC_E_ARG, "kind must be SWPC_SNAP_XY_V or _U");
    return swpc_gpu_fetch_section(sim, SWPC_SEC_XY, kind == SWPC_SNAP_XY_V ? SWPC_SNAPK_V : SWPC_SNAPK_U, frame, out);
}

int swpc_gpu_vmax(swpc_sim* sim, float out[3]) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument");
    out[0] = out[1] = out[2] = 0;
    if (s->vmax_args.ntdec_r <= 0 || s->rep_host.empty()) return 0;
    int rc = swpc_gpu_sync(sim);
    int r = s->it_done / s->vmax_args.ntdec_r - 1;
    if (r < 0) return rc;
    r = std::min(r, s->vmax_args.nrep - 1);
    for (int c = 0; c < 3; ++c) {
        float v;
        std::memcpy(&v, &s->rep_host[3 * r + c], 4);
        out[c] = (float)((double)v * s->dims.UC * s->dims.M0);
    }
    return rc;
}

int swpc_gpu_fetch_field(swpc_sim* sim, int which, double* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out || which < 0 || which > 13) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_fetch_field");
    const Geo& g = s->p.g;
    size_t n = (size_t)g.nx * g.ny * g.nz;
    double* d = nullptr;
    CK(cudaMallocAsync(&d, n * 8, s->stream));
    const dim3 tg((g.nz + 31) / 32, (g.nx + 31) / 32, g.ny), tb(32, 8);
    if (which < 3) k_gather_d<<<tg, tb, 0, s->stream>>>(s->V, d, g, 3, which);
    else if (which < 9) k_gather_d<<<tg, tb, 0, s->stream>>>(s->S, d, g, 6, which - 3);
    else k_gather_d<<<tg, tb, 0, s->stream>>>(s->M, d, g, 5, which - 9);
    ++s->launches;
    CK(cudaMemcpyAsync(out, d, n * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaFreeAsync(d, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

// ---------------------------------------------------------------------------
// Field read-back without any device allocation.
//
// swpc_gpu_fetch_field gathers a field into a temporary device buffer that it
// allocates and frees on every call.  Some callers cannot allow that: a host
// that has committed the whole device to resident wavefields under an HBM
// budget (the temporary allocation would fail on a full device, or would
// break the budget's accounting), and frameworks whose own allocator owns all
// device memory and forbids side allocations.  For them the gather goes
// through this fixed scratch array instead.  It lives in the library image:
// every GPU that loads the library holds its 32 MiB until the process exits.
// Fields larger than SWPC_STATIC_FIELD_MAX points are rejected.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_field_scratch[SWPC_STATIC_FIELD_MAX];

// Device address of g_field_scratch on device `dev` (the simulation's), looked
// up once per device with that device current.  In host code the symbol name
// is only a host-side stand-in, never a device address.
static int static_scratch(int dev, double** out) {
    static std::mutex mu;
    static void* addr[128] = {};
    if (dev < 0 || dev >= 128) return set_err(SWPC_E_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        int cur = 0;
        CK(cudaGetDevice(&cur));
        if (cur != dev) CK(cudaSetDevice(dev));
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_field_scratch);
        if (cur != dev) cudaSetDevice(cur);
        if (e != cudaSuccess || !p)
            return set_err(SWPC_E_CUDA, std::string("cudaGetSymbolAddress(g_field_scratch): ") + cudaGetErrorString(e));
        addr[dev] = p;
    }
    *out = (double*)addr[dev];
    return 0;
}

extern "C" int swpc_gpu_fetch_field_static(swpc_sim* sim, int which, double* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument to swpc_gpu_fetch_field_static");
    if (which < 0 || which > 8)
        return set_err(SWPC_E_ARG, "swpc_gpu_fetch_field_static reads the wavefields 0..8 (Vx .. Sxy) only; "
                                   "use swpc_gpu_fetch_field for the medium fields");
    const Geo& g = s->p.g;
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    if (n > (size_t)SWPC_STATIC_FIELD_MAX)
        return set_err(SWPC_E_ARG, "grid of " + std::to_string(n) + " points exceeds the static read-back limit of " +
                                       std::to_string((long long)SWPC_STATIC_FIELD_MAX) + " points; use swpc_gpu_fetch_field");
    double* d = nullptr;
    int rc = static_scratch(s->device, &d);  // the scratch of the device the simulation lives on
    if (rc) return rc;
    // every one of the n elements copied back is written by the gather first,
    // so the array needs no clearing
    const dim3 tg((g.nz + 31) / 32, (g.nx + 31) / 32, g.ny), tb(32, 8);
    if (which < 3) k_gather_d<<<tg, tb, 0, s->stream>>>(s->V, d, g, 3, which);
    else k_gather_d<<<tg, tb, 0, s->stream>>>(s->S, d, g, 6, which - 3);
    ++s->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d, n * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return 0;
}

int swpc_gpu_selftest_wait(double* seconds) {
    int* err = nullptr;
    CK(cudaMalloc(&err, sizeof(int)));
    int h = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemset(err, 0, sizeof(int));
    cudaEventRecord(e0);
    k_wait_selftest<<<1, 32>>>(err);
    cudaEventRecord(e1);
    cudaError_t e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (seconds) *seconds = ms / 1e3;
    if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
    return h == 1 ? set_err(SWPC_E_TIMEOUT, "bounded wait gave up as designed") : 0;
}

int swpc_gpu_get_dims(swpc_sim* sim, swpc_dims* out) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !out) return set_err(SWPC_E_ARG, "null argument");
    *out = s->dims;
    return 0;
}

int swpc_gpu_reset(swpc_sim* sim) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemsetAsync(s->V, 0, s->p.nV * 4, s->stream));
    CK(cudaMemsetAsync(s->S, 0, s->p.nS * 4, s->stream));
    CK(cudaMemsetAsync(s->R, 0, s->p.nR * s->p.rbytes, s->stream));
    if (s->adeV) CK(cudaMemsetAsync(s->adeV, 0, s->p.nade * 4, s->stream));
    if (s->adeS) CK(cudaMemsetAsync(s->adeS, 0, s->p.nade * 4, s->stream));
    const TapArgs& t = s->tap_args;
    if (t.n > 0) {
        const size_t w3 = (size_t)t.ntw * 3 * t.n * 4, w6 = (size_t)t.ntw * 6 * t.n * 4;
        if (t.wav_v) CK(cudaMemsetAsync(t.wav_v, 0, w3, s->stream));
        if (t.wav_u) CK(cudaMemsetAsync(t.wav_u, 0, w3, s->stream));
        if (t.wav_s) CK(cudaMemsetAsync(t.wav_s, 0, w6, s->stream));
        if (t.wav_e) CK(cudaMemsetAsync(t.wav_e, 0, w6, s->stream));
        if (t.acc) CK(cudaMemsetAsync(t.acc, 0, (size_t)9 * t.n * 8, s->stream));
    }
    const SnapArgs& a = s->snap_args;
    const GreenArgs& gr = s->green_args;
    if (gr.n) {
        CK(cudaMemsetAsync(gr.acc, 0, (size_t)12 * gr.n * 8, s->stream));
        CK(cudaMemsetAsync(gr.gf, 0, (size_t)gr.ntw * gr.ncmp * gr.n * 4, s->stream));
    }
    for (int q = 0; q < a.n; ++q) {
        const SnapPlane& P = a.pl[q];
        const size_t pix = (size_t)P.n1 * P.n2;
        CK(cudaMemsetAsync(P.frames, 0, (size_t)a.maxframes * P.nc * pix * 4, s->stream));
        if (P.uacc) CK(cudaMemsetAsync(P.uacc, 0, 3 * pix * 8, s->stream));
    }
    if (s->vmax_args.rep) CK(cudaMemsetAsync(s->vmax_args.rep, 0, (size_t)s->vmax_args.nrep * 12, s->stream));
    CK(cudaMemsetAsync(s->d_err, 0, 4, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->it_done = 0;
    s->diverged = false;
    return 0;
}

int swpc_gpu_profile(swpc_sim* sim, int enable) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    int rc = s->drain_events();
    if (rc) return rc;
    s->profiling = enable != 0;
    for (int c = 0; c < Sim::NPROF; ++c) { s->prof_ms[c] = 0; s->prof_n[c] = 0; }
    return 0;
}

int swpc_gpu_profile_read_pml(swpc_sim* sim, double* ms, long long* n, long long* points, long long* axis_points) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    int rc = s->drain_events();
    if (rc) return rc;
    for (int c = 0; c < 2 * PML_NCLASS; ++c) {
        if (ms) ms[c] = s->prof_ms[6 + c];
        if (n) n[c] = s->prof_n[6 + c];
    }
    for (int q = 0; q < PML_NCLASS; ++q) {
        if (points) points[q] = s->pml_pts[q];
        if (axis_points) axis_points[q] = s->pml_axpts[q];
    }
    return 0;
}

int swpc_gpu_profile_read(swpc_sim* sim, double* ms, long long* n) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    int rc = s->drain_events();
    if (rc) return rc;
    for (int c = 0; c < 6; ++c) {
        if (ms) ms[c] = s->prof_ms[c];
        if (n) n[c] = s->prof_n[c];
    }
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Sim methods
// ---------------------------------------------------------------------------
Sim::~Sim() {
    if (stream) cudaStreamSynchronize(stream);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (void* q : allocs) cudaFree(q);
    for (auto& q : pending) { ev_pool.push_back(q.a); ev_pool.push_back(q.b); }
    for (auto& e : ev_pool) if (e) cudaEventDestroy(e);
    if (stream2) { cudaStreamSynchronize(stream2); cudaStreamDestroy(stream2); }
    for (cudaEvent_t e : {ev_fork, ev_join, ev_fork2, ev_join2}) if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
}

int Sim::dalloc(void** ptr, size_t bytes) {
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(SWPC_E_NOMEM, std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    }
    allocs.push_back(*ptr);
    e = cudaMemsetAsync(*ptr, 0, bytes ? bytes : 16, stream);
    if (e != cudaSuccess) return set_err(SWPC_E_CUDA, cudaGetErrorString(e));
    return 0;
}

int Sim::allocate() {
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_fork2, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_join2, cudaEventDisableTiming));
    int rc;
    // the large arrays are carved out of one allocation: freeing one 72 GB
    // block took 26 ms on a GB300, freeing the same bytes in 4 to 16 blocks
    // 45 to 53 ms (and one allocation maps faster too)
    {
        size_t off = 0;
        auto carve = [&](size_t bytes) {
            const size_t o = off;
            off += (bytes + 4095) / 4096 * 4096;  // 4 KB aligned bases (tensor maps want 16 B)
            return o;
        };
        const size_t oV = carve(p.nV * 4), oS = carve(p.nS * 4), oM = carve(p.nM * 4), oR = carve(p.nR * p.rbytes);
        const size_t oAV = p.pml ? carve(p.nade * 4) : 0, oAS = p.pml ? carve(p.nade * 4) : 0;
        const size_t oSH = p.pml ? carve(p.nshm * 4) : 0;
        char* arena = nullptr;
        if ((rc = dalloc((void**)&arena, off))) return rc;
        V = reinterpret_cast<float*>(arena + oV);
        S = reinterpret_cast<float*>(arena + oS);
        M = reinterpret_cast<float*>(arena + oM);
        R = arena + oR;
        if (p.pml) {
            adeV = reinterpret_cast<float*>(arena + oAV);
            adeS = reinterpret_cast<float*>(arena + oAS);
            shm = reinterpret_cast<float*>(arena + oSH);
        }
    }
    if ((rc = dalloc((void**)&band, 16 * (size_t)p.nxi * p.nyi))) return rc;
    if ((rc = dalloc((void**)&d_it, 16))) return rc;
    if ((rc = dalloc((void**)&d_kob, 4 * (size_t)p.g.nx * p.g.ny))) return rc;
    if ((rc = dalloc((void**)&d_kfs, 4 * (size_t)p.g.nx * p.g.ny))) return rc;
    // z chunking: enough blocks to fill the GPU at least ~8 times; then the
    // stress kernels take chunks of at most 6 planes with FP32 memory
    // variables, 32 with 16-bit ones (neighbouring blocks sweep the same
    // planes at the same time and share their V halo rows in L2:
    // 1024x1024x512 FP32 stress 15.91, 15.64, 15.44, 15.52, 15.65, 15.77 ms
    // with 4, 5, 6, 8, 10, 12 planes in the grouped block order (17.6 ms with
    // 492 in the plain order); FP16 12.18, 11.57, 11.35 ms with 8, 16, 32
    // planes) and the velocity kernels chunks of at most 96 planes (its
    // longer start-up costs more at 16 planes, 4.95 ms; 4.27 ms at 123,
    // 4.256 at 99 and 82, 4.254 at 70)
    int dev = 0, nsm = 148;
    cudaGetDevice(&dev);
    device = dev;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    variant = dims.reserved[0] == 1 ? 1 : 0;
    pml_np = dims.reserved[2] == 2 ? 2 : 1;
    // reserved[3] = 2: the TMA tile kernels sweep the PML shell too (interior
    // and shell-tile kernels); otherwise the shell runs in launches of its own
    pml_fused = p.pml && variant == 0 && p.nbox == 5 && dims.reserved[3] == 2;
    const int nzs = p.nzi;  // chunks of the interior's planes (the planes below take chunks of the same depth)
    long long cols = (long long)((p.nxi + TBX - 1) / TBX) * ((p.nyi + TBY - 1) / TBY);
    long long want = 8LL * nsm;
    int nchunk = (int)std::max(1LL, std::min((long long)(nzs / 8), (want + cols - 1) / cols));
    const int kfill = (nzs + nchunk - 1) / nchunk;
    auto even = [&](int cap) {  // equal chunks of at most cap planes
        const int nc = (nzs + cap - 1) / cap;
        return (nzs + nc - 1) / nc;
    };
    kchunk = kchunk_auto = even(std::min(kfill, p.rbytes == 4 ? 6 : 32));
    kchunk_v = kchunk_v_auto = even(std::min(kfill, 96));
    graph_steps = 8;
    if ((rc = dalloc((void**)&d_err, 16))) return rc;
    // PML shell beside the interior: pays off only when the interior launch
    // cannot fill the GPU by itself (measured: 128x128x64 0.134 vs 0.16 ms per
    // step; 1024x1024x512 27.9 serial vs 28.3 ms concurrent)
    {
        const long long tiles = (long long)((p.nxi + 31) / 32) * ((p.nyi + ty_s - 1) / ty_s) * ((nzs + kfill - 1) / kfill);
        concurrent = dims.reserved[1] == 2 || (dims.reserved[1] == 0 && tiles < 4LL * nsm);
    }
    if ((rc = build_tensor_maps())) return rc;
    return 0;
}

// Device address of a pinned (page-locked, device-mapped) host array, or
// null for any other memory.  The transpose kernels read pinned arrays
// directly over the CPU-GPU link instead of staging them in device memory
// first; the callers synchronise before they return, as the ABI's copy
// semantics require.
static const float* pinned_view(const float* h) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost && at.devicePointer ? static_cast<const float*>(at.devicePointer) : nullptr;
}

// Split the PML boxes into parts with the same damped axes at every point
// and sort the parts into the launch classes of PML_CLASS_MASK (x, y or z
// alone; anything else).  An axis index counts as damped when g4 of its
// centre or edge profile is not zero, read from the profiles themselves, so
// the split is exact whatever the rounding of the layer edges.  When the
// damped indices of an axis are not its two end runs, or a class would hold
// more than PML_MAXPART parts, every box goes to the general class whole.
void Sim::plan_pml_parts(const std::vector<float>& prof) {
    const PArgs& a = pml_args;
    const int n[3] = {p.g.nx, p.g.ny, p.g.nz};
    const int oc[3] = {a.pxc, a.pyc, a.pzc}, oe[3] = {a.pxe, a.pye, a.pze};
    std::vector<char> damp[3];
    bool ends_only = true;
    for (int ax = 0; ax < 3; ++ax) {
        damp[ax].resize(n[ax]);
        for (int i = 0; i < n[ax]; ++i)
            damp[ax][i] = prof[oc[ax] + 4 * i + 3] != 0.f || prof[oe[ax] + 4 * i + 3] != 0.f;
        int i = 0;  // damped run at the start, undamped middle, damped run at the end
        while (i < n[ax] && damp[ax][i]) ++i;
        while (i < n[ax] && !damp[ax][i]) ++i;
        while (i < n[ax] && damp[ax][i]) ++i;
        if (i != n[ax]) ends_only = false;
    }
    // the shell-tile kernels test damping by index ranges: every profile's
    // damped indices must be its two end runs (else the shell keeps its own
    // launches)
    {
        const int offs[6] = {a.pxc, a.pxe, a.pyc, a.pye, a.pzc, a.pze};
        bool runs = true;
        for (int q = 0; q < 6; ++q) {
            const int n1 = n[q / 2];
            auto d = [&](int i) { return prof[offs[q] + 4 * i + 3] != 0.f; };
            int lo = 0, hi = n1;
            while (lo < n1 && d(lo)) ++lo;
            while (hi > lo && d(hi - 1)) --hi;
            for (int i = lo; i < hi; ++i) runs = runs && !d(i);
            shell_dlo[q] = lo;
            shell_dhi[q] = hi;
        }
        if (!runs) pml_fused = false;
    }
    std::vector<PmlPart> cls[PML_NCLASS];
    long long cls_pts[PML_NCLASS] = {}, cls_ax[PML_NCLASS] = {};
    bool fits = ends_only;
    if (ends_only) {
        for (int b = 0; b < p.nbox; ++b) {
            const PmlBox& B = p.box[b];
            const int o[3] = {B.x0, B.y0, B.z0}, m[3] = {B.nx, B.ny, B.nz};
            std::vector<int> cut[3];  // run boundaries of damped-ness along each axis of the box
            for (int ax = 0; ax < 3; ++ax) {
                cut[ax].push_back(0);
                for (int i = 1; i < m[ax]; ++i)
                    if (damp[ax][o[ax] + i] != damp[ax][o[ax] + i - 1]) cut[ax].push_back(i);
                cut[ax].push_back(m[ax]);
            }
            for (size_t kz = 0; kz + 1 < cut[2].size(); ++kz)
                for (size_t jy = 0; jy + 1 < cut[1].size(); ++jy)
                    for (size_t ix = 0; ix + 1 < cut[0].size(); ++ix) {
                        PmlPart P{};
                        P.b = b;
                        P.x0 = cut[0][ix]; P.nx = cut[0][ix + 1] - P.x0;
                        P.y0 = cut[1][jy]; P.ny = cut[1][jy + 1] - P.y0;
                        P.z0 = cut[2][kz]; P.nz = cut[2][kz + 1] - P.z0;
                        const int mask = (damp[0][o[0] + P.x0] ? 1 : 0) | (damp[1][o[1] + P.y0] ? 2 : 0) |
                                         (damp[2][o[2] + P.z0] ? 4 : 0);
                        int c = PML_NCLASS - 1;
                        for (int q = 0; q < PML_NCLASS - 1; ++q)
                            if (PML_CLASS_MASK[q] == mask) c = q;
                        cls[c].push_back(P);
                        const long long np = (long long)P.nx * P.ny * P.nz;
                        cls_pts[c] += np;
                        cls_ax[c] += np * ((mask & 1) + (mask >> 1 & 1) + (mask >> 2 & 1));
                    }
        }
        for (int q = 0; q < PML_NCLASS; ++q)
            if ((int)cls[q].size() > PML_MAXPART) fits = false;
    }
    if (!fits) {
        for (auto& v : cls) v.clear();
        for (int b = 0; b < p.nbox; ++b) {
            const PmlBox& B = p.box[b];
            cls[PML_NCLASS - 1].push_back(PmlPart{b, 0, 0, 0, B.nx, B.ny, B.nz, 0});
        }
    }
    // a single simulation's step launches the classes separately only when
    // its shell is large enough for each launch to fill the GPU; a small
    // shell takes one launch of the general kernel over the whole boxes
    // (the batched form always splits: its launches span every member)
    pml_all = pml_args;
    pml_all.npart = p.nbox;
    pml_all.nblocks = 0;
    for (int b = 0; b < p.nbox; ++b) {
        const PmlBox& B = p.box[b];
        pml_all.part[b] = PmlPart{b, 0, 0, 0, B.nx, B.ny, B.nz, pml_all.nblocks};
        pml_all.nblocks += (int)(((long long)B.nx * B.ny * B.nz + PTPB - 1) / PTPB);
    }
    pml_split = p.npml >= 4000000LL;
    // shell points and damped-axis points per launch class, for the byte
    // count of each class (one general launch: everything in the last class)
    for (int q = 0; q < PML_NCLASS; ++q) pml_pts[q] = pml_axpts[q] = 0;
    if (pml_split && fits) {
        for (int q = 0; q < PML_NCLASS; ++q) { pml_pts[q] = cls_pts[q]; pml_axpts[q] = cls_ax[q]; }
    } else {
        for (int b = 0; b < p.nbox; ++b) {
            const PmlBox& B = p.box[b];
            long long sx = 0, sy = 0, sz = 0;
            for (int i = 0; i < B.nx; ++i) sx += damp[0][B.x0 + i];
            for (int j = 0; j < B.ny; ++j) sy += damp[1][B.y0 + j];
            for (int k = 0; k < B.nz; ++k) sz += damp[2][B.z0 + k];
            pml_pts[PML_NCLASS - 1] += (long long)B.nx * B.ny * B.nz;
            pml_axpts[PML_NCLASS - 1] += sx * B.ny * B.nz + sy * (long long)B.nx * B.nz + sz * (long long)B.nx * B.ny;
        }
    }
    for (int q = 0; q < PML_NCLASS; ++q) {
        PArgs& c = pml_cls[q];
        c = pml_args;
        c.npart = (int)cls[q].size();
        c.nblocks = 0;
        for (int t = 0; t < c.npart; ++t) {
            c.part[t] = cls[q][t];
            c.part[t].first_block = c.nblocks;
            const long long np = (long long)c.part[t].nx * c.part[t].ny * c.part[t].nz;
            c.nblocks += (int)((np + PTPB - 1) / PTPB);
        }
    }
}

int Sim::upload_medium(const float* rho, const float* lam, const float* mu, const float* taup, const float* taus,
                       const int* kfs, const int* kob, const int* kfs_top, const int* kfs_bot, const int* kob_top,
                       const int* kob_bot, const double* ts, bool column) {
    const Geo& g = p.g;
    const float* fields[5] = {rho, lam, mu, taup, taus};
    if (column) {  // one column of nz + 6 values per field, spread over every (i, j) on the device
        const size_t nc = (size_t)g.nz + 6;
        float* stage = nullptr;
        CK(cudaMallocAsync((void**)&stage, 5 * nc * 4, stream));
        for (int f = 0; f < 5; ++f)
            CK(cudaMemcpyAsync(stage + f * nc, fields[f], nc * 4, cudaMemcpyHostToDevice, stream));
        k_spread_col<<<2048, 256, 0, stream>>>(stage, M, g);
        ++launches;
        CK(cudaFreeAsync(stage, stream));
    } else {
        const size_t n3 = (size_t)(g.nz + 6) * (g.nx + 6) * (g.ny + 6);
        float* stage = nullptr;
        for (int f = 0; f < 5; ++f) {
            const float* src = pinned_view(fields[f]);
            if (!src) {
                if (!stage) CK(cudaMallocAsync((void**)&stage, n3 * 4, stream));
                CK(cudaMemcpyAsync(stage, fields[f], n3 * 4, cudaMemcpyHostToDevice, stream));
                src = stage;
            }
            k_scatter_t<<<dim3((g.nz + 6 + 31) / 32, (g.nx + 6 + 31) / 32, g.ny + 6), dim3(32, 8), 0, stream>>>(src, M, g, 5, f, 0);
            ++launches;
        }
        if (stage) CK(cudaFreeAsync(stage, stream));
    }
    // band table over the interior columns and the kob map
    const int mx = g.nx + 6;
    auto at = [&](const int* m, int i, int j) { return m[(size_t)(j + 2) * mx + (i + 2)]; };  // 1-based i, j
    std::vector<int> bnd(4 * (size_t)p.nxi * p.nyi);
    for (int jj = 0; jj < p.nyi; ++jj)
        for (int ii = 0; ii < p.nxi; ++ii) {
            int i = p.x0 + ii + 1, j = p.y0 + jj + 1;
            size_t q = 4 * ((size_t)jj * p.nxi + ii);
            bnd[q] = at(kfs_top, i, j); bnd[q + 1] = at(kfs_bot, i, j);
            bnd[q + 2] = at(kob_top, i, j); bnd[q + 3] = at(kob_bot, i, j);
        }
    // per-column kob and kfs (1-based, clamped to 0..nz-1 so that k+1 is a
    // valid 0-based plane index plus one)
    std::vector<int> kb((size_t)g.nx * g.ny), kf((size_t)g.nx * g.ny);
    for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
            kb[(size_t)j * g.nx + i] = std::max(0, std::min(g.nz - 1, at(kob, i + 1, j + 1)));
            kf[(size_t)j * g.nx + i] = std::max(0, std::min(g.nz - 1, at(kfs, i + 1, j + 1)));
        }
    CK(cudaMemcpyAsync(band, bnd.data(), bnd.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_kob, kb.data(), kb.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_kfs, kf.data(), kf.size() * 4, cudaMemcpyHostToDevice, stream));
    // the host arrays must stay readable until the copies are done
    CK(cudaStreamSynchronize(stream));
    return finish_medium(ts);
}

// The medium of a layered model with a random perturbation, built on the
// device from the background column and the periodic field (medium.cuh):
// cells, absorber band, tau-method and relaxation in FP64, surface maps and
// the interior band table.  maps6 (optional) receives the six surface maps
// of the halo plane (kfs, kob, kfs_top, kfs_bot, kob_top, kob_bot, each
// (nx+6) x (ny+6), i fastest); ts the relaxation times.
int Sim::build_medium_rmed(const float* bg, const float* xi, int nxc, int nyc, int nzc, int kxi0, double vmin,
                           double vmax, double rhomin, double fq_min, double fq_max, double fq_ref, int* maps6,
                           double* ts) {
    const Geo& g = p.g;
    visco::relaxation_times(NM, fq_min, fq_max, ts);
    const double zeta = visco::constq_zeta(NM, fq_min, fq_max, ts);
    RmedArgs a{};
    a.g = g; a.M = M;
    a.nxc = nxc; a.nyc = nyc; a.nzc = nzc; a.kxi0 = kxi0; a.na = dims.na;
    a.vmin = (float)vmin; a.vmax = (float)vmax; a.rhomin = (float)rhomin;
    // Q depends on depth only: the tau-method ratios and the relaxation
    // factors of every k, in the FP64 sequence of the host set-up
    double cr, ci;
    visco::zener_c(NM, fq_ref, ts, cr, ci);
    const int nk = g.nz + 6;
    std::vector<double> kq(4 * (size_t)nk);
    for (int k = 0; k < nk; ++k) {
        const double tp = NM * zeta / (double)bg[3 * nk + k], tsv = NM * zeta / (double)bg[4 * nk + k];
        kq[k] = tp;
        kq[nk + k] = tsv;
        kq[2 * nk + k] = visco::relax_factor(cr, ci, tsv);
        kq[3 * nk + k] = visco::relax_factor(cr, ci, tp);
    }
    const size_t nbg = 5 * (size_t)nk, nfield = (size_t)nxc * nyc * nzc;
    const size_t n2 = (size_t)(g.nx + 6) * (g.ny + 6);
    const size_t bytes = kq.size() * 8 + (nbg + nfield) * 4 + 6 * n2 * 4;
    char* stage = nullptr;
    CK(cudaMallocAsync((void**)&stage, bytes, stream));
    double* dkq = reinterpret_cast<double*>(stage);
    float* dbg = reinterpret_cast<float*>(dkq + kq.size());
    float* dxi = dbg + nbg;
    int* dm = reinterpret_cast<int*>(dxi + nfield);
    CK(cudaMemcpyAsync(dkq, kq.data(), kq.size() * 8, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dbg, bg, nbg * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dxi, xi, nfield * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(dm, 0, 6 * n2 * 4, stream));
    a.bg = dbg;
    a.xi = dxi;
    a.kq = dkq;
    k_rmed_medium<<<4096, 256, 0, stream>>>(a);
    int* kfs = dm; int* kob = dm + n2; int* kft = dm + 2 * n2; int* kfb = dm + 3 * n2; int* kot = dm + 4 * n2;
    int* kobb = dm + 5 * n2;
    const int ncol = (g.nx + 3) * (g.ny + 3);
    k_rmed_surface<<<(ncol + 255) / 256, 256, 0, stream>>>(M, g, kfs, kob);
    k_rmed_ranges<<<(g.nx * g.ny + 255) / 256, 256, 0, stream>>>(kfs, kob, g, kft, kfb, kot, kobb);
    const int nt = std::max(p.nxi * p.nyi, g.nx * g.ny);
    k_rmed_tables<<<(nt + 255) / 256, 256, 0, stream>>>(kfs, kob, kft, kfb, kot, kobb, g, p.x0, p.y0, p.nxi, p.nyi,
                                                      band, d_kob, d_kfs);
    launches += 4;
    CK(cudaGetLastError());
    if (maps6) CK(cudaMemcpyAsync(maps6, dm, 6 * n2 * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaFreeAsync(stage, stream));
    CK(cudaStreamSynchronize(stream));
    return finish_medium(ts);
}

// Coefficients, absorber profiles and the divergence check once the medium
// and the surface maps are on the device.
int Sim::finish_medium(const double* ts) {
    const Geo& g = p.g;
    // FD and Zener coefficients in FP64 (m_kernel.f90:43-67)
    const double dt = dims.dt, dx = dims.dx, dy = dims.dy, dz = dims.dz;
    coef.e4x0 = (float)(18.0 / 16.0 / dx); coef.e4x1 = (float)(2.0 / 48.0 / dx);
    coef.e4y0 = (float)(18.0 / 16.0 / dy); coef.e4y1 = (float)(2.0 / 48.0 / dy);
    coef.e4z0 = (float)(18.0 / 16.0 / dz); coef.e4z1 = (float)(2.0 / 48.0 / dz);
    coef.e2x = (float)(1.0 / dx); coef.e2y = (float)(1.0 / dy); coef.e2z = (float)(1.0 / dz);
    // FP16 storage of the memory variables keeps them scaled by a power of two
    // rscale, folded into c2 (R is built from c2 terms) and d1 (R enters the
    // stress through d1); both products stay exact in FP32, so only where the
    // 16-bit rounding happens changes.  The stress next to a unit source
    // reaches about 1/(dx dy dz) and R about 0.05 of that, so
    // rscale = 4096 dx dy dz puts the largest R near 200 (overflow at 65504)
    // and keeps R down to ~1e-6 of its peak in the normal FP16 range.
    double rscale = 1.0;
    if (dims.store == SWPC_STORE_FP16)
        rscale = std::ldexp(1.0, std::max(0, std::min(20, (int)std::lround(std::log2(4096.0 * dx * dy * dz)))));
    double d2 = 0;
    for (int m = 0; m < NM; ++m) {
        coef.c1[m] = (float)((2 * ts[m] - dt) / (2 * ts[m] + dt));
        coef.c2[m] = (float)(2.0 / (2 * ts[m] + dt) / NM * rscale);
        coef.d1[m] = (float)(2 * ts[m] / (2 * ts[m] - dt) / rscale);
        d2 += dt / (2 * ts[m] - dt);
    }
    coef.d2 = (float)(d2 / NM);
    coef.dt = (float)dt;

    // absorbing boundary profiles in FP64
    if (p.pml) {
        std::vector<float> prof;
        auto add = [&](int n, double beg, double d) {
            int o0 = (int)prof.size();
            prof.resize(prof.size() + 8 * (size_t)n);
            const double H = dims.na * d, end = beg + n * d;
            for (int q = 0; q < n; ++q) {
                double xc = beg + (q + 0.5) * d;
                damping_profile(xc, H, beg, end, dims.na, dims.fcut, dt, &prof[o0 + 4 * q]);
                damping_profile(xc + d / 2, H, beg, end, dims.na, dims.fcut, dt, &prof[o0 + 4 * n + 4 * q]);
            }
            return o0;
        };
        PArgs& a = pml_args;
        a.pxc = add(g.nx, dims.xbeg, dx); a.pxe = a.pxc + 4 * g.nx;
        a.pyc = add(g.ny, dims.ybeg, dy); a.pye = a.pyc + 4 * g.ny;
        a.pzc = add(g.nz, dims.zbeg, dz); a.pze = a.pzc + 4 * g.nz;
        float* dp = nullptr;
        int rc = dalloc((void**)&dp, prof.size() * 4);
        if (rc) return rc;
        CK(cudaMemcpyAsync(dp, prof.data(), prof.size() * 4, cudaMemcpyHostToDevice, stream));
        a.g = g; a.V = V; a.S = S; a.M = M; a.adeV = adeV; a.adeS = adeS; a.prof = dp; a.shm = shm;
        a.nbox = p.nbox;
        for (int b = 0; b < p.nbox; ++b) a.box[b] = p.box[b];
        a.npart = 0;
        a.nblocks = 0;
        a.r20x = (float)(1.0 / dx); a.r20y = (float)(1.0 / dy); a.r20z = (float)(1.0 / dz); a.dt = (float)dt;
        plan_pml_parts(prof);
        // the shell's harmonic means and buoyancies, once per medium
        if (pml_all.nblocks) {
            k_shell_medium<<<pml_all.nblocks, PTPB, 0, stream>>>(pml_all, shm);
            ++launches;
            CK(cudaGetLastError());
        }
    } else {
        std::vector<float> c, b, all;
        int n[3] = {g.nx, g.ny, g.nz};
        double d[3] = {dx, dy, dz};
        for (int ax = 0; ax < 3; ++ax) {
            cerjan_profile(n[ax], dims.na, d[ax], c, b, ax == 2);
            cer_off[2 * ax] = (int)all.size(); all.insert(all.end(), c.begin(), c.end());
            cer_off[2 * ax + 1] = (int)all.size(); all.insert(all.end(), b.begin(), b.end());
        }
        int rc = dalloc((void**)&cer, all.size() * 4);
        if (rc) return rc;
        CK(cudaMemcpyAsync(cer, all.data(), all.size() * 4, cudaMemcpyHostToDevice, stream));
    }
    // divergence check (m_report.f90:120-152)
    VmaxArgs& v = vmax_args;
    v.g = g; v.V = V; v.kob = d_kob; v.it = d_it;
    v.ntdec_r = dims.ntdec_r;
    const int ibk = p.x0 + 1, iek = p.x0 + p.nxi, jbk = p.y0 + 1, jek = p.y0 + p.nyi;
    v.i0 = std::max(dims.na + 5 + 1, ibk) - 1; v.i1 = std::min(g.nx - dims.na - 5, iek) - 1;
    v.j0 = std::max(dims.na + 5 + 1, jbk) - 1; v.j1 = std::min(g.ny - dims.na - 5, jek) - 1;
    if (v.i1 < v.i0 || v.j1 < v.j0) v.ntdec_r = 0;
    if (v.ntdec_r > 0) {
        v.nrep = std::max(1, dims.nt / v.ntdec_r + 1);
        int rc = dalloc((void**)&v.rep, (size_t)v.nrep * 12);
        if (rc) return rc;
        rep_host.assign((size_t)v.nrep * 3, 0u);
    }
    CK(cudaStreamSynchronize(stream));
    medium_ready = true;
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    return 0;
}

int Sim::set_sources(int n, const int* ijk, const double* mo, const double* mij, const double* fxyz, const double* prm,
                     int stftype, bool bf) {
    SrcArgs& a = src_args;
    a.g = p.g; a.V = V; a.S = S; a.M = M; a.it = d_it;
    a.n = n; a.stf = stftype;
    a.tbeg = (float)dims.tbeg; a.dt = (float)dims.dt;
    a.dt_dxyz = (float)(dims.dt / (dims.dx * dims.dy * dims.dz));
    a.bf = bf ? 1 : 0;
    bf_mode = bf;
    if (n == 0) return 0;
    std::vector<int> q(3 * (size_t)n);
    std::vector<float> m6(6 * (size_t)n, 0.f), f3(3 * (size_t)n, 0.f), pr(2 * (size_t)n);
    for (int s = 0; s < n; ++s) {
        for (int c = 0; c < 3; ++c) {
            q[3 * s + c] = ijk[3 * s + c] - 1;
            int lim = c == 0 ? p.g.nx : c == 1 ? p.g.ny : p.g.nz;
            if (q[3 * s + c] < -2 || q[3 * s + c] > lim + 1) return set_err(SWPC_E_ARG, "source grid point outside the model sleeve");
        }
        if (bf) for (int c = 0; c < 3; ++c) f3[3 * s + c] = (float)fxyz[3 * s + c];
        else for (int c = 0; c < 6; ++c) m6[6 * s + c] = (float)(mo[s] * mij[6 * s + c]);
        pr[2 * s] = (float)prm[2 * s];
        pr[2 * s + 1] = (float)prm[2 * s + 1];
    }
    int* di; float *dm, *df, *dp;
    int rc;
    if ((rc = dalloc((void**)&di, q.size() * 4))) return rc;
    if ((rc = dalloc((void**)&dm, m6.size() * 4))) return rc;
    if ((rc = dalloc((void**)&df, f3.size() * 4))) return rc;
    if ((rc = dalloc((void**)&dp, pr.size() * 4))) return rc;
    CK(cudaMemcpyAsync(di, q.data(), q.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dm, m6.data(), m6.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(df, f3.data(), f3.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(dp, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    a.ijk = di; a.mij = dm; a.fxyz = df; a.prm = dp;
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    return 0;
}

int Sim::set_receivers(int n, const int* ijk, int ntdec_w, int flags) {
    TapArgs& a = tap_args;
    a.g = p.g; a.V = V; a.S = S; a.it = d_it;
    a.n = n; a.ntdec_w = ntdec_w; a.flags = flags;
    a.ntw = (int)std::floor((float)(dims.nt - 1) / (float)ntdec_w + 1.0f);
    a.dt = (float)dims.dt;
    a.vscale = (float)(dims.M0 * dims.UC * 1e9);
    a.sscale = (float)(dims.M0 * dims.UC * 1e6);
    a.escale = (float)(dims.M0 * dims.UC * 1e-3);
    a.r40x = (float)(9.0 / 8.0 / dims.dx); a.r40y = (float)(9.0 / 8.0 / dims.dy); a.r40z = (float)(9.0 / 8.0 / dims.dz);
    a.r41x = (float)(1.0 / 24.0 / dims.dx); a.r41y = (float)(1.0 / 24.0 / dims.dy); a.r41z = (float)(1.0 / 24.0 / dims.dz);
    if (n == 0 || flags == 0) { a.n = 0; return 0; }
    std::vector<int> q(3 * (size_t)n);
    for (int s = 0; s < n; ++s)
        for (int c = 0; c < 3; ++c) {
            q[3 * s + c] = ijk[3 * s + c] - 1;
            int lim = c == 0 ? p.g.nx : c == 1 ? p.g.ny : p.g.nz;
            if (q[3 * s + c] < 0 || q[3 * s + c] >= lim) return set_err(SWPC_E_ARG, "receiver outside the grid");
        }
    int rc;
    int* di;
    if ((rc = dalloc((void**)&di, q.size() * 4))) return rc;
    CK(cudaMemcpyAsync(di, q.data(), q.size() * 4, cudaMemcpyHostToDevice, stream));
    a.ijk = di;
    const size_t w3 = (size_t)a.ntw * 3 * n, w6 = (size_t)a.ntw * 6 * n;
    a.wav_v = a.wav_u = a.wav_s = a.wav_e = nullptr;
    if ((flags & 1) && (rc = dalloc((void**)&a.wav_v, w3 * 4))) return rc;
    if ((flags & 2) && (rc = dalloc((void**)&a.wav_u, w3 * 4))) return rc;
    if ((flags & 4) && (rc = dalloc((void**)&a.wav_s, w6 * 4))) return rc;
    if ((flags & 8) && (rc = dalloc((void**)&a.wav_e, w6 * 4))) return rc;
    if ((rc = dalloc((void**)&a.acc, 9 * (size_t)n * 8))) return rc;
    CK(cudaStreamSynchronize(stream));
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    return 0;
}

// Snapshot planes (snap__setup, m_snap.f90:95-207): every plane shares the
// frame interval ntdec_s; adding a plane of the same section and kind again
// replaces its geometry.
int Sim::add_snapshot(int sec, int kind, int fix, int d1, int d2, int ntdec_s) {
    SnapArgs& a = snap_args;
    if (a.n > 0 && ntdec_s != a.ntdec_s) return set_err(SWPC_E_ARG, "all snapshots share one ntdec_s");
    const Geo& g = p.g;
    a.g = g; a.V = V; a.S = S; a.M = M; a.kfs = d_kfs; a.kob = d_kob; a.it = d_it;
    a.ntdec_s = ntdec_s;
    a.maxframes = (dims.nt - 1) / ntdec_s + 1;
    a.UC = (float)dims.UC; a.M0 = (float)dims.M0; a.dt = (float)dims.dt;
    a.r20x = (float)(1.0 / dims.dx); a.r20y = (float)(1.0 / dims.dy); a.r20z = (float)(1.0 / dims.dz);
    int q = 0;
    while (q < a.n && !(a.pl[q].sec == sec && a.pl[q].kind == kind)) ++q;
    if (q == MAX_SNAP) return set_err(SWPC_E_ARG, "too many snapshot planes");
    SnapPlane P{};
    P.sec = sec; P.kind = kind; P.d1 = d1; P.d2 = d2; P.nc = kind == SNAP_PS ? 4 : 3;
    const int nxs = (g.nx + d1 / 2) / d1;
    switch (sec) {  // nxs, nys, nzs of m_snap.f90:131-133
    case SEC_YZ: P.n1 = (g.ny + d1 / 2) / d1; P.n2 = (g.nz + d2 / 2) / d2; P.fix = fix - 1; break;
    case SEC_XZ: P.n1 = nxs; P.n2 = (g.nz + d2 / 2) / d2; P.fix = fix - 1; break;
    default: P.n1 = nxs; P.n2 = (g.ny + d2 / 2) / d2; P.fix = fix - 1; break;
    }
    const size_t pix = (size_t)P.n1 * P.n2;
    const bool same = q < a.n && a.pl[q].n1 == P.n1 && a.pl[q].n2 == P.n2;
    if (same) {
        P.frames = a.pl[q].frames;
        P.uacc = a.pl[q].uacc;
    } else {
        int rc;
        if ((rc = dalloc((void**)&P.frames, (size_t)a.maxframes * P.nc * pix * 4))) return rc;
        if (kind == SNAP_U && (rc = dalloc((void**)&P.uacc, 3 * pix * 8))) return rc;
    }
    if (kind == SNAP_U && !P.uacc) {
        int rc = dalloc((void**)&P.uacc, 3 * pix * 8);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(P.frames, 0, (size_t)a.maxframes * P.nc * pix * 4, stream));
    if (P.uacc) CK(cudaMemsetAsync(P.uacc, 0, 3 * pix * 8, stream));
    a.pl[q] = P;
    if (q == a.n) ++a.n;
    a.maxpix = 0;
    for (int r = 0; r < a.n; ++r) a.maxpix = std::max(a.maxpix, a.pl[r].n1 * a.pl[r].n2);
    CK(cudaStreamSynchronize(stream));
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    return 0;
}

const SnapPlane* Sim::find_plane(int sec, int kind) const {
    for (int q = 0; q < snap_args.n; ++q)
        if (snap_args.pl[q].sec == sec && snap_args.pl[q].kind == kind) return &snap_args.pl[q];
    return nullptr;
}

// Green's-function points (m_green.f90:67-404): n points at 1-based ijk,
// samples every ntdec_w steps, with (bforce) or without displacement output
int Sim::set_green(int n, const int* ijk, int ntdec_w, int bforce) {
    GreenArgs& a = green_args;
    a = GreenArgs{};
    if (n <= 0) return 0;
    a.g = p.g; a.V = V; a.it = d_it;
    a.n = n; a.ncmp = bforce ? 9 : 6; a.ntdec_w = ntdec_w;
    a.ntw = (dims.nt - 1) / ntdec_w + 1;
    a.dt = (float)dims.dt;
    a.r40x = (float)(9.0 / 8.0 / dims.dx); a.r41x = (float)(1.0 / 24.0 / dims.dx);
    a.r40y = (float)(9.0 / 8.0 / dims.dy); a.r41y = (float)(1.0 / 24.0 / dims.dy);
    a.r40z = (float)(9.0 / 8.0 / dims.dz); a.r41z = (float)(1.0 / 24.0 / dims.dz);
    std::vector<int> q(3 * (size_t)n);
    for (int m = 0; m < n; ++m) {
        const int i = ijk[3 * m], j = ijk[3 * m + 1], k = ijk[3 * m + 2];
        // the 4th-order stencils reach two cells on either side
        if (i < 1 || i > dims.nx || j < 1 || j > dims.ny || k < 1 || k > dims.nz)
            return set_err(SWPC_E_ARG, "Green's-function point outside the grid");
        q[3 * m] = i - 1; q[3 * m + 1] = j - 1; q[3 * m + 2] = k - 1;
    }
    int rc;
    int* dq = nullptr;
    if ((rc = dalloc((void**)&dq, q.size() * 4))) return rc;
    if ((rc = dalloc((void**)&a.acc, (size_t)12 * n * 8))) return rc;
    if ((rc = dalloc((void**)&a.gf, (size_t)a.ntw * a.ncmp * n * 4))) return rc;
    a.ijk = dq;
    CK(cudaMemcpyAsync(dq, q.data(), q.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(a.acc, 0, (size_t)12 * n * 8, stream));
    CK(cudaMemsetAsync(a.gf, 0, (size_t)a.ntw * a.ncmp * n * 4, stream));
    CK(cudaStreamSynchronize(stream));
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    return 0;
}

int Sim::nframes_done() const {
    if (!snap_args.n || it_done < 1) return 0;
    return std::min(snap_args.maxframes, (it_done - 1) / std::max(1, snap_args.ntdec_s) + 1);
}

// ---------------------------------------------------------------------------
// Batched form: many independent simulations advanced by one fused launch per
// phase of the time step (stress interior + PML shell, sources, velocity
// interior + PML shell, taps), captured as a CUDA graph.  Every launch walks a
// block table that spans all members, so small grids that would leave most of
// the GPU idle alone fill it together.
// ---------------------------------------------------------------------------
struct Batch {
    std::vector<Sim*> sims;
    cudaStream_t stream = nullptr, stream2 = nullptr;
    cudaEvent_t ev[4] = {};
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 8;
    int rbytes = 4, store = 0;
    std::vector<void*> allocs;
    TArgs* d_targs = nullptr;
    PArgs* d_pargs[PML_NCLASS] = {};  // per launch class: every member's PML arguments
    SrcArgs* d_src = nullptr;
    TapArgs* d_tap = nullptr;
    SnapArgs* d_snap = nullptr;
    GreenArgs* d_green = nullptr;
    int max_green = 0;
    std::vector<Sim*> pw_members;  // plane-wave members: lateral ghost extrapolation before the PML updates
    VmaxArgs* d_vmax = nullptr;
    int** d_its = nullptr;
    int4* d_tblocks = nullptr;   // stress tiles (interior kernels)
    int4* d_tblocks_v = nullptr; // velocity tiles
    int4* d_tblocks_sh = nullptr;   // stress shell tiles (members whose tile kernels sweep the shell)
    int4* d_tblocks_vsh = nullptr;  // velocity shell tiles
    int n_tblocks_sh = 0, n_tblocks_vsh = 0;
    TArgs* d_targs_np = nullptr;        // the persistent form's view of every member (interior box)
    PArgs* d_pargs_np[PML_NCLASS] = {}; // and its PML blocks
    int2* d_pblocks[PML_NCLASS] = {}; // per launch class: (member, block of its launch)
    int n_pblocks[PML_NCLASS] = {};
    int n_tblocks = 0, n_tblocks_v = 0, max_nst = 0, max_src = 0, max_pix = 0, max_planes = 0;
    bool any_vmax = false, any_snap = false, any_bf = false, any_mt = false;
    size_t smem_stress = 0, smem_vel = 0, smem_stress_sh = 0, smem_vel_sh = 0;
    long long launches = 0, launches_per_graph = 0;
    // persistent fused form: the work queue of one time step of every
    // member, the per-member finished counters and the launch shape
    bool persistent = false;
    int ty_s = TTY, ty_v = TTY;  // tile rows shared by every member
    PersistArgs pargs{};
    int n_items = 0, persist_grid = 0;
    size_t smem_persist = 0;
    int* d_ctr = nullptr;  // [0] head, [1] error word, [2..] per-member finished counters
    ~Batch() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph) cudaGraphExecDestroy(graph);
        for (void* q : allocs) cudaFree(q);
        for (auto e : ev) if (e) cudaEventDestroy(e);
        if (stream2) cudaStreamDestroy(stream2);
        if (stream) cudaStreamDestroy(stream);
    }
    template <class T>
    int upload(T** dst, const std::vector<T>& v) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(16, v.size() * sizeof(T)));
        if (e != cudaSuccess) return set_err(SWPC_E_NOMEM, std::string("batch table: ") + cudaGetErrorString(e));
        allocs.push_back(q);
        if (!v.empty()) CK(cudaMemcpy(q, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        *dst = (T*)q;
        return 0;
    }
    // The work queue of the persistent form (persist.cuh): phase by phase,
    // every member's items of that phase, each with the number of the
    // member's items in earlier phases that must be finished first.
    int build_queue(const std::vector<int4>& tb, const std::vector<int4>& tbv, const std::vector<PArgs>* pa) {
        const int n = (int)sims.size();
        const int T = PERSIST_THREADS;
        auto chunks = [T](long long units) { return (int)((units + T - 1) / T); };
        std::vector<int4> items;
        std::vector<int> need;
        std::vector<int> cnt(n, 0);
        // tiles of each member, in the order of the phase launches' tables
        std::vector<std::vector<int4>> st(n), vt(n);
        for (const int4& e : tb) st[e.x].push_back(e);
        for (const int4& e : tbv) vt[e.x].push_back(e);
        auto item = [](int type, int m, int y, int z, int w) { return make_int4(type | (m << 4), y, z, w); };
        for (int phase = 0; phase < 8; ++phase) {
            for (int m = 0; m < n; ++m) {
                Sim* s = sims[m];
                const size_t first = items.size();
                const bool pw = s->pw && s->p.pml;
                switch (phase) {
                case 0: {  // taps, Green's-function taps, snapshot pixels
                    long long u = s->tap_args.n + s->green_args.n;
                    for (int q = 0; q < s->snap_args.n; ++q) u += (long long)s->snap_args.pl[q].n1 * s->snap_args.pl[q].n2;
                    for (int c = 0; c < chunks(u); ++c) items.push_back(item(IT_PRE, m, c, 0, 0));
                    break;
                }
                case 1:
                    if (pw) for (int c = 0; c < chunks(pw_ghost_units(s->p.g, 3)); ++c) items.push_back(item(IT_PW_V, m, c, 0, 0));
                    break;
                case 2:
                    if (s->p.pml)
                        for (int c = 0; c < PML_NCLASS; ++c)
                            for (int k = 0; k < (pa[c][m].nblocks + PML_ITEM_BLOCKS - 1) / PML_ITEM_BLOCKS; ++k)
                                items.push_back(item(IT_PML_S, m, c, k, 0));
                    for (const int4& e : st[m]) items.push_back(item(IT_STRESS, m, e.y, e.z, e.w));
                    break;
                case 3:
                    if (s->src_args.n > 0 && !s->bf_mode)
                        for (int c = 0; c < chunks(s->src_args.n); ++c) items.push_back(item(IT_SRC_S, m, c, 0, 0));
                    break;
                case 4:
                    if (pw) for (int c = 0; c < chunks(pw_ghost_units(s->p.g, 6)); ++c) items.push_back(item(IT_PW_S, m, c, 0, 0));
                    break;
                case 5:
                    if (s->p.pml)
                        for (int c = 0; c < PML_NCLASS; ++c)
                            for (int k = 0; k < (pa[c][m].nblocks + PML_ITEM_BLOCKS - 1) / PML_ITEM_BLOCKS; ++k)
                                items.push_back(item(IT_PML_V, m, c, k, 0));
                    for (const int4& e : vt[m]) items.push_back(item(IT_VEL, m, e.y, e.z, e.w));
                    break;
                case 6:
                    if (s->src_args.n > 0 && s->bf_mode)
                        for (int c = 0; c < chunks(s->src_args.n); ++c) items.push_back(item(IT_SRC_V, m, c, 0, 0));
                    break;
                default:
                    items.push_back(item(IT_ADV, m, 0, 0, 0));
                    break;
                }
                need.insert(need.end(), items.size() - first, cnt[m]);
                cnt[m] += (int)(items.size() - first);
            }
        }
        int rc;
        int4* d_items = nullptr;
        int* d_need = nullptr;
        if ((rc = upload(&d_items, items)) || (rc = upload(&d_need, need))) return rc;
        std::vector<int> zero(2 + n, 0);
        if ((rc = upload(&d_ctr, zero))) return rc;
        n_items = (int)items.size();
        PersistArgs& P = pargs;
        P.items = d_items; P.need = d_need; P.n_items = n_items;
        P.head = d_ctr; P.err = d_ctr + 1; P.done = d_ctr + 2;
        P.targs = d_targs_np;
        for (int c = 0; c < PML_NCLASS; ++c) P.pargs[c] = d_pargs_np[c];
        P.src = d_src; P.tap = d_tap; P.snap = d_snap; P.green = d_green; P.its = d_its;
        // one block of the 8-row tile kernels' shape holds either tile's rings
        smem_persist = std::max(rbytes == 4 ? sizeof(StressSmem<float>) : sizeof(StressSmem<__half>), sizeof(VelSmem<>));
        int dev = 0, nsm = 0, occ = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        const void* fn = rbytes == 4 ? (const void*)k_batch_persistent<float>
                         : store == SWPC_STORE_FP16 ? (const void*)k_batch_persistent<__half>
                                                    : (const void*)k_batch_persistent<__nv_bfloat16>;
        CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_persist));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, PERSIST_THREADS, smem_persist));
        persist_grid = std::max(1, std::min(n_items, nsm * std::max(1, occ)));
        return 0;
    }
    bool any_pml() const {
        for (int q = 0; q < PML_NCLASS; ++q)
            if (n_pblocks[q]) return true;
        return false;
    }
    void launch_pml(bool stress) {
        for (int q = 0; q < PML_NCLASS; ++q) {
            if (!n_pblocks[q]) continue;
            const unsigned nb = (unsigned)n_pblocks[q];
            const PArgs* a = d_pargs[q];
            const int2* t = d_pblocks[q];
            switch (PML_CLASS_MASK[q]) {
            case 1: stress ? k_stress_pml_batch<1><<<nb, PTPB, 0, stream2>>>(a, t) : k_vel_pml_batch<1><<<nb, PTPB, 0, stream2>>>(a, t); break;
            case 2: stress ? k_stress_pml_batch<2><<<nb, PTPB, 0, stream2>>>(a, t) : k_vel_pml_batch<2><<<nb, PTPB, 0, stream2>>>(a, t); break;
            case 4: stress ? k_stress_pml_batch<4><<<nb, PTPB, 0, stream2>>>(a, t) : k_vel_pml_batch<4><<<nb, PTPB, 0, stream2>>>(a, t); break;
            default: stress ? k_stress_pml_batch<7><<<nb, PTPB, 0, stream2>>>(a, t) : k_vel_pml_batch<7><<<nb, PTPB, 0, stream2>>>(a, t); break;
            }
            ++launches;
        }
    }
    int launch_persistent() {
        const int n = (int)sims.size();
        if (any_vmax) { k_vmax_batch<<<dim3(64, n), 256, 0, stream>>>(d_vmax); ++launches; }
        // head and finished counters back to zero, the error word kept
        CK(cudaMemsetAsync(d_ctr, 0, sizeof(int), stream));
        CK(cudaMemsetAsync(d_ctr + 2, 0, sizeof(int) * (size_t)n, stream));
        const dim3 tblk(32, TTY);  // the persistent form runs 8-row tiles only
        if (rbytes == 4) k_batch_persistent<float><<<persist_grid, tblk, smem_persist, stream>>>(pargs);
        else if (store == SWPC_STORE_FP16) k_batch_persistent<__half><<<persist_grid, tblk, smem_persist, stream>>>(pargs);
        else k_batch_persistent<__nv_bfloat16><<<persist_grid, tblk, smem_persist, stream>>>(pargs);
        ++launches;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
        return 0;
    }
    int launch_step() {
        if (persistent) return launch_persistent();
        const int n = (int)sims.size();
        if (any_vmax) { k_vmax_batch<<<dim3(64, n), 256, 0, stream>>>(d_vmax); ++launches; }
        if (max_nst) { k_taps_batch<<<dim3((max_nst + 127) / 128, n), 128, 0, stream>>>(d_tap); ++launches; }
        if (max_green) { k_green_batch<<<dim3((max_green + 127) / 128, n), 128, 0, stream>>>(d_green); ++launches; }
        if (any_snap) { k_snap_batch<<<dim3((max_pix + 127) / 128, max_planes, n), 128, 0, stream>>>(d_snap); ++launches; }
        const dim3 tblk(32, ty_s), tblk_v(32, ty_v);
        for (Sim* m : pw_members) { k_pw_ghost<<<256, 256, 0, stream>>>(m->V, m->p.g, 3); ++launches; }
        const bool pml = any_pml();
        if (pml) {
            cudaEventRecord(ev[0], stream);
            cudaStreamWaitEvent(stream2, ev[0], 0);
            launch_pml(true);
            cudaEventRecord(ev[1], stream2);
        }
        if (n_tblocks_sh) {  // shell tiles of the members whose tile kernels sweep the shell
            if (ty_s == 16) {
                if (rbytes == 4) k_stress_tma_batch<float, 16, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
                else if (store == SWPC_STORE_FP16)
                    k_stress_tma_batch<__half, 16, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
                else k_stress_tma_batch<__nv_bfloat16, 16, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
            } else {
                if (rbytes == 4) k_stress_tma_batch<float, 8, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
                else if (store == SWPC_STORE_FP16)
                    k_stress_tma_batch<__half, 8, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
                else k_stress_tma_batch<__nv_bfloat16, 8, true><<<n_tblocks_sh, tblk, smem_stress_sh, stream>>>(d_targs, d_tblocks_sh);
            }
            ++launches;
        }
        if (n_tblocks == 0) {
            // every tile of every member went to the shell-tile kernel
        } else if (ty_s == 16) {
            if (rbytes == 4) k_stress_tma_batch<float, 16><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
            else if (store == SWPC_STORE_FP16)
                k_stress_tma_batch<__half, 16><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
            else k_stress_tma_batch<__nv_bfloat16, 16><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
        } else {
            if (rbytes == 4) k_stress_tma_batch<float><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
            else if (store == SWPC_STORE_FP16) k_stress_tma_batch<__half><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
            else k_stress_tma_batch<__nv_bfloat16><<<n_tblocks, tblk, smem_stress, stream>>>(d_targs, d_tblocks);
        }
        if (n_tblocks) ++launches;
        if (pml) cudaStreamWaitEvent(stream, ev[1], 0);
        if (any_mt) { k_stressglut_batch<<<dim3((max_src + 127) / 128, n), 128, 0, stream>>>(d_src); ++launches; }
        for (Sim* m : pw_members) { k_pw_ghost<<<256, 256, 0, stream>>>(m->S, m->p.g, 6); ++launches; }
        if (pml) {
            cudaEventRecord(ev[2], stream);
            cudaStreamWaitEvent(stream2, ev[2], 0);
            launch_pml(false);
            cudaEventRecord(ev[3], stream2);
        }
        if (n_tblocks_vsh) {
            if (ty_v == 16) k_vel_tma_batch<16, true><<<n_tblocks_vsh, tblk_v, smem_vel_sh, stream>>>(d_targs, d_tblocks_vsh);
            else if (ty_v == 12) k_vel_tma_batch<12, true><<<n_tblocks_vsh, tblk_v, smem_vel_sh, stream>>>(d_targs, d_tblocks_vsh);
            else k_vel_tma_batch<8, true><<<n_tblocks_vsh, tblk_v, smem_vel_sh, stream>>>(d_targs, d_tblocks_vsh);
            ++launches;
        }
        if (n_tblocks_v) {
            if (ty_v == 16) k_vel_tma_batch<16><<<n_tblocks_v, tblk_v, smem_vel, stream>>>(d_targs, d_tblocks_v);
            else if (ty_v == 12) k_vel_tma_batch<12><<<n_tblocks_v, tblk_v, smem_vel, stream>>>(d_targs, d_tblocks_v);
            else k_vel_tma_batch<><<<n_tblocks_v, tblk_v, smem_vel, stream>>>(d_targs, d_tblocks_v);
            ++launches;
        }
        if (pml) cudaStreamWaitEvent(stream, ev[3], 0);
        if (any_bf) { k_bodyforce_batch<<<dim3((max_src + 127) / 128, n), 128, 0, stream>>>(d_src); ++launches; }
        k_advance_batch<<<(n + 127) / 128, 128, 0, stream>>>(d_its, n); ++launches;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
        return 0;
    }
};

extern "C" {

int swpc_gpu_set_zchunks(swpc_sim* sim, int kstress, int kvel) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || kstress < 0 || kvel < 0) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_set_zchunks");
    if (kstress == 0) kstress = s->kchunk_auto;
    if (kvel == 0) kvel = s->kchunk_v_auto;
    s->kchunk = std::max(1, std::min(kstress, s->p.nzi));
    s->kchunk_v = std::max(1, std::min(kvel, s->p.nzi));
    if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
    return 0;
}

int swpc_gpu_set_zchunk(swpc_sim* sim, int kchunk) { return swpc_gpu_set_zchunks(sim, kchunk, kchunk); }

int swpc_gpu_pml_fused(swpc_sim* sim) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    return s->pml_fused ? 1 : 0;
}

int swpc_gpu_set_tiles(swpc_sim* sim, int rows_stress, int rows_vel) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s) return set_err(SWPC_E_ARG, "null simulation");
    if (rows_stress == 0) rows_stress = TTY;
    if (rows_vel == 0) rows_vel = TTY;
    if ((rows_stress != 8 && rows_stress != 16) || (rows_vel != 8 && rows_vel != 12 && rows_vel != 16))
        return set_err(SWPC_E_ARG, "tile rows must be 8 or 16 for the stress kernels, 8, 12 or 16 for the velocity "
                                   "kernels (0: the default 8)");
    CK(cudaStreamSynchronize(s->stream));
    s->ty_s = rows_stress;
    s->ty_v = rows_vel;
    int rc = s->build_tensor_maps();
    if (rc) return rc;
    if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
    return 0;
}

int swpc_gpu_get_tiles(swpc_sim* sim, int* rows_stress, int* rows_vel) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !rows_stress || !rows_vel) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_get_tiles");
    *rows_stress = s->ty_s;
    *rows_vel = s->ty_v;
    return 0;
}

int swpc_gpu_get_zchunks(swpc_sim* sim, int* kstress, int* kvel) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    if (!s || !kstress || !kvel) return set_err(SWPC_E_ARG, "bad arguments to swpc_gpu_get_zchunks");
    *kstress = s->kchunk;
    *kvel = s->kchunk_v;
    return 0;
}

int swpc_gpu_get_zchunk(swpc_sim* sim) {
    Sim* s = reinterpret_cast<Sim*>(sim);
    return s ? s->kchunk : set_err(SWPC_E_ARG, "null simulation");
}

int swpc_batch_create(swpc_sim* const* sims, int n, swpc_batch** out) {
    if (!sims || n <= 0 || !out) return set_err(SWPC_E_ARG, "bad arguments to swpc_batch_create");
    *out = nullptr;
    Batch* b = new Batch();
    auto fail = [&](int rc) { delete b; return rc; };
    for (int q = 0; q < n; ++q) {
        Sim* s = reinterpret_cast<Sim*>(sims[q]);
        if (!s || !s->medium_ready) return fail(set_err(SWPC_E_STATE, "every member must have its medium uploaded"));
        if (s->variant != 0) return fail(set_err(SWPC_E_ARG, "batched members must use the TMA interior kernels"));
        if (q && s->dims.store != b->store) return fail(set_err(SWPC_E_ARG, "batched members must share one storage precision"));
        if (q && (s->ty_s != b->ty_s || s->ty_v != b->ty_v))
            return fail(set_err(SWPC_E_ARG, "batched members must share their tile shapes"));
        b->ty_s = s->ty_s;
        b->ty_v = s->ty_v;
        for (int r = 0; r < q; ++r)
            if (b->sims[r] == s) return fail(set_err(SWPC_E_ARG, "a simulation appears twice in the batch"));
        b->store = s->dims.store;
        b->rbytes = s->p.rbytes;
        b->sims.push_back(s);
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_err(SWPC_E_CUDA, "stream creation failed"));
    for (auto& e : b->ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(set_err(SWPC_E_CUDA, "event creation failed"));
    // ta, pa, tb, tbv, tbs, tbvs: the phase launches (a member whose tile
    // kernels sweep its shell has interior and shell-tile blocks and no PML
    // blocks); ta_np, pa_np, tb_np, tbv_np: the persistent form, which runs
    // every member's interior tiles and PML blocks
    std::vector<TArgs> ta(n), ta_np(n);
    std::vector<PArgs> pa[PML_NCLASS], pa_np[PML_NCLASS];
    std::vector<SrcArgs> sa(n);
    std::vector<TapArgs> tp(n);
    std::vector<SnapArgs> sn(n);
    std::vector<GreenArgs> gr(n);
    std::vector<VmaxArgs> vm(n);
    std::vector<int*> its(n);
    std::vector<int4> tb, tbv, tbs, tbvs, tb_np, tbv_np;
    std::vector<int2> pb[PML_NCLASS];
    // interior tiles of a member's view: stress in the grouped order of the
    // single-simulation launch, velocity x fastest; entries (member, bx, by,
    // first plane of the chunk)
    auto interior_lists = [&](int q, const Sim* s, const ZArgs& z, std::vector<int4>& st, std::vector<int4>& vt) {
        int bxl, bxh, byl, byh;
        interior_tiles(z, s->ty_s, bxl, bxh, byl, byh);
        const int gz = (s->p.nzi + s->kchunk - 1) / s->kchunk;
        for (int y0 = byl; y0 < byh; y0 += STRESS_YGROUP)
            for (int bz = 0; bz < gz; ++bz)
                for (int by = y0; by < std::min(byh, y0 + STRESS_YGROUP); ++by)
                    for (int bx = bxl; bx < bxh; ++bx) st.push_back(make_int4(q, bx, by, bz * s->kchunk));
        interior_tiles(z, s->ty_v, bxl, bxh, byl, byh);
        const int gzv = (s->p.nzi + s->kchunk_v - 1) / s->kchunk_v;
        for (int bz = 0; bz < gzv; ++bz)
            for (int by = byl; by < byh; ++by)
                for (int bx = bxl; bx < bxh; ++bx) vt.push_back(make_int4(q, bx, by, bz * s->kchunk_v));
    };
    for (int q = 0; q < n; ++q) {
        Sim* s = b->sims[q];
        CK(cudaStreamSynchronize(s->stream));
        ZArgs z, znp;
        s->fill_zargs(z);
        s->fill_zargs(znp, false);
        ta[q] = s->targs;
        ta[q].z = z;
        ta_np[q] = s->targs;
        ta_np[q].z = znp;
        for (int c = 0; c < PML_NCLASS; ++c) {
            pa_np[c].push_back(s->pml_cls[c]);
            if (!s->p.pml) pa_np[c].back().nblocks = 0;
            pa[c].push_back(pa_np[c].back());
            if (s->pml_fused) pa[c].back().nblocks = 0;
            for (int bk = 0; bk < pa[c].back().nblocks; ++bk) pb[c].push_back(make_int2(q, bk));
        }
        interior_lists(q, s, z, tb, tbv);
        interior_lists(q, s, znp, tb_np, tbv_np);
        for (int L = 0, ns = shell_tile_count(z, s->ty_s, s->kchunk); L < ns; ++L) {
            int bx, by, kz0;
            shell_tile(z, s->ty_s, s->kchunk, L, bx, by, kz0);
            tbs.push_back(make_int4(q, bx, by, kz0));
        }
        for (int L = 0, ns = shell_tile_count(z, s->ty_v, s->kchunk_v); L < ns; ++L) {
            int bx, by, kz0;
            shell_tile(z, s->ty_v, s->kchunk_v, L, bx, by, kz0);
            tbvs.push_back(make_int4(q, bx, by, kz0));
        }
        sa[q] = s->src_args;
        tp[q] = s->tap_args;
        sn[q] = s->snap_args;
        gr[q] = s->green_args;
        b->max_green = std::max(b->max_green, s->green_args.n);
        if (s->pw && s->p.pml) b->pw_members.push_back(s);
        vm[q] = s->vmax_args;
        its[q] = s->d_it;
        b->max_nst = std::max(b->max_nst, s->tap_args.n);
        b->max_src = std::max(b->max_src, s->src_args.n);
        if (s->src_args.n > 0) { if (s->bf_mode) b->any_bf = true; else b->any_mt = true; }
        if (s->vmax_args.ntdec_r > 0) b->any_vmax = true;
        if (s->snap_args.n) {
            b->any_snap = true;
            b->max_pix = std::max(b->max_pix, s->snap_args.maxpix);
            b->max_planes = std::max(b->max_planes, s->snap_args.n);
        }
    }
    int rc;
    for (int c = 0; c < PML_NCLASS; ++c)
        if ((rc = b->upload(&b->d_pargs[c], pa[c])) || (rc = b->upload(&b->d_pblocks[c], pb[c])) ||
            (rc = b->upload(&b->d_pargs_np[c], pa_np[c])))
            return fail(rc);
    if ((rc = b->upload(&b->d_targs, ta)) || (rc = b->upload(&b->d_targs_np, ta_np)) || (rc = b->upload(&b->d_src, sa)) ||
        (rc = b->upload(&b->d_tap, tp)) || (rc = b->upload(&b->d_snap, sn)) || (rc = b->upload(&b->d_green, gr)) || (rc = b->upload(&b->d_vmax, vm)) ||
        (rc = b->upload(&b->d_its, its)) || (rc = b->upload(&b->d_tblocks, tb)) || (rc = b->upload(&b->d_tblocks_v, tbv)) ||
        (rc = b->upload(&b->d_tblocks_sh, tbs)) || (rc = b->upload(&b->d_tblocks_vsh, tbvs)))
        return fail(rc);
    if (((uintptr_t)b->d_targs & 127) != 0 || ((uintptr_t)b->d_targs_np & 127) != 0)
        return fail(set_err(SWPC_E_CUDA, "tensor-map table is not 128-byte aligned"));
    b->n_tblocks = (int)tb.size();
    b->n_tblocks_v = (int)tbv.size();
    b->n_tblocks_sh = (int)tbs.size();
    b->n_tblocks_vsh = (int)tbvs.size();
    for (int c = 0; c < PML_NCLASS; ++c) b->n_pblocks[c] = (int)pb[c].size();
    b->smem_stress = b->sims[0]->smem_stress;
    b->smem_vel = b->sims[0]->smem_vel;
    b->smem_stress_sh = b->sims[0]->smem_stress_sh;
    b->smem_vel_sh = b->sims[0]->smem_vel_sh;
    if ((rc = b->build_queue(tb_np, tbv_np, pa_np))) return fail(rc);
    *out = reinterpret_cast<swpc_batch*>(b);
    return 0;
}

int swpc_batch_run(swpc_batch* batch, int nsteps) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || nsteps < 0) return set_err(SWPC_E_ARG, "bad arguments to swpc_batch_run");
    // every member continues from its own next step; the members' own
    // streams are drained first so their state is current
    for (Sim* s : b->sims) {
        if (s->diverged) return set_err(SWPC_E_DIVERGED, "a batch member has diverged");
        CK(cudaStreamSynchronize(s->stream));
        k_set_it<<<1, 1, 0, b->stream>>>(s->d_it, s->it_done + 1);
        ++b->launches;
    }
    int n = nsteps, rc = 0;
    if (n >= b->graph_steps && !b->graph) {
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        long long l0 = b->launches;
        for (int q = 0; q < b->graph_steps && rc == 0; ++q) rc = b->launch_step();
        cudaGraph_t gr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &gr);
        if (rc) return rc;
        if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return set_err(SWPC_E_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
        b->launches_per_graph = b->launches - l0;
        b->launches = l0;
    }
    while (b->graph && n >= b->graph_steps) {
        CK(cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->launches_per_graph;
        n -= b->graph_steps;
    }
    for (int q = 0; q < n && rc == 0; ++q) rc = b->launch_step();
    for (Sim* s : b->sims) s->it_done += nsteps;
    return rc;
}

int swpc_batch_sync(swpc_batch* batch) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b) return set_err(SWPC_E_ARG, "null batch");
    CK(cudaStreamSynchronize(b->stream));
    if (b->d_ctr) {
        int e = 0;
        CK(cudaMemcpy(&e, b->d_ctr + 1, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) return set_err(SWPC_E_TIMEOUT, "a bounded wait of the persistent batch launch ran out");
    }
    for (Sim* s : b->sims) {
        int rc = s->check_divergence();
        if (rc) return rc;
    }
    return 0;
}

int swpc_batch_set_persistent(swpc_batch* batch, int on) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b) return set_err(SWPC_E_ARG, "null batch");
    if (on && (b->ty_s != TTY || b->ty_v != TTY))
        return set_err(SWPC_E_ARG, "the persistent batch form runs 8-row tiles; the members use other tile shapes");
    CK(cudaStreamSynchronize(b->stream));
    if (b->persistent != (on != 0) && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->persistent = on != 0;
    return 0;
}

int swpc_batch_item_count(swpc_batch* batch) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    return b ? b->n_items : set_err(SWPC_E_ARG, "null batch");
}

void* swpc_batch_stream(swpc_batch* batch) { return batch ? (void*)reinterpret_cast<Batch*>(batch)->stream : nullptr; }

long long swpc_batch_launch_count(swpc_batch* batch) { return batch ? reinterpret_cast<Batch*>(batch)->launches : -1; }

int swpc_batch_destroy(swpc_batch* batch) {
    delete reinterpret_cast<Batch*>(batch);
    return 0;
}

}  // extern "C"
