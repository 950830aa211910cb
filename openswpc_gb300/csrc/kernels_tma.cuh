// kernels_tma.cuh -- TMA-fed z-sweep kernels for the viscoelastic interior.
//
// Each block owns a 32 x TY column tile and sweeps z.  One elected thread
// streams whole plane tiles into shared-memory rings with
// cp.async.bulk.tensor (4-D tensor maps over the row-interleaved [kz][jy][f][x]
// groups: one copy brings every field of a group for the tile), completing on
// one mbarrier per ring slot.  Several planes are in flight per block, so
// the HBM pipe stays full without the register cost of software prefetch.
// All threads compute from shared memory and store results with coalesced
// 128-byte stores.  Every mbarrier wait is bounded; a wait that runs out sets
// the error word, the block drains its own copies (again bounded) and returns.
#pragma once
#include <cuda.h>
#include "kernels.cuh"

namespace swpc {

constexpr int TTY = 8;            // default tile rows of the TMA kernels (8 or 16 per kernel)
constexpr int WAIT_LIMIT = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// Tensor maps and scalars of the TMA kernels.  The maps must stay 64-byte
// aligned and are read from the kernel parameter space (__grid_constant__).
struct TArgs {
    // boxes for tile rows TY (the stress kernel's for the first four, the
    // velocity kernel's for the last three)
    CUtensorMap tmV;    // V group, box (40, 3, TY+4, 1)
    CUtensorMap tmS;    // S group, box (32, 6, TY, 1)
    CUtensorMap tmM;    // M group fields lam..taus, box (36, 4, TY+1, 1)
    CUtensorMap tmR;    // memory variables, box (32, 18, TY, 1)
    CUtensorMap tmSh;   // S group with halo, box (40, 6, TY+4, 1)
    CUtensorMap tmRho;  // M group field rho, box (36, 1, TY+1, 1)
    CUtensorMap tmVc;   // V group centre, box (32, 3, TY, 1)
    ZArgs z;
    int* err;           // error word (bounded wait ran out)
};

// Every ring slot is a TMA destination and must start on a 128-byte
// boundary: each slot is its own 128-byte-aligned struct, so its size is
// padded to a multiple of 128 bytes.
template <class T, int A, int B, int C>
struct alignas(128) Slot3 { T d[A][B][C]; };
template <class T, int A, int B>
struct alignas(128) Slot2 { T d[A][B]; };

template <class RT, int TY = TTY>
struct StressSmem {
    Slot3<RT, TY, 18, 32> R[2];
    Slot3<float, TY, 6, 32> S[2];
    Slot3<float, TY + 1, 4, 36> M[3];
    Slot3<float, TY + 4, 3, 40> V[6];
    alignas(8) uint64_t barRS[2], barM[3], barV[6];
    int bad;
};

// Velocity kernel S ring: planes k .. k+2 are live (the tile of plane k for
// the x/y stencils, single values of k+1 and k+2 for the z stencil rolled in
// registers), the other VRING - 3 slots are in flight.  VRING = 5 keeps the
// block at 74 KB so three blocks fit on an SM.
#ifndef VEL_RING
#define VEL_RING 5
#endif
#ifndef VEL_MINB
#define VEL_MINB 3
#endif
constexpr int VRING = VEL_RING;
constexpr int VMINB = VEL_MINB;
static_assert(VRING >= 5, "the velocity S ring needs planes k-2 .. k+2 at start-up");
template <int TY = TTY>
struct VelSmem {
    Slot3<float, TY + 4, 6, 40> S[VRING];
    Slot2<float, TY + 1, 36> M[3];
    Slot3<float, TY, 3, 32> V[4];
    alignas(8) uint64_t barS[VRING], barM[3], barV[4];
    int bad;
};
// blocks per SM the tile kernels are built for: 8-row tiles two (stress) and
// VMINB (velocity), 16-row tiles one (their rings take 181 and 125 KB)
template <int TY> struct TileOcc { static constexpr int stress = 2, vel = VMINB; };
template <> struct TileOcc<16> { static constexpr int stress = 1, vel = 1; };
// 12-row tiles (velocity only): two 99 KB blocks per SM, the same 80
// registers per thread as three 8-row blocks, a third less S halo per point
template <> struct TileOcc<12> { static constexpr int stress = 1, vel = 2; };
static_assert(sizeof(Slot3<float, TTY + 1, 4, 36>) % 128 == 0, "slot size");
static_assert(sizeof(Slot2<float, TTY + 1, 36>) % 128 == 0, "slot size");
static_assert(sizeof(Slot3<__half, TTY, 18, 32>) % 128 == 0, "slot size");
static_assert(sizeof(Slot3<float, TTY + 4, 6, 40>) % 128 == 0, "slot size");
static_assert(sizeof(Slot3<float, 17, 4, 36>) % 128 == 0 && sizeof(Slot2<float, 17, 36>) % 128 == 0, "slot size");
static_assert(sizeof(StressSmem<float, 16>) <= 227 * 1024 && sizeof(VelSmem<16>) <= 227 * 1024, "16-row rings fit");
static_assert(2 * sizeof(VelSmem<12>) <= 226 * 1024, "two 12-row velocity blocks fit on an SM");
static_assert(sizeof(Slot3<float, 16, 6, 40>) % 128 == 0 && sizeof(Slot3<float, 12, 3, 32>) % 128 == 0, "slot size");

// Shell-tile kernels: the auxiliaries of every thread's shell point staged one
// plane ahead by cp.async (nine words per thread), after the rings.
template <int TY> struct AuxStage { float a[9][32 * TY]; };
template <class RT, int TY, bool SHELL> struct StressSm : StressSmem<RT, TY> {};
template <class RT, int TY> struct StressSm<RT, TY, true> : StressSmem<RT, TY> { AuxStage<TY> aux; };
template <int TY, bool SHELL> struct VelSm : VelSmem<TY> {};
template <int TY> struct VelSm<TY, true> : VelSmem<TY> { AuxStage<TY> aux; };
// blocks per SM of the shell-tile kernels (8-row tiles two; 12- and 16-row
// tiles one)
template <int TY> struct ShellOcc { static constexpr int stress = 2, vel = 2; };
template <> struct ShellOcc<16> { static constexpr int stress = 1, vel = 1; };
template <> struct ShellOcc<12> { static constexpr int stress = 1, vel = 1; };
static_assert(2 * sizeof(StressSm<float, 8, true>) <= 226 * 1024 && 2 * sizeof(VelSm<8, true>) <= 226 * 1024,
              "two shell-tile blocks fit on an SM");

// 4-byte asynchronous copy global -> shared; with `read` false the word is
// zero-filled and the source is not read
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool read) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(read ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Damped flags of index i for the profiles of PmlShell: bit p set when
// profile p (x centre, x edge, y c, y e, z c, z e) damps i.
__device__ __forceinline__ int damped_bit(const PmlShell& sh, int p, int i) {
    return (i < sh.dlo[p] || i >= sh.dhi[p]) ? (1 << p) : 0;
}
// the profile (bit of the flags above) whose g4 keeps auxiliary q live, in
// the auxiliary order of the stress update (axVx ayVy azVz ayVx azVx axVy
// azVy axVz ayVz) and of the velocity update (axSxx aySxy azSxz axSxy aySyy
// azSyz axSxz aySyz azSzz)
__host__ __device__ constexpr int aux_prof(bool vel, int q) {
    return vel ? (q == 0 ? 1 : q == 1 ? 2 : q == 2 ? 4 : q == 3 ? 0 : q == 4 ? 3 : q == 5 ? 4 : q == 6 ? 0 : q == 7 ? 2 : 5)
               : (q == 0 ? 0 : q == 1 ? 2 : q == 2 ? 4 : q == 3 ? 3 : q == 4 ? 5 : q == 5 ? 1 : q == 6 ? 5 : q == 7 ? 1 : 3);
}
// Stage the nine auxiliaries of a shell point (ADE address A, stride qs)
// with damped flags fl into the thread's slots: dead ones as zeros.
template <bool VEL, int TY>
__device__ __forceinline__ void stage_aux(AuxStage<TY>& st, int tid, const float* A, long long qs, int fl) {
#pragma unroll
    for (int q = 0; q < 9; ++q) cp_async4(&st.a[q][tid], A + q * qs, (fl >> aux_prof(VEL, q)) & 1);
    cp_async_commit();
}

// The tiles of a sweep grid run by the interior kernels: with the shell
// swept too, the tiles whose columns all lie inside the interior box (the
// others go to the shell-tile kernels); without, every tile of the interior
// box, the last ones partly filled.
__host__ __device__ inline void interior_tiles(const ZArgs& a, int TY, int& bxl, int& bxh, int& byl, int& byh) {
    if (a.sh.prof) {
        bxl = (a.x0 - a.tx0 + 31) / 32;
        bxh = max(bxl, (a.x0 + a.nxi - a.tx0) / 32);
        byl = (a.y0 - a.ty0 + TY - 1) / TY;
        byh = max(byl, (a.y0 + a.nyi - a.ty0) / TY);
    } else {
        bxl = 0;
        bxh = (a.nxi + 31) / 32;
        byl = 0;
        byh = (a.nyi + TY - 1) / TY;
    }
}
// end of the z chunk that starts at kz0 (chunks never cross the interior's
// last plane)
__host__ __device__ inline int chunk_end(const ZArgs& a, int kz0, int kc) {
    return min(kz0 + kc, kz0 < a.nzi ? a.nzi : a.kz_end);
}

// The shell tiles of a sweep over the shell too, for chunks of kc planes:
// over the interior's chunks every tile outside interior_tiles (rows above,
// the left and right edge tiles of the middle rows, rows below), then every
// tile over the chunks of the planes below the interior.  Tile L of that list
// -> (bx, by, kz0); the count of the list.
__host__ __device__ inline int shell_tile_count(const ZArgs& a, int TY, int kc) {
    if (!a.sh.prof) return 0;
    int bxl, bxh, byl, byh;
    interior_tiles(a, TY, bxl, bxh, byl, byh);
    const int ntx = (a.sx + 31) / 32, nty = (a.sy + TY - 1) / TY;
    const int edge = ntx * nty - (bxh - bxl) * (byh - byl);
    const int nci = (a.nzi + kc - 1) / kc, ncz = (a.kz_end - a.nzi + kc - 1) / kc;
    return nci * edge + ncz * ntx * nty;
}
__host__ __device__ inline void shell_tile(const ZArgs& a, int TY, int kc, int L, int& bx, int& by, int& kz0) {
    int bxl, bxh, byl, byh;
    interior_tiles(a, TY, bxl, bxh, byl, byh);
    const int ntx = (a.sx + 31) / 32, nty = (a.sy + TY - 1) / TY;
    const int edge = ntx * nty - (bxh - bxl) * (byh - byl);
    const int nci = (a.nzi + kc - 1) / kc;
    if (L < nci * edge) {
        const int c = L / edge;
        int r = L - c * edge;
        kz0 = c * kc;
        const int top = byl * ntx;
        if (r < top) {
            by = r / ntx;
            bx = r - by * ntx;
            return;
        }
        r -= top;
        const int w = ntx - (bxh - bxl), mid = (byh - byl) * w;
        if (r < mid) {
            const int q = r / w, e = r - q * w;
            by = byl + q;
            bx = e < bxl ? e : bxh + (e - bxl);
            return;
        }
        r -= mid;
        by = byh + r / ntx;
        bx = r - (r / ntx) * ntx;
        return;
    }
    L -= nci * edge;
    const int c = L / (ntx * nty), r = L - c * (ntx * nty);
    kz0 = a.nzi + c * kc;
    by = r / ntx;
    bx = r - by * ntx;
}

// Start-up check of a TMA destination (128-byte boundary) and of the
// innermost box coordinate (a multiple of 16 bytes; the edge tiles of a
// sweep over the PML shell load from x < 0, which the copy fills with zeros);
// a block that fails it issues no copy at all.
__device__ __forceinline__ bool tma_ok(const void* dst, int x, int esize) {
    return (smem_u32(dst) & 127u) == 0 && ((x * esize) & 15) == 0;
}

// Position of a plane in a ring of N slots that is filled in plane order:
// the slot and the parity of the fill it belongs to.
template <int N>
struct RingPos {
    int slot;
    uint32_t par;
    __device__ __forceinline__ void advance() {
        if (++slot == N) { slot = 0; par ^= 1u; }
    }
};

// Producer bookkeeping for the bounded drain: bit s of `used` marks a slot
// that has been filled, bit s of `last` the parity of its latest fill.
struct FillLog {
    uint32_t used = 0, last = 0;
    __device__ __forceinline__ void note(int s, uint32_t par) {
        used |= 1u << s;
        last = (last & ~(1u << s)) | (par << s);
    }
    __device__ __forceinline__ void drain(uint64_t* bars, int n) const {
        for (int s = 0; s < n; ++s)
            if (used & (1u << s)) mbar_wait(&bars[s], (last >> s) & 1u);
    }
};

// Column (ix, jy) of a tile: interior, PML shell (inside the grid, outside
// the interior box; only when the tile kernels sweep the shell) or neither,
// and the shell box holding its ADE storage (box 4, the z layer below the
// interior, for an interior column).
struct ShellCol {
    bool interior, shell;
    int box;
};
__device__ __forceinline__ ShellCol shell_col(const ZArgs& a, int ix, int jy) {
    ShellCol c;
    const bool inx = ix >= a.x0 && ix < a.x0 + a.nxi, iny = jy >= a.y0 && jy < a.y0 + a.nyi;
    c.interior = inx && iny;
    c.shell = a.sh.prof != nullptr && !c.interior && ix >= 0 && ix < a.g.nx && jy >= 0 && jy < a.g.ny;
    c.box = ix < a.x0 ? 0 : ix >= a.x0 + a.nxi ? 1 : jy < a.y0 ? 2 : jy >= a.y0 + a.nyi ? 3 : 4;
    return c;
}

// ---------------------------------------------------------------------------
// Interior stress update (m_kernel.f90:142-348), TMA pipeline.
//   R+S ring: 2 planes (k, k+1 in flight)
//   M ring:   3 planes (k, k+1 for mu(k+1), k+2 in flight)
//   V ring:   6 planes (k-2 .. k+2 for the z stencil, k+3 in flight)
// ---------------------------------------------------------------------------
// One 32 x TY column tile (bx, by) of the sweep grid and the z chunk that
// starts at plane kz0, of one simulation; `ta` lives in kernel parameter
// space (single simulation) or in global memory (batched launch).  SHELL:
// the tile may hold PML shell points (shell-tile kernels), updated as in the
// shell launches from the same staged planes, with their auxiliaries staged
// one plane ahead.
// Returns whether the block initialised its mbarriers (a caller that reuses
// the shared memory for other work invalidates them first).
template <class RT, int TY = TTY, bool SHELL = false>
__device__ __forceinline__ bool stress_tma_tile(const TArgs& ta, const int bx, const int by, const int kz0) {
    extern __shared__ __align__(128) unsigned char smraw[];
    StressSm<RT, TY, SHELL>& sm = *reinterpret_cast<StressSm<RT, TY, SHELL>*>(smraw);
    int& bad = sm.bad;
    const ZArgs& a = ta.z;
    const Coef cf = a.c;
    const Geo& g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int xt = a.tx0 + bx * 32, yt = a.ty0 + by * TY;
    const int ix = xt + tx, jy = yt + ty;
    const ShellCol sc = shell_col(a, ix, jy);
    const bool act = sc.interior;
    const int kz1 = chunk_end(a, kz0, a.kchunk);
    if (kz0 >= kz1 || kz0 < 0) return false;

    constexpr uint32_t BR = sizeof(RT) * TY * 18 * 32, BS = 4 * TY * 6 * 32;
    constexpr uint32_t BM = 4 * (TY + 1) * 4 * 36, BV = 4 * (TY + 4) * 3 * 40;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) mbar_init(&sm.barRS[s], 1);
        for (int s = 0; s < 3; ++s) mbar_init(&sm.barM[s], 1);
        for (int s = 0; s < 6; ++s) mbar_init(&sm.barV[s], 1);
        fence_barrier_init();
        bad = 0;
    }
    const int gxS = xt + g.hx, gyS = yt + HYT;
    if (tid == 0) {
        bool ok = true;
        for (int s = 0; s < 2; ++s) ok &= tma_ok(&sm.R[s], xt - a.x0, (int)sizeof(RT)) && tma_ok(&sm.S[s], gxS, 4);
        for (int s = 0; s < 3; ++s) ok &= tma_ok(&sm.M[s], gxS, 4);
        for (int s = 0; s < 6; ++s) ok &= tma_ok(&sm.V[s], gxS - 4, 4);
        if (!ok) { bad = 1; atomicExch(ta.err, 2); }
    }
    __syncthreads();
    if (bad) return true;

    // producer (thread 0): next plane and ring position of every stream
    int nRS = kz0, nM = kz0, nV = kz0 - 2;
    RingPos<2> pRS{0, 0u};
    RingPos<3> pM{0, 0u};
    RingPos<6> pV{0, 0u};
    FillLog lRS, lM, lV;
    auto issueRS = [&]() {
        const int s = pRS.slot;
        mbar_expect_tx(&sm.barRS[s], BR + BS);
        tma_load_4d(&sm.R[s], &ta.tmR, &sm.barRS[s], xt - a.x0, 0, yt - a.y0, nRS);
        tma_load_4d(&sm.S[s], &ta.tmS, &sm.barRS[s], gxS, 0, gyS, nRS + HZT);
        lRS.note(s, pRS.par);
        pRS.advance();
        ++nRS;
    };
    auto issueM = [&]() {
        const int s = pM.slot;
        mbar_expect_tx(&sm.barM[s], BM);
        tma_load_4d(&sm.M[s], &ta.tmM, &sm.barM[s], gxS, 1, gyS, nM + HZT);
        lM.note(s, pM.par);
        pM.advance();
        ++nM;
    };
    auto issueV = [&]() {
        const int s = pV.slot;
        mbar_expect_tx(&sm.barV[s], BV);
        tma_load_4d(&sm.V[s], &ta.tmV, &sm.barV[s], gxS - 4, 0, gyS - 2, nV + HZT);
        lV.note(s, pV.par);
        pV.advance();
        ++nV;
    };
    if (tid == 0) {
        while (nRS <= min(kz0 + 1, kz1 - 1)) issueRS();
        while (nM <= min(kz0 + 2, kz1)) issueM();
        while (nV <= min(kz0 + 3, kz1 + 1)) issueV();
    }

    int4 band = make_int4(0, -1, 0, -1);
    if (act) band = a.band[(size_t)(jy - a.y0) * a.nxi + (ix - a.x0)];
    const float dt = cf.dt;
    const float eps = 1.1920928955078125e-07f;
    const long long planeS = 6LL * g.pitch * g.nyp;
    const long long bS = (long long)goff(g, 6, 0, ix, jy, 0);
    const long long rrow = 18LL * a.rpitch, rplane = rrow * a.nyi;
    const long long bR = (long long)(jy - a.y0) * rrow + (ix - a.x0);
    float* __restrict__ Sg = a.S;
    RT* __restrict__ Rg = (RT*)a.R;
    const int P = g.pitch;

    // shell point of this thread in the chunk (a chunk never crosses the
    // interior's last plane, so a thread is a shell point on every plane of
    // its chunk or on none): ADE column, damped flags, auxiliaries of the
    // first plane staged
    const bool shl = SHELL && (sc.shell || (act && kz0 >= a.nzi));
    const float* Ab = nullptr;
    long long aqs = 0, apl = 0;
    int az0 = 0, fxy = 0;
    if constexpr (SHELL) {
        if (shl) {
            const PmlBox& B = a.sh.box[sc.box];
            Ab = a.sh.adeV + B.off + (long long)(jy - B.y0) * B.pitch + (ix - B.x0);
            aqs = B.qs;
            apl = (long long)B.ny * B.pitch;
            az0 = B.z0;
            fxy = damped_bit(a.sh, 0, ix) | damped_bit(a.sh, 1, ix) | damped_bit(a.sh, 2, jy) | damped_bit(a.sh, 3, jy);
            stage_aux<false, TY>(sm.aux, tid, Ab + (kz0 - az0) * apl, aqs,
                                 fxy | damped_bit(a.sh, 4, kz0) | damped_bit(a.sh, 5, kz0));
        }
    }

    // consumer ring positions: R+S of plane k, M of plane k+1, V of plane k+2;
    // the slots of M(k) and of V(k-2 .. k+1) ride along
    RingPos<2> cRS{0, 0u};
    RingPos<3> cM1{1, 0u};
    RingPos<6> cV2{4, 0u};
    int sM0 = 0, sV[5] = {0, 1, 2, 3, 4};
    bool ok = mbar_wait(&sm.barM[0], 0u);
    for (int q = 0; q < 4; ++q) ok &= mbar_wait(&sm.barV[q], 0u);

    for (int k = kz0; k < kz1; ++k) {
        ok &= mbar_wait(&sm.barRS[cRS.slot], cRS.par);
        ok &= mbar_wait(&sm.barM[cM1.slot], cM1.par);
        ok &= mbar_wait(&sm.barV[cV2.slot], cV2.par);
        if (!ok) bad = 1;
        const int sRS = cRS.slot, sM1 = cM1.slot;
        sV[4] = cV2.slot;
        const int lx = tx + 4, ly = ty + 2;
        if (act && !shl && ok) {
            const int kk = k + 1;
            const bool nb = in_band(kk, band);
            const float e40x = nb ? cf.e2x : cf.e4x0, e41x = nb ? 0.f : cf.e4x1;
            const float e40y = nb ? cf.e2y : cf.e4y0, e41y = nb ? 0.f : cf.e4y1;
            const float e40z = nb ? cf.e2z : cf.e4z0, e41z = nb ? 0.f : cf.e4z1;
            // V(k) plane tile: [y][c][x]
            float (*Vk)[3][40] = sm.V[sV[2]].d;
            auto X = [&](int dy, int dx) { return Vk[ly + dy][0][lx + dx]; };
            auto Y = [&](int dy, int dx) { return Vk[ly + dy][1][lx + dx]; };
            auto Z = [&](int dy, int dx) { return Vk[ly + dy][2][lx + dx]; };
            auto zc = [&](int d, int c) { return sm.V[sV[d + 2]].d[ly][c][lx]; };  // own column at plane k+d

            const float dxVx = (X(0, 0) - X(0, -1)) * e40x - (X(0, 1) - X(0, -2)) * e41x;
            const float dyVy = (Y(0, 0) - Y(-1, 0)) * e40y - (Y(1, 0) - Y(-2, 0)) * e41y;
            const float dzVz = (zc(0, 2) - zc(-1, 2)) * e40z - (zc(1, 2) - zc(-2, 2)) * e41z;
            const float dxVy_dyVx = (Y(0, 1) - Y(0, 0)) * e40x - (Y(0, 2) - Y(0, -1)) * e41x
                                  + (X(1, 0) - X(0, 0)) * e40y - (X(2, 0) - X(-1, 0)) * e41y;
            const float dxVz_dzVx = (Z(0, 1) - Z(0, 0)) * e40x - (Z(0, 2) - Z(0, -1)) * e41x
                                  + (zc(1, 0) - zc(0, 0)) * e40z - (zc(2, 0) - zc(-1, 0)) * e41z;
            const float dyVz_dzVy = (Z(1, 0) - Z(0, 0)) * e40y - (Z(2, 0) - Z(-1, 0)) * e41y
                                  + (zc(1, 1) - zc(0, 1)) * e40z - (zc(2, 1) - zc(-1, 1)) * e41z;

            float (*M0)[4][36] = sm.M[sM0].d;
            float (*M1)[4][36] = sm.M[sM1].d;
            const float lam = M0[ty][0][tx], tp = M0[ty][2][tx], ts = M0[ty][3][tx];
            const float m000 = M0[ty][1][tx], m100 = M1[ty][1][tx];
            const float m010 = M0[ty][1][tx + 1], m110 = M1[ty][1][tx + 1];
            const float m001 = M0[ty + 1][1][tx], m101 = M1[ty + 1][1][tx];
            const float m011 = M0[ty + 1][1][tx + 1];

            float r[18];
#pragma unroll
            for (int f = 0; f < 18; ++f) r[f] = St<RT>::ld(&sm.R[sRS].d[ty][f][tx]);
            float (*Sk)[32] = sm.S[sRS].d[ty];
            float sxx = Sk[0][tx], syy = Sk[1][tx], szz = Sk[2][tx], syz = Sk[3][tx], sxz = Sk[4][tx], sxy = Sk[5][tx];

            const float mu2 = 2.f * m000, lam2mu = lam + mu2;
            const float d3v3 = dxVx + dyVy + dzVz;
            const float sx = dyVy + dzVz, sy = dxVx + dzVz, sz = dxVx + dyVy;
            const float A = lam2mu * tp * d3v3;
            const float Bx = A - mu2 * ts * sx, By = A - mu2 * ts * sy, Bz = A - mu2 * ts * sz;
            float rxn = 0.f, ryn = 0.f, rzn = 0.f;
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                r[m] = cf.c1[m] * r[m] - cf.c2[m] * Bx * dt;
                r[3 + m] = cf.c1[m] * r[3 + m] - cf.c2[m] * By * dt;
                r[6 + m] = cf.c1[m] * r[6 + m] - cf.c2[m] * Bz * dt;
                rxn += cf.d1[m] * r[m];
                ryn += cf.d1[m] * r[3 + m];
                rzn += cf.d1[m] * r[6 + m];
            }
            const float tp1 = 1.f + tp * (1.f + cf.d2), ts1 = 1.f + ts * (1.f + cf.d2);
            const float P2 = lam2mu * tp1 * d3v3;
            sxx += (P2 - mu2 * ts1 * sx + rxn) * dt;
            syy += (P2 - mu2 * ts1 * sy + ryn) * dt;
            szz += (P2 - mu2 * ts1 * sz + rzn) * dt;
            const float muxz = 4.f * m000 * m100 * m010 * m110 /
                               (m000 * m100 * m010 + m000 * m100 * m110 + m000 * m010 * m110 + m100 * m010 * m110 + eps);
            const float muxy = 4.f * m000 * m010 * m001 * m011 /
                               (m000 * m010 * m001 + m000 * m010 * m011 + m000 * m001 * m011 + m010 * m001 * m011 + eps);
            const float muyz = 4.f * m000 * m100 * m001 * m101 /
                               (m000 * m100 * m001 + m000 * m100 * m101 + m000 * m001 * m101 + m100 * m001 * m101 + eps);
            float ryzn = 0.f, rxzn = 0.f, rxyn = 0.f;
            const float qyz = muyz * ts * dyVz_dzVy, qxz = muxz * ts * dxVz_dzVx, qxy = muxy * ts * dxVy_dyVx;
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                r[9 + m] = cf.c1[m] * r[9 + m] - cf.c2[m] * qyz * dt;
                r[12 + m] = cf.c1[m] * r[12 + m] - cf.c2[m] * qxz * dt;
                r[15 + m] = cf.c1[m] * r[15 + m] - cf.c2[m] * qxy * dt;
                ryzn += cf.d1[m] * r[9 + m];
                rxzn += cf.d1[m] * r[12 + m];
                rxyn += cf.d1[m] * r[15 + m];
            }
            syz += (muyz * ts1 * dyVz_dzVy + ryzn) * dt;
            sxz += (muxz * ts1 * dxVz_dzVx + rxzn) * dt;
            sxy += (muxy * ts1 * dxVy_dyVx + rxyn) * dt;
            if (a.cer) {  // Cerjan sponge epilogue (m_absorb_c.f90:113-168)
                const float gxc = a.cer[a.cer_off[0] + ix], gxb = a.cer[a.cer_off[1] + ix];
                const float gyc = a.cer[a.cer_off[2] + jy], gyb = a.cer[a.cer_off[3] + jy];
                const float gzc = a.cer[a.cer_off[4] + k], gzb = a.cer[a.cer_off[5] + k];
                const float gcc = gxc * gyc * gzc;
                sxx *= gcc; syy *= gcc; szz *= gcc;
                syz = syz * gxc * gyb * gzb;
                sxz = sxz * gxb * gyc * gzb;
                sxy = sxy * gxb * gyb * gzc;
            }
            const long long oS = bS + k * planeS;
            Sg[oS] = sxx; Sg[oS + P] = syy; Sg[oS + 2 * P] = szz;
            Sg[oS + 3 * P] = syz; Sg[oS + 4 * P] = sxz; Sg[oS + 5 * P] = sxy;
            const long long oR = bR + k * rplane;
#pragma unroll
            for (int f = 0; f < 18; ++f) St<RT>::st(Rg + oR + (long long)f * a.rpitch, r[f]);
        }
        if constexpr (SHELL) {
            if (shl && ok) {
                // PML shell point (m_absorb_p.f90:429-531): the same
                // explicitly rounded update as the shell launches, from the
                // staged tiles and auxiliaries
                const PmlShell& sh = a.sh;
                PmlSIn L;
                L.S = Sg + bS + k * planeS;
                L.P = P;
                L.A = const_cast<float*>(Ab) + (k - az0) * apl;
                L.AP = (int)aqs;
                L.gxc = ld4(sh.prof + sh.pxc + 4 * ix); L.gxe = ld4(sh.prof + sh.pxe + 4 * ix);
                L.gyc = ld4(sh.prof + sh.pyc + 4 * jy); L.gye = ld4(sh.prof + sh.pye + 4 * jy);
                L.gzc = ld4(sh.prof + sh.pzc + 4 * k); L.gze = ld4(sh.prof + sh.pze + 4 * k);
                float (*Vk)[3][40] = sm.V[sV[2]].d;
                L.vx = Vk[ly][0][lx]; L.vy = Vk[ly][1][lx]; L.vz = Vk[ly][2][lx];
                L.vxw = Vk[ly][0][lx - 1]; L.vys = Vk[ly - 1][1][lx]; L.vzu = sm.V[sV[1]].d[ly][2][lx];
                L.vye = Vk[ly][1][lx + 1]; L.vze = Vk[ly][2][lx + 1];
                L.vxn = Vk[ly + 1][0][lx]; L.vzn = Vk[ly + 1][2][lx];
                L.vxd = sm.V[sV[3]].d[ly][0][lx]; L.vyd = sm.V[sV[3]].d[ly][1][lx];
                float (*M0)[4][36] = sm.M[sM0].d;
                float (*M1)[4][36] = sm.M[sM1].d;
                L.lamv = M0[ty][0][tx]; L.m000 = M0[ty][1][tx];
                L.muxz = pml_hmean(L.m000, M1[ty][1][tx], M0[ty][1][tx + 1], M1[ty][1][tx + 1]);
                L.muxy = pml_hmean(L.m000, M0[ty][1][tx + 1], M0[ty + 1][1][tx], M0[ty + 1][1][tx + 1]);
                L.muyz = pml_hmean(L.m000, M1[ty][1][tx], M0[ty + 1][1][tx], M1[ty + 1][1][tx]);
#pragma unroll
                for (int q = 0; q < 6; ++q) L.sv[q] = sm.S[sRS].d[ty][q][tx];
                cp_async_wait_all();
#pragma unroll
                for (int q = 0; q < 9; ++q) L.ad[q] = sm.aux.a[q][tid];
                stress_pml_store(sh, L);
                // the stores above used every staged word: refill for k + 1
                if (k + 1 < kz1)
                    stage_aux<false, TY>(sm.aux, tid, Ab + (k + 1 - az0) * apl, aqs,
                                         fxy | damped_bit(sh, 4, k + 1) | damped_bit(sh, 5, k + 1));
            }
        }
        __syncthreads();  // every thread is done with R/S(k), M(k), V(k-2)
        if (bad) break;
        if (tid == 0) {
            fence_proxy_async();
            if (nRS <= kz1 - 1) issueRS();
            if (nM <= kz1) issueM();
            if (nV <= kz1 + 1) issueV();
        }
        cRS.advance();
        sM0 = sM1;
        cM1.advance();
        for (int q = 0; q < 4; ++q) sV[q] = sV[q + 1];
        cV2.advance();
    }
    if constexpr (SHELL) cp_async_wait_all();  // no staged copy outlives the block
    if (bad && tid == 0) {
        atomicExch(ta.err, 1);
        // drain this block's copies still in flight (bounded)
        lRS.drain(sm.barRS, 2);
        lM.drain(sm.barM, 3);
        lV.drain(sm.barV, 6);
    }
    return true;
}

// PML shell point of the velocity tile (m_absorb_p.f90:246-317): the
// operations of the shell launches, one component at a time, from the
// staged plane k (Sk), the point's Sxz, Syz at k - 1 and Szz at k + 1, and
// its staged auxiliaries aux[q * stride] (ADE address A, stride AP).
__device__ __forceinline__ void vel_shell_point(const PmlShell& sh, int ix, int jy, int k, int tx, int ty,
                                             float (*Sk)[6][40], float sxz_u, float syz_u, float szz_d,
                                             float (*R0)[36], float (*R1)[36], float (*Vk)[3][32], float* Vo, int P,
                                             const float* aux, int stride, float* A, long long AP) {
    const int lx = tx + 4, ly = ty + 2;
    const float r0 = R0[ty][tx];
    const float4 gxc = ld4(sh.prof + sh.pxc + 4 * ix), gyc = ld4(sh.prof + sh.pyc + 4 * jy);
    const float4 gzc = ld4(sh.prof + sh.pzc + 4 * k);
    {
        const float4 gxe = ld4(sh.prof + sh.pxe + 4 * ix);
        const float dxSxx = __fmul_rn(__fsub_rn(Sk[ly][0][lx + 1], Sk[ly][0][lx]), sh.r20x);
        const float dySxy = __fmul_rn(__fsub_rn(Sk[ly][5][lx], Sk[ly - 1][5][lx]), sh.r20y);
        const float dzSxz = __fmul_rn(__fsub_rn(Sk[ly][4][lx], sxz_u), sh.r20z);
        const float b = __fdiv_rn(2.f, __fadd_rn(r0, R0[ty][tx + 1]));
        vel_pml_component(sh.dt, gxe, dxSxx, gyc, dySxy, gzc, dzSxz, aux[0], aux[stride], aux[2 * stride], A, AP, 0,
                          1, 2, b, Vk[ty][0][tx], Vo);
    }
    {
        const float4 gye = ld4(sh.prof + sh.pye + 4 * jy);
        const float dxSxy = __fmul_rn(__fsub_rn(Sk[ly][5][lx], Sk[ly][5][lx - 1]), sh.r20x);
        const float dySyy = __fmul_rn(__fsub_rn(Sk[ly + 1][1][lx], Sk[ly][1][lx]), sh.r20y);
        const float dzSyz = __fmul_rn(__fsub_rn(Sk[ly][3][lx], syz_u), sh.r20z);
        const float b = __fdiv_rn(2.f, __fadd_rn(r0, R0[ty + 1][tx]));
        vel_pml_component(sh.dt, gxc, dxSxy, gye, dySyy, gzc, dzSyz, aux[3 * stride], aux[4 * stride],
                          aux[5 * stride], A, AP, 3, 4, 5, b, Vk[ty][1][tx], Vo + P);
    }
    {
        const float4 gze = ld4(sh.prof + sh.pze + 4 * k);
        const float dxSxz = __fmul_rn(__fsub_rn(Sk[ly][4][lx], Sk[ly][4][lx - 1]), sh.r20x);
        const float dySyz = __fmul_rn(__fsub_rn(Sk[ly][3][lx], Sk[ly - 1][3][lx]), sh.r20y);
        const float dzSzz = __fmul_rn(__fsub_rn(szz_d, Sk[ly][2][lx]), sh.r20z);
        const float b = __fdiv_rn(2.f, __fadd_rn(r0, R1[ty][tx]));
        vel_pml_component(sh.dt, gxc, dxSxz, gyc, dySyz, gze, dzSzz, aux[6 * stride], aux[7 * stride],
                          aux[8 * stride], A, AP, 6, 7, 8, b, Vk[ty][2][tx], Vo + 2 * P);
    }
}

// ---------------------------------------------------------------------------
// Interior velocity update (m_kernel.f90:75-140), TMA pipeline.
//   S ring:   VRING planes (k .. k+2 live, k+3 .. k+VRING-1 in flight; the
//             start-up planes k-2, k-1 only seed the register z columns)
//   rho ring: 3 planes (k, k+1, k+2 in flight)
//   V ring:   4 planes (k, k+1 .. k+3 in flight)
// ---------------------------------------------------------------------------
template <int TY = TTY, bool SHELL = false>
__device__ __forceinline__ bool vel_tma_tile(const TArgs& ta, const int bx, const int by, const int kz0) {
    extern __shared__ __align__(128) unsigned char smraw[];
    VelSm<TY, SHELL>& sm = *reinterpret_cast<VelSm<TY, SHELL>*>(smraw);
    int& bad = sm.bad;
    const ZArgs& a = ta.z;
    const Coef cf = a.c;
    const Geo& g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int xt = a.tx0 + bx * 32, yt = a.ty0 + by * TY;
    const int ix = xt + tx, jy = yt + ty;
    const ShellCol sc = shell_col(a, ix, jy);
    const bool act = sc.interior;
    const int kz1 = chunk_end(a, kz0, a.kchunk_v);
    if (kz0 >= kz1 || kz0 < 0) return false;

    constexpr uint32_t BSH = 4 * (TY + 4) * 6 * 40, BRHO = 4 * (TY + 1) * 36, BVC = 4 * TY * 3 * 32;
    if (tid == 0) {
        for (int s = 0; s < VRING; ++s) mbar_init(&sm.barS[s], 1);
        for (int s = 0; s < 3; ++s) mbar_init(&sm.barM[s], 1);
        for (int s = 0; s < 4; ++s) mbar_init(&sm.barV[s], 1);
        fence_barrier_init();
        bad = 0;
    }
    const int gx = xt + g.hx, gy = yt + HYT;
    if (tid == 0) {
        bool ok = true;
        for (int s = 0; s < VRING; ++s) ok &= tma_ok(&sm.S[s], gx - 4, 4);
        for (int s = 0; s < 3; ++s) ok &= tma_ok(&sm.M[s], gx, 4);
        for (int s = 0; s < 4; ++s) ok &= tma_ok(&sm.V[s], gx, 4);
        if (!ok) { bad = 1; atomicExch(ta.err, 2); }
    }
    __syncthreads();
    if (bad) return true;

    int nS = kz0 - 2, nM = kz0, nV = kz0;
    RingPos<VRING> pS{0, 0u};
    RingPos<3> pM{0, 0u};
    RingPos<4> pV{0, 0u};
    FillLog lS, lM, lV;
    auto issueS = [&]() {
        const int s = pS.slot;
        mbar_expect_tx(&sm.barS[s], BSH);
        tma_load_4d(&sm.S[s], &ta.tmSh, &sm.barS[s], gx - 4, 0, gy - 2, nS + HZT);
        lS.note(s, pS.par);
        pS.advance();
        ++nS;
    };
    auto issueM = [&]() {
        const int s = pM.slot;
        mbar_expect_tx(&sm.barM[s], BRHO);
        tma_load_4d(&sm.M[s], &ta.tmRho, &sm.barM[s], gx, 0, gy, nM + HZT);
        lM.note(s, pM.par);
        pM.advance();
        ++nM;
    };
    auto issueV = [&]() {
        const int s = pV.slot;
        mbar_expect_tx(&sm.barV[s], BVC);
        tma_load_4d(&sm.V[s], &ta.tmVc, &sm.barV[s], gx, 0, gy, nV + HZT);
        lV.note(s, pV.par);
        pV.advance();
        ++nV;
    };
    if (tid == 0) {
        // every slot: planes kz0-2 .. kz0+VRING-3
        while (nS <= min(kz0 + VRING - 3, kz1 + 1)) issueS();
        while (nM <= min(kz0 + 2, kz1)) issueM();
        while (nV <= min(kz0 + 3, kz1 - 1)) issueV();
    }

    int4 band = make_int4(0, -1, 0, -1);
    if (act) band = a.band[(size_t)(jy - a.y0) * a.nxi + (ix - a.x0)];
    const float dt = cf.dt;
    const long long planeV = 3LL * g.pitch * g.nyp;
    const long long bV = (long long)goff(g, 3, 0, ix, jy, 0);
    float* __restrict__ Vg = a.V;
    const int P = g.pitch;

    // shell point of this thread in the chunk, as in the stress tile
    const bool shl = SHELL && (sc.shell || (act && kz0 >= a.nzi));
    float* Ab = nullptr;
    long long aqs = 0, apl = 0;
    int az0 = 0, fxy = 0;
    if constexpr (SHELL) {
        if (shl) {
            const PmlBox& B = a.sh.box[sc.box];
            Ab = a.sh.adeS + B.off + (long long)(jy - B.y0) * B.pitch + (ix - B.x0);
            aqs = B.qs;
            apl = (long long)B.ny * B.pitch;
            az0 = B.z0;
            fxy = damped_bit(a.sh, 0, ix) | damped_bit(a.sh, 1, ix) | damped_bit(a.sh, 2, jy) | damped_bit(a.sh, 3, jy);
            stage_aux<true, TY>(sm.aux, tid, Ab + (kz0 - az0) * apl, aqs,
                                fxy | damped_bit(a.sh, 4, kz0) | damped_bit(a.sh, 5, kz0));
        }
    }

    // consumer positions: S of plane k+2 (slots of k-2 .. k+1 ride along),
    // rho of plane k+1 (slot of rho(k) rides along), V of plane k
    RingPos<VRING> cS2{4, 0u};
    RingPos<3> cM1{1, 0u};
    RingPos<4> cV{0, 0u};
    int sS[5] = {0, 1, 2, 3, 4}, sM0 = 0;
    bool ok = mbar_wait(&sm.barM[0], 0u);
    for (int q = 0; q < 4; ++q) ok &= mbar_wait(&sm.barS[q], 0u);
    const int lx = tx + 4, ly = ty + 2;
    // z stencil columns rolled in registers: Sxz and Syz of planes k-2..k+1,
    // Szz of planes k-1..k+2 (slots 0..3 hold planes kz0-2..kz0+1)
    float cxz[4], cyz[4], czz[4];
    for (int q = 0; q < 4; ++q) {
        cxz[q] = sm.S[q].d[ly][4][lx];
        cyz[q] = sm.S[q].d[ly][3][lx];
    }
    for (int q = 0; q < 3; ++q) czz[q] = sm.S[q + 1].d[ly][2][lx];
    // planes kz0-2 and kz0-1 only seeded the columns: refill their slots
    // (unless a start-up wait ran out, when a copy may still be landing)
    const bool all_ok = __syncthreads_and(ok);
    if (tid == 0) {
        if (!all_ok) {
            bad = 1;
        } else {
            fence_proxy_async();
            for (int q = 0; q < 2; ++q)
                if (nS <= kz1 + 1) issueS();
        }
    }

    for (int k = kz0; k < kz1; ++k) {
        ok &= mbar_wait(&sm.barS[cS2.slot], cS2.par);
        ok &= mbar_wait(&sm.barM[cM1.slot], cM1.par);
        ok &= mbar_wait(&sm.barV[cV.slot], cV.par);
        if (!ok) bad = 1;
        sS[4] = cS2.slot;
        const int sM1 = cM1.slot;
        czz[3] = sm.S[sS[4]].d[ly][2][lx];
        if (act && !shl && ok) {
            const int kk = k + 1;
            const bool nb = in_band(kk, band);
            const float e40x = nb ? cf.e2x : cf.e4x0, e41x = nb ? 0.f : cf.e4x1;
            const float e40y = nb ? cf.e2y : cf.e4y0, e41y = nb ? 0.f : cf.e4y1;
            const float e40z = nb ? cf.e2z : cf.e4z0, e41z = nb ? 0.f : cf.e4z1;
            float (*Sk)[6][40] = sm.S[sS[2]].d;
            // plane-k tile fields: 0 Sxx 1 Syy 2 Szz 3 Syz 4 Sxz 5 Sxy
            auto T = [&](int f, int dy, int dx) { return Sk[ly + dy][f][lx + dx]; };
            const float d3Sx3 = (T(0, 0, 1) - T(0, 0, 0)) * e40x - (T(0, 0, 2) - T(0, 0, -1)) * e41x
                              + (T(5, 0, 0) - T(5, -1, 0)) * e40y - (T(5, 1, 0) - T(5, -2, 0)) * e41y
                              + (cxz[2] - cxz[1]) * e40z - (cxz[3] - cxz[0]) * e41z;
            const float d3Sy3 = (T(5, 0, 0) - T(5, 0, -1)) * e40x - (T(5, 0, 1) - T(5, 0, -2)) * e41x
                              + (T(1, 1, 0) - T(1, 0, 0)) * e40y - (T(1, 2, 0) - T(1, -1, 0)) * e41y
                              + (cyz[2] - cyz[1]) * e40z - (cyz[3] - cyz[0]) * e41z;
            const float d3Sz3 = (T(4, 0, 0) - T(4, 0, -1)) * e40x - (T(4, 0, 1) - T(4, 0, -2)) * e41x
                              + (T(3, 0, 0) - T(3, -1, 0)) * e40y - (T(3, 1, 0) - T(3, -2, 0)) * e41y
                              + (czz[2] - czz[1]) * e40z - (czz[3] - czz[0]) * e41z;
            float (*R0)[36] = sm.M[sM0].d;
            float (*R1)[36] = sm.M[sM1].d;
            const float r0 = R0[ty][tx];
            float (*Vk)[3][32] = sm.V[cV.slot].d;
            // 2/(rho_a + rho_b) with the fast (approximate, 2-ulp) division
            // intrinsic: the kernel is issue-bound and the correctly rounded
            // quotient costs a Newton step and a range check per component
            // (5.8 % of the kernel's time); a 2-ulp buoyancy changes the
            // receiver traces by far less than the 1e-5 parity bar
            float vx = Vk[ty][0][tx] + __fdividef(2.f, r0 + R0[ty][tx + 1]) * d3Sx3 * dt;
            float vy = Vk[ty][1][tx] + __fdividef(2.f, r0 + R0[ty + 1][tx]) * d3Sy3 * dt;
            float vz = Vk[ty][2][tx] + __fdividef(2.f, r0 + R1[ty][tx]) * d3Sz3 * dt;
            if (a.cer) {  // Cerjan sponge epilogue (m_absorb_c.f90:170-198)
                const float gxc = a.cer[a.cer_off[0] + ix], gxb = a.cer[a.cer_off[1] + ix];
                const float gyc = a.cer[a.cer_off[2] + jy], gyb = a.cer[a.cer_off[3] + jy];
                const float gzc = a.cer[a.cer_off[4] + k], gzb = a.cer[a.cer_off[5] + k];
                vx = vx * gxb * gyc * gzc;
                vy = vy * gxc * gyb * gzc;
                vz = vz * gxc * gyc * gzb;
            }
            const long long oV = bV + k * planeV;
            Vg[oV] = vx; Vg[oV + P] = vy; Vg[oV + 2 * P] = vz;
        }
        if constexpr (SHELL) {
            if (shl && ok) {
                // the z neighbours come from the rolled columns: the slots of
                // planes below k are refilled early at the start of a chunk
                cp_async_wait_all();
                vel_shell_point(a.sh, ix, jy, k, tx, ty, sm.S[sS[2]].d, cxz[1], cyz[1], czz[2], sm.M[sM0].d,
                                sm.M[sM1].d, sm.V[cV.slot].d, Vg + bV + k * planeV, P, &sm.aux.a[0][tid], 32 * TY,
                                Ab + (k - az0) * apl, aqs);
                // every staged word went into the stores above: refill for k + 1
                if (k + 1 < kz1)
                    stage_aux<true, TY>(sm.aux, tid, Ab + (k + 1 - az0) * apl, aqs,
                                        fxy | damped_bit(a.sh, 4, k + 1) | damped_bit(a.sh, 5, k + 1));
            }
        }
        __syncthreads();  // every thread is done with S(k), rho(k), V(k)
        if (bad) break;
        if (tid == 0) {
            fence_proxy_async();
            if (nS <= kz1 + 1) issueS();
            if (nM <= kz1) issueM();
            if (nV <= kz1 - 1) issueV();
        }
        for (int q = 0; q < 4; ++q) sS[q] = sS[q + 1];
        for (int q = 0; q < 3; ++q) {
            cxz[q] = cxz[q + 1];
            cyz[q] = cyz[q + 1];
            czz[q] = czz[q + 1];
        }
        // plane k+2 (now at sS[3]) supplies the new Sxz, Syz column entries
        cxz[3] = sm.S[sS[3]].d[ly][4][lx];
        cyz[3] = sm.S[sS[3]].d[ly][3][lx];
        cS2.advance();
        sM0 = sM1;
        cM1.advance();
        cV.advance();
    }
    if constexpr (SHELL) cp_async_wait_all();  // no staged copy outlives the block
    if (bad && tid == 0) {
        atomicExch(ta.err, 1);
        lS.drain(sm.barS, VRING);
        lM.drain(sm.barM, 3);
        lV.drain(sm.barV, 4);
    }
    return true;
}

// Block order of the single-simulation stress launch (a 1-D grid): groups of
// STRESS_YGROUP tile rows; inside a group the z chunks, then the rows, then
// x.  The blocks resident at one time then cover a few neighbouring chunks
// of a band of rows, so the V planes shared by consecutive chunks and the
// halo rows shared by neighbouring tiles are still in L2 when the second
// block reads them (1024x1024x512: 15.98 -> 15.53 ms with groups of 8 rows,
// against the x-fastest order of a 3-D grid).  The velocity kernel keeps the
// plain order: grouped it was slower (4.27 -> 4.34 ms).
#ifndef STRESS_YGROUP
#define STRESS_YGROUP 8
#endif
__device__ __forceinline__ void grouped_tile(int L, int tx, int ty, int nzc, int& bx, int& by, int& bz) {
    const int full = tx * STRESS_YGROUP * nzc;  // blocks of a full group
    const int g = L / full;
    const int r = L - g * full;
    const int rows = min(STRESS_YGROUP, ty - g * STRESS_YGROUP);
    const int layer = tx * rows;                // blocks of one chunk layer of the group
    bz = r / layer;
    const int r2 = r - bz * layer;
    by = g * STRESS_YGROUP + r2 / tx;
    bx = r2 - (r2 / tx) * tx;
}
// Interior kernels: the tiles of interior_tiles over the interior's chunks
// (stress in the grouped order, velocity in a 3-D grid).
template <class RT, int TY = TTY>
__global__ void __launch_bounds__(32 * TY, TileOcc<TY>::stress) k_stress_tma(const __grid_constant__ TArgs ta) {
    const ZArgs& a = ta.z;
    int bxl, bxh, byl, byh;
    interior_tiles(a, TY, bxl, bxh, byl, byh);
    const int ntx = bxh - bxl, nty = byh - byl, ntz = (a.nzi + a.kchunk - 1) / a.kchunk;
    if ((int)blockIdx.x >= ntx * nty * ntz) return;
    int bx, by, bz;
    grouped_tile(blockIdx.x, ntx, nty, ntz, bx, by, bz);
    stress_tma_tile<RT, TY, false>(ta, bxl + bx, byl + by, bz * a.kchunk);
}
template <int TY = TTY>
__global__ void __launch_bounds__(32 * TY, TileOcc<TY>::vel) k_vel_tma(const __grid_constant__ TArgs ta) {
    int bxl, bxh, byl, byh;
    interior_tiles(ta.z, TY, bxl, bxh, byl, byh);
    vel_tma_tile<TY, false>(ta, bxl + blockIdx.x, byl + blockIdx.y, blockIdx.z * ta.z.kchunk_v);
}
// Shell-tile kernels: block b sweeps tile b of the shell_tile list.
template <class RT, int TY = TTY>
__global__ void __launch_bounds__(32 * TY, ShellOcc<TY>::stress) k_stress_tma_shell(const __grid_constant__ TArgs ta) {
    if ((int)blockIdx.x >= shell_tile_count(ta.z, TY, ta.z.kchunk)) return;
    int bx, by, kz0;
    shell_tile(ta.z, TY, ta.z.kchunk, blockIdx.x, bx, by, kz0);
    stress_tma_tile<RT, TY, true>(ta, bx, by, kz0);
}
template <int TY = TTY>
__global__ void __launch_bounds__(32 * TY, ShellOcc<TY>::vel) k_vel_tma_shell(const __grid_constant__ TArgs ta) {
    if ((int)blockIdx.x >= shell_tile_count(ta.z, TY, ta.z.kchunk_v)) return;
    int bx, by, kz0;
    shell_tile(ta.z, TY, ta.z.kchunk_v, blockIdx.x, bx, by, kz0);
    vel_tma_tile<TY, true>(ta, bx, by, kz0);
}

// Self-test of the bounded wait: an mbarrier that expects one arrival which
// never comes.  Every thread's wait gives up after WAIT_LIMIT polls and the
// block records the time-out in the error word, as the TMA kernels do.
__global__ void k_wait_selftest(int* err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    const bool ok = mbar_wait(&bar, 0u);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
}

// Batched launches: every simulation's tensor maps live in `all` (global
// memory, 128-byte aligned).
// The tables were written by host copies, so the issuing thread makes the
// tensor maps visible to the TMA unit with a system-scope tensormap-proxy
// acquire fence before the first copy.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap* m) {
    asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"((uint64_t)m) : "memory");
}
__device__ __forceinline__ void tmaps_acquire(const TArgs& t) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        tmap_acquire(&t.tmV);
        tmap_acquire(&t.tmS);
        tmap_acquire(&t.tmM);
        tmap_acquire(&t.tmR);
        tmap_acquire(&t.tmSh);
        tmap_acquire(&t.tmRho);
        tmap_acquire(&t.tmVc);
    }
}
// Batched launches: block b sweeps tile (e.y, e.z) of simulation e.x over
// the chunk that starts at plane e.w, e = blocks[b]; SHELL: the shell tiles.
template <class RT, int TY = TTY, bool SHELL = false>
__global__ void __launch_bounds__(32 * TY, SHELL ? ShellOcc<TY>::stress : TileOcc<TY>::stress)
    k_stress_tma_batch(const TArgs* __restrict__ all, const int4* __restrict__ blocks) {
    const int4 e = blocks[blockIdx.x];
    tmaps_acquire(all[e.x]);
    stress_tma_tile<RT, TY, SHELL>(all[e.x], e.y, e.z, e.w);
}
template <int TY = TTY, bool SHELL = false>
__global__ void __launch_bounds__(32 * TY, SHELL ? ShellOcc<TY>::vel : TileOcc<TY>::vel)
    k_vel_tma_batch(const TArgs* __restrict__ all, const int4* __restrict__ blocks) {
    const int4 e = blocks[blockIdx.x];
    tmaps_acquire(all[e.x]);
    vel_tma_tile<TY, SHELL>(all[e.x], e.y, e.z, e.w);
}

}  // namespace swpc
