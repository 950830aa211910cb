// persist.cuh -- one persistent fused launch per time step for a batch of
// independent simulations.
//
// Every piece of work of one time step of every member is an item of a device
// work queue: the receiver/snapshot taps, the plane-wave ghost planes, the
// interior stress tiles and PML stress blocks, the stress-glut sources, the
// interior velocity tiles and PML velocity blocks, the body forces and the
// step counter.  Resident blocks take items in queue order with one atomic
// increment, wait until the items their item depends on are finished, do the
// item and count it finished for its member.
//
// The step of one member runs in phases (main.f90:119-139):
//   0 taps, Green's-function taps, snapshots (read the previous step's fields)
//   1 plane-wave ghost planes of V
//   2 stress: interior tiles + PML blocks
//   3 stress-glut sources
//   4 plane-wave ghost planes of S
//   5 velocity: interior tiles + PML blocks
//   6 body forces
//   7 step counter
// An item of phase p of member m needs every item of member m in phases < p:
// its `need` is that count, and it waits until the member's finished counter
// reaches it.  The queue lists phase 0 of every member, then phase 1 of every
// member, and so on, so an item depends only on items earlier in the queue.
// Those were taken by blocks that are already running and that wait only on
// still earlier items, so the launch cannot deadlock whatever the number of
// resident blocks.  Every wait is bounded: after WAIT_NS nanoseconds it sets
// the error word, and once the error word is set no wait blocks again.
#pragma once
#include "kernels.cuh"
#include "kernels_tma.cuh"

namespace swpc {

enum { IT_PRE = 0, IT_PW_V = 1, IT_STRESS = 2, IT_PML_S = 3, IT_SRC_S = 4, IT_PW_S = 5, IT_VEL = 6, IT_PML_V = 7,
       IT_SRC_V = 8, IT_ADV = 9 };
constexpr int PERSIST_THREADS = 32 * TTY;  // 256: the 8-row tile kernels' block (every member uses 8-row tiles)

struct PersistArgs {
    const int4* items;  // x = type | member << 4; y, z, w: tile (bx, by, bz), PML (class, pair), chunk
    const int* need;    // items of the same member to be finished first
    int n_items;
    int* head;          // next item (0 before the launch)
    int* done;          // per member: items finished (0 before the launch)
    int* err;           // 3: a dependency wait ran out
    const TArgs* targs;
    const PArgs* pargs[PML_NCLASS];
    const SrcArgs* src;
    const TapArgs* tap;
    const SnapArgs* snap;
    const GreenArgs* green;
    int* const* its;
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s

// Bounded wait of one thread until *cnt >= need (acquire); false when it ran
// out or an earlier wait of the launch had run out.
__device__ __forceinline__ bool wait_count(const int* cnt, int need, int* err) {
    if (ld_acquire_gpu(cnt) >= need) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        __nanosleep(128);
        if (ld_acquire_gpu(cnt) >= need) return true;
        if (*(volatile int*)err != 0) return false;
        if (global_ns() - t0 > WAIT_NS) {
            atomicExch(err, 3);
            return false;
        }
    }
}

template <class RT>
__device__ __forceinline__ void inval_stress_bars() {
    extern __shared__ __align__(128) unsigned char smraw[];
    StressSmem<RT, TTY>& sm = *reinterpret_cast<StressSmem<RT, TTY>*>(smraw);
    for (int s = 0; s < 2; ++s) mbar_inval(&sm.barRS[s]);
    for (int s = 0; s < 3; ++s) mbar_inval(&sm.barM[s]);
    for (int s = 0; s < 6; ++s) mbar_inval(&sm.barV[s]);
}
__device__ __forceinline__ void inval_vel_bars() {
    extern __shared__ __align__(128) unsigned char smraw[];
    VelSmem<TTY>& sm = *reinterpret_cast<VelSmem<TTY>*>(smraw);
    for (int s = 0; s < VRING; ++s) mbar_inval(&sm.barS[s]);
    for (int s = 0; s < 3; ++s) mbar_inval(&sm.barM[s]);
    for (int s = 0; s < 4; ++s) mbar_inval(&sm.barV[s]);
}

// taps, Green's-function taps and snapshot pixels of one member, numbered one
// after the other; unit u of them
__device__ __forceinline__ void pre_unit(const PersistArgs& P, int m, int u) {
    const TapArgs& T = P.tap[m];
    if (u < T.n) { taps_one(T, u); return; }
    u -= T.n;
    const GreenArgs& G = P.green[m];
    if (u < G.n) { green_pt(G, u); return; }
    u -= G.n;
    const SnapArgs& S = P.snap[m];
    for (int q = 0; q < S.n; ++q) {
        const int np = S.pl[q].n1 * S.pl[q].n2;
        if (u < np) { snap_pix(S, S.pl[q], u); return; }
        u -= np;
    }
}

// A PML item covers PML_ITEM_BLOCKS blocks of PTPB points of one launch
// class (two blocks per pass of the 256 threads).
constexpr int PML_ITEM_BLOCKS = 16;
template <int MASK>
__device__ __forceinline__ void pml_pair(const PArgs& a, int item, int tid, bool stress) {
    for (int r = 0; r < PML_ITEM_BLOCKS / 2; ++r) {
        const int blk = item * PML_ITEM_BLOCKS + 2 * r + (tid >> 7);
        if (blk >= a.nblocks) break;
        PmlPt c;
        if (pml_point(a, blk, tid & (PTPB - 1), c)) {
            if (stress) stress_pml_at<MASK>(a, c);
            else vel_pml_at<MASK>(a, c);
        }
    }
}
__device__ __forceinline__ void pml_item(const PersistArgs& P, int m, int cls, int pair, int tid, bool stress) {
    const PArgs& a = P.pargs[cls][m];
    static_assert(PML_NCLASS == 4 && PML_CLASS_MASK[0] == 1 && PML_CLASS_MASK[1] == 2 && PML_CLASS_MASK[2] == 4,
                  "launch classes x, y, z, general");
    switch (cls) {
    case 0: pml_pair<1>(a, pair, tid, stress); break;
    case 1: pml_pair<2>(a, pair, tid, stress); break;
    case 2: pml_pair<4>(a, pair, tid, stress); break;
    default: pml_pair<7>(a, pair, tid, stress); break;
    }
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <class RT>
__global__ void __launch_bounds__(PERSIST_THREADS, 2) k_batch_persistent(const __grid_constant__ PersistArgs P) {
    static_assert(PTPB * 2 == PERSIST_THREADS, "a PML pass is two PML blocks");
    __shared__ int s_item, s_ok;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid == 0) s_item = atomicAdd(P.head, 1);
    __syncthreads();
    for (;;) {
        const int q = s_item;
        if (q >= P.n_items) break;
        // take the following item now; its index is only needed after this
        // one, so the atomic's latency hides behind the work (a block holds
        // at most one item ahead, which keeps the queue order argument:
        // the first unfinished item is always the current item of a block)
        int nxt = 0;
        if (tid == 0) nxt = atomicAdd(P.head, 1);
        const int4 it = P.items[q];
        const int type = it.x & 15, m = it.x >> 4;
        if (tid == 0) {
            const int nd = P.need[q];
            s_ok = nd <= 0 || wait_count(P.done + m, nd, P.err);
            // order this block's coming reads through the TMA unit after the
            // acquire that made the other blocks' stores visible
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
        __syncthreads();
        if (s_ok) {
            switch (type) {
            case IT_PRE: pre_unit(P, m, it.y * PERSIST_THREADS + tid); break;
            case IT_PW_V: {
                const ZArgs& z = P.targs[m].z;
                const long long u = (long long)it.y * PERSIST_THREADS + tid;
                if (u < pw_ghost_units(z.g, 3)) pw_ghost_unit(z.V, z.g, 3, u);
                break;
            }
            case IT_STRESS: {
                tmaps_acquire(P.targs[m]);
                const bool bars = stress_tma_tile<RT, TTY, false>(P.targs[m], it.y, it.z, it.w);
                __syncthreads();
                if (bars && tid == 0) inval_stress_bars<RT>();
                break;
            }
            case IT_PML_S: pml_item(P, m, it.y, it.z, tid, true); break;
            case IT_SRC_S: stressglut_one(P.src[m], it.y * PERSIST_THREADS + tid); break;
            case IT_PW_S: {
                const ZArgs& z = P.targs[m].z;
                const long long u = (long long)it.y * PERSIST_THREADS + tid;
                if (u < pw_ghost_units(z.g, 6)) pw_ghost_unit(z.S, z.g, 6, u);
                break;
            }
            case IT_VEL: {
                tmaps_acquire(P.targs[m]);
                const bool bars = vel_tma_tile<TTY, false>(P.targs[m], it.y, it.z, it.w);
                __syncthreads();
                if (bars && tid == 0) inval_vel_bars();
                break;
            }
            case IT_PML_V: pml_item(P, m, it.y, it.z, tid, false); break;
            case IT_SRC_V: bodyforce_one(P.src[m], it.y * PERSIST_THREADS + tid); break;
            default:
                if (tid == 0) *P.its[m] += 1;
                break;
            }
        }
        // make this block's stores visible to the generic and the TMA reads
        // of other blocks, then count the item finished with a release
        asm volatile("fence.proxy.async.global;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            red_release_add(P.done + m, 1);
            s_item = nxt;
        }
        __syncthreads();
    }
}

}  // namespace swpc
