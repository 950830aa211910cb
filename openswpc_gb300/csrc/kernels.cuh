// kernels.cuh -- sm_103a kernels of the swpc_3d time step.
//
// Device layout (see Geo): every 3-D quantity is a group of nf fields stored
// row-interleaved, [kz][jy][f][x], x fastest, with a padded row pitch.  One
// base address per (kz, jy) row then reaches every field of the group through
// immediate offsets f*pitch, and each warp access along x is one coalesced
// 128-byte line.  Groups: V (Vx Vy Vz), S (Sxx Syy Szz Syz Sxz Sxy), M (rho
// lam mu taup taus).  The memory variables R live only on the viscoelastic
// interior box (18 fields, [kz][jy'][f][x']); the 18 ADE auxiliaries live
// only on the five PML boxes of the absorbing shell.
//
// Ghost cells around the physical grid are zero and never written: with one
// domain the reference's halo exchange (m_global.f90:391-607) only ever
// copies zeros into them.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace swpc {

constexpr int HYT = 3;   // rows above jy = 0
constexpr int HZT = 3;   // planes above kz = 0
constexpr int TBX = 32;  // tile width (one warp)
constexpr int TBY = 8;   // tile height of the interior sweep kernels
constexpr int NM = 3;    // Zener bodies (m_global.f90:31)

struct Geo {
    int nx, ny, nz, na;
    int hx;     // left x halo, chosen so the interior box starts on a 128-byte boundary
    int pitch;  // floats per row
    int nyp;    // rows per plane
    int nzp;    // planes
};

__host__ __device__ __forceinline__ size_t goff(const Geo& g, int nf, int f, int ix, int jy, int kz) {
    return ((size_t)((kz + HZT) * g.nyp + (jy + HYT)) * nf + f) * (size_t)g.pitch + (size_t)(ix + g.hx);
}

// storage conversion for the memory variables / medium (precision form)
template <class T> struct St;
template <> struct St<float> {
    static __device__ __forceinline__ float ld(const float* p) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
};
template <> struct St<__half> {
    static __device__ __forceinline__ float ld(const __half* p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
};
template <> struct St<__nv_bfloat16> {
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
};

struct Coef {
    float e4x0, e4x1, e4y0, e4y1, e4z0, e4z1;  // 4th order: 9/8/d, 1/24/d
    float e2x, e2y, e2z;                       // 2nd order near surfaces: 1/d, 0
    float c1[NM], c2[NM], d1[NM], d2;          // Zener (m_kernel.f90:58-67)
    float dt;
};

// One box of the PML shell and its compact ADE storage (the shell's layout
// is described with the PML kernels below).
struct PmlBox {
    int x0, y0, z0, nx, ny, nz;
    int pitch;           // ADE row pitch (= nx: rows stored without padding)
    int qs;              // stride between the box's nine auxiliary arrays (nx * ny * nz)
    long long off;       // offset of this box in the ADE buffers (elements)
    long long moff;      // offset of the box's six medium arrays in the shell-medium buffer
};

// The PML shell swept by the TMA tile kernels together with the interior:
// damping profiles, ADE storage and the five boxes in a fixed order
// (x < x0, x >= x0 + nxi, y < y0, y >= y0 + nyi, z >= nzi).
struct PmlShell {
    const float* prof;  // null: the shell runs in launches of its own
    float* adeV;
    float* adeS;
    int pxc, pxe, pyc, pye, pzc, pze;
    // damped indices of the six profiles (x centre, x edge, y c, y e, z c,
    // z e): i is damped (g4 != 0) exactly when i < dlo or i >= dhi
    int dlo[6], dhi[6];
    float r20x, r20y, r20z, dt;
    PmlBox box[5];
};

// Interior (viscoelastic, 4th-order) sweep arguments.
struct ZArgs {
    Geo g;
    float* V;
    float* S;
    const float* M;
    void* R;           // memory variables, storage type per template
    const int4* band;  // per interior column: kfs_top, kfs_bot, kob_top, kob_bot (1-based k)
    int x0, y0, nxi, nyi;  // interior box (0-based origin, extent)
    int kz_end;            // planes [0, kz_end) swept by the tile kernels
    int nzi;               // interior planes [0, nzi)
    int tx0, ty0;          // origin of the tile grid (the interior's, or left of it when the shell is swept too)
    int sx, sy;            // extent of the swept box from (tx0, ty0) in x and y (tiles: ceil(sx / 32), ceil(sy / TY))
    int kchunk;            // planes per block in z (stress kernels)
    int kchunk_v;          // planes per block in z (velocity kernels)
    int rpitch;            // R row pitch (elements)
    const float* cer;      // Cerjan profiles (null for PML): xc xb yc yb zc zb, each padded
    int cer_off[6];
    Coef c;
    PmlShell sh;           // sh.prof null: interior only
};

// 2nd-order band test of m_kernel.f90:103-111 / 188-196: inside a free-surface
// or ocean-bottom band (product >= 0, Fortran sign(1,0) = +1) the stencil is
// 2nd order.
__device__ __forceinline__ bool in_band(int k, int4 b) {
    int a = (k - b.x) * (b.y - k);
    int c = (k - b.z) * (b.w - k);
    return max(a, c) >= 0;
}

// Halo cells of a (TBX+4) x (TBY+4) plane tile without its corners:
// two full rows above and below (x in [2, 34)) plus two cells left and right
// of every middle row.  Returns the tile coordinate of halo index h.
__device__ __forceinline__ void halo_xy(int h, int& lx, int& ly) {
    if (h < 4 * TBX) {
        int r = h / TBX;  // 0,1 top; 2,3 bottom
        lx = 2 + (h - r * TBX);
        ly = (r < 2) ? r : (TBY + r);
    } else {
        int q = h - 4 * TBX;
        int c = q & 3;
        ly = 2 + (q >> 2);
        lx = (c < 2) ? c : (TBX + c);
    }
}
constexpr int NHALO = 4 * TBX + 4 * TBY;

// ---------------------------------------------------------------------------
// Interior stress update: m_kernel.f90:142-348 (normal + shear fused).
// One thread per (i, j) column, sweeping z.  The x/y neighbours of V come from
// a shared-memory plane tile (double buffered), the z neighbours of the own
// column from a 4-deep register window, mu from a 3-plane shared ring.
// ---------------------------------------------------------------------------
template <class RT>
__global__ void __launch_bounds__(TBX * TBY, 2) k_stress_interior(const ZArgs a) {
    __shared__ float sV[2][3][TBY + 4][TBX + 4];
    __shared__ float sMu[3][TBY + 1][TBX + 1];

    const Geo& g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TBX + tx;
    const int xt = a.x0 + blockIdx.x * TBX, yt = a.y0 + blockIdx.y * TBY;
    const int ix = xt + tx, jy = yt + ty;
    const bool act = (ix < a.x0 + a.nxi) && (jy < a.y0 + a.nyi);
    const int kz0 = blockIdx.z * a.kchunk;
    const int kz1 = min(kz0 + a.kchunk, a.kz_end);
    if (kz0 >= kz1) return;

    const long long planeV = 3LL * g.pitch * g.nyp;
    const long long planeS = 6LL * g.pitch * g.nyp;
    const long long planeM = 5LL * g.pitch * g.nyp;
    const float* __restrict__ V = a.V;
    const float* __restrict__ M = a.M;
    float* __restrict__ S = a.S;
    RT* __restrict__ R = (RT*)a.R;
    const int P = g.pitch;

    // column base addresses at kz = 0
    const long long bV = (long long)goff(g, 3, 0, ix, jy, 0);
    const long long bS = (long long)goff(g, 6, 0, ix, jy, 0);
    const long long bM = (long long)goff(g, 5, 0, ix, jy, 0);
    const long long rrow = 18LL * a.rpitch, rplane = rrow * a.nyi;
    const long long bR = (long long)(jy - a.y0) * rrow + (ix - a.x0);

    int4 band = make_int4(0, -1, 0, -1);
    if (act) band = a.band[(size_t)(jy - a.y0) * a.nxi + (ix - a.x0)];

    // z window of the own column: vx,vy at k-1..k+2, vz at k-2..k+1
    float vx[4], vy[4], vz[4];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        vx[q + 1] = V[bV + (kz0 - 1 + q) * planeV];
        vy[q + 1] = V[bV + P + (kz0 - 1 + q) * planeV];
        vz[q + 1] = V[bV + 2 * P + (kz0 - 2 + q) * planeV];
    }

    // mu plane kz0 into ring slot 0
    int s0 = 0, s1 = 1, s2 = 2;
    for (int h = tid; h < (TBX + 1) * (TBY + 1); h += TBX * TBY) {
        int lx = h % (TBX + 1), ly = h / (TBX + 1);
        sMu[s0][ly][lx] = M[goff(g, 5, 2, xt + lx, yt + ly, kz0)];
    }

    const float dt = a.c.dt;
    const float eps = 1.1920928955078125e-07f;  // epsilon(1.0)

    for (int kz = kz0; kz < kz1; ++kz) {
        const int b = kz & 1;
        // advance the window
#pragma unroll
        for (int q = 0; q < 3; ++q) { vx[q] = vx[q + 1]; vy[q] = vy[q + 1]; vz[q] = vz[q + 1]; }
        vx[3] = V[bV + (kz + 2) * planeV];
        vy[3] = V[bV + P + (kz + 2) * planeV];
        vz[3] = V[bV + 2 * P + (kz + 1) * planeV];

        // per-point streams of this plane (issued before the barrier)
        float sxx = 0, syy = 0, szz = 0, syz = 0, sxz = 0, sxy = 0, lam = 0, tp = 0, ts = 0;
        float r[18];
        const long long oS = bS + kz * planeS, oM = bM + kz * planeM, oR = bR + kz * rplane;
        if (act) {
            sxx = S[oS]; syy = S[oS + P]; szz = S[oS + 2 * P];
            syz = S[oS + 3 * P]; sxz = S[oS + 4 * P]; sxy = S[oS + 5 * P];
            lam = M[oM + P]; tp = M[oM + 3 * P]; ts = M[oM + 4 * P];
#pragma unroll
            for (int f = 0; f < 18; ++f) r[f] = St<RT>::ld(R + oR + (long long)f * a.rpitch);
        }

        // plane tile of V (center from the window, halo from global)
        sV[b][0][ty + 2][tx + 2] = vx[1];
        sV[b][1][ty + 2][tx + 2] = vy[1];
        sV[b][2][ty + 2][tx + 2] = vz[2];
        for (int h = tid; h < 3 * NHALO; h += TBX * TBY) {
            int c = h / NHALO, lx, ly;
            halo_xy(h - c * NHALO, lx, ly);
            sV[b][c][ly][lx] = V[goff(g, 3, c, xt - 2 + lx, yt - 2 + ly, kz)];
        }
        // mu plane kz+1 into slot s1
        for (int h = tid; h < (TBX + 1) * (TBY + 1); h += TBX * TBY) {
            int lx = h % (TBX + 1), ly = h / (TBX + 1);
            sMu[s1][ly][lx] = M[goff(g, 5, 2, xt + lx, yt + ly, kz + 1)];
        }
        __syncthreads();

        if (act) {
            const int k = kz + 1;  // reference 1-based k
            const bool nb = in_band(k, band);
            const float e40x = nb ? a.c.e2x : a.c.e4x0, e41x = nb ? 0.f : a.c.e4x1;
            const float e40y = nb ? a.c.e2y : a.c.e4y0, e41y = nb ? 0.f : a.c.e4y1;
            const float e40z = nb ? a.c.e2z : a.c.e4z0, e41z = nb ? 0.f : a.c.e4z1;
            const int lx = tx + 2, ly = ty + 2;
            float (*X)[TBX + 4] = sV[b][0];
            float (*Y)[TBX + 4] = sV[b][1];
            float (*Z)[TBX + 4] = sV[b][2];

            const float dxVx = (X[ly][lx] - X[ly][lx - 1]) * e40x - (X[ly][lx + 1] - X[ly][lx - 2]) * e41x;
            const float dyVy = (Y[ly][lx] - Y[ly - 1][lx]) * e40y - (Y[ly + 1][lx] - Y[ly - 2][lx]) * e41y;
            const float dzVz = (vz[2] - vz[1]) * e40z - (vz[3] - vz[0]) * e41z;
            const float dxVy_dyVx = (Y[ly][lx + 1] - Y[ly][lx]) * e40x - (Y[ly][lx + 2] - Y[ly][lx - 1]) * e41x
                                  + (X[ly + 1][lx] - X[ly][lx]) * e40y - (X[ly + 2][lx] - X[ly - 1][lx]) * e41y;
            const float dxVz_dzVx = (Z[ly][lx + 1] - Z[ly][lx]) * e40x - (Z[ly][lx + 2] - Z[ly][lx - 1]) * e41x
                                  + (vx[2] - vx[1]) * e40z - (vx[3] - vx[0]) * e41z;
            const float dyVz_dzVy = (Z[ly + 1][lx] - Z[ly][lx]) * e40y - (Z[ly + 2][lx] - Z[ly - 1][lx]) * e41y
                                  + (vy[2] - vy[1]) * e40z - (vy[3] - vy[0]) * e41z;

            // mu at (k,k+1) x (i,i+1) x (j,j+1)
            const float m000 = sMu[s0][ty][tx], m100 = sMu[s1][ty][tx];
            const float m010 = sMu[s0][ty][tx + 1], m110 = sMu[s1][ty][tx + 1];
            const float m001 = sMu[s0][ty + 1][tx], m101 = sMu[s1][ty + 1][tx];
            const float m011 = sMu[s0][ty + 1][tx + 1];

            // normal components (m_kernel.f90:198-238)
            const float mu2 = 2.f * m000, lam2mu = lam + mu2;
            const float d3v3 = dxVx + dyVy + dzVz;
            const float sx = dyVy + dzVz, sy = dxVx + dzVz, sz = dxVx + dyVy;
            const float A = lam2mu * tp * d3v3;
            const float Bx = A - mu2 * ts * sx, By = A - mu2 * ts * sy, Bz = A - mu2 * ts * sz;
            float rxn = 0.f, ryn = 0.f, rzn = 0.f;
#pragma unroll
            for (int m = 0; m < NM; ++m) {
                r[m] = a.c.c1[m] * r[m] - a.c.c2[m] * Bx * dt;
                r[3 + m] = a.c.c1[m] * r[3 + m] - a.c.c2[m] * By * dt;
                r[6 + m] = a.c.c1[m] * r[6 + m] - a.c.c2[m] * Bz * dt;
                rxn += a.c.d1[m] * r[m];
                ryn += a.c.d1[m] * r[3 + m];
                rzn += a.c.d1[m] * r[6 + m];
            }
            const float tp1 = 1.f + tp * (1.f + a.c.d2), ts1 = 1.f + ts * (1.f + a.c.d2);
            const float P2 = lam2mu * tp1 * d3v3;
            sxx += (P2 - mu2 * ts1 * sx + rxn) * dt;
            syy += (P2 - mu2 * ts1 * sy + ryn) * dt;
            szz += (P2 - mu2 * ts1 * sz + rzn) * dt;

            // shear components with harmonic means of mu (m_kernel.f90:285-333)
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
                r[9 + m] = a.c.c1[m] * r[9 + m] - a.c.c2[m] * qyz * dt;
                r[12 + m] = a.c.c1[m] * r[12 + m] - a.c.c2[m] * qxz * dt;
                r[15 + m] = a.c.c1[m] * r[15 + m] - a.c.c2[m] * qxy * dt;
                ryzn += a.c.d1[m] * r[9 + m];
                rxzn += a.c.d1[m] * r[12 + m];
                rxyn += a.c.d1[m] * r[15 + m];
            }
            syz += (muyz * ts1 * dyVz_dzVy + ryzn) * dt;
            sxz += (muxz * ts1 * dxVz_dzVx + rxzn) * dt;
            sxy += (muxy * ts1 * dxVy_dyVx + rxyn) * dt;

            if (a.cer) {  // Cerjan sponge epilogue (m_absorb_c.f90:113-168)
                const float gxc = a.cer[a.cer_off[0] + ix], gxb = a.cer[a.cer_off[1] + ix];
                const float gyc = a.cer[a.cer_off[2] + jy], gyb = a.cer[a.cer_off[3] + jy];
                const float gzc = a.cer[a.cer_off[4] + kz], gzb = a.cer[a.cer_off[5] + kz];
                const float gcc = gxc * gyc * gzc;
                sxx *= gcc; syy *= gcc; szz *= gcc;
                syz = syz * gxc * gyb * gzb;
                sxz = sxz * gxb * gyc * gzb;
                sxy = sxy * gxb * gyb * gzc;
            }
            S[oS] = sxx; S[oS + P] = syy; S[oS + 2 * P] = szz;
            S[oS + 3 * P] = syz; S[oS + 4 * P] = sxz; S[oS + 5 * P] = sxy;
#pragma unroll
            for (int f = 0; f < 18; ++f) St<RT>::st(R + oR + (long long)f * a.rpitch, r[f]);
        }
        // rotate the mu ring: next iteration needs (kz+1, kz+2)
        int t = s0; s0 = s1; s1 = s2; s2 = t;
    }
}

// ---------------------------------------------------------------------------
// Interior velocity update: m_kernel.f90:75-140.
// Plane tile in shared memory: Sxx Syy Sxy Sxz Syz rho (x/y neighbours);
// register window for Szz (k-1..k+2), Sxz, Syz (k-2..k+1), rho (k, k+1).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TBX * TBY, 2) k_vel_interior(const ZArgs a) {
    __shared__ float sT[2][6][TBY + 4][TBX + 4];
    const Geo& g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TBX + tx;
    const int xt = a.x0 + blockIdx.x * TBX, yt = a.y0 + blockIdx.y * TBY;
    const int ix = xt + tx, jy = yt + ty;
    const bool act = (ix < a.x0 + a.nxi) && (jy < a.y0 + a.nyi);
    const int kz0 = blockIdx.z * a.kchunk_v;
    const int kz1 = min(kz0 + a.kchunk_v, a.kz_end);
    if (kz0 >= kz1) return;

    const long long planeV = 3LL * g.pitch * g.nyp;
    const long long planeS = 6LL * g.pitch * g.nyp;
    const long long planeM = 5LL * g.pitch * g.nyp;
    float* __restrict__ V = a.V;
    const float* __restrict__ S = a.S;
    const float* __restrict__ M = a.M;
    const int P = g.pitch;
    const long long bV = (long long)goff(g, 3, 0, ix, jy, 0);
    const long long bS = (long long)goff(g, 6, 0, ix, jy, 0);
    const long long bM = (long long)goff(g, 5, 0, ix, jy, 0);

    int4 band = make_int4(0, -1, 0, -1);
    if (act) band = a.band[(size_t)(jy - a.y0) * a.nxi + (ix - a.x0)];

    float wzz[4], wxz[4], wyz[4], wr[2];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        wzz[q + 1] = S[bS + 2 * P + (kz0 - 1 + q) * planeS];
        wxz[q + 1] = S[bS + 4 * P + (kz0 - 2 + q) * planeS];
        wyz[q + 1] = S[bS + 3 * P + (kz0 - 2 + q) * planeS];
    }
    wr[1] = M[bM + kz0 * planeM];
    const float dt = a.c.dt;
    // shared tile component -> (group, field) for halo loads
    for (int kz = kz0; kz < kz1; ++kz) {
        const int b = kz & 1;
#pragma unroll
        for (int q = 0; q < 3; ++q) { wzz[q] = wzz[q + 1]; wxz[q] = wxz[q + 1]; wyz[q] = wyz[q + 1]; }
        wzz[3] = S[bS + 2 * P + (kz + 2) * planeS];
        wxz[3] = S[bS + 4 * P + (kz + 1) * planeS];
        wyz[3] = S[bS + 3 * P + (kz + 1) * planeS];
        wr[0] = wr[1];
        wr[1] = M[bM + (kz + 1) * planeM];
        const float cxx = S[bS + kz * planeS], cyy = S[bS + P + kz * planeS], cxy = S[bS + 5 * P + kz * planeS];
        float vxo = 0, vyo = 0, vzo = 0;
        const long long oV = bV + kz * planeV;
        if (act) { vxo = V[oV]; vyo = V[oV + P]; vzo = V[oV + 2 * P]; }

        sT[b][0][ty + 2][tx + 2] = cxx;
        sT[b][1][ty + 2][tx + 2] = cyy;
        sT[b][2][ty + 2][tx + 2] = cxy;
        sT[b][3][ty + 2][tx + 2] = wxz[2];
        sT[b][4][ty + 2][tx + 2] = wyz[2];
        sT[b][5][ty + 2][tx + 2] = wr[0];
        for (int h = tid; h < 6 * NHALO; h += TBX * TBY) {
            int c = h / NHALO, lx, ly;
            halo_xy(h - c * NHALO, lx, ly);
            int gx = xt - 2 + lx, gy = yt - 2 + ly;
            float v;
            if (c == 5) v = M[goff(g, 5, 0, gx, gy, kz)];
            else v = S[goff(g, 6, c < 2 ? c : 7 - c, gx, gy, kz)];  // Sxx Syy Sxy Sxz Syz
            sT[b][c][ly][lx] = v;
        }
        __syncthreads();
        if (act) {
            const int k = kz + 1;
            const bool nb = in_band(k, band);
            const float e40x = nb ? a.c.e2x : a.c.e4x0, e41x = nb ? 0.f : a.c.e4x1;
            const float e40y = nb ? a.c.e2y : a.c.e4y0, e41y = nb ? 0.f : a.c.e4y1;
            const float e40z = nb ? a.c.e2z : a.c.e4z0, e41z = nb ? 0.f : a.c.e4z1;
            const int lx = tx + 2, ly = ty + 2;
            float (*XX)[TBX + 4] = sT[b][0];
            float (*YY)[TBX + 4] = sT[b][1];
            float (*XY)[TBX + 4] = sT[b][2];
            float (*XZ)[TBX + 4] = sT[b][3];
            float (*YZ)[TBX + 4] = sT[b][4];
            float (*RH)[TBX + 4] = sT[b][5];
            const float d3Sx3 = (XX[ly][lx + 1] - XX[ly][lx]) * e40x - (XX[ly][lx + 2] - XX[ly][lx - 1]) * e41x
                              + (XY[ly][lx] - XY[ly - 1][lx]) * e40y - (XY[ly + 1][lx] - XY[ly - 2][lx]) * e41y
                              + (wxz[2] - wxz[1]) * e40z - (wxz[3] - wxz[0]) * e41z;
            const float d3Sy3 = (XY[ly][lx] - XY[ly][lx - 1]) * e40x - (XY[ly][lx + 1] - XY[ly][lx - 2]) * e41x
                              + (YY[ly + 1][lx] - YY[ly][lx]) * e40y - (YY[ly + 2][lx] - YY[ly - 1][lx]) * e41y
                              + (wyz[2] - wyz[1]) * e40z - (wyz[3] - wyz[0]) * e41z;
            const float d3Sz3 = (XZ[ly][lx] - XZ[ly][lx - 1]) * e40x - (XZ[ly][lx + 1] - XZ[ly][lx - 2]) * e41x
                              + (YZ[ly][lx] - YZ[ly - 1][lx]) * e40y - (YZ[ly + 1][lx] - YZ[ly - 2][lx]) * e41y
                              + (wzz[2] - wzz[1]) * e40z - (wzz[3] - wzz[0]) * e41z;
            const float r0 = RH[ly][lx];
            float vx = vxo + 2.f / (r0 + RH[ly][lx + 1]) * d3Sx3 * dt;
            float vy = vyo + 2.f / (r0 + RH[ly + 1][lx]) * d3Sy3 * dt;
            float vz = vzo + 2.f / (r0 + wr[1]) * d3Sz3 * dt;
            if (a.cer) {  // Cerjan sponge epilogue (m_absorb_c.f90:170-198)
                const float gxc = a.cer[a.cer_off[0] + ix], gxb = a.cer[a.cer_off[1] + ix];
                const float gyc = a.cer[a.cer_off[2] + jy], gyb = a.cer[a.cer_off[3] + jy];
                const float gzc = a.cer[a.cer_off[4] + kz], gzb = a.cer[a.cer_off[5] + kz];
                vx = vx * gxb * gyc * gzc;
                vy = vy * gxc * gyb * gzc;
                vz = vz * gxc * gyc * gzb;
            }
            V[oV] = vx; V[oV + P] = vy; V[oV + 2 * P] = vz;
        }
    }
}

// ---------------------------------------------------------------------------
// PML shell (ADE-CFS, m_absorb_p.f90).  The shell is five boxes; each has its
// own compact ADE storage [9][z][y][x] (one array per auxiliary, so the rows
// of the 20-cell x-side boxes run on without gaps) for the V-derivative
// auxiliaries (used by the stress update) and for the S-derivative
// auxiliaries (used by the velocity update).  One thread per shell point.
// ---------------------------------------------------------------------------

// threads (shell points) per block of the PML kernels
#ifndef PML_TPB
#define PML_TPB 128
#endif
constexpr int PTPB = PML_TPB;

// A launch of a PML kernel covers a list of parts: sub-boxes of the five ADE
// boxes in which the set of damped axes is the same at every point.  Each
// part starts on a block boundary, so a block belongs to one part.
constexpr int PML_MAXPART = 40;
struct PmlPart {
    int b;             // parent box (ADE storage and origin)
    int x0, y0, z0;    // origin inside the parent box
    int nx, ny, nz;    // extents
    int first_block;   // first block of this part in its launch
};

struct PArgs {
    Geo g;
    float* V;
    float* S;
    const float* M;
    float* adeV;        // axVx ayVy azVz ayVx azVx axVy azVy axVz ayVz
    float* adeS;        // axSxx aySxy azSxz axSxy aySyy azSyz axSxz aySyz azSzz
    const float* prof;  // gxc gxe (4 x nx each, l-major), gyc gye, gzc gze
    const float* shm;   // shell medium per box [6][z][y][x]: mu_xz mu_xy mu_yz (harmonic means), bx by bz
    int pxc, pxe, pyc, pye, pzc, pze;  // offsets of each profile (array of 4*n, l fastest)
    PmlBox box[5];
    int nbox;
    PmlPart part[PML_MAXPART];
    int npart;
    int nblocks;        // blocks of this launch (0: nothing to do)
    float r20x, r20y, r20z, dt;
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// Block blk, thread t of a launch -> shell point (box, x, y, z in the box):
// the block's part is found by a binary search over the parts' first blocks
// (the same for every thread of the block); inside the part, points run x
// fastest.  False for the threads past the end of the part.
struct PmlPt {
    int b, lx, ly, lz;
};
__device__ __forceinline__ bool pml_point(const PArgs& a, int blk, int t, PmlPt& r) {
    int lo = 0, hi = a.npart - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.part[mid].first_block <= blk) lo = mid;
        else hi = mid - 1;
    }
    const PmlPart& P = a.part[lo];
    const unsigned q = (unsigned)((blk - P.first_block) * PTPB + t);
    if (q >= (unsigned)P.nx * (unsigned)P.ny * (unsigned)P.nz) return false;
    const unsigned u = q / (unsigned)P.nx;
    const unsigned lz = u / (unsigned)P.ny;
    r.b = P.b;
    r.lx = P.x0 + (int)(q - u * (unsigned)P.nx);
    r.ly = P.y0 + (int)(u - lz * (unsigned)P.ny);
    r.lz = P.z0 + (int)lz;
    return true;
}

// Damping profile (g1 g2 g3 g4) of one axis at index i.  An axis that is not
// damped anywhere in a part (bit clear in MASK) has g1 = 1 and g4 = 0 at
// every point of it, so its ADE auxiliaries stay zero: it takes the constant
// (1, -1, 1, 0) instead of loading, which yields the same results bit for
// bit (g2 and g3 only ever multiply the zero auxiliaries).
template <int MASK, int AX>
__device__ __forceinline__ float4 pml_prof(const PArgs& a, int off, int i) {
    if (MASK & (1 << AX)) return ld4(a.prof + off + 4 * i);
    return make_float4(1.f, -1.f, 1.f, 0.f);
}

// PML stress update (m_absorb_p.f90:429-531) at shell point c, in two stages:
// stress_pml_load issues every load of the point (about 40 independent
// words; the kernel is bound by load latency, so all of them go out before
// any arithmetic or store), stress_pml_store does the arithmetic and the
// stores.  A thread may load two points before storing either.
struct PmlSIn {
    float* S;
    float* A;
    int P, AP;
    float4 gxc, gxe, gyc, gye, gzc, gze;
    float vx, vy, vz, vxw, vys, vzu, vye, vze, vxn, vzn, vxd, vyd;
    float lamv, m000, muxz, muxy, muyz;
    float ad[9], sv[6];
};
// Harmonic mean of four moduli, 4 m1 m2 m3 m4 / (sum of the triple products
// + eps) (m_absorb_p.f90:477-518), in explicitly rounded operations.
__device__ __forceinline__ float pml_hmean(float m1, float m2, float m3, float m4) {
    const float eps = 1.1920928955078125e-07f;
    const float num = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(4.f, m1), m2), m3), m4);
    const float m12 = __fmul_rn(m1, m2);
    float den = __fmul_rn(m12, m3);
    den = __fadd_rn(den, __fmul_rn(m12, m4));
    den = __fadd_rn(den, __fmul_rn(__fmul_rn(m1, m3), m4));
    den = __fadd_rn(den, __fmul_rn(__fmul_rn(m2, m3), m4));
    return __fdiv_rn(num, __fadd_rn(den, eps));
}
// the auxiliaries of point L (its profiles and ADE address set)
__device__ __forceinline__ void stress_pml_aux(PmlSIn& L) {
    const bool live[9] = {L.gxc.w != 0.f, L.gyc.w != 0.f, L.gzc.w != 0.f, L.gye.w != 0.f, L.gze.w != 0.f,
                          L.gxe.w != 0.f, L.gze.w != 0.f, L.gxe.w != 0.f, L.gye.w != 0.f};
    const float* __restrict__ A = L.A;
#pragma unroll
    for (int q = 0; q < 9; ++q) L.ad[q] = live[q] ? A[(long long)q * L.AP] : 0.f;
}
template <int MASK>
__device__ __forceinline__ void stress_pml_load(const PArgs& a, const PmlPt c, PmlSIn& L) {
    const PmlBox& B = a.box[c.b];
    const Geo& g = a.g;
    const int P = g.pitch;
    const long long rowV = 3LL * P, planeV = rowV * g.nyp;
    const int ix = B.x0 + c.lx, jy = B.y0 + c.ly, kz = B.z0 + c.lz;
    const long long oV = (long long)goff(g, 3, 0, ix, jy, kz);
    const long long oM = (long long)goff(g, 5, 0, ix, jy, kz);
    const long long oS = (long long)goff(g, 6, 0, ix, jy, kz);
    const long long oA = B.off + ((long long)c.lz * B.ny + c.ly) * B.pitch + c.lx;
    const float* __restrict__ V = a.V + oV;
    const float* __restrict__ M = a.M + oM;
    L.S = a.S + oS;
    L.A = a.adeV + oA;
    L.P = P;
    L.AP = B.qs;
    L.gxc = pml_prof<MASK, 0>(a, a.pxc, ix); L.gxe = pml_prof<MASK, 0>(a, a.pxe, ix);
    L.gyc = pml_prof<MASK, 1>(a, a.pyc, jy); L.gye = pml_prof<MASK, 1>(a, a.pye, jy);
    L.gzc = pml_prof<MASK, 2>(a, a.pzc, kz); L.gze = pml_prof<MASK, 2>(a, a.pze, kz);
    L.vx = V[0]; L.vy = V[P]; L.vz = V[2 * P];
    L.vxw = V[-1]; L.vys = V[P - rowV]; L.vzu = V[2 * P - planeV];
    L.vye = V[P + 1]; L.vze = V[2 * P + 1]; L.vxn = V[rowV]; L.vzn = V[2 * P + rowV];
    L.vxd = V[planeV]; L.vyd = V[P + planeV];
    L.lamv = M[P]; L.m000 = M[2 * P];
    // the shear moduli at the edges, precomputed once per medium
    const float* __restrict__ H = a.shm + B.moff + ((long long)c.lz * B.ny + c.ly) * B.pitch + c.lx;
    L.muxz = H[0]; L.muxy = H[B.qs]; L.muyz = H[2LL * B.qs];
    // an auxiliary variable whose axis has no damping here (g4 = 0, the
    // point lies outside that axis's layer) starts at zero and its update
    // g3 * 0 + 0 keeps it zero: it is neither loaded nor stored.  Order:
    // axVx ayVy azVz ayVx azVx axVy azVy axVz ayVz
    stress_pml_aux(L);
    const float* __restrict__ S = L.S;
#pragma unroll
    for (int q = 0; q < 6; ++q) L.sv[q] = S[q * P];
}
// K: any argument block with dt, r20x, r20y, r20z (the PML launches' or the
// tile kernels' shell arguments)
template <class K>
__device__ __forceinline__ void stress_pml_store(const K& a, const PmlSIn& L) {
    const int P = L.P, AP = L.AP;
    float* __restrict__ S = L.S;
    float* __restrict__ A = L.A;
    const float4 gxc = L.gxc, gxe = L.gxe, gyc = L.gyc, gye = L.gye, gzc = L.gzc, gze = L.gze;
    const bool live[9] = {gxc.w != 0.f, gyc.w != 0.f, gzc.w != 0.f, gye.w != 0.f, gze.w != 0.f,
                          gxe.w != 0.f, gze.w != 0.f, gxe.w != 0.f, gye.w != 0.f};
    const float* ad = L.ad;
    const float* sv = L.sv;
    const float vx = L.vx, vy = L.vy, vz = L.vz;
    // every operation below is an explicitly rounded intrinsic, so that the
    // kernels specialised to one damped axis (profile constants 1, -1, 1, 0)
    // and the general kernel produce the same bits: the compiler may not
    // contract or reorder them differently around the constants
    const float dt = a.dt;
    // normal part (m_absorb_p.f90:453-474)
    const float dxVx = __fmul_rn(__fsub_rn(vx, L.vxw), a.r20x);
    const float dyVy = __fmul_rn(__fsub_rn(vy, L.vys), a.r20y);
    const float dzVz = __fmul_rn(__fsub_rn(vz, L.vzu), a.r20z);
    const float lam2mu = __fmaf_rn(2.f, L.m000, L.lamv);
    const float lamR = __fmaf_rn(-2.f, L.m000, lam2mu);
    const float dxa = __fmaf_rn(gxc.y, ad[0], __fmul_rn(gxc.x, dxVx));
    const float dya = __fmaf_rn(gyc.y, ad[1], __fmul_rn(gyc.x, dyVy));
    const float dza = __fmaf_rn(gzc.y, ad[2], __fmul_rn(gzc.x, dzVz));
    S[0] = __fmaf_rn(__fmaf_rn(lam2mu, dxa, __fmul_rn(lamR, __fadd_rn(dya, dza))), dt, sv[0]);
    S[P] = __fmaf_rn(__fmaf_rn(lam2mu, dya, __fmul_rn(lamR, __fadd_rn(dxa, dza))), dt, sv[1]);
    S[2 * P] = __fmaf_rn(__fmaf_rn(lam2mu, dza, __fmul_rn(lamR, __fadd_rn(dxa, dya))), dt, sv[2]);
    auto ade = [dt](float4 gp, float aux, float d) { return __fmaf_rn(gp.z, aux, __fmul_rn(__fmul_rn(gp.w, d), dt)); };
    if (live[0]) A[0] = ade(gxc, ad[0], dxVx);
    if (live[1]) A[1LL * AP] = ade(gyc, ad[1], dyVy);
    if (live[2]) A[2LL * AP] = ade(gzc, ad[2], dzVz);
    // shear part (m_absorb_p.f90:477-518)
    const float dxVy = __fmul_rn(__fsub_rn(L.vye, vy), a.r20x);
    const float dxVz = __fmul_rn(__fsub_rn(L.vze, vz), a.r20x);
    const float dyVx = __fmul_rn(__fsub_rn(L.vxn, vx), a.r20y);
    const float dyVz = __fmul_rn(__fsub_rn(L.vzn, vz), a.r20y);
    const float dzVx = __fmul_rn(__fsub_rn(L.vxd, vx), a.r20z);
    const float dzVy = __fmul_rn(__fsub_rn(L.vyd, vy), a.r20z);
    const float muxz = L.muxz, muxy = L.muxy, muyz = L.muyz;
    const float ayVx = ad[3], azVx = ad[4], axVy = ad[5], azVy = ad[6], axVz = ad[7], ayVz = ad[8];
    // (g1 d1 + g1' d2 + g2 a1 + g2' a2) in a fixed order
    auto sum4 = [](float4 p, float d1, float4 q, float d2, float a1, float a2) {
        float t = __fmul_rn(p.x, d1);
        t = __fmaf_rn(q.x, d2, t);
        t = __fmaf_rn(p.y, a1, t);
        return __fmaf_rn(q.y, a2, t);
    };
    S[3 * P] = __fmaf_rn(__fmul_rn(muyz, sum4(gye, dyVz, gze, dzVy, ayVz, azVy)), dt, sv[3]);
    S[4 * P] = __fmaf_rn(__fmul_rn(muxz, sum4(gxe, dxVz, gze, dzVx, axVz, azVx)), dt, sv[4]);
    S[5 * P] = __fmaf_rn(__fmul_rn(muxy, sum4(gxe, dxVy, gye, dyVx, axVy, ayVx)), dt, sv[5]);
    if (live[3]) A[3LL * AP] = ade(gye, ayVx, dyVx);
    if (live[4]) A[4LL * AP] = ade(gze, azVx, dzVx);
    if (live[5]) A[5LL * AP] = ade(gxe, axVy, dxVy);
    if (live[6]) A[6LL * AP] = ade(gze, azVy, dzVy);
    if (live[7]) A[7LL * AP] = ade(gxe, axVz, dxVz);
    if (live[8]) A[8LL * AP] = ade(gye, ayVz, dyVz);
}
template <int MASK>
__device__ __forceinline__ void stress_pml_at(const PArgs& a, const PmlPt c) {
    PmlSIn L;
    stress_pml_load<MASK>(a, c, L);
    stress_pml_store(a, L);
}

// PML velocity update (m_absorb_p.f90:246-317) at shell point c, in the same
// two stages.
struct PmlVIn {
    float* V;
    float* A;
    int P, AP;
    float4 gxc, gxe, gyc, gye, gzc, gze;
    float sxx, syy, szz, syz, sxz, sxy, sxxe, syyn, szzd, syzs, syzu, sxzw, sxzu, sxyw, sxys;
    float bx, by, bz;  // buoyancies 2 / (rho + rho') at the faces, precomputed once per medium
    float ad[9], v0, v1, v2;
};
__device__ __forceinline__ void vel_pml_aux(PmlVIn& L) {
    const bool live[9] = {L.gxe.w != 0.f, L.gyc.w != 0.f, L.gzc.w != 0.f, L.gxc.w != 0.f, L.gye.w != 0.f,
                          L.gzc.w != 0.f, L.gxc.w != 0.f, L.gyc.w != 0.f, L.gze.w != 0.f};
    const float* __restrict__ A = L.A;
#pragma unroll
    for (int q = 0; q < 9; ++q) L.ad[q] = live[q] ? A[(long long)q * L.AP] : 0.f;
}
template <int MASK>
__device__ __forceinline__ void vel_pml_load(const PArgs& a, const PmlPt c, PmlVIn& L) {
    const PmlBox& B = a.box[c.b];
    const Geo& g = a.g;
    const int P = g.pitch;
    const long long rowS = 6LL * P, planeS = rowS * g.nyp;
    const int ix = B.x0 + c.lx, jy = B.y0 + c.ly, kz = B.z0 + c.lz;
    const long long oV = (long long)goff(g, 3, 0, ix, jy, kz);
    const long long oS = (long long)goff(g, 6, 0, ix, jy, kz);
    const long long oA = B.off + ((long long)c.lz * B.ny + c.ly) * B.pitch + c.lx;
    const float* __restrict__ S = a.S + oS;
    L.V = a.V + oV;
    L.A = a.adeS + oA;
    L.P = P;
    L.AP = B.qs;
    L.gxc = pml_prof<MASK, 0>(a, a.pxc, ix); L.gxe = pml_prof<MASK, 0>(a, a.pxe, ix);
    L.gyc = pml_prof<MASK, 1>(a, a.pyc, jy); L.gye = pml_prof<MASK, 1>(a, a.pye, jy);
    L.gzc = pml_prof<MASK, 2>(a, a.pzc, kz); L.gze = pml_prof<MASK, 2>(a, a.pze, kz);
    L.sxx = S[0]; L.syy = S[P]; L.szz = S[2 * P]; L.syz = S[3 * P]; L.sxz = S[4 * P]; L.sxy = S[5 * P];
    L.sxxe = S[1]; L.syyn = S[P + rowS]; L.szzd = S[2 * P + planeS];
    L.syzs = S[3 * P - rowS]; L.syzu = S[3 * P - planeS];
    L.sxzw = S[4 * P - 1]; L.sxzu = S[4 * P - planeS];
    L.sxyw = S[5 * P - 1]; L.sxys = S[5 * P - rowS];
    const float* __restrict__ H = a.shm + B.moff + ((long long)c.lz * B.ny + c.ly) * B.pitch + c.lx;
    L.bx = H[3LL * B.qs]; L.by = H[4LL * B.qs]; L.bz = H[5LL * B.qs];
    // auxiliaries of undamped axes stay zero (as in the stress update).
    // Order: axSxx aySxy azSxz axSxy aySyy azSyz axSxz aySyz azSzz
    vel_pml_aux(L);
    const float* __restrict__ V = L.V;
    L.v0 = V[0]; L.v1 = V[P]; L.v2 = V[2 * P];
}
template <class K>
__device__ __forceinline__ void vel_pml_store(const K& a, const PmlVIn& L) {
    const int P = L.P, AP = L.AP;
    float* __restrict__ V = L.V;
    float* __restrict__ A = L.A;
    const float4 gxc = L.gxc, gxe = L.gxe, gyc = L.gyc, gye = L.gye, gzc = L.gzc, gze = L.gze;
    const bool live[9] = {gxe.w != 0.f, gyc.w != 0.f, gzc.w != 0.f, gxc.w != 0.f, gye.w != 0.f,
                          gzc.w != 0.f, gxc.w != 0.f, gyc.w != 0.f, gze.w != 0.f};
    // explicitly rounded operations, as in the stress update
    const float dt = a.dt;
    // m_absorb_p.f90:265-305
    const float dxSxx = __fmul_rn(__fsub_rn(L.sxxe, L.sxx), a.r20x);
    const float dySyy = __fmul_rn(__fsub_rn(L.syyn, L.syy), a.r20y);
    const float dzSzz = __fmul_rn(__fsub_rn(L.szzd, L.szz), a.r20z);
    const float dySyz = __fmul_rn(__fsub_rn(L.syz, L.syzs), a.r20y);
    const float dzSyz = __fmul_rn(__fsub_rn(L.syz, L.syzu), a.r20z);
    const float dxSxz = __fmul_rn(__fsub_rn(L.sxz, L.sxzw), a.r20x);
    const float dzSxz = __fmul_rn(__fsub_rn(L.sxz, L.sxzu), a.r20z);
    const float dxSxy = __fmul_rn(__fsub_rn(L.sxy, L.sxyw), a.r20x);
    const float dySxy = __fmul_rn(__fsub_rn(L.sxy, L.sxys), a.r20y);
    const float bx = L.bx, by = L.by, bz = L.bz;
    const float* ad = L.ad;
    const float axSxx = ad[0], aySxy = ad[1], azSxz = ad[2], axSxy = ad[3], aySyy = ad[4];
    const float azSyz = ad[5], axSxz = ad[6], aySyz = ad[7], azSzz = ad[8];
    // (g1 d1 + g1' d2 + g1'' d3 + g2 a1 + g2' a2 + g2'' a3) in a fixed order
    auto sum6 = [](float4 p, float d1, float4 q, float d2, float4 r, float d3, float a1, float a2, float a3) {
        float t = __fmul_rn(p.x, d1);
        t = __fmaf_rn(q.x, d2, t);
        t = __fmaf_rn(r.x, d3, t);
        t = __fmaf_rn(p.y, a1, t);
        t = __fmaf_rn(q.y, a2, t);
        return __fmaf_rn(r.y, a3, t);
    };
    V[0] = __fmaf_rn(__fmul_rn(bx, sum6(gxe, dxSxx, gyc, dySxy, gzc, dzSxz, axSxx, aySxy, azSxz)), dt, L.v0);
    V[P] = __fmaf_rn(__fmul_rn(by, sum6(gxc, dxSxy, gye, dySyy, gzc, dzSyz, axSxy, aySyy, azSyz)), dt, L.v1);
    V[2 * P] = __fmaf_rn(__fmul_rn(bz, sum6(gxc, dxSxz, gyc, dySyz, gze, dzSzz, axSxz, aySyz, azSzz)), dt, L.v2);
    auto ade = [dt](float4 gp, float aux, float d) { return __fmaf_rn(gp.z, aux, __fmul_rn(__fmul_rn(gp.w, d), dt)); };
    if (live[0]) A[0] = ade(gxe, axSxx, dxSxx);
    if (live[1]) A[1LL * AP] = ade(gyc, aySxy, dySxy);
    if (live[2]) A[2LL * AP] = ade(gzc, azSxz, dzSxz);
    if (live[3]) A[3LL * AP] = ade(gxc, axSxy, dxSxy);
    if (live[4]) A[4LL * AP] = ade(gye, aySyy, dySyy);
    if (live[5]) A[5LL * AP] = ade(gzc, azSyz, dzSyz);
    if (live[6]) A[6LL * AP] = ade(gxc, axSxz, dxSxz);
    if (live[7]) A[7LL * AP] = ade(gyc, aySyz, dySyz);
    if (live[8]) A[8LL * AP] = ade(gze, azSzz, dzSzz);
}
// One component of the velocity shell update (the tile kernels update the
// three components one after the other):
// V = v0 + b (p.x d1 + q.x d2 + r.x d3 + p.y a1 + q.y a2 + r.y a3) dt, with
// the auxiliaries a1..a3 (arrays q1..q3 of A; zero where g4 of their profile
// is zero, and then neither stored) advanced as in vel_pml_store, whose
// operations and order this repeats bit for bit.
__device__ __forceinline__ void vel_pml_component(float dt, float4 p, float d1, float4 q, float d2, float4 r, float d3,
                                                  float a1, float a2, float a3, float* __restrict__ A, long long AP,
                                                  int q1, int q2, int q3, float b, float v0, float* __restrict__ out) {
    float t = __fmul_rn(p.x, d1);
    t = __fmaf_rn(q.x, d2, t);
    t = __fmaf_rn(r.x, d3, t);
    t = __fmaf_rn(p.y, a1, t);
    t = __fmaf_rn(q.y, a2, t);
    t = __fmaf_rn(r.y, a3, t);
    *out = __fmaf_rn(__fmul_rn(b, t), dt, v0);
    auto ade = [dt](float4 gp, float aux, float d) { return __fmaf_rn(gp.z, aux, __fmul_rn(__fmul_rn(gp.w, d), dt)); };
    if (p.w != 0.f) A[q1 * AP] = ade(p, a1, d1);
    if (q.w != 0.f) A[q2 * AP] = ade(q, a2, d2);
    if (r.w != 0.f) A[q3 * AP] = ade(r, a3, d3);
}

template <int MASK>
__device__ __forceinline__ void vel_pml_at(const PArgs& a, const PmlPt c) {
    PmlVIn L;
    vel_pml_load<MASK>(a, c, L);
    vel_pml_store(a, L);
}

// Two points per thread: both points' loads go out before either point's
// arithmetic and stores (points of blocks 2b and 2b + 1 of the launch).
template <int MASK>
__device__ __forceinline__ void stress_pml_two(const PArgs& a, int b2, int t) {
    PmlPt c0, c1;
    const bool o0 = pml_point(a, 2 * b2, t, c0);
    const bool o1 = 2 * b2 + 1 < a.nblocks && pml_point(a, 2 * b2 + 1, t, c1);
    PmlSIn L0, L1;
    if (o0) stress_pml_load<MASK>(a, c0, L0);
    if (o1) stress_pml_load<MASK>(a, c1, L1);
    if (o0) stress_pml_store(a, L0);
    if (o1) stress_pml_store(a, L1);
}
template <int MASK>
__device__ __forceinline__ void vel_pml_two(const PArgs& a, int b2, int t) {
    PmlPt c0, c1;
    const bool o0 = pml_point(a, 2 * b2, t, c0);
    const bool o1 = 2 * b2 + 1 < a.nblocks && pml_point(a, 2 * b2 + 1, t, c1);
    PmlVIn L0, L1;
    if (o0) vel_pml_load<MASK>(a, c0, L0);
    if (o1) vel_pml_load<MASK>(a, c1, L1);
    if (o0) vel_pml_store(a, L0);
    if (o1) vel_pml_store(a, L1);
}

// The shell's medium terms that the PML updates take from several cells --
// the harmonic-mean shear moduli at the cell edges (m_absorb_p.f90:477-518)
// and the buoyancies at the faces (m_absorb_p.f90:265-305) -- computed once
// per medium with the operations the updates used, so that the updates give
// the same bits: one thread per shell point of the whole boxes (a.part[] with
// one part per box, as the general launch).
__global__ void k_shell_medium(const PArgs a, float* __restrict__ shm) {
    PmlPt c;
    if (!pml_point(a, blockIdx.x, threadIdx.x, c)) return;
    const PmlBox& B = a.box[c.b];
    const Geo& g = a.g;
    const int P = g.pitch;
    const long long rowM = 5LL * P, planeM = rowM * g.nyp;
    const int ix = B.x0 + c.lx, jy = B.y0 + c.ly, kz = B.z0 + c.lz;
    const float* __restrict__ M = a.M + (long long)goff(g, 5, 0, ix, jy, kz);
    const float m000 = M[2 * P], m100 = M[2 * P + planeM], m010 = M[2 * P + 1], m110 = M[2 * P + planeM + 1];
    const float m001 = M[2 * P + rowM], m011 = M[2 * P + rowM + 1], m101 = M[2 * P + planeM + rowM];
    const float r0 = M[0], rx = M[1], ry = M[rowM], rz = M[planeM];
    float* H = shm + B.moff + ((long long)c.lz * B.ny + c.ly) * B.pitch + c.lx;
    const long long q = B.qs;
    H[0] = pml_hmean(m000, m100, m010, m110);
    H[q] = pml_hmean(m000, m010, m001, m011);
    H[2 * q] = pml_hmean(m000, m100, m001, m101);
    H[3 * q] = __fdiv_rn(2.f, __fadd_rn(r0, rx));
    H[4 * q] = __fdiv_rn(2.f, __fadd_rn(r0, ry));
    H[5 * q] = __fdiv_rn(2.f, __fadd_rn(r0, rz));
}

// One thread per shell point.  MASK: the axes damped somewhere in the parts
// of the launch (7 = any, checked per point).  With one damped axis the
// kernels skip two thirds of the auxiliaries and profiles and fit 64
// registers without spilling (8 blocks per SM); the general kernels fit 72
// (7 blocks; the general velocity kernel, which took 85 registers and 6
// blocks unbounded, runs its corners 12 % faster so: 0.121 -> 0.106 ms on
// the 1024x1024x512 grid, the 64-member batch step 17.63 -> 17.37 ms).
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 7 : 8) k_stress_pml(const PArgs a) {
    PmlPt c;
    if (pml_point(a, blockIdx.x, threadIdx.x, c)) stress_pml_at<MASK>(a, c);
}
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 7 : 8) k_vel_pml(const PArgs a) {
    PmlPt c;
    if (pml_point(a, blockIdx.x, threadIdx.x, c)) vel_pml_at<MASK>(a, c);
}
// two points per thread (block b covers blocks 2b and 2b + 1 of the parts)
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 4 : 5) k_stress_pml2(const PArgs a) { stress_pml_two<MASK>(a, blockIdx.x, threadIdx.x); }
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 4 : 5) k_vel_pml2(const PArgs a) { vel_pml_two<MASK>(a, blockIdx.x, threadIdx.x); }
// batched: block b is block e.y of member e.x's launch, e = blocks[b]
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 7 : 8) k_stress_pml_batch(const PArgs* __restrict__ all, const int2* __restrict__ blocks) {
    const int2 e = blocks[blockIdx.x];
    PmlPt c;
    if (pml_point(all[e.x], e.y, threadIdx.x, c)) stress_pml_at<MASK>(all[e.x], c);
}
template <int MASK>
__global__ void __launch_bounds__(PTPB, MASK == 7 ? 7 : 8) k_vel_pml_batch(const PArgs* __restrict__ all, const int2* __restrict__ blocks) {
    const int2 e = blocks[blockIdx.x];
    PmlPt c;
    if (pml_point(all[e.x], e.y, threadIdx.x, c)) vel_pml_at<MASK>(all[e.x], c);
}
// the launch classes: x only, y only, z only, any
constexpr int PML_NCLASS = 4;
constexpr int PML_CLASS_MASK[PML_NCLASS] = {1, 2, 4, 7};

// ---------------------------------------------------------------------------
// Sources, receivers, snapshots, divergence check
// ---------------------------------------------------------------------------

// m_fdtool.f90:339-497
__device__ __forceinline__ float momentrate(float t, int stf, float ts, float tr) {
    const float pi = 3.14159265358979f;
    switch (stf) {
    case 0: return (ts <= t && t <= ts + tr) ? 1.f / tr : 0.f;
    case 1:
        if (ts <= t && t <= ts + tr / 2) return 4 * (t - ts) / (tr * tr);
        if (ts + tr / 2 < t && t <= ts + tr) return -4 * (t - ts - tr) / (tr * tr);
        return 0.f;
    case 2: {
        float t1 = ts + tr / 4, t2 = ts + 3 * tr / 4;
        if (ts <= t && t < t1) return 16 * (t - ts) * (t - ts) / (tr * tr * tr);
        if (t1 <= t && t < t2) return -2 * (8 * (t * t + tr * ts + ts * ts - t * tr - 2 * t * ts) + tr * tr) / (tr * tr * tr);
        if (t2 <= t && t <= ts + tr) return 16 * (ts + tr - t) * (ts + tr - t) / (tr * tr * tr);
        return 0.f;
    }
    case 4: return (ts <= t && t <= ts + tr) ? (1 - cosf(2 * pi * (t - ts) / tr)) / tr : 0.f;
    case 5: {
        if (ts <= t) { float tt = t - ts; return (2 * pi) * (2 * pi) * tt / (tr * tr) * expf(-2 * pi * tt / tr); }
        return 0.f;
    }
    default: {
        if (ts <= t && t <= ts + tr) { float s = sinf(pi * (t - ts) / tr); return 3 * pi * s * s * s / (4 * tr); }
        return 0.f;
    }
    }
}

struct SrcArgs {
    Geo g;
    float* V;
    float* S;
    const float* M;
    const int* ijk;      // 3n, 0-based
    const float* mij;    // 6n (xx yy zz yz xz xy) multiplied by mo
    const float* fxyz;   // 3n
    const float* prm;    // 2n
    int n, stf;
    int bf;              // 1: body forces (velocity), 0: moment tensors (stress)
    float tbeg, dt, dt_dxyz;
    const int* it;       // device step counter
};

// Ghost planes in x/y are never stored to: the reference zeroes the ones the
// stencils read right after injection (m_global.f90:458-488, 569-601).
__device__ __forceinline__ bool in_xy(const Geo& g, int ix, int jy) { return ix >= 0 && ix < g.nx && jy >= 0 && jy < g.ny; }

// m_source.f90:776-848
__device__ __forceinline__ void stressglut_one(const SrcArgs& a, const int s) {
    if (s >= a.n || a.bf) return;
    const int it = *a.it;
    const float t = a.tbeg + ((float)it - 0.5f) * a.dt;
    const float st = momentrate(t, a.stf, a.prm[2 * s], a.prm[2 * s + 1]);
    const float sdrop = st * a.dt_dxyz;
    const int i = a.ijk[3 * s], j = a.ijk[3 * s + 1], k = a.ijk[3 * s + 2];
    const float* m = a.mij + 6 * s;
    const Geo& g = a.g;
    auto add = [&](int f, int ii, int jj, int kk, float v) {
        if (in_xy(g, ii, jj)) atomicAdd(a.S + goff(g, 6, f, ii, jj, kk), -v);
    };
    add(0, i, j, k, m[0] * sdrop);
    add(1, i, j, k, m[1] * sdrop);
    add(2, i, j, k, m[2] * sdrop);
    const float qyz = m[3] * sdrop / 4, qxz = m[4] * sdrop / 4, qxy = m[5] * sdrop / 4;
    add(5, i, j, k, qxy); add(5, i, j - 1, k, qxy); add(5, i - 1, j, k, qxy); add(5, i - 1, j - 1, k, qxy);
    add(4, i, j, k, qxz); add(4, i, j, k - 1, qxz); add(4, i - 1, j, k, qxz); add(4, i - 1, j, k - 1, qxz);
    add(3, i, j, k, qyz); add(3, i, j, k - 1, qyz); add(3, i, j - 1, k, qyz); add(3, i, j - 1, k - 1, qyz);
}

// m_source.f90:850-898
__device__ __forceinline__ void bodyforce_one(const SrcArgs& a, const int s) {
    if (s >= a.n || !a.bf) return;
    const int it = *a.it;
    const float st = momentrate(a.tbeg + (float)it * a.dt, a.stf, a.prm[2 * s], a.prm[2 * s + 1]);
    const int i = a.ijk[3 * s], j = a.ijk[3 * s + 1], k = a.ijk[3 * s + 2];
    const Geo& g = a.g;
    const float* f = a.fxyz + 3 * s;
    auto rho = [&](int ii, int jj, int kk) { return a.M[goff(g, 5, 0, ii, jj, kk)]; };
    auto add = [&](int c, int ii, int jj, int kk, float b, float fc) {
        if (in_xy(g, ii, jj)) atomicAdd(a.V + goff(g, 3, c, ii, jj, kk), b * fc * st * a.dt_dxyz / 2);
    };
    const float r0 = rho(i, j, k);
    add(0, i, j, k, 2.f / (r0 + rho(i + 1, j, k)), f[0]);
    add(0, i - 1, j, k, 2.f / (r0 + rho(i - 1, j, k)), f[0]);
    add(1, i, j, k, 2.f / (r0 + rho(i, j + 1, k)), f[1]);
    add(1, i, j - 1, k, 2.f / (r0 + rho(i, j - 1, k)), f[1]);
    add(2, i, j, k, 2.f / (r0 + rho(i, j, k + 1)), f[2]);
    add(2, i, j, k - 1, 2.f / (r0 + rho(i, j, k - 1)), f[2]);
}

__global__ void k_stressglut(const SrcArgs a) { stressglut_one(a, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_bodyforce(const SrcArgs a) { bodyforce_one(a, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_stressglut_batch(const SrcArgs* __restrict__ all) { stressglut_one(all[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_bodyforce_batch(const SrcArgs* __restrict__ all) { bodyforce_one(all[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x); }

struct TapArgs {
    Geo g;
    const float* V;
    const float* S;
    const int* ijk;   // 3n, 0-based
    int n, ntw, ntdec_w, flags;
    float* wav_v;     // (ntw, 3, n)
    float* wav_u;
    float* wav_s;     // (ntw, 6, n)
    float* wav_e;
    double* acc;      // 9n: ux uy uz exx eyy ezz eyz exz exy (FP64 time integration)
    float vscale, sscale, escale;  // M0*UC*1e9, M0*UC*1e6, M0*UC*1e-3
    float dt;
    float r40x, r40y, r40z, r41x, r41y, r41z;  // 9/8/d, 1/24/d
    const int* it;
};

// m_wav.f90:397-625: taps of the *previous* step's velocity/stress
__device__ __forceinline__ void taps_one(const TapArgs& a, const int n) {
    if (n >= a.n) return;
    const int it = *a.it;
    const Geo& g = a.g;
    const int i = a.ijk[3 * n], j = a.ijk[3 * n + 1], k = a.ijk[3 * n + 2];
    auto v = [&](int c, int ii, int jj, int kk) { return a.V[goff(g, 3, c, ii, jj, kk)]; };
    auto s = [&](int f, int ii, int jj, int kk) { return a.S[goff(g, 6, f, ii, jj, kk)]; };
    double* acc = a.acc + 9 * n;
    if (a.flags & 2) {  // displacement by time integration (FP64)
        acc[0] += ((double)v(0, i, j, k) + (double)v(0, i - 1, j, k)) * 0.5 * (double)a.dt;
        acc[1] += ((double)v(1, i, j, k) + (double)v(1, i, j - 1, k)) * 0.5 * (double)a.dt;
        acc[2] -= ((double)v(2, i, j, k) + (double)v(2, i, j, k - 1)) * 0.5 * (double)a.dt;
    }
    if (a.flags & 8) {  // strain (4th order, m_wav.f90:465-504)
        auto D = [&](int c, int di, int dj, int dk, int ax, float r40, float r41) {
            // forward difference along axis ax at offset (di,dj,dk): (f(+1)-f(0))*r40 - (f(+2)-f(-1))*r41
            int ei = (ax == 0), ej = (ax == 1), ek = (ax == 2);
            int ii = i + di, jj = j + dj, kk = k + dk;
            return (v(c, ii + ei, jj + ej, kk + ek) - v(c, ii, jj, kk)) * r40 -
                   (v(c, ii + 2 * ei, jj + 2 * ej, kk + 2 * ek) - v(c, ii - ei, jj - ej, kk - ek)) * r41;
        };
        const float dxVx = D(0, -1, 0, 0, 0, a.r40x, a.r41x);
        const float dyVy = D(1, 0, -1, 0, 1, a.r40y, a.r41y);
        const float dzVz = D(2, 0, 0, -1, 2, a.r40z, a.r41z);
        const float dxVy = (D(1, 0, 0, 0, 0, a.r40x, a.r41x) + D(1, 0, -1, 0, 0, a.r40x, a.r41x) +
                            D(1, -1, 0, 0, 0, a.r40x, a.r41x) + D(1, -1, -1, 0, 0, a.r40x, a.r41x)) / 4.f;
        const float dxVz = (D(2, 0, 0, 0, 0, a.r40x, a.r41x) + D(2, 0, 0, -1, 0, a.r40x, a.r41x) +
                            D(2, -1, 0, 0, 0, a.r40x, a.r41x) + D(2, -1, 0, -1, 0, a.r40x, a.r41x)) / 4.f;
        const float dyVx = (D(0, 0, 0, 0, 1, a.r40y, a.r41y) + D(0, -1, 0, 0, 1, a.r40y, a.r41y) +
                            D(0, 0, -1, 0, 1, a.r40y, a.r41y) + D(0, -1, -1, 0, 1, a.r40y, a.r41y)) / 4.f;
        const float dyVz = (D(2, 0, 0, 0, 1, a.r40y, a.r41y) + D(2, 0, 0, -1, 1, a.r40y, a.r41y) +
                            D(2, 0, -1, 0, 1, a.r40y, a.r41y) + D(2, 0, -1, -1, 1, a.r40y, a.r41y)) / 4.f;
        const float dzVx = (D(0, 0, 0, 0, 2, a.r40z, a.r41z) + D(0, -1, 0, 0, 2, a.r40z, a.r41z) +
                            D(0, 0, 0, -1, 2, a.r40z, a.r41z) + D(0, -1, 0, -1, 2, a.r40z, a.r41z)) / 4.f;
        const float dzVy = (D(1, 0, 0, 0, 2, a.r40z, a.r41z) + D(1, 0, -1, 0, 2, a.r40z, a.r41z) +
                            D(1, 0, 0, -1, 2, a.r40z, a.r41z) + D(1, 0, -1, -1, 2, a.r40z, a.r41z)) / 4.f;
        acc[3] += (double)dxVx * a.dt;
        acc[4] += (double)dyVy * a.dt;
        acc[5] += (double)dzVz * a.dt;
        acc[6] += (double)((dyVz + dzVy) / 2.f) * a.dt;
        acc[7] += (double)((dxVz + dzVx) / 2.f) * a.dt;
        acc[8] += (double)((dxVy + dyVx) / 2.f) * a.dt;
    }
    if ((it - 1) % a.ntdec_w != 0) return;
    const int itw = (it - 1) / a.ntdec_w;
    if (itw >= a.ntw) return;
    if (a.flags & 1) {
        float* w = a.wav_v + (size_t)n * 3 * a.ntw + itw;
        w[0] = (v(0, i, j, k) + v(0, i - 1, j, k)) / 2.f * a.vscale;
        w[a.ntw] = (v(1, i, j, k) + v(1, i, j - 1, k)) / 2.f * a.vscale;
        w[2 * a.ntw] = -(v(2, i, j, k) + v(2, i, j, k - 1)) / 2.f * a.vscale;
    }
    if (a.flags & 2) {
        float* w = a.wav_u + (size_t)n * 3 * a.ntw + itw;
        for (int c = 0; c < 3; ++c) w[c * a.ntw] = (float)acc[c] * a.vscale;
    }
    if (a.flags & 4) {
        float* w = a.wav_s + (size_t)n * 6 * a.ntw + itw;
        w[0] = s(0, i, j, k) * a.sscale;
        w[a.ntw] = s(1, i, j, k) * a.sscale;
        w[2 * a.ntw] = s(2, i, j, k) * a.sscale;
        w[3 * a.ntw] = (s(3, i, j, k) + s(3, i, j - 1, k) + s(3, i, j, k - 1) + s(3, i, j - 1, k - 1)) / 4.f * a.sscale;
        w[4 * a.ntw] = (s(4, i, j, k) + s(4, i - 1, j, k) + s(4, i, j, k - 1) + s(4, i - 1, j, k - 1)) / 4.f * a.sscale;
        w[5 * a.ntw] = (s(5, i, j, k) + s(5, i, j - 1, k) + s(5, i - 1, j, k) + s(5, i - 1, j - 1, k)) / 4.f * a.sscale;
    }
    if (a.flags & 8) {
        float* w = a.wav_e + (size_t)n * 6 * a.ntw + itw;
        for (int c = 0; c < 6; ++c) w[c * a.ntw] = (float)acc[3 + c] * a.escale;
    }
}

__global__ void k_taps(const TapArgs a) { taps_one(a, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_taps_batch(const TapArgs* __restrict__ all) { taps_one(all[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x); }

// Snapshot sections (m_snap.f90:95-473): xy at k0, yz at i0, xz at j0, and
// the free-surface / ocean-bottom maps at kfs+1 / kob+1 of every column;
// kinds: velocity, displacement (integrated every step), and divergence /
// rotation with the medium and shear-stress masks.
enum { SEC_XY = 0, SEC_YZ = 1, SEC_XZ = 2, SEC_FS = 3, SEC_OB = 4 };
enum { SNAP_V = 0, SNAP_U = 1, SNAP_PS = 2 };
constexpr int MAX_SNAP = 15;

struct SnapPlane {
    int sec, kind;
    int n1, n2;         // pixels along the first and second axis
    int d1, d2;         // decimation along them
    int fix;            // 0-based k (xy), i (yz) or j (xz)
    int nc;             // 3 (v, u) or 4 (ps)
    float* frames;      // (maxframes, nc, n2, n1)
    double* uacc;       // (3, n2, n1) running displacement (u only)
};

struct SnapArgs {
    Geo g;
    const float* V;
    const float* S;
    const float* M;
    const int* kfs;     // (nx, ny) 1-based kfs of each column, 0-based map
    const int* kob;     // same for kob
    int n, ntdec_s, maxframes, maxpix;
    float UC, M0, dt, r20x, r20y, r20z;
    SnapPlane pl[MAX_SNAP];
    const int* it;
};

// wbuf_{xy,yz,xz,fs,ob}_{v,u,ps} (m_snap.f90:981-2205) for pixel q of plane P
__device__ __forceinline__ void snap_pix(const SnapArgs& a, const SnapPlane& P, const int q) {
    if (q >= P.n1 * P.n2) return;
    const int it = *a.it;
    const Geo& g = a.g;
    const int p1 = q % P.n1, p2 = q / P.n1;
    auto dec = [](int pp, int d) { return (pp + 1) * d - d / 2 - 1; };  // 0-based cell of pixel pp
    int i, j, k;
    switch (P.sec) {
    case SEC_YZ: i = P.fix; j = dec(p1, P.d1); k = dec(p2, P.d2); break;
    case SEC_XZ: i = dec(p1, P.d1); j = P.fix; k = dec(p2, P.d2); break;
    default:
        i = dec(p1, P.d1); j = dec(p2, P.d2);
        k = P.sec == SEC_XY ? P.fix : (P.sec == SEC_FS ? a.kfs : a.kob)[(size_t)j * g.nx + i];  // (kfs|kob)+1, 1-based
        break;
    }
    const size_t pl = (size_t)P.n1 * P.n2;
    const bool frame = (it - 1) % a.ntdec_s == 0 && (it - 1) / a.ntdec_s < a.maxframes;
    float* out = P.frames + (frame ? (size_t)((it - 1) / a.ntdec_s) * P.nc * pl : 0) + q;
    const float* V = a.V;
    auto v = [&](int c, int di, int dj, int dk) { return V[goff(g, 3, c, i + di, j + dj, k + dk)]; };
    if (P.kind == SNAP_V) {
        if (!frame) return;
        for (int c = 0; c < 3; ++c) out[c * pl] = v(c, 0, 0, 0) * a.UC * a.M0;
    } else if (P.kind == SNAP_U) {
        // integrated every step; FP64 accumulation (the reference sums in FP32)
        for (int c = 0; c < 3; ++c) {
            double u = P.uacc[c * pl + q] + (double)(v(c, 0, 0, 0) * a.UC * a.M0) * (double)a.dt;
            P.uacc[c * pl + q] = u;
            if (frame) out[c * pl] = (float)u;
        }
    } else {
        if (!frame) return;
        const float eps = 1.1920928955078125e-07f;
        const float vx = v(0, 0, 0, 0), vy = v(1, 0, 0, 0), vz = v(2, 0, 0, 0);
        float div = (vx - v(0, -1, 0, 0)) * a.r20x + (vy - v(1, 0, -1, 0)) * a.r20y + (vz - v(2, 0, 0, -1)) * a.r20z;
        float rx = (v(2, 0, 1, 0) - vz) * a.r20y - (v(1, 0, 0, 1) - vy) * a.r20z;
        float ry = (v(0, 0, 0, 1) - vx) * a.r20z - (v(2, 1, 0, 0) - vz) * a.r20x;
        float rz = (v(1, 1, 0, 0) - vy) * a.r20x - (v(0, 0, 1, 0) - vx) * a.r20y;
        const float lam = a.M[goff(g, 5, 1, i, j, k)];
        const float syz = a.S[goff(g, 6, 3, i, j, k)], sxz = a.S[goff(g, 6, 4, i, j, k)], sxy = a.S[goff(g, 6, 5, i, j, k)];
        div = div * lam / fabsf(lam + eps);
        if (P.sec == SEC_YZ) {  // wbuf_yz_ps masks with |S| / |S + eps| (m_snap.f90:1027-1030)
            rx = rx * fabsf(syz) / fabsf(syz + eps);
            ry = ry * fabsf(sxz) / fabsf(sxz + eps);
            rz = rz * fabsf(sxy) / fabsf(sxy + eps);
        } else {
            rx = rx * fabsf(syz) / (fabsf(syz) + eps);
            ry = ry * fabsf(sxz) / (fabsf(sxz) + eps);
            rz = rz * fabsf(sxy) / (fabsf(sxy) + eps);
        }
        out[0] = div * a.UC * a.M0 * 1e-3f;
        out[pl] = rx * a.UC * a.M0 * 1e-3f;
        out[2 * pl] = ry * a.UC * a.M0 * 1e-3f;
        out[3 * pl] = rz * a.UC * a.M0 * 1e-3f;
    }
}

__global__ void k_snap(const SnapArgs a) { snap_pix(a, a.pl[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_snap_batch(const SnapArgs* __restrict__ all) {
    const SnapArgs& a = all[blockIdx.z];
    if ((int)blockIdx.y < a.n) snap_pix(a, a.pl[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x);
}

// Green's-function taps (src/swpc_3d/m_green.f90:406-551): at every grid
// point of the list, the nine displacement gradients (four-point averages of
// the 4th-order staggered derivatives for the off-diagonal ones) and, with
// body-force output, the displacement, integrated every step; every ntdec_w
// steps the six strain-like combinations (and the displacement) are stored.
struct GreenArgs {
    Geo g;
    const float* V;
    int n, ncmp, ntdec_w, ntw;
    const int* ijk;     // 3n, 0-based i, j, k
    double* acc;        // (12, n): dxUx dxUy dxUz dyUx dyUy dyUz dzUx dzUy dzUz Ux Uy Uz
    float* gf;          // (ntw, ncmp, n) Fortran order
    float dt, r40x, r41x, r40y, r41y, r40z, r41z;
    const int* it;
};

__device__ __forceinline__ void green_pt(const GreenArgs& a, const int n) {
    if (n >= a.n) return;
    const int it = *a.it;
    const Geo& g = a.g;
    const int i = a.ijk[3 * n], j = a.ijk[3 * n + 1], k = a.ijk[3 * n + 2];
    auto V = [&](int c, int kk, int ii, int jj) { return a.V[goff(g, 3, c, ii, jj, kk)]; };
    // (V(k1,i1,j1) - V(k0,i0,j0)) r0 - (V(k2,i2,j2) - V(k3,i3,j3)) r1 along x, y or z
    auto dx = [&](int c, int kk, int jj, int i0) {  // derivative between i0 and i0 + 1
        return (V(c, kk, i0 + 1, jj) - V(c, kk, i0, jj)) * a.r40x - (V(c, kk, i0 + 2, jj) - V(c, kk, i0 - 1, jj)) * a.r41x;
    };
    auto dy = [&](int c, int kk, int ii, int j0) {
        return (V(c, kk, ii, j0 + 1) - V(c, kk, ii, j0)) * a.r40y - (V(c, kk, ii, j0 + 2) - V(c, kk, ii, j0 - 1)) * a.r41y;
    };
    auto dz = [&](int c, int ii, int jj, int k0) {
        return (V(c, k0 + 1, ii, jj) - V(c, k0, ii, jj)) * a.r40z - (V(c, k0 + 2, ii, jj) - V(c, k0 - 1, ii, jj)) * a.r41z;
    };
    const float dxVx = dx(0, k, j, i - 1), dyVy = dy(1, k, i, j - 1), dzVz = dz(2, i, j, k - 1);
    const float dxVy = (dx(1, k, j, i) + dx(1, k, j - 1, i) + dx(1, k, j, i - 1) + dx(1, k, j - 1, i - 1)) * 0.25f;
    const float dxVz = (dx(2, k, j, i) + dx(2, k - 1, j, i) + dx(2, k, j, i - 1) + dx(2, k - 1, j, i - 1)) * 0.25f;
    const float dyVx = (dy(0, k, i, j) + dy(0, k, i - 1, j) + dy(0, k, i, j - 1) + dy(0, k, i - 1, j - 1)) * 0.25f;
    const float dyVz = (dy(2, k, i, j) + dy(2, k - 1, i, j) + dy(2, k, i, j - 1) + dy(2, k - 1, i, j - 1)) * 0.25f;
    const float dzVx = (dz(0, i, j, k) + dz(0, i - 1, j, k) + dz(0, i, j, k - 1) + dz(0, i - 1, j, k - 1)) * 0.25f;
    const float dzVy = (dz(1, i, j, k) + dz(1, i, j - 1, k) + dz(1, i, j, k - 1) + dz(1, i, j - 1, k - 1)) * 0.25f;
    const float g9[9] = {dxVx, dxVy, dxVz, dyVx, dyVy, dyVz, dzVx, dzVy, dzVz};
    double* acc = a.acc;
    const size_t N = a.n;
    // time integration in FP64 (the reference sums in FP32)
    for (int c = 0; c < 9; ++c) acc[c * N + n] += (double)(g9[c] * a.dt);
    if (a.ncmp == 9) {
        acc[9 * N + n] += (double)(0.5f * (V(0, k, i, j) + V(0, k, i - 1, j)) * a.dt);
        acc[10 * N + n] += (double)(0.5f * (V(1, k, i, j) + V(1, k, i, j - 1)) * a.dt);
        acc[11 * N + n] += (double)(0.5f * (V(2, k, i, j) + V(2, k - 1, i, j)) * a.dt);
    }
    if ((it - 1) % a.ntdec_w != 0) return;
    const int itw = (it - 1) / a.ntdec_w;
    if (itw >= a.ntw) return;
    auto A = [&](int c) { return (float)acc[c * N + n]; };
    float* gf = a.gf + (size_t)n * a.ncmp * a.ntw + itw;
    const float ud = 1e-15f, ub = 1e-12f, nm = 1e9f;  // UC_DERIV, UC_BF (m_green.f90:31-32), m -> nm
    gf[0] = A(0) * ud * nm;
    gf[(size_t)a.ntw] = A(4) * ud * nm;
    gf[(size_t)2 * a.ntw] = A(8) * ud * nm;
    gf[(size_t)3 * a.ntw] = (A(5) + A(7)) * ud * nm;
    gf[(size_t)4 * a.ntw] = (A(2) + A(6)) * ud * nm;
    gf[(size_t)5 * a.ntw] = (A(1) + A(3)) * ud * nm;
    if (a.ncmp == 9) {
        gf[(size_t)6 * a.ntw] = A(9) * ub * nm;
        gf[(size_t)7 * a.ntw] = A(10) * ub * nm;
        gf[(size_t)8 * a.ntw] = A(11) * ub * nm;
    }
}
__global__ void k_green(const GreenArgs a) { green_pt(a, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_green_batch(const GreenArgs* __restrict__ all) {
    green_pt(all[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x);
}

struct VmaxArgs {
    Geo g;
    const float* V;
    const int* kob;        // (nx, ny) 1-based kob of each column, 0-based map
    int i0, i1, j0, j1;    // 0-based inclusive ranges
    int ntdec_r, nrep;
    unsigned int* rep;     // (nrep, 3) float bits of max |V|
    const int* it;
};

// m_kernel.f90:350-374 (+ the NaN check the report's divergence test implies)
__device__ __forceinline__ void vmax_block(const VmaxArgs& a) {
    const int it = *a.it;
    if (a.ntdec_r <= 0 || it % a.ntdec_r != 0) return;
    const int r = it / a.ntdec_r - 1;
    if (r >= a.nrep) return;
    float m[3] = {0.f, 0.f, 0.f};
    const int ni = a.i1 - a.i0 + 1, nj = a.j1 - a.j0 + 1;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ni * nj; p += gridDim.x * blockDim.x) {
        int i = a.i0 + p % ni, j = a.j0 + p / ni;
        int kz = a.kob[j * a.g.nx + i];  // kob + 1 (1-based) == kob (0-based)
        for (int c = 0; c < 3; ++c) {
            float v = fabsf(a.V[goff(a.g, 3, c, i, j, kz)]);
            if (v != v) v = __int_as_float(0x7fc00000);
            m[c] = (v != v || v > m[c]) ? v : m[c];
        }
    }
    for (int c = 0; c < 3; ++c) {
        float v = m[c];
        for (int o = 16; o > 0; o >>= 1) {
            float w = __shfl_xor_sync(0xffffffffu, v, o);
            v = (w != w || w > v) ? w : v;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(a.rep + 3 * r + c, __float_as_uint(v));
    }
}

__global__ void k_vmax(const VmaxArgs a) { vmax_block(a); }
__global__ void k_vmax_batch(const VmaxArgs* __restrict__ all) { vmax_block(all[blockIdx.y]); }

__global__ void k_set_it(int* it, int v) { *it = v; }
__global__ void k_advance(int* it) { *it += 1; }
__global__ void k_advance_batch(int* const* __restrict__ its, int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) *its[q] += 1;
}

// Fortran (k,i,j) halo array -> one field of a device group, as a tiled
// transpose: a block stages a 32 (k) x 32 (i) tile of one j row in shared
// memory, reading along k and writing along x, so that both the read and the
// write are coalesced.  cols_only leaves the x/y ghost columns untouched
// (every k of the halo range is written).  Grid (ceil((nz+6)/32),
// ceil((nx+6)/32), ny+6), block (32, 8).
__global__ void __launch_bounds__(256) k_scatter_t(const float* __restrict__ src, float* __restrict__ dst, Geo g, int nf,
                                                    int f, int cols_only) {
    __shared__ float t[32][33];
    const int nk = g.nz + 6, ni = g.nx + 6;
    const int k0 = blockIdx.x * 32, i0 = blockIdx.y * 32, jh = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        const int ih = i0 + r, kh = k0 + tx;
        if (ih < ni && kh < nk) t[r][tx] = src[((size_t)jh * ni + ih) * nk + kh];
    }
    __syncthreads();
    const int j = jh - 3;
    if (cols_only && (j < 0 || j >= g.ny)) return;
    for (int r = ty; r < 32; r += 8) {
        const int kh = k0 + r, ih = i0 + tx;
        if (kh >= nk || ih >= ni) continue;
        const int i = ih - 3;
        if (cols_only && (i < 0 || i >= g.nx)) continue;
        dst[goff(g, nf, f, i, j, kh - 3)] = t[tx][r];
    }
}

// Depth-only medium: five columns of nz + 6 values (k = -2 .. nz+3; rho lam
// mu taup taus) copied into every (i, j) of the halo grid of the M group,
// walking the destination in its own order (x fastest).
__global__ void k_spread_col(const float* __restrict__ col, float* __restrict__ M, Geo g) {
    const int nk = g.nz + 6, ni = g.nx + 6, nj = g.ny + 6;
    const long long n = (long long)nk * nj * 5 * ni;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const int ih = (int)(p % ni);
        long long q = p / ni;
        const int f = (int)(q % 5);
        q /= 5;
        const int jh = (int)(q % nj);
        const int kh = (int)(q / nj);
        M[goff(g, 5, f, ih - 3, jh - 3, kh - 3)] = col[f * nk + kh];
    }
}

// Plane-wave mode: the lateral ghost planes of every field of a group are
// extrapolated linearly from the two outermost cells before the PML update
// reads them (src/swpc_3d/m_absorb_p.f90:137-244 for S, 332-427 for V):
// x sides for j = 1..ny, y sides for i = 1..nx, k = 1..nz; corners untouched.
__host__ __device__ __forceinline__ long long pw_ghost_units(const Geo& g, int nf) {
    return (2LL * g.ny * g.nz + 2LL * g.nx * g.nz) * nf;
}
__device__ __forceinline__ void pw_ghost_unit(float* F, const Geo& g, int nf, long long p) {
    const long long nxs = (long long)g.ny * g.nz, nys = (long long)g.nx * g.nz;
    {
        const int f = (int)(p % nf);
        long long q = p / nf;
        int side;
        if (q < 2 * nxs) { side = (int)(q / nxs); q %= nxs; }
        else { q -= 2 * nxs; side = 2 + (int)(q / nys); q %= nys; }
        const int k = (int)(q % g.nz);
        const int t = (int)(q / g.nz);  // j for the x sides, i for the y sides (0-based)
        int gi, i1, i2, gj, j1, j2;
        switch (side) {
        case 0: gi = -1; i1 = 0; i2 = 1; gj = j1 = j2 = t; break;
        case 1: gi = g.nx; i1 = g.nx - 1; i2 = g.nx - 2; gj = j1 = j2 = t; break;
        case 2: gj = -1; j1 = 0; j2 = 1; gi = i1 = i2 = t; break;
        default: gj = g.ny; j1 = g.ny - 1; j2 = g.ny - 2; gi = i1 = i2 = t; break;
        }
        F[goff(g, nf, f, gi, gj, k)] = 2 * F[goff(g, nf, f, i1, j1, k)] - F[goff(g, nf, f, i2, j2, k)];
    }
}
__global__ void k_pw_ghost(float* F, Geo g, int nf) {
    const long long n = pw_ghost_units(g, nf);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        pw_ghost_unit(F, g, nf, p);
}

// one field of a device group -> Fortran (nz, nx, ny) physical-grid double
// array, as a tiled transpose (read along x, write along k).  Grid
// (ceil(nz/32), ceil(nx/32), ny), block (32, 8).
__global__ void __launch_bounds__(256) k_gather_d(const float* __restrict__ src, double* __restrict__ dst, Geo g, int nf,
                                                   int f) {
    __shared__ float t[32][33];
    const int k0 = blockIdx.x * 32, i0 = blockIdx.y * 32, j = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, i = i0 + tx;
        if (k < g.nz && i < g.nx) t[r][tx] = src[goff(g, nf, f, i, j, k)];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, k = k0 + tx;
        if (k < g.nz && i < g.nx) dst[((size_t)j * g.nx + i) * g.nz + k] = (double)t[tx][r];
    }
}

}  // namespace swpc
