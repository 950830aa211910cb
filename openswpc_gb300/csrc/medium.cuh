// medium.cuh -- the medium set-up of a layered model with a random
// perturbation, on the device.
//
// vmodel_lhm_rmed / vmodel_lgm_rmed (src/swpc_3d/m_vmodel_lhm_rmed.f90:21-229)
// build every cell from a background column (layers or gradients) and a
// perturbation field xi that repeats periodically over the grid
// (src/shared/m_rdrmed.f90:73-134): rho = rho0 (1 + 0.8 xi), vp = vp0 (1 + xi),
// vs = vs0 (1 + xi), kept inside [vmin, vmax] and above rhomin by vcheck
// (src/shared/m_fdtool.f90:15-48).  medium__setup (src/swpc_3d/m_medium.f90)
// then homogenises the absorber band (:124-190), applies the tau-method
// (:192-207) and relaxes the moduli to fq_ref (:231-271, in FP64), and finds
// the free surface and the ocean bottom of every column (:339-394).
//
// Here one thread builds one cell from the column and the field (the band
// copies become a clamp of the cell index), post-processes it in FP64 with
// the column's tau-method ratios and relaxation factors (Q depends on depth
// only) and writes the medium group; two more kernels detect the surfaces
// and their 6 x 6 ranges.  Single-precision steps use explicitly rounded operations in
// the reference's order and the FP64 steps the sequence of visco.hpp, so the
// result equals the host set-up bit for bit.
#pragma once
#include "kernels.cuh"

namespace swpc {

struct RmedArgs {
    Geo g;
    float* M;           // medium group: rho lam mu taup taus
    const float* bg;    // 5 x (nz+6): rho0 vp0 vs0 qp0 qs0 at k = -2 .. nz+3
    const float* xi;    // nzc x nyc x nxc, x fastest
    int nxc, nyc, nzc;
    int kxi0;           // the perturbation applies from this 1-based k down (the solid below the topography)
    int na;
    float vmin, vmax, rhomin;
    // per k of the column (Q depends on depth only): the tau-method ratios
    // and 1 / chi^2 of mu and of lambda + 2 mu, in FP64 (visco.hpp)
    const double* kq;   // 4 x (nz+6): taup, taus, 1/chi_mu^2, 1/chi_lam^2
};

// 0-based index of the periodic field for a 1-based grid index
__device__ __forceinline__ int rmed_wrap(int i, int n) {
    int r = (i - 1) % n;
    return r < 0 ? r + n : r;
}

// vcheck of src/shared/m_fdtool.f90:15-48 in single precision
__device__ __forceinline__ void rmed_vcheck(float& vp, float& vs, float& rho, float xi, float vmin, float vmax,
                                            float rhomin) {
    float gamma = __fdiv_rn(vp, vs);
    if (gamma < 1.1920928955078125e-07f) gamma = 1.7320508075688772f;  // sqrt(3.)
    if (vp > vmax || vs > vmax) {
        const float xi2 = __fsub_rn(__fdiv_rn(__fmul_rn(__fadd_rn(1.f, xi), vmax), vp), 1.f);
        vp = vmax;
        vs = __fdiv_rn(vmax, gamma);
        rho = __fdiv_rn(__fmul_rn(rho, __fadd_rn(1.f, __fmul_rn(0.8f, xi2))), __fadd_rn(1.f, __fmul_rn(0.8f, xi)));
    }
    if (vp < vmin || vs < vmin) {
        vs = vmin;
        vp = __fmul_rn(vmin, gamma);
    }
    if (rho < rhomin) rho = rhomin;
}

// every cell of the halo grid, x fastest
__global__ void k_rmed_medium(const RmedArgs a) {
    const Geo& g = a.g;
    const int ni = g.nx + 6, nj = g.ny + 6, nk = g.nz + 6;
    const long long n = (long long)ni * nj * nk;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const int ih = (int)(p % ni);
        const long long q = p / ni;
        const int jh = (int)(q % nj), kh = (int)(q / nj);
        const int i = ih - 2, j = jh - 2, k = kh - 2;  // 1-based halo indices
        // the absorber band holds the medium of its inner edge (m_medium.f90:124-190)
        const int ic = min(max(i, a.na + 1), g.nx - a.na), jc = min(max(j, a.na + 1), g.ny - a.na);
        const int kc = min(k, g.nz - a.na);
        const int kq = kc + 2;
        const float r0 = a.bg[kq], vp0 = a.bg[nk + kq], vs0 = a.bg[2 * nk + kq];
        float rho = r0, vp = vp0, vs = vs0;
        if (kc >= a.kxi0) {
            const float x = a.xi[((size_t)rmed_wrap(kc, a.nzc) * a.nyc + rmed_wrap(jc, a.nyc)) * a.nxc + rmed_wrap(ic, a.nxc)];
            const float one = __fadd_rn(1.f, x);
            rho = __fmul_rn(r0, __fadd_rn(1.f, __fmul_rn(0.8f, x)));
            vp = __fmul_rn(vp0, one);
            vs = __fmul_rn(vs0, one);
            if (vp0 > 0.f && vs0 > 0.f) rmed_vcheck(vp, vs, rho, x, a.vmin, a.vmax, a.rhomin);
        }
        const float mu = __fmul_rn(__fmul_rn(rho, vs), vs);
        const float lam = __fmul_rn(rho, __fsub_rn(__fmul_rn(vp, vp), __fmul_rn(__fmul_rn(2.f, vs), vs)));
        // tau-method and relaxation to fq_ref in FP64 (m_medium.f90:192-271)
        const int nk2 = nk;
        const double tp = a.kq[kq], tsv = a.kq[nk2 + kq], rcm = a.kq[2 * nk2 + kq], rcl = a.kq[3 * nk2 + kq];
        const double ra2 = __dadd_rn((double)lam, __dmul_rn(2.0, (double)mu));
        const double m2 = __dmul_rn((double)mu, rcm);
        const double l2 = __dsub_rn(__dmul_rn(ra2, rcl), __dmul_rn(2.0, m2));
        float* const M = a.M;
        M[goff(g, 5, 0, i - 1, j - 1, k - 1)] = rho;
        M[goff(g, 5, 1, i - 1, j - 1, k - 1)] = (float)l2;
        M[goff(g, 5, 2, i - 1, j - 1, k - 1)] = (float)m2;
        M[goff(g, 5, 3, i - 1, j - 1, k - 1)] = (float)tp;
        M[goff(g, 5, 4, i - 1, j - 1, k - 1)] = (float)tsv;
    }
}

// surface_detection (m_medium.f90:339-394): per column i = 0 .. nx+2,
// j = 0 .. ny+2 (1-based) the last k with |mu(k)| < eps < |mu(k+1)| (ocean
// bottom kob) and the same for lambda (free surface kfs); maps over the halo
// (nx+6) x (ny+6) with i fastest, 0 where there is none
__global__ void k_rmed_surface(const float* __restrict__ M, Geo g, int* kfs, int* kob) {
    const int ni = g.nx + 3, nj = g.ny + 3;  // i = 0 .. nx+2
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj) return;
    const int i = t % ni, j = t / ni;
    const float eps = 1.1920928955078125e-07f;
    int fs = 0, ob = 0;
    float lam0 = M[goff(g, 5, 1, i - 1, j - 1, 0)], mu0 = M[goff(g, 5, 2, i - 1, j - 1, 0)];
    for (int k = 1; k <= g.nz - 1; ++k) {
        const float lam1 = M[goff(g, 5, 1, i - 1, j - 1, k)], mu1 = M[goff(g, 5, 2, i - 1, j - 1, k)];
        if (fabsf(mu0) < eps && fabsf(mu1) > eps) ob = k;
        if (fabsf(lam0) < eps && fabsf(lam1) > eps) fs = k;
        lam0 = lam1;
        mu0 = mu1;
    }
    const size_t q = (size_t)(j + 2) * (g.nx + 6) + (i + 2);
    kfs[q] = fs;
    kob[q] = ob;
}

// kfs_top/bot, kob_top/bot over the 6 x 6 neighbourhood (i-2 .. i+3,
// j-2 .. j+3) of every physical column, clamped to 1 .. nz
__global__ void k_rmed_ranges(const int* __restrict__ kfs, const int* __restrict__ kob, Geo g, int* kft, int* kfb,
                              int* kot, int* kobb) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nx * g.ny) return;
    const int i = t % g.nx + 1, j = t / g.nx + 1;
    const int mx = g.nx + 6;
    int a = 1 << 30, b = -(1 << 30), c = 1 << 30, d = -(1 << 30);
    for (int jj = j - 2; jj <= j + 3; ++jj)
        for (int ii = i - 2; ii <= i + 3; ++ii) {
            const size_t q = (size_t)(jj + 2) * mx + (ii + 2);
            a = min(a, kfs[q]); b = max(b, kfs[q]);
            c = min(c, kob[q]); d = max(d, kob[q]);
        }
    const size_t q = (size_t)(j + 2) * mx + (i + 2);
    kft[q] = max(a - 2, 1); kfb[q] = min(b + 2, g.nz);
    kot[q] = max(c - 2, 1); kobb[q] = min(d + 2, g.nz);
}

// the interior band table and the clamped per-column kob and kfs of the
// time-step kernels, from the maps
__global__ void k_rmed_tables(const int* __restrict__ kfs, const int* __restrict__ kob, const int* __restrict__ kft,
                              const int* __restrict__ kfb, const int* __restrict__ kot, const int* __restrict__ kobb,
                              Geo g, int x0, int y0, int nxi, int nyi, int4* band, int* d_kob, int* d_kfs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int mx = g.nx + 6;
    if (t < nxi * nyi) {
        const int i = x0 + t % nxi + 1, j = y0 + t / nxi + 1;
        const size_t q = (size_t)(j + 2) * mx + (i + 2);
        band[t] = make_int4(kft[q], kfb[q], kot[q], kobb[q]);
    }
    if (t < g.nx * g.ny) {
        const int i = t % g.nx + 1, j = t / g.nx + 1;
        const size_t q = (size_t)(j + 2) * mx + (i + 2);
        d_kob[t] = max(0, min(g.nz - 1, kob[q]));
        d_kfs[t] = max(0, min(g.nz - 1, kfs[q]));
    }
}

}  // namespace swpc
