// sim.hpp -- per-simulation device state behind the swpc_sim handle.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/swpc_gpu.h"
#include "kernels.cuh"
#include "kernels_tma.cuh"

namespace swpc {

int set_err(int code, const std::string& msg);

// Geometry and sizes of one simulation's device state.
struct Plan {
    Geo g;
    bool pml;
    int x0, y0, nxi, nyi, nzi;  // viscoelastic interior box
    int rpitch, rbytes;
    long long nV, nS, nM, nR, nade, nshm, npml, bytes;
    PmlBox box[5];
    int nbox;
};

struct Sim {
    swpc_dims dims;
    Plan p;
    int device = 0;  // CUDA device the simulation was created on
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // PML shell kernels, joined back into `stream` every phase
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_fork2 = nullptr, ev_join2 = nullptr;
    bool concurrent = true;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 8;
    long long launches = 0, launches_per_graph = 0;
    std::vector<void*> allocs;

    float *V = nullptr, *S = nullptr, *M = nullptr;
    void* R = nullptr;
    int4* band = nullptr;
    float *adeV = nullptr, *adeS = nullptr;
    float* shm = nullptr;  // the shell's precomputed medium terms (k_shell_medium)
    float* cer = nullptr;
    int cer_off[6] = {0, 0, 0, 0, 0, 0};
    int* d_it = nullptr;
    int* d_kob = nullptr;
    int* d_kfs = nullptr;
    int* d_err = nullptr;   // set by a kernel whose bounded wait ran out
    Coef coef{};
    int kchunk = 1, kchunk_auto = 1;      // z-sweep depth of the stress kernels
    int kchunk_v = 1, kchunk_v_auto = 1;  // and of the velocity kernels
    int variant = 0;        // 0: TMA-fed interior kernels, 1: shared-memory sweep without TMA
    int ty_s = TTY, ty_v = TTY;  // tile rows of the stress and velocity TMA kernels (8 or 16)
    int pml_np = 0;              // shell points per thread of the PML kernels (2; 0 or 1: one)
    bool pml_fused = false;      // the TMA tile kernels sweep the PML shell (interior and shell-tile kernels)
    int shell_dlo[6] = {}, shell_dhi[6] = {};  // damped index runs of the six profiles (PmlShell::dlo, dhi)
    TArgs targs;            // tensor maps of the TMA kernels (64-byte aligned)
    size_t smem_stress = 0, smem_vel = 0;
    size_t smem_stress_sh = 0, smem_vel_sh = 0;  // shell-tile kernels (rings + staged auxiliaries)

    PArgs pml_args{};                 // pointers, profiles and boxes of the PML kernels
    PArgs pml_cls[PML_NCLASS]{};      // the same with the parts of each launch class
    PArgs pml_all{};                  // the same with the whole boxes, for one general launch
    bool pml_split = false;           // launch the classes separately
    SrcArgs src_args{};
    TapArgs tap_args{};
    SnapArgs snap_args{};
    GreenArgs green_args{};
    VmaxArgs vmax_args{};
    std::vector<unsigned int> rep_host;
    bool bf_mode = false, medium_ready = false, diverged = false, profiling = false;
    bool pw = false;        // plane-wave mode: extrapolate the lateral ghost planes before the PML updates
    int it_done = 0;

    struct Pending { int cls; cudaEvent_t a, b; };
    std::vector<cudaEvent_t> ev_pool;
    std::vector<Pending> pending;
    // timing classes: 0..5 as swpc_gpu_profile_read, then the PML launch
    // classes (PML_CLASS_MASK order) of the stress (6..9) and velocity
    // (10..13) updates
    static constexpr int NPROF = 6 + 2 * PML_NCLASS;
    double prof_ms[NPROF] = {};
    long long prof_n[NPROF] = {};
    // shell points of each PML launch class and the sum over them of the
    // number of damped axes (the auxiliaries kept per point)
    long long pml_pts[PML_NCLASS] = {}, pml_axpts[PML_NCLASS] = {};

    ~Sim();
    int dalloc(void** ptr, size_t bytes);
    int allocate();
    void plan_pml_parts(const std::vector<float>& prof);
    void launch_pml(bool stress, cudaStream_t st, bool timed = false);
    int upload_medium(const float* rho, const float* lam, const float* mu, const float* taup, const float* taus,
                      const int* kfs, const int* kob, const int* kfs_top, const int* kfs_bot, const int* kob_top,
                      const int* kob_bot, const double* ts, bool column);
    int finish_medium(const double* ts);
    int build_medium_rmed(const float* bg, const float* xi, int nxc, int nyc, int nzc, int kxi0, double vmin,
                          double vmax, double rhomin, double fq_min, double fq_max, double fq_ref, int* maps6,
                          double* ts);
    int set_sources(int n, const int* ijk, const double* mo, const double* mij, const double* fxyz, const double* prm,
                    int stftype, bool bf);
    int set_receivers(int n, const int* ijk, int ntdec_w, int flags);
    int add_snapshot(int sec, int kind, int fix, int d1, int d2, int ntdec_s);
    int set_green(int n, const int* ijk, int ntdec_w, int bforce);
    const SnapPlane* find_plane(int sec, int kind) const;
    int nframes_done() const;
    // shell_view: with pml_fused, the sweep over the whole grid (its x
    // origin moved left so that the interior starts on a tile boundary) for
    // the interior and shell-tile kernels; otherwise the interior box
    void fill_zargs(ZArgs& z, bool shell_view = true) const;
    int launch_step(bool timed);
    int ensure_graph();
    int check_divergence();
    cudaEvent_t get_event();
    int drain_events();
    int build_tensor_maps();
};

}  // namespace swpc
