/*
 * swpc_gpu.h -- C ABI of the GB300-native swpc_3d time-stepping library.
 *
 * This ABI replaces the zero-argument step routines that swpc_3d's driver
 * loop calls (src/swpc_3d/main.f90:119-139) and the module arrays they
 * communicate through (src/swpc_3d/m_global.f90:34-41, 86, 93-98).  A host
 * that keeps the reference's set-up chain (m_global / m_medium / m_source /
 * m_wav / m_snap, main.f90:64-78) hands the prepared arrays to this library
 * once, then calls swpc_gpu_run() in place of the loop.  Every entry point
 * returns 0 on success or a negative code (SWPC_E_*); the message of the
 * last failure is available from swpc_gpu_last_error().  Nothing throws
 * across the ABI and nothing calls exit().
 *
 * Array conventions (all host pointers; every call copies):
 *   3-D medium arrays use the reference's Fortran layout A(k,i,j), k fastest,
 *   with the 3-cell halo k in [-2,nz+3], i in [-2,nx+3], j in [-2,ny+3]
 *   (m_global.f90:295-300 for one rank): (nz+6)*(nx+6)*(ny+6) floats.
 *   2-D maps M(i,j) use i in [-2,nx+3], j in [-2,ny+3]: (nx+6)*(ny+6) ints.
 *   Grid indices (sources, stations, snapshot planes) are the reference's
 *   1-based i, j, k.
 */
#ifndef SWPC_GPU_H
#define SWPC_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct swpc_sim swpc_sim;

enum {
    SWPC_OK = 0,
    SWPC_E_ARG = -1,       /* invalid argument or unsupported option */
    SWPC_E_CUDA = -2,      /* CUDA runtime failure (message has the CUDA error) */
    SWPC_E_NOMEM = -3,     /* device allocation failed or exceeds the budget */
    SWPC_E_STATE = -4,     /* call out of order (e.g. run before upload) */
    SWPC_E_DIVERGED = -5,  /* max |V| * UC > 1e5 or NaN (m_report.f90:142-151) */
    SWPC_E_IO = -6,        /* file could not be read or written */
    SWPC_E_TIMEOUT = -7    /* a bounded device wait gave up */
};

enum { SWPC_ABC_PML = 0, SWPC_ABC_CERJAN = 1 };

/* Storage precision of the memory variables and medium coefficients.
 * Arithmetic is FP32 in every mode. */
enum { SWPC_STORE_FP32 = 0, SWPC_STORE_FP16 = 1, SWPC_STORE_BF16 = 2 };

/* Receiver outputs (m_wav.f90:31-34) */
enum { SWPC_WAV_V = 1, SWPC_WAV_U = 2, SWPC_WAV_STRESS = 4, SWPC_WAV_STRAIN = 8 };

/* xy-section snapshot kinds of swpc_gpu_set_snapshot (m_snap.f90:105-119) */
enum { SWPC_SNAP_XY_V = 1, SWPC_SNAP_XY_U = 2 };

/* Snapshot sections and kinds of swpc_gpu_add_snapshot (m_snap.f90:105-119):
 * xy at k0_xy, yz at i0_yz, xz at j0_xz, fs at kfs+1 and ob at kob+1 of
 * every column; velocity, displacement, divergence/rotation ("ps"). */
enum { SWPC_SEC_XY = 0, SWPC_SEC_YZ = 1, SWPC_SEC_XZ = 2, SWPC_SEC_FS = 3, SWPC_SEC_OB = 4 };
enum { SWPC_SNAPK_V = 0, SWPC_SNAPK_U = 1, SWPC_SNAPK_PS = 2 };

/* Source time functions (m_fdtool.f90:472-497) */
enum { SWPC_STF_BOXCAR = 0, SWPC_STF_TRIANGLE = 1, SWPC_STF_HERRMANN = 2,
       SWPC_STF_KUPPER = 3, SWPC_STF_COSINE = 4, SWPC_STF_TEXP = 5 };

typedef struct swpc_dims {
    int nx, ny, nz;      /* global grid (m_global.f90:52) */
    int nt;              /* number of time steps (sizes the receiver buffers) */
    int na;              /* absorber thickness in cells */
    int nm;              /* Zener bodies; must be 3 (m_global.f90:31) */
    int abc_type;        /* SWPC_ABC_PML or SWPC_ABC_CERJAN */
    int store;           /* SWPC_STORE_* */
    double dx, dy, dz;   /* grid spacing [km] (real(MP) in m_global.f90:54) */
    double dt;           /* time step [s] */
    double xbeg, ybeg, zbeg, tbeg;
    double fcut;         /* PML a0 = pi * fcut (m_absorb_p.f90:554; fcut from m_source.f90:184-188) */
    double M0;           /* total moment (m_source.f90:190-198) */
    double UC;           /* unit conversion (m_global.f90:29; x1e3 in body-force mode) */
    int ntdec_r;         /* divergence-check interval (m_report.f90:134); 0 = off */
    int reserved[7];     /* 0 (all zero: library defaults); [0] 1 = interior kernels without TMA,
                            [1] 1/2 = PML kernels in series/beside the interior ones,
                            [2] 2 = two PML shell points per thread (0 or 1: one),
                            [3] 2 = the TMA tile kernels sweep the PML shell too (interior
                            kernels over the tiles inside the interior, shell-tile kernels over
                            the rest; 0 or 1: the shell in launches of its own) */
} swpc_dims;

/* Create a simulation and allocate its device state on the current CUDA
 * device.  Replaces kernel__setup's memory_allocate (m_kernel.f90:376-400)
 * and absorb_p__setup's ADE allocation (m_absorb_p.f90:98-116). */
int swpc_gpu_create(const swpc_dims* dims, swpc_sim** out);

/* Device bytes swpc_gpu_create() would allocate for these dims (no GPU call). */
long long swpc_gpu_required_bytes(const swpc_dims* dims);

/* Upload the prepared medium: rho, lam, mu (relaxed moduli) and the tau-method
 * ratios taup, taus after medium__setup (m_medium.f90:192-229), the surface
 * maps of surface_detection (m_medium.f90:339-394), and the nm relaxation
 * times ts (m_fdtool.f90:691-727).  The library derives the Zener
 * coefficients (m_kernel.f90:58-67) and the PML or Cerjan profiles
 * (m_absorb_p.f90:74-93, m_absorb_c.f90:27-111) in FP64 here.  Arrays in
 * pinned (page-locked) host memory are read by the device directly over the
 * CPU-GPU link; other memory is staged through a device copy.  Either way
 * the call returns after the arrays have been read. */
int swpc_gpu_upload_medium(swpc_sim* sim, const float* rho, const float* lam, const float* mu,
                           const float* taup, const float* taus,
                           const int* kfs, const int* kob, const int* kfs_top, const int* kfs_bot,
                           const int* kob_top, const int* kob_bot, const double* ts);

/* The same upload for a medium that depends on depth only (the uni, lhm
 * and lgm models of m_vmodel_*): rho .. taus are single columns of nz+6
 * values (k = -2 .. nz+3) after the medium post-processing, which the device
 * copies into every (i, j); the surface maps are full 2-D arrays as above.
 * Spares the host building and sending nx*ny copies of the column. */
int swpc_gpu_upload_medium_column(swpc_sim* sim, const float* rho, const float* lam, const float* mu,
                                  const float* taup, const float* taus,
                                  const int* kfs, const int* kob, const int* kfs_top, const int* kfs_bot,
                                  const int* kob_top, const int* kob_bot, const double* ts);

/* The medium of a layered model with a random perturbation built on the
 * device (vmodel_lhm_rmed / vmodel_lgm_rmed, src/swpc_3d/m_vmodel_lhm_rmed.f90:
 * 21-229, followed by medium__setup, m_medium.f90:124-394), in place of
 * building the halo arrays on the host and uploading them.
 *   bg:  5 x (nz+6) floats, the background column at k = -2 .. nz+3:
 *        rho0, vp0, vs0, Qp, Qs (layers or gradients as the host reads them).
 *   xi:  the perturbation, nzc planes of nyc rows of nxc values (x fastest),
 *        repeated periodically over the grid as src/shared/m_rdrmed.f90:73-134
 *        wraps a field smaller than the grid.
 *   kxi0: first 1-based k of the solid; cells above keep the column (air,
 *        water).  Below: rho = rho0 (1 + 0.8 xi), vp = vp0 (1 + xi),
 *        vs = vs0 (1 + xi), kept inside [vmin, vmax] and above rhomin by
 *        vcheck (src/shared/m_fdtool.f90:15-48).
 * The device then homogenises the absorber band, applies the tau-method,
 * relaxes the moduli to fq_ref in FP64, finds the free surface and ocean
 * bottom of every column and sets the coefficients as swpc_gpu_upload_medium
 * does; the result equals host set-up (swpc_host_medium) of the same cells
 * bit for bit.  maps6 (optional) receives the six surface maps kfs, kob,
 * kfs_top, kfs_bot, kob_top, kob_bot, each (nx+6) x (ny+6) ints as in
 * swpc_gpu_upload_medium, for placing stations and sources on the host; ts
 * receives the nm relaxation times.  Host traffic: the column and the field
 * instead of five full halo arrays. */
int swpc_gpu_build_medium_rmed(swpc_sim* sim, const float* bg, const float* xi, int nxc, int nyc, int nzc, int kxi0,
                               double vmin, double vmax, double rhomin, double fq_min, double fq_max, double fq_ref,
                               int* maps6, double* ts);

/* Sources (replaces source__stressglut / source__bodyforce state,
 * m_source.f90:26-36).  ijk: 3n grid indices.  mo: n normalised moments
 * (mo/M0).  mij: 6n components xx yy zz yz xz xy.  fxyz: 3n normalised body
 * forces.  prm: 2n (start time, rise time).  bf_mode selects body force. */
int swpc_gpu_set_sources(swpc_sim* sim, int n, const int* ijk, const double* mo, const double* mij,
                         const double* fxyz, const double* prm, int stftype, int bf_mode);

/* Receivers (m_wav.f90:54-139): n stations at ijk (3n), sampled every
 * ntdec_w steps; flags is a mask of SWPC_WAV_*. */
int swpc_gpu_set_receivers(swpc_sim* sim, int n, const int* ijk, int ntdec_w, int flags);

/* xy-section snapshot (m_snap.f90:95-160, 1587-1653, 1963-2025): plane k0,
 * decimation idec/jdec, every ntdec_s steps; kinds is a mask of SWPC_SNAP_*. */
int swpc_gpu_set_snapshot(swpc_sim* sim, int kinds, int k0, int idec, int jdec, int ntdec_s);

/* Any of the fifteen snapshots of m_snap.f90 (wbuf_{xy,yz,xz,fs,ob}_{v,u,ps},
 * :981-2205): section SWPC_SEC_*, kind SWPC_SNAPK_*, fix = the 1-based k0
 * (xy), i0 (yz) or j0 (xz) (ignored for fs/ob), decimation along the
 * section's first and second axis (xy/fs/ob: idec, jdec; yz: jdec, kdec;
 * xz: idec, kdec), frames at it = 1, 1+ntdec_s, ... (every snapshot shares
 * ntdec_s).  A frame holds nc planes of (n1, n2) floats: nc = 3 (Vx Vy Vz,
 * Ux Uy Uz) or 4 (div, rot_x, rot_y, rot_z), scaled as the reference
 * writes them.  Adding the same section and kind again replaces it. */
int swpc_gpu_add_snapshot(swpc_sim* sim, int section, int kind, int fix, int dec1, int dec2, int ntdec_s);
int swpc_gpu_query_snapshot(swpc_sim* sim, int section, int kind, int* n1, int* n2, int* nframes);
int swpc_gpu_fetch_section(swpc_sim* sim, int section, int kind, int frame, float* out);

/* Overwrite one state field (which = 0..8 for Vx Vy Vz Sxx Syy Szz Syz Sxz
 * Sxy) from a Fortran halo array A(k,i,j) (the layout of the medium arrays):
 * every cell of the physical columns, including the z halo planes; the x/y
 * ghost columns stay zero.  Used for the plane-wave initial condition
 * (pw_setup, m_source.f90:316-466). */
int swpc_gpu_set_field(swpc_sim* sim, int which, const float* field);

/* Plane-wave mode (pw_mode): before each PML update the lateral ghost
 * planes are extrapolated linearly from the two outermost cells
 * (m_absorb_p.f90:137-244, 332-427).  Needs the PML absorber. */
int swpc_gpu_set_plane_wave(swpc_sim* sim, int on);

/* Reciprocal Green's-function taps (green__store, m_green.f90:406-551): n
 * grid points at 1-based ijk (3n); every ntdec_w steps the combinations
 * dxUx, dyUy, dzUz, dyUz+dzUy, dxUz+dzUx, dxUy+dyUx of the time-integrated
 * displacement gradients (scaled by 1e-15 * 1e9) and, with bforce, the
 * displacement Ux, Uy, Uz (scaled by 1e-12 * 1e9).  The pseudo source is an
 * ordinary body-force source (swpc_gpu_set_sources, bf_mode = 1). */
int swpc_gpu_set_green(swpc_sim* sim, int n, const int* ijk, int ntdec_w, int bforce);
/* Green's-function traces (ntw, ncmp, n) in Fortran order; with out null
 * only *n, *ncmp and *ntw are set. */
int swpc_gpu_fetch_green(swpc_sim* sim, float* out, int* n, int* ncmp, int* ntw);

/* One time step it (main.f90:120-138 minus host I/O). */
int swpc_gpu_step(swpc_sim* sim, int it);

/* Steps it0..it1 inclusive, replayed through a captured CUDA graph. */
int swpc_gpu_run(swpc_sim* sim, int it0, int it1);

/* Block until the simulation's stream is idle; checks divergence. */
int swpc_gpu_sync(swpc_sim* sim);

/* Receiver traces, Fortran order (ntw, ncmp, nst); kind is one SWPC_WAV_*
 * bit; ncmp = 3 for V/U, 6 for stress/strain (m_wav.f90:105-123). */
int swpc_gpu_fetch_waveforms(swpc_sim* sim, int kind, float* out);

/* Snapshot frame `frame` (0-based) of one kind: (nxs, nys, 3) Fortran order. */
int swpc_gpu_fetch_snapshot(swpc_sim* sim, int kind, int frame, float* out);

/* Number of samples per trace and snapshot geometry. */
int swpc_gpu_query(swpc_sim* sim, int* ntw, int* nst, int* nxs, int* nys, int* nframes);

/* Max |V| at kob+1 (kernel__vmax, m_kernel.f90:350-374) for the latest
 * report step, already multiplied by UC * M0 as the progress line prints it. */
int swpc_gpu_vmax(swpc_sim* sim, float out[3]);

/* One state field over the physical grid, Fortran (nz, nx, ny) order, as
 * double: which = 0..8 for Vx Vy Vz Sxx Syy Szz Syz Sxz Sxy, 9..13 for the
 * uploaded medium rho lam mu taup taus. */
int swpc_gpu_fetch_field(swpc_sim* sim, int which, double* out);

/* The read-back of swpc_gpu_fetch_field for the nine wavefields only
 * (which = 0..8, Vx .. Sxy; the medium fields 9..13 are refused with
 * SWPC_E_ARG), for callers that cannot allocate device memory (a host whose
 * device is fully committed under an HBM budget, or whose allocator forbids
 * side allocations).  No counterpart in the reference.  It calls no
 * cudaMalloc/cudaFree: the gather goes through a fixed 32 MiB scratch array
 * in the library image that every GPU loading the library holds until exit.
 * Grids above SWPC_STATIC_FIELD_MAX points are rejected with SWPC_E_ARG.  The
 * first call for a device looks the array up on the simulation's device;
 * make it before any stream capture.  All calls share the one array: calls
 * that overlap on the GPU (from different threads or streams) race. */
#define SWPC_STATIC_FIELD_MAX (4 * 1024 * 1024)
int swpc_gpu_fetch_field_static(swpc_sim* sim, int which, double* out);

/* Optional per-kernel timing with CUDA events on the simulation's stream:
 * enable = 1 records every launch of the interior and PML kernels (graph
 * replay is bypassed while enabled).  ms[0..5] = accumulated milliseconds of
 * stress-interior, velocity-interior, stress-PML, velocity-PML, taps,
 * sources; launches[0..5] the matching counts. */
int swpc_gpu_profile(swpc_sim* sim, int enable);
int swpc_gpu_profile_read(swpc_sim* sim, double* ms, long long* launches);
/* The PML time of swpc_gpu_profile_read split by launch class (the shell
 * parts damped along x only, y only, z only, and the rest): ms[0..3] and
 * launches[0..3] for the stress update, ms[4..7] and launches[4..7] for the
 * velocity update; points[0..3] the shell points of each class and
 * axis_points[0..3] the sum over those points of the number of damped axes
 * (each damped axis keeps three stress and three velocity auxiliaries per
 * point, m_absorb_p.f90:99-116).  A small shell runs as one launch of the
 * last class.  No counterpart in the reference. */
int swpc_gpu_profile_read_pml(swpc_sim* sim, double* ms, long long* launches, long long* points,
                              long long* axis_points);

/* The cudaStream_t the simulation launches on (as void*). */
void* swpc_gpu_stream(swpc_sim* sim);

/* Number of this library's kernels launched since creation. */
long long swpc_gpu_launch_count(swpc_sim* sim);

int swpc_gpu_destroy(swpc_sim* sim);

/* Self-test of the bounded device waits used by the TMA kernels: launches
 * one block that waits on a barrier nothing completes.  Returns
 * SWPC_E_TIMEOUT when the wait gave up and reported, as designed (0 would
 * mean the barrier completed, which cannot happen); *seconds receives how
 * long the wait took.  The device stays usable afterwards.  No counterpart
 * in the reference. */
int swpc_gpu_selftest_wait(double* seconds);

/* The dims the simulation was created with. */
int swpc_gpu_get_dims(swpc_sim* sim, swpc_dims* out);

/* Return the simulation to its initial state (all wavefields, memory
 * variables, PML auxiliaries, receiver and snapshot buffers zero; next step
 * is it = 1) while keeping medium, sources, receivers and snapshot set-up.
 * Used by the autotuner, which times steps on the real simulations. */
int swpc_gpu_reset(swpc_sim* sim);

/* z-sweep depth (planes per block) of the interior stress and velocity
 * kernels; 0 restores the automatic choice (at most 6 planes for the stress
 * kernel with FP32 memory variables, 32 with 16-bit ones, 96 for the
 * velocity kernel, fewer when the grid is too small to fill the GPU).  The autotuner (openswpc_gb300/autotune.py) sets them.
 * set_zchunk sets both to one depth; get_zchunk returns the stress depth. */
int swpc_gpu_set_zchunks(swpc_sim* sim, int kstress, int kvel);
/* Tile shape of the interior stress and velocity kernels: 32 columns by 8
 * (default) or 16 rows each, or 12 rows for the velocity kernels; with
 * 8-row tiles two stress blocks or three velocity blocks share an SM, with
 * 12-row velocity tiles two, with 16-row tiles one (fewer halo rows per
 * point, fewer blocks); 0 restores 8.  The autotuner sets them together with
 * the z-sweep depths.  Batched members must share their tile shapes, and the
 * persistent batch form runs 8-row tiles.  No counterpart in the reference. */
int swpc_gpu_set_tiles(swpc_sim* sim, int rows_stress, int rows_vel);
int swpc_gpu_get_tiles(swpc_sim* sim, int* rows_stress, int* rows_vel);

/* 1 when the simulation's TMA tile kernels sweep the PML shell too
 * (swpc_dims.reserved[3] = 2 with a PML and the TMA kernels: per phase one
 * launch over the tiles inside the interior and one over the tiles that
 * hold shell points), 0 when the shell runs in launches of its own; < 0 on a
 * bad handle.  Either form gives the same bits (absorb_p__update_stress /
 * __update_vel of m_absorb_p.f90:246-317, 429-531). */
int swpc_gpu_pml_fused(swpc_sim* sim);
int swpc_gpu_get_zchunks(swpc_sim* sim, int* kstress, int* kvel);
int swpc_gpu_set_zchunk(swpc_sim* sim, int kchunk);
int swpc_gpu_get_zchunk(swpc_sim* sim);

/* ------------------------------------------------------------------------
 * Batched form: n independent simulations (same storage precision, medium
 * uploaded) advanced together, one fused launch per phase of the time step,
 * replayed through a CUDA graph.  No counterpart in the reference, which runs
 * one simulation per process; it replaces running the reference once per
 * input file (e.g. the Green's-function runs of example/green/).  Each
 * member continues from its own next step; members keep their own receivers,
 * snapshots and divergence checks.  Destroying the batch leaves the members.
 * ---------------------------------------------------------------------- */
typedef struct swpc_batch swpc_batch;
int swpc_batch_create(swpc_sim* const* sims, int n, swpc_batch** out);
int swpc_batch_run(swpc_batch* batch, int nsteps);
int swpc_batch_sync(swpc_batch* batch);
/* How the batch advances a time step.  on = 1: one persistent fused launch
 * per time step; resident blocks take every member's stress tiles, PML
 * blocks, sources, velocity tiles, taps and snapshots from a device work
 * queue in phase order, each item waiting (bounded) until the items of its
 * member it depends on are done (8-row tiles only).  on = 0 (the default):
 * one launch per phase of the step over a block table spanning all members.
 * Both give the same results bit for bit.  No counterpart in the reference. */
int swpc_batch_set_persistent(swpc_batch* batch, int on);
/* Items in the persistent form's work queue for one time step. */
int swpc_batch_item_count(swpc_batch* batch);
void* swpc_batch_stream(swpc_batch* batch);
long long swpc_batch_launch_count(swpc_batch* batch);
int swpc_batch_destroy(swpc_batch* batch);

/* Copy the last error message into buf; returns its length. */
int swpc_gpu_last_error(char* buf, size_t n);

/* ------------------------------------------------------------------------
 * Host driver layer: reads the reference's input files and performs the
 * reference's host-side set-up (m_global, m_medium, m_source, m_wav, m_snap
 * set-up routines) in FP64, then creates and uploads the simulation.
 * ---------------------------------------------------------------------- */

/* Parse input.inf (and the files it names) and return a ready simulation.
 * Relative file names in input.inf are resolved against the directory of
 * inf_path. */
int swpc_host_prepare(const char* inf_path, swpc_sim** out);

/* Two-phase form of swpc_host_prepare, for callers that decide when a
 * simulation may take device memory (the serving loop below):
 * swpc_host_load runs the whole host set-up (medium, sources, stations) and
 * touches no GPU; swpc_host_request_bytes gives the device bytes the
 * simulation will hold; swpc_host_materialize creates and uploads it (the
 * request can be materialised more than once); swpc_host_request_free
 * releases the host copy.  Together they equal swpc_host_prepare
 * (src/swpc_3d/main.f90:48-117). */
typedef struct swpc_request swpc_request;
int swpc_host_load(const char* inf_path, swpc_request** out);
long long swpc_host_request_bytes(const swpc_request* req);
int swpc_host_request_dims(const swpc_request* req, swpc_dims* out);
int swpc_host_materialize(const swpc_request* req, swpc_sim** out);
int swpc_host_request_free(swpc_request* req);

/* Run the whole host set-up of swpc_host_prepare without touching a GPU and
 * write a JSON summary (grid, M0, fcut, relaxation times, source and station
 * grid indices) into summary.  Returns the summary length or a negative
 * error code. */
int swpc_host_check(const char* inf_path, char* summary, size_t n);

/* Number of time steps nt read from input.inf by swpc_host_prepare (0 if the
 * simulation was not made by it). */
int swpc_host_nt(swpc_sim* sim);

/* Progress-report interval ntdec_r read from input.inf (report__setup,
 * src/swpc_3d/m_report.f90:47, default 10); 0 if the simulation was not
 * made by swpc_host_prepare. */
int swpc_host_ntdec_r(swpc_sim* sim);

/* The run banner of report__setup (src/swpc_3d/m_report.f90:64-88): grid,
 * MPI partitioning of input.inf, memory estimate (memory_size_3d,
 * src/shared/m_fdtool.f90:137-187), stability number c and wavelength
 * number r (m_fdtool.f90:81-134) from the velocity range of the processed
 * medium (velocity_minmax, m_medium.f90:396-427) and the maximum
 * frequency, formatted as the reference prints it.  Copies the text into
 * buf and returns its length. */
int swpc_host_banner(swpc_sim* sim, char* buf, size_t n);

/* Medium post-processing of medium__setup (m_medium.f90:124-394) in FP64 for
 * hosts that bring their own velocity model.  On entry rho, lam, mu, qp_taup
 * and qs_taus hold density, unrelaxed moduli and Qp, Qs over the halo grid;
 * on return the absorber band is homogenised, lam/mu are relaxed to fq_ref,
 * qp_taup/qs_taus hold the tau-method ratios, the six surface maps are
 * filled and ts[3] holds the relaxation times.  Host memory only. */
int swpc_host_medium(int nx, int ny, int nz, int na, double fq_min, double fq_max, double fq_ref,
                     float* rho, float* lam, float* mu, float* qp_taup, float* qs_taus,
                     int* kfs, int* kob, int* kfs_top, int* kfs_bot, int* kob_top, int* kob_bot, double* ts);

/* Write the receiver traces as SAC files named
 * odir/wav/<title>.3d.<station>.<cmp>.sac (m_wav.f90:782-792). */
int swpc_host_write_sac(swpc_sim* sim, const char* odir);

/* Green's-function mode (green_mode = .true.): write the traces of every
 * point of fn_glst as SAC files odir/green/<stnm>/<title>__<id8>__<stnm>__
 * <cmp>__<mxx..fz_>__.sac or as one CSF file (wav_format = 'csf'), with the
 * headers of green__setup and the sign flip of a vertical force
 * (green__export, m_green.f90:318-398, 553-612).  Does nothing outside that
 * mode. */
int swpc_host_write_green(swpc_sim* sim, const char* odir);

/* Write the xy-section snapshots as the reference's native .snp files
 * odir/<title>.3d.xy.v.snp and .xy.u.snp: header version 6
 * (m_snap.f90:846-892), the rho/lam/mu planes at k0_xy and the topography
 * (newfile_xy, m_snap.f90:413-473), then one (nxs, nys) plane per component
 * per frame (wbuf_xy_v / wbuf_xy_u, m_snap.f90:1587-1653, 1963-2025).
 * Does nothing when the input asked for no xy snapshot. */
int swpc_host_write_snp(swpc_sim* sim, const char* odir);

/* ------------------------------------------------------------------------
 * Serving form: a request loop with continuous batching.  No counterpart in
 * the reference (one simulation per mpiexec).  Requests are input.inf paths;
 * host threads run their set-up as they arrive, a request takes device memory
 * only once the admitted simulations leave room for it inside hbm_budget
 * (first come, first served), and every admitted simulation is advanced by
 * one batched launch sequence per quantum of time steps.  Between quanta the
 * finished simulations hand back their receiver traces and free their memory,
 * and the requests that became ready join the batch, so new work overlaps
 * the work already on the GPU.  Wavefields stay resident from admission to
 * completion.  All functions are thread-safe.
 * ---------------------------------------------------------------------- */
typedef struct swpc_server swpc_server;
typedef struct {
    double hbm_budget;  /* device bytes the admitted simulations may hold (0: 80% of free memory) */
    int max_active;     /* most simulations advanced together (0: 128) */
    int quantum;        /* time steps between scheduling points (0: 50) */
    int prep_threads;   /* host threads running request set-up (0: 4) */
    int write_sac;      /* 1: also write each request's SAC files into its odir */
    int reserved[8];
} swpc_serve_config;

enum { SWPC_REQ_QUEUED = 0, SWPC_REQ_LOADING = 1, SWPC_REQ_WAITING = 2, SWPC_REQ_RUNNING = 3, SWPC_REQ_DONE = 4 };

int swpc_serve_create(const swpc_serve_config* cfg, swpc_server** out);
/* Queue one input.inf; *id identifies the request from then on. */
int swpc_serve_submit(swpc_server* srv, const char* inf_path, long long* id);
/* State of a request: SWPC_REQ_* or the negative error code it failed with. */
int swpc_serve_state(swpc_server* srv, long long id);
/* Block until the request is done or failed, or timeout_s passes (< 0: no
 * limit); returns its state. */
int swpc_serve_wait(swpc_server* srv, long long id, double timeout_s);
/* Receiver traces of a finished request in the layout of
 * swpc_gpu_fetch_waveforms (Fortran order (ntw, ncmp, nst)); with buf null
 * only *nst and *ntw are set.  n_floats is the room in buf. */
int swpc_serve_result(swpc_server* srv, long long id, int kind, float* buf, size_t n_floats, int* nst, int* ntw);
/* Error message of a failed request; returns its length. */
int swpc_serve_error(swpc_server* srv, long long id, char* buf, size_t n);
/* Server-clock seconds at submission, admission (device memory granted),
 * first time step and completion. */
int swpc_serve_times(swpc_server* srv, long long id, double* t4);
/* Forget a finished request and its traces. */
int swpc_serve_release(swpc_server* srv, long long id);
/* Block until every submitted request is done or failed. */
int swpc_serve_drain(swpc_server* srv);
/* st[0..9]: done, failed, running, waiting or loading, queued, device bytes
 * granted, peak device bytes granted, quanta run, batch rebuilds, grid-point
 * updates performed. */
int swpc_serve_stats(swpc_server* srv, double* st);
int swpc_serve_destroy(swpc_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* SWPC_GPU_H */
