/*
 * baorec_gb300.h — C ABI of the GB300 (sm_103a) BAO reconstruction library.
 *
 * Each entry point replaces one function of BAOrec.jl's reconstruction path;
 * the comment above it names the Julia method (file:line inside the BAOrec.jl
 * project) whose behaviour it reproduces.  A Julia package binds these with
 * `ccall`, Python with ctypes (baorec.jl_gb300/baorec/_lib.py).
 *
 * Conventions
 *  - Every function returns a baorec_status (0 = success).  On failure
 *    baorec_last_error(ctx) returns a message that stays valid until the next
 *    call on the same context.
 *  - Meshes are FP32 arrays on the device, x fastest: element (ix, iy, iz) of
 *    an n1 x n2 x n3 mesh is at ix + n1*(iy + n2*iz) — the memory order of a
 *    Julia Array{Float32,3}(n1, n2, n3).  Indices are 0-based here; the
 *    reference's ρ[i, j, k] is element (i-1, j-1, k-1).
 *  - Particle arrays are FP32 structure-of-arrays (x, y, z, w).  They live on
 *    the host when BAOREC_HOST is set in `flags`, else on the device.  They
 *    are borrowed for the call only.
 *  - A context owns one CUDA stream, its cuFFT plans and all work buffers.
 *    Calls on one context must not overlap (not thread-safe); separate
 *    contexts are independent.  Without BAOREC_ASYNC a call returns after its
 *    work has finished on the GPU, like the reference's `wait(ev)`.
 */
#ifndef BAOREC_GB300_H
#define BAOREC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BAOREC_OK = 0,
  BAOREC_ERR_ARG = 1,           /* invalid argument (reference: MethodError / AssertionError) */
  BAOREC_ERR_CUDA = 2,          /* CUDA runtime error */
  BAOREC_ERR_CUFFT = 3,         /* cuFFT error */
  BAOREC_ERR_NOT_CONVERGED = 4, /* residual-driven solve hit its cycle cap */
  BAOREC_ERR_OOB = 5,           /* particle outside the mesh (reference: BoundsError) */
  BAOREC_ERR_STATE = 6,         /* call order error, e.g. no result yet */
  BAOREC_ERR_NOMEM = 7,         /* device allocation failed */
  BAOREC_ERR_TOO_LARGE = 8      /* input exceeds the fixed scratch of a no-allocation entry point */
} baorec_status;

/* flags */
#define BAOREC_HOST       0x1u  /* particle pointers are host memory */
#define BAOREC_ASYNC      0x2u  /* do not wait for the GPU before returning */
#define BAOREC_WRITEBACK  0x4u  /* paint with wrap writes wrapped positions back (reference mutates its inputs) */
#define BAOREC_DETERMINISTIC 0x8u /* paint through the tile counting sort with fixed-point sums: the same mesh
                                     bits on every run (no reference counterpart) */

/* method / option enums */
#define BAOREC_ITERATIVE  0
#define BAOREC_MULTIGRID  1
#define BAOREC_LOS_LOCAL  0     /* los = nothing: radial line of sight from the origin */
#define BAOREC_LOS_GLOBAL 1     /* fixed line-of-sight vector */
#define BAOREC_MAS_CIC    0
#define BAOREC_MAS_TSC    1     /* no reference counterpart */
#define BAOREC_MG_REFERENCE  0  /* FMG, damped Jacobi, fixed cycles (src/multigrid.jl:722-752) */
#define BAOREC_MG_CONVERGENT 1  /* residual-driven V-cycles to rtol (no reference counterpart) */
#define BAOREC_START_ZERO     0 /* convergent mode: V-cycles from a zero potential (plain multigrid) */
#define BAOREC_START_SPECTRAL 1 /* convergent mode: FFT-preconditioned corrections first (no reference counterpart) */
#define BAOREC_START_LEARNED  2 /* convergent mode: CNN initial guess, then as SPECTRAL; with a fixed line of
                                   sight the FFT start is exact and is the learned start (no reference counterpart) */
#define BAOREC_FIELD_DISP 0     /* :disp */
#define BAOREC_FIELD_RSD  1     /* :rsd  */
#define BAOREC_FIELD_SUM  2     /* :sum  */

/* Reconstruction parameters: the fields of IterativeRecon / MultigridRecon
 * (src/recon.jl:2-33) plus the options this library adds. */
typedef struct {
  int32_t method;            /* BAOREC_ITERATIVE | BAOREC_MULTIGRID */
  int32_t n[3];              /* mesh size (grid_size of run!) */
  float box_size[3];         /* recon.box_size */
  float box_min[3];          /* recon.box_min */
  int32_t los_mode;          /* BAOREC_LOS_LOCAL (los = nothing) | BAOREC_LOS_GLOBAL */
  float los[3];              /* recon.los when global */
  float bias;                /* recon.bias */
  float f;                   /* recon.f (growth rate) */
  float smoothing_radius;    /* recon.smoothing_radius */
  float beta;                /* recon.β; <= 0 means f / bias as the reference default */
  int32_t n_iter;            /* IterativeRecon.n_iter (default 3) */
  float jacobi_damping_factor;   /* MultigridRecon (default 0.4) */
  int32_t jacobi_niterations;    /* MultigridRecon (default 5) */
  int32_t vcycle_niterations;    /* MultigridRecon (default 6) */
  float ran_min;             /* setup_overdensity! randoms threshold (default 0.01) */
  /* additions */
  int32_t mas;               /* BAOREC_MAS_CIC (default) | BAOREC_MAS_TSC */
  int32_t mg_mode;           /* BAOREC_MG_REFERENCE (default) | BAOREC_MG_CONVERGENT */
  int32_t nu1, nu2;          /* convergent mode: pre/post red-black Gauss-Seidel sweeps (2, 2) */
  float rtol;                /* convergent mode: relative residual target (1e-6) */
  int32_t max_cycles;        /* convergent mode: V-cycle cap (50) */
  int32_t mg_start;          /* convergent mode: BAOREC_START_ZERO (default) | _SPECTRAL | _LEARNED */
  float start_rate;          /* spectral corrections continue while each shrinks the residual
                                by at least this factor (0.5); then V-cycles take over */
} baorec_config;

/* Solver statistics of the last multigrid solve. */
typedef struct {
  int32_t cycles;            /* V-cycles run */
  int32_t spectral_steps;    /* FFT-preconditioned corrections run before the V-cycles */
  double rel_residual;       /* |f - a*1 - A phi| / |f - a*1| after the last cycle (FP64) */
  double alpha;              /* constant shift a removed from the right-hand side */
  double rel_residual_initial;
} baorec_solve_stats;

typedef struct baorec_ctx baorec_ctx;

/* Fill `cfg` with the reference defaults (n_iter 3, damping 0.4, 5 Jacobi
 * sweeps, 6 V-cycles, ran_min 0.01, CIC, reference MG schedule, 2+2 sweeps,
 * rtol 1e-6, 50 cycles). */
void baorec_config_default(baorec_config* cfg);

/* Create a context: allocates the mesh buffers and cuFFT plans for cfg->n on
 * the current CUDA device.  Replaces setup_fft! (src/recon.jl:35-37), which
 * plans the FFT on every run!. */
int baorec_create(const baorec_config* cfg, baorec_ctx** out);
int baorec_destroy(baorec_ctx* ctx);
const char* baorec_last_error(const baorec_ctx* ctx);
/* Update box_size / box_min (run! with randoms overrides them). */
int baorec_set_box(baorec_ctx* ctx, const float box_size[3], const float box_min[3]);
int baorec_get_box(const baorec_ctx* ctx, float box_size[3], float box_min[3]);
/* The CUDA stream the context launches on (cudaStream_t as void*). */
void* baorec_stream(baorec_ctx* ctx);
/* Number of kernels this context has launched since creation. */
int64_t baorec_kernel_launches(const baorec_ctx* ctx);
/* This library's kernel launches in the process so far, every context (a
 * batch graph's kernels counted once, when captured). */
int64_t baorec_total_kernel_launches(void);
/* Device pointer of the context's result field (result_cache), or NULL. */
float* baorec_result_ptr(baorec_ctx* ctx);

/* setup_box (src/utils.jl:100-109): box_min = min - pad/2, cubic box_size of
 * the largest extent of max - min + pad.  Device min/max reduction. */
int baorec_setup_box(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                     int64_t n, float pad, uint32_t flags,
                     float box_size_out[3], float box_min_out[3]);

/* Bounding box without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot let the
 * library call cudaMalloc: hosts whose pool allocator (CUDA.jl, PyTorch)
 * already owns the device memory budget, and latency-sensitive pipelines that
 * cannot afford the device-wide synchronisation of cudaMalloc / cudaFree.
 * It computes what baorec_setup_box computes, needs no context, and keeps its
 * partial results in a fixed 24.6 KB device array that every GPU loading the
 * library holds until exit.  x, y, z are device arrays of n particles; at most
 * 16,777,216 particles per call (larger n returns BAOREC_ERR_TOO_LARGE, n < 1
 * BAOREC_ERR_ARG).  x, y, z must be device or managed memory of the current
 * device (anything else is BAOREC_ERR_ARG).  The outputs are host arrays.
 * Work runs on `stream` (cudaStream_t, NULL = legacy default stream) and the
 * call is synchronous: it waits for that stream, so it cannot be recorded
 * into a CUDA graph, and a call on a stream that is being captured returns
 * BAOREC_ERR_ARG without touching the capture.  The first call on each device
 * looks up the array's device address (with that device current) and caches
 * it; after cudaDeviceReset of a device the cached address is stale, so do
 * not call this entry point on that device again in the same process.
 * All calls share the one array: calls that overlap on the GPU race. */
int baorec_setup_box_noalloc(const float* x, const float* y, const float* z, int64_t n, float pad,
                             void* stream, float box_size_out[3], float box_min_out[3]);

/* cic! (src/mas.jl:1-52 CPU, :53-107 GPU): add the CIC weights of n particles
 * to `mesh` (device, not cleared).  wrap != 0 applies the reference's
 * periodic rules; with BAOREC_WRITEBACK the wrapped positions are written back
 * into x, y, z like the reference mutates its inputs.  Particles whose cell
 * falls outside the mesh are skipped and reported as BAOREC_ERR_OOB. */
int baorec_cic(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z,
               const float* w, int64_t n, int wrap, uint32_t flags);

/* Triangular-shaped-cloud paint (no reference counterpart; same node and wrap
 * conventions as cic!). */
int baorec_tsc(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z,
               const float* w, int64_t n, int wrap, uint32_t flags);

/* The lower CIC cell of every particle (int32 keys ix + n1*(iy + n2*iz)) and
 * the particle count per cell (int32 mesh, cleared first), computed by the
 * paint's own binning; integer outputs, bit-exact with src/mas.jl:13-35.
 * Either output may be NULL. */
int baorec_cell_bins(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                     int64_t n, int wrap, uint32_t flags, int32_t* keys_out, int32_t* counts_out);

/* smooth! (src/utils.jl:45-56, :85-96): Gaussian smoothing of a device mesh
 * in place, exp(-R^2 k^2 / 2) in k space. */
int baorec_smooth(baorec_ctx* ctx, float* mesh);

/* setup_overdensity!, data only (src/recon.jl:42-57): paint (wrap), smooth,
 * delta = (delta/mean - 1)/b.  `delta` (device) must be zero on entry. */
int baorec_setup_overdensity(baorec_ctx* ctx, float* delta, float* x, float* y, float* z,
                             const float* w, int64_t n, int wrap, uint32_t flags);

/* setup_overdensity!, data + randoms (src/recon.jl:60-91).  `delta` must be
 * zero on entry. */
int baorec_setup_overdensity_randoms(baorec_ctx* ctx, float* delta,
                                     const float* x, const float* y, const float* z,
                                     const float* w, int64_t n,
                                     const float* rx, const float* ry, const float* rz,
                                     const float* rw, int64_t nr, uint32_t flags);

/* iterate! (src/iterative.jl:5-67, :151-211): one iterative-FFT step with the
 * 1-based counter `iter`; delta_r is updated in place from delta_s. */
int baorec_iterate(baorec_ctx* ctx, float* delta_r, const float* delta_s, int iter);

/* Multigrid primitives on one level of size nl[3] (src/multigrid.jl). */
/* jacobi! (:14-135, :193-210): niter damped-Jacobi sweeps on v. */
int baorec_mg_jacobi(baorec_ctx* ctx, float* v, const float* f, const int32_t nl[3], int niter);
/* residual! (:213-326, :378-395): r = f - A v. */
int baorec_mg_residual(baorec_ctx* ctx, float* r, const float* v, const float* f, const int32_t nl[3]);
/* reduce! (:520-584, :641-651): full-weighting restriction fine -> coarse (nl = fine size). */
int baorec_mg_reduce(baorec_ctx* ctx, float* coarse, const float* fine, const int32_t nl[3]);
/* prolong! (:398-453, :511-518): trilinear prolongation coarse -> fine (nl = fine size), overwrites fine. */
int baorec_mg_prolong(baorec_ctx* ctx, float* fine, const float* coarse, const int32_t nl[3]);
/* vcycle! (:654-719): one V-cycle on v (level size nl). */
int baorec_mg_vcycle(baorec_ctx* ctx, float* v, const float* f, const int32_t nl[3]);
/* fmg (:722-752): full multigrid on the context mesh size; phi is overwritten. */
int baorec_mg_fmg(baorec_ctx* ctx, const float* f, float* phi);
/* Residual-driven solve (no reference counterpart): V-cycles with red-black
 * Gauss-Seidel smoothing until |f - a*1 - A phi| <= rtol |f - a*1|, the shift
 * `a` making the singular periodic system consistent.  phi0 (device, may be
 * NULL = zero start) is the initial guess; phi receives the solution.  stats
 * may be NULL.  Returns BAOREC_ERR_NOT_CONVERGED at the cycle cap (phi holds
 * the last iterate). */
int baorec_mg_solve(baorec_ctx* ctx, const float* f, float* phi, const float* phi0,
                    baorec_solve_stats* stats);

/* Measurement hook (no reference counterpart): launch one finest-level kernel
 * `reps` times on the context's scratch buffers between two CUDA events on
 * the context stream and report the mean duration and the kernel's
 * algorithmic bytes per launch.  which: 0 = red-black sweep (both colours),
 * 1 = accurate residual with solution update, 2 = damped-Jacobi sweep
 * (reference schedule), 3 = FP32 difference-form running residual of the FFT
 * corrections, 4 and 5 = the streaming forms of 1 and 3, 6 = one V-cycle of
 * the residual-driven solve (nu1 + nu2 red-black sweeps per level, the small
 * levels in one cooperative kernel, FP64 coarsest solve), 7 = one V-cycle of
 * the reference schedule (vcycle!: jacobi_niterations damped-Jacobi sweeps
 * before and after on every level); for 6 and 7 the bytes are those of every
 * level's sweeps, residual, restriction and prolongation; 8 and 9 = the
 * batched 2-D forward (real to half spectrum) and inverse transforms of the
 * finest mesh's xy planes (meshes of 256 z planes), by the autotuner's
 * current choice (baorec_set_tune_xy): the fused cluster kernels or cuFFT.
 * Needs a multigrid context. */
int baorec_profile_kernel(baorec_ctx* ctx, int which, int reps, float* avg_ms, double* bytes_per_launch);

/* Statistics of the context's last residual-driven solve. */
int baorec_last_solve_stats(const baorec_ctx* ctx, baorec_solve_stats* stats);
/* Convergence history of the last residual-driven solve: for each outer step
 * the relative residual before it (rho[i]) and the correction that followed
 * (kind[i]: 0 = V-cycle, m > 0 = m FFT corrections, -1 = none, the last
 * entry).  Copies min(count, cap) entries and returns count (or < 0 on error). */
int baorec_solve_history(const baorec_ctx* ctx, double* rho, int32_t* kind, int cap);
/* Relative residual |r - mean r| / |f - mean f| of the start of kind
 * BAOREC_START_* (zero, FFT, learned) for the right-hand side f (device mesh). */
int baorec_start_residual(baorec_ctx* ctx, const float* f, int start, double* rel_residual);
/* Whether the FFT start's k-space multiply runs as a cuFFT LTO load callback
 * (1), as a separate kernel (-1: not requested or unavailable, *note says
 * which) or is requested and not set up yet (0). */
int baorec_fft_callbacks(const baorec_ctx* ctx, const char** note);
/* Request (1) or drop (0, the default) the callback form; a request that
 * cuFFT cannot honour leaves the kernel form in use. */
int baorec_set_fft_callbacks(baorec_ctx* ctx, int enable);

/* reconstructed_overdensity! (src/recon.jl:93-132): overdensity then n_iter
 * iterations into the context result.  rx.. may be NULL (data only). */
int baorec_reconstructed_overdensity(baorec_ctx* ctx, float* x, float* y, float* z,
                                     const float* w, int64_t n,
                                     const float* rx, const float* ry, const float* rz,
                                     const float* rw, int64_t nr, uint32_t flags);
/* reconstructed_potential! (src/recon.jl:184-212): overdensity then the
 * multigrid solve (cfg.mg_mode) into the context result. */
int baorec_reconstructed_potential(baorec_ctx* ctx, float* x, float* y, float* z,
                                   const float* w, int64_t n,
                                   const float* rx, const float* ry, const float* rz,
                                   const float* rw, int64_t nr, uint32_t flags);

/* run! (src/recon.jl:134-261): with randoms the box is first replaced by
 * setup_box(randoms, 500); then reconstructed_overdensity! (iterative) or
 * reconstructed_potential! (multigrid) into the context result. */
int baorec_run(baorec_ctx* ctx, float* x, float* y, float* z, const float* w, int64_t n,
               const float* rx, const float* ry, const float* rz, const float* rw, int64_t nr,
               uint32_t flags);

/* Copy the result field (recon.result_cache) to `out` (host if BAOREC_HOST). */
int baorec_get_result(baorec_ctx* ctx, float* out, uint32_t flags);
/* Replace the result field (the 5-argument read_shifts takes a field). */
int baorec_set_result(baorec_ctx* ctx, const float* in, uint32_t flags);

/* The three displacement meshes of compute_displacements
 * (src/iterative.jl:253-275 / src/multigrid.jl:755-773) for the result field;
 * device outputs. */
int baorec_displacement_meshes(baorec_ctx* ctx, float* psi_x, float* psi_y, float* psi_z);

/* Gradient of the multigrid potential for the displacements and shifts:
 * BAOREC_GRADIENT_FFT (default, compute_displacements of
 * src/multigrid.jl:755-773) or BAOREC_GRADIENT_FD, the periodic
 * central-difference gradient that read_grad_cic (src/mas.jl:388-466, not
 * wired into the reference) interpolates: one stencil pass instead of one R2C
 * and three C2R transforms; the results differ from the FFT gradient by the
 * discretisation error.  Multigrid contexts only. */
#define BAOREC_GRADIENT_FFT 0
#define BAOREC_GRADIENT_FD  1
int baorec_set_gradient(baorec_ctx* ctx, int32_t mode);

/* read_cic! (src/mas.jl:218-269): trilinear read of a device mesh at n
 * particles (wrap = true as the reference's callers use). */
int baorec_read_cic(baorec_ctx* ctx, const float* mesh, const float* x, const float* y,
                    const float* z, int64_t n, float* out, uint32_t flags);

/* read_shifts (src/recon.jl:264-364): shifts of kind `field` at n particles
 * from the context result. */
int baorec_read_shifts(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                       int64_t n, int field, float* sx, float* sy, float* sz, uint32_t flags);

/* reconstructed_positions (src/recon.jl:366-388): p - shift(field). */
int baorec_reconstructed_positions(baorec_ctx* ctx, const float* x, const float* y,
                                   const float* z, int64_t n, int field,
                                   float* ox, float* oy, float* oz, uint32_t flags);
/* Two reconstructed_positions calls on the same particles (the examples'
 * :sum and :disp randoms, test_helpers' "sym" and "iso" catalogs) from one
 * gather of the displacement: outputs bit-identical to the two calls. */
int baorec_reconstructed_positions2(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                                    int field_a, float* oxa, float* oya, float* oza,
                                    int field_b, float* oxb, float* oyb, float* ozb, uint32_t flags);

/* ---- Catalog I/O (examples/lightcone.jl:22-23, examples/simulation.jl:13
 * read catalogs with CSV.jl; examples/simulation.jl:38-40 write the shifted
 * positions with npzwrite) ----------------------------------------------
 * Both work without a context (ctx NULL; baorec_last_error(NULL) holds the
 * message) for host arrays; device arrays need one.
 *
 * baorec_read_ascii: whitespace-delimited numbers, one row per line; the
 * first `skip` lines are dropped, then blank lines and lines whose first
 * non-blank character is `comment` (0: none).  Columns `cols` (0-based) of
 * every row go to out[0..ncols) as FP32, correctly rounded (strtof in the C
 * locale).  With out NULL only *n_rows is set (the row count); with out, the
 * columns need room for n_max rows (BAOREC_ERR_TOO_LARGE otherwise).  A row
 * with too few fields or a field that is not a number is BAOREC_ERR_ARG,
 * with the file line in the message. */
int baorec_read_ascii(baorec_ctx* ctx, const char* path, const int32_t* cols, int32_t ncols, int32_t skip,
                      int32_t comment, float** out, int64_t n_max, int64_t* n_rows, uint32_t flags);
/* baorec_write_npy: an (n, ncols) float32 .npy file with fortran_order True
 * (columns stored one after the other, as npzwrite writes hcat(x, y, z));
 * cols on the device unless BAOREC_HOST. */
int baorec_write_npy(baorec_ctx* ctx, const char* path, const float* const* cols, int32_t ncols, int64_t n,
                     uint32_t flags);

/* ---- Power-spectrum multipoles (the science check of the reference's test
 * helpers, which call the external pypowspec: compute_auto_box,
 * compute_auto_box_rand, compute_auto_lc in test_helpers/simulation.py:40-55
 * and test_helpers/lightcone.py:48-75) ------------------------------------
 * On this context's mesh and box.  The catalogs are painted (CIC or TSC,
 * nodes at box_min + i L/n, periodic) into F = Σ w_d - α Σ w_r with
 * α = Σw_d / Σw_r (F = Σ w_d without randoms), transformed, compensated for
 * the assignment window Π sinc(k_a Δ_a / 2)^p and binned in |k| shells
 * [kmin + b dk, kmin + (b+1) dk).
 *   BAOREC_POWER_BOX     periodic box, fixed unit line of sight `los`;
 *                        P(k, μ) = |F_k|² / I - shot, I = (Σw_d)² / V,
 *                        shot = (Σw_d² + α² Σw_r²) / I; optional interlacing
 *                        (a second paint shifted by half a cell).
 *   BAOREC_POWER_SURVEY  local line of sight from the origin (Yamamoto
 *                        estimator through FFTs: A_0 = FFT[F],
 *                        A_2 = k̂_i k̂_j FFT[r̂_i r̂_j F],
 *                        A_4 = k̂_i k̂_j k̂_k k̂_l FFT[r̂_i r̂_j r̂_k r̂_l F] with r̂
 *                        at the mesh nodes); P_0 = <|A_0|²>/I - shot,
 *                        P_2 = 5/2 <Re A_0 (3 A_2 - A_0)*>/I,
 *                        P_4 = 9/8 <Re A_0 (35 A_4 - 30 A_2 + 3 A_0)*>/I with
 *                        I = α Σ_r n(z)_r w_r² from the randoms' n(z) (rnz);
 *                        weights are the total (e.g. FKP) weights.
 * Outputs (host, nbins each): mean |k| of the modes in the bin, P_0, P_2,
 * P_4 and the mode count; *shot and *norm get the shot noise and I.  Shot
 * noise is subtracted from P_0 only.  Particles outside the box are an error
 * for the survey geometry (BAOREC_ERR_OOB) and wrap for the box. */
#define BAOREC_POWER_BOX    0
#define BAOREC_POWER_SURVEY 1
typedef struct {
  int32_t geometry;          /* BAOREC_POWER_BOX | BAOREC_POWER_SURVEY */
  int32_t mas;               /* BAOREC_MAS_CIC | BAOREC_MAS_TSC */
  int32_t interlace;         /* 0 | 1 (box geometry) */
  int32_t nbins;
  float kmin, dk;            /* h/Mpc */
  float los[3];              /* box geometry: line of sight (normalised internally) */
  int32_t reserved;
} baorec_power_config;

int baorec_power_multipoles(baorec_ctx* ctx, const baorec_power_config* pc,
                            const float* x, const float* y, const float* z, const float* w, int64_t n,
                            const float* rx, const float* ry, const float* rz, const float* rw,
                            const float* rnz, int64_t nr,
                            double* k_mean, double* p0, double* p2, double* p4, int64_t* nmodes,
                            double* shot, double* norm, uint32_t flags);

/* ---- Learned initial guess (no reference counterpart) ----------------------
 * A 3-level 3-D U-Net (16/32/64 channels, BF16 weights and activations, FP32
 * accumulation) predicts the error of the FFT start of the residual-driven
 * solve; BAOREC_START_LEARNED uses it.  Meshes must be cubic with n % 4 == 0.
 * Training draws sub-boxes of `region` with this context's box size, fills
 * each with a lognormal field (Gaussian field with P(k) ∝ k^pk_slope smoothed
 * with the context's smoothing radius, RMS sigma_g before the transform) in
 * the survey window (comoving r, RA, Dec in degrees; the observer at the
 * origin), divides by the bias, and solves it to `rtol` for the target. */
typedef struct {
  int32_t steps, batch;      /* Adam steps; fields per step */
  float lr;                  /* Adam learning rate */
  uint32_t seed;
  float sigma_g, pk_slope;
  float region_min[3], region_size[3];
  float r_min, r_max, ra_min, ra_max, dec_min, dec_max;
  float rtol;                /* solver tolerance of the targets */
  int32_t loss;              /* 0: MSE of the potential error; 1: MSE of its 7-point Laplacian */
} baorec_guess_train_config;

int64_t baorec_guess_num_params(void);
/* He-initialised weights (the head starts near zero: the guess starts as the FFT start). */
int baorec_guess_init(baorec_ctx* ctx, uint32_t seed);
/* FP32 parameters, host arrays of baorec_guess_num_params() values. */
int baorec_guess_set_params(baorec_ctx* ctx, const float* params, int64_t n);
int baorec_guess_get_params(baorec_ctx* ctx, float* params, int64_t n);
/* Network forward on device features (N x 8 FP32, channels fastest) into
 * out (N, device); with a target (N, device) also the loss (loss_kind as in
 * baorec_guess_train_config.loss) and, when grads (host, num_params) is
 * given, the parameter gradients. */
int baorec_guess_eval(baorec_ctx* ctx, const float* features, const float* target, float* out,
                      float* grads, double* loss, int loss_kind);
/* phi0 = FFT start + learned correction for the right-hand side f (device meshes). */
int baorec_guess_apply(baorec_ctx* ctx, const float* f, float* phi0);
/* Where the network runs: level 0 (default) on this context's mesh; level 1
 * on the first restriction of the mesh (n/2 per axis, same box), the way a
 * multigrid coarse level sees it: the right-hand side is restricted with the
 * full-weighting operator of reduce! (src/multigrid.jl:520-584), the
 * network's correction is computed there against the FFT start of that
 * coarse problem and brought back with the trilinear prolongation of
 * prolong! (src/multigrid.jl:398-453) onto this mesh's FFT start.  Level 1
 * needs a cubic mesh with n % 8 == 0; it creates a child context at n/2 that
 * owns the network from then on (every baorec_guess_* call on this context
 * acts on the child's network; parameters set before the switch move with
 * it).  Returns BAOREC_ERR_ARG for other levels. */
int baorec_guess_set_level(baorec_ctx* ctx, int32_t level);
int32_t baorec_guess_level(const baorec_ctx* ctx);
/* One training pair (device meshes f and its solution phi); moves the box. */
int baorec_guess_sample(baorec_ctx* ctx, const baorec_guess_train_config* tc, int64_t index,
                        float* f, float* phi);
/* Train on the device; loss_history (host, steps values) may be NULL. */
int baorec_guess_train(baorec_ctx* ctx, const baorec_guess_train_config* tc, float* loss_history);
/* Convolution kernels of the network: tensor_core 1 (default) runs the 3x3x3
 * layers whose shape has one on the tcgen05 kernel (TMA-staged operands, TMEM
 * accumulators; the 3x3x3 shapes 8->16, 16->16, 16->32, 32->16, 32->32,
 * 32->64, 64->32 on grids with n % 128 == 0 or n == 64), 0 runs every
 * layer on the mma.sync kernels. */
int baorec_guess_set_conv_path(baorec_ctx* ctx, int32_t tensor_core);
/* Convolutions of the last network forward that ran on tcgen05 (-1: no network). */
int32_t baorec_guess_tc_layers(baorec_ctx* ctx);
/* One 3x3x3 zero-padded convolution of the network on device arrays: x is
 * n^3 x cin BF16 (channels fastest, x fastest among voxels), w FP32
 * [27][cin][cout] with tap t = dx + 3 dy + 9 dz, bias FP32 [cout] or NULL,
 * add n^3 x cout BF16 or NULL; y = relu?(conv(x) + bias + add) as BF16.
 * path 0: mma.sync kernel, 1: tcgen05 kernel with TMA-box slab loads (the
 * network's path), 2: tcgen05 kernel with cp.async slab loads
 * (BAOREC_ERR_ARG for 1 and 2 if the shape or n has none). */
int baorec_guess_conv3(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n, const void* x, const float* w,
                       const float* bias, const void* add, void* y, int32_t relu, int32_t path);
/* Test hook of the bounded device waits (no reference counterpart): one
 * tcgen05 convolution (zero input and weights, cin -> cout on an n^3 grid)
 * whose slab loader is held back, so that no slab ever arrives and the
 * pipeline's waits, limited to wait_ns each, expire.  The kernel records the
 * timeout in the context's device error word, every role stops, the block
 * waits for its weight copy and frees its TMEM, and the call returns
 * BAOREC_ERR_CUDA with a "timed out" message; the context stays usable.
 * BAOREC_ERR_ARG for shapes without a tcgen05 kernel. */
int baorec_guess_conv3_held_back(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n, int64_t wait_ns);
/* Average device time (CUDA events on the context's stream) of `reps`
 * launches of one network convolution cin -> cout on an n^3 grid (path as in
 * baorec_guess_conv3) and its algorithmic FLOPs, 2 * 27 * cin * cout * n^3. */
int baorec_guess_profile_conv(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n, int32_t path, int32_t reps,
                              float* avg_ms, double* flops);

/* ---- Batched box reconstructions in one CUDA graph (no reference counterpart) ----
 * Each item is one periodic-box mock (device arrays; positions in [0, box),
 * wrapped in place by the paint as cic! with wrap does) reconstructed with
 * the iterative method of `base` (bias, f, los, n_iter) on its own mesh,
 * box, mass assignment and smoothing radius; its shifted positions (field
 * BAOREC_FIELD_*) go to out_x/y/z.  Items sharing (mesh, box_size) share one
 * context.  baorec_batch_create runs the batch once and captures it as a
 * graph; baorec_batch_launch replays all of it asynchronously on `stream`
 * (cudaStream_t; NULL = the batch's own, baorec_batch_stream) and
 * baorec_batch_sync waits for that stream and checks for errors.
 * On failure of create, *out still holds the batch for baorec_batch_last_error
 * and must be destroyed. */
typedef struct {
  float *x, *y, *z;
  const float* w;
  int64_t n;
  int32_t mesh;              /* cubic mesh edge */
  float box_size;            /* cubic box edge, box_min = 0 */
  int32_t mas;               /* BAOREC_MAS_CIC | BAOREC_MAS_TSC */
  float smoothing_radius;
  int32_t field;             /* BAOREC_FIELD_DISP | _RSD | _SUM */
  float *out_x, *out_y, *out_z;
} baorec_batch_item;
typedef struct baorec_batch baorec_batch;

int baorec_batch_create(const baorec_config* base, const baorec_batch_item* items, int count,
                        baorec_batch** out);
int baorec_batch_launch(baorec_batch* b, void* stream);
int baorec_batch_sync(baorec_batch* b, void* stream);
void* baorec_batch_stream(baorec_batch* b);
/* Kernels of this library one replay launches (cuFFT's not counted). */
int64_t baorec_batch_kernel_launches(const baorec_batch* b);
const char* baorec_batch_last_error(const baorec_batch* b);
int baorec_batch_destroy(baorec_batch* b);

/* ---- Autotuner (no reference counterpart) ---------------------------------
 * Times candidate launch shapes on this context's meshes and keeps the
 * fastest for every later call: BAOREC_TUNE_STENCIL picks 32x8x8 or 32x16x16
 * tiles per multigrid level (multigrid contexts); BAOREC_TUNE_PAINT picks the
 * deterministic paint's tile edge (4, 8 or 16).  Outputs (may be NULL): the
 * paint tile and 16 per-level tile choices (-1 = not tuned, 0 = 8x8, 1 = 16x16). */
#define BAOREC_TUNE_STENCIL 0x1u
#define BAOREC_TUNE_PAINT   0x2u
int baorec_autotune(baorec_ctx* ctx, uint32_t what, int32_t* paint_tile, int32_t* big_tiles);
/* Set the shapes explicitly (paint tile edge 1..16; per-level choices as above, NULL keeps them). */
int baorec_set_tune(baorec_ctx* ctx, int32_t paint_tile, const int32_t* big_tiles);
/* Finest-level residual kernels of the convergent solve: 1 streaming (z-marching,
 * cp.async-pipelined), 0 tiled, -1 not tuned (streaming where the mesh allows). */
int baorec_tune_stream(const baorec_ctx* ctx);
int baorec_set_tune_stream(baorec_ctx* ctx, int stream);
/* FP32 running residual of the FFT corrections: 1 two z-adjacent cells per
 * thread in packed FP32x2 arithmetic on 32x16x16 tiles (default), 0 one cell
 * per thread, 2 and 3 the packed form with the window streamed through a ring
 * of plane pairs in blocks of 16 and 32 z planes, 4 and 5 two x-adjacent cells
 * per thread on 64x16 columns of 32 and 16 z planes with every operand staged
 * in shared memory by TMA (n[0] % 64 == 0, n[1] % 16 == 0; elsewhere form 1
 * runs), 6 form 1 on 32x8x16 tiles of 256 threads (four blocks per SM).
 * Forms 1-6 give the same bits.  The stencil autotune times all seven. */
int baorec_tune_pairs(const baorec_ctx* ctx);
int baorec_set_tune_pairs(baorec_ctx* ctx, int pairs);
/* FP32 paint (cic! / tsc! without BAOREC_DETERMINISTIC): 0 one float atomic
 * per weight into the mesh (default), 1 binned (particles sorted by 16^3 or
 * 32^3 mesh tile with an integer counting sort, each tile painted in shared
 * memory and written once).  The same weights; the paint autotune times both. */
int baorec_tune_binned(const baorec_ctx* ctx);
int baorec_set_tune_binned(baorec_ctx* ctx, int binned);
/* Accurate residual (double-float solution update) of the residual-driven
 * solve on the finest level: 0 blocks of 512 threads on the level's tiles
 * (default), 1 and 2 blocks of 256 threads on 32x8x8 and 32x8x16 tiles.  The
 * same results; the stencil autotune times all three. */
int baorec_tune_acc(const baorec_ctx* ctx);
int baorec_set_tune_acc(baorec_ctx* ctx, int acc);
/* FFT preconditioner of the residual-driven solve where n[2] = 256: 1 batched
 * 2-D transforms of the xy planes around one kernel that transforms along z,
 * multiplies by S^-1(k) and transforms back (default), 2 the same with the
 * z kernel's registers capped for three resident blocks per SM, 0 3-D
 * transforms with a separate multiply.  The stencil autotune times all three. */
int baorec_tune_zpass(const baorec_ctx* ctx);
int baorec_set_tune_zpass(baorec_ctx* ctx, int zpass);
/* The xy transforms of the z-pass paths (preconditioner, smoothing,
 * displacement) for 256 x 256 planes: 0 cuFFT's batched 2-D transforms,
 * 1 (default) one fused kernel per direction (a cluster of four CTAs per
 * plane, the rows <-> columns transposition through distributed shared
 * memory: each plane read and written once).  The stencil autotune times
 * both and keeps the faster (on a GB300 the fused kernels: about 49 / 52 us
 * per 256-plane transform against 62 us). */
int baorec_tune_xy(const baorec_ctx* ctx);
int baorec_set_tune_xy(baorec_ctx* ctx, int xy);

/* ---- Catalog coordinates (examples/lightcone.jl:30-82) ------------------------
 * sky_to_cartesian (lightcone.jl:30-47): ra, dec in degrees and redshift z ->
 * comoving x, y, z in Mpc/h; cartesian_to_sky (lightcone.jl:50-80) the
 * inverse, with the script's ra convention ((lon - 360) rem 360).  The host
 * passes the comoving-distance table r(z) (Mpc, FP64, ntab values on a uniform
 * grid z_min..z_max, as comoving_distance_interp of src/cosmo.jl:83-90 tabulates
 * it) and h; values outside the table return BAOREC_ERR_OOB (the reference's
 * interpolation throws).  fkp_weights (lightcone.jl:82): w = 1/(1 + nz P0). */
int baorec_sky_to_cartesian(baorec_ctx* ctx, const float* ra, const float* dec, const float* z, int64_t n,
                            const double* r_table, int32_t ntab, double z_min, double z_max, float h,
                            float* x, float* y, float* zc, uint32_t flags);
int baorec_cartesian_to_sky(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                            const double* r_table, int32_t ntab, double z_min, double z_max, float h,
                            float* ra, float* dec, float* red, uint32_t flags);
int baorec_fkp_weights(baorec_ctx* ctx, const float* nz, int64_t n, float P0, float* w, uint32_t flags);

#ifdef __cplusplus
}
#endif
#endif /* BAOREC_GB300_H */
