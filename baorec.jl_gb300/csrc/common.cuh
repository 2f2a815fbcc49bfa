// Internal declarations shared by the translation units of libbaorec_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "baorec_gb300.h"

namespace baorec {

constexpr int kNumSMs = 152;          // GB300: 2 dies x 76 SMs
constexpr size_t kRedCapacity = 1u << 17;   // FP64 entries of the reduction-partials buffer

// Device-side error word bits (set by kernels, read after a sync).
enum : unsigned {
  kErrOOB = 1u,        // particle index outside the mesh
  kErrTimeout = 2u,    // a bounded device-side wait gave up (pipeline stalled)
};

struct Level {                        // one multigrid level
  int n[3];
  size_t N;
  float* f;                            // right-hand side
  float* v;                            // solution / correction
  float* r;                            // residual / scratch
  float* ax[3];                        // p tables (x_vec / cell) of this level (device, FP32)
  std::vector<float> ptab[3];          // host copies of the p tables
  bool needs_clamp = false;            // some cell next to the observer needs a clamped coefficient
};

struct DevBuf {                       // a growable device buffer
  void* p = nullptr;
  size_t bytes = 0;
};

struct GuessNet;                      // capture-safe device forms of the iterative reconstruction and the read-out (api.cu)
int reconstruct_iterative_device(baorec_ctx* ctx, float* x, float* y, float* z, const float* w, int64_t n);
int positions_device(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n, int field,
                     float* ox, float* oy, float* oz);
// learned initial guess (guess_net.cu)

}  // namespace baorec

struct baorec_ctx {
  baorec_config cfg;
  int n1, n2, n3, n1h;
  size_t N, Nk;                        // real cells, complex (halved) cells
  cudaStream_t stream;
  cufftHandle plan_r2c = 0, plan_c2r = 0, plan_r2c2 = 0, plan_c2r2 = 0, plan_c2r3 = 0, plan_c2r6 = 0;
  void* fft_work = nullptr;            // one work area shared by all plans
  size_t fft_work_bytes = 0;
  // FFT preconditioner: inverse transform with the k-space multiply as a cuFFT
  // load callback (LTO, linked at plan creation); state 0 untried, 1 in use,
  // -1 unavailable or not requested (the separate multiply kernel runs instead)
  cufftHandle plan_c2r_spec = 0;
  int spec_cb_state = -1;
  void* spec_cb = nullptr;             // device copy of the callback's parameters
  void* spec_work = nullptr;           // its own work area when the shared one is too small
  char spec_cb_note[256] = "not requested (baorec_set_fft_callbacks)";
  // FFT preconditioner over 256 z planes: batched 2-D transforms of the xy
  // planes around one kernel doing the z transform, the k-space multiply and
  // the inverse z transform (state 0 untried, 1 ready, -1 unavailable)
  cufftHandle plan_r2c_xy = 0, plan_c2r_xy = 0;
  void* xy_work = nullptr;             // their own work area when the shared one is too small
  int xy_state = 0;
  // persistent meshes: mesh3 = three adjacent meshes A | B | C
  float* mesh3 = nullptr;
  float* result = nullptr;             // recon.result_cache (= A)
  bool has_result = false;
  float* psi = nullptr;                // 6 real meshes (displacements / iterative parts)
  bool psi_valid = false;              // psi[0..2] hold the displacement of `result`
  // set by the composed reconstruction: the solve computes the displacement
  // of its last iterate while the host reads the final residual (psi_ahead:
  // it did, and that iterate is the solution)
  bool want_psi_ahead = false, psi_ahead = false;
  cudaEvent_t ev_red = nullptr;          // the solve's partial sums have reached the host
  // chunked host read-out: copy-in and copy-out streams beside `stream`, the
  // events that order them per staging slot, and the double-buffered staging
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev_in[2] = {}, ev_k[2] = {}, ev_out[2] = {}, ev_begin = nullptr, ev_done = nullptr;
  baorec::DevBuf pipe_buf;
  int grad_mode = BAOREC_GRADIENT_FFT;  // multigrid displacement: spectral or finite-difference gradient
  cufftComplex* ck = nullptr;          // complex work: 6 spectra
  float* xvec[3] = {nullptr, nullptr, nullptr};   // x_vec of the mesh (device)
  float* stab = nullptr;               // per-axis sine tables of the FFT preconditioner (device)
  float* phi_lo = nullptr;             // low part of the double-float solution
  float* phi_lo2 = nullptr;            // ping-pong partners of the solution pair
  float* phi_hi2 = nullptr;
  // multigrid levels (level 0 = finest)
  int nlev = 0;
  baorec::Level lev[16];
  double* coarse_M = nullptr;          // dense FP64 inverse of level dense_level (or null)
  int dense_level = -1;                // first level with at most 512 cells
  bool coarse_dirty = true;            // coarse_M / dense_level need rebuilding
  baorec::GuessNet* net = nullptr;     // learned initial guess (weights, workspace)
  // learned guess on the first restriction (guess_level 1): a context at n/2
  // per axis over the same box owns the network; events order its stream
  // after this context's and back
  baorec_ctx* guess_child = nullptr;
  int guess_level = 0;
  cudaEvent_t ev_guess[2] = {nullptr, nullptr};
  // deterministic paint scratch: tile keys, permutation, tile counts/offsets, fixed-point mesh
  baorec::DevBuf sort_keys, sort_perm, sort_tiles, fix_mesh;
  baorec::DevBuf bin_parts;            // binned paint: particles (x, y, z, w) ordered by mesh tile
  baorec::DevBuf pw_mesh, pw_spec, pw_part, pw_nz;   // power-spectrum scratch (power.cu)
  struct Tune {                        // launch shapes (defaults, or chosen by baorec_autotune)
    int paint_tile = 8;                // tile edge of the deterministic paint
    int binned = 0;                    // FP32 paint: 0 global atomics, 1 binned (tile sort + shared-memory tiles)
    int stream0 = -1;                  // finest-level residuals: -1 default (streaming), 0 tile, 1 streaming
    int pairs = 1;                     // form of the FP32 running residual (baorec_set_tune_pairs)
    int acc = 0;                       // form of the accurate residual (baorec_set_tune_acc)
    int zpass = 1;                     // FFT preconditioner: 1 (2: capped registers) xy transforms + fused z pass where n3 = 256, 0 3-D transforms
    int xy = 1;                        // xy transforms of the z-pass paths: 0 cuFFT, 1 fused kernels (256 x 256 planes)
    int big_tiles[16] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};   // per level: -1 heuristic, 0/1
    bool tuned = false;
  } tune;
  // reductions
  double* dred = nullptr;              // device FP64 partial sums
  double* dfsum = nullptr;             // per-block (Σf, Σf²) of the normalised overdensity, for the solve
  double* hred = nullptr;              // pinned host mirror
  unsigned* derr = nullptr;            // device error word
  unsigned* herr = nullptr;            // pinned host copy
  // particle staging (host inputs)
  baorec::DevBuf stage[11];
  // statistics
  int64_t launches = 0;
  baorec_solve_stats last_stats;
  std::vector<double> hist_rho;        // per outer step of the last solve
  std::vector<int32_t> hist_kind;
  char msg[512];
};

namespace baorec {

int set_error(baorec_ctx* c, int code, const char* fmt, ...);
int set_error_noctx(int code, const char* fmt, ...);
int cuda_fail(baorec_ctx* c, cudaError_t e, const char* what);
int cufft_fail(baorec_ctx* c, cufftResult e, const char* what);
int ensure(baorec_ctx* c, DevBuf& b, size_t bytes);
int finish(baorec_ctx* c, uint32_t flags);   // sync unless async; check device error word

// Stage host particle arrays to the device (slot s..s+k-1); device pointers pass through.
int stage_in(baorec_ctx* c, int slot, const float* p, int64_t n, uint32_t flags, const float** out);
int stage_out_alloc(baorec_ctx* c, int slot, int64_t n, uint32_t flags, float* user, float** dev);
int stage_out_copy(baorec_ctx* c, float* user, const float* dev, int64_t n, uint32_t flags);

inline unsigned grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  return (unsigned)(g > 0x7fffffffu ? 0x7fffffffu : (g == 0 ? 1 : g));
}

#define BAOREC_LAUNCHED(c) ((c)->launches++)

// Process-wide count of this library's kernel launches (every context, the
// launches captured into a batch graph counted once): each launch site is
// the expression (kernel<<<...>>>(...), count_launch()).
int64_t count_launch();

#define CK(call)                                                         \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::baorec::cuda_fail(ctx, _e, #call);   \
  } while (0)

#define CKLAUNCH()                                                       \
  do {                                                                   \
    ctx->launches++;                                                     \
    cudaError_t _e = cudaGetLastError();                                 \
    if (_e != cudaSuccess) return ::baorec::cuda_fail(ctx, _e, "kernel launch"); \
  } while (0)

#define CKFFT(call)                                                      \
  do {                                                                   \
    cufftResult _r = (call);                                             \
    if (_r != CUFFT_SUCCESS) return ::baorec::cufft_fail(ctx, _r, #call); \
  } while (0)

#define CKS(call)                                                        \
  do {                                                                   \
    int _s = (call);                                                     \
    if (_s != BAOREC_OK) return _s;                                      \
  } while (0)

// ---- geometry helpers shared by kernels ---------------------------------

// Mesh geometry passed by value to kernels.
struct Geom {
  int n1, n2, n3;
  float L[3];
  float bmin[3];
};

inline Geom geom_of(const baorec_ctx* c) {
  Geom g;
  g.n1 = c->n1; g.n2 = c->n2; g.n3 = c->n3;
  for (int a = 0; a < 3; ++a) { g.L[a] = c->cfg.box_size[a]; g.bmin[a] = c->cfg.box_min[a]; }
  return g;
}

// ---- entry points implemented per translation unit ------------------------
// paint.cu
int paint_sorted(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n, int wrap,
                 int mas, uint32_t flags);
// FP32 paint by tile sort and shared-memory tiles (paint_sorted.cu)
bool paint_binned_ok(const baorec_ctx* ctx, int64_t n);
int paint_binned(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n, int wrap,
                 int mas, uint32_t flags);
int paint(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w,
          int64_t n, int wrap, int mas, uint32_t flags);
int minmax3(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
            float mn[3], float mx[3]);
// fft.cu
int smooth(baorec_ctx* ctx, float* mesh);
int normalize_data(baorec_ctx* ctx, float* delta);
// fpart (optional, kFsumBlocks pairs): per-block (Σδ, Σδ²) of the normalised mesh
constexpr int kFsumBlocks = 8 * kNumSMs;
int normalize_randoms(baorec_ctx* ctx, float* delta, const float* ran, int64_t nr, double* fpart = nullptr);
int iterate(baorec_ctx* ctx, float* delta_r, const float* delta_s, int iter);
int displacement_meshes(baorec_ctx* ctx, const float* field, float* psi3);
int spectral_correction(baorec_ctx* ctx, const float* r, float* e);
int zpass_prepare(baorec_ctx* ctx);   // batched xy plans of the z pass (n3 = 256)
// fused 2-D real transforms of 256 x 256 xy planes (xyfft.cu)
bool xy_fused_ok(const baorec_ctx* ctx);
int xy_fused_prepare(baorec_ctx* ctx);
int xy_r2c(baorec_ctx* ctx, const float* in, cufftComplex* out, int planes);
int xy_c2r(baorec_ctx* ctx, const cufftComplex* in, float* out, int planes);
int xy_profile(baorec_ctx* ctx, int inverse, const float* r, float* out);
// Unit line of sight the FFT preconditioner uses (false: isotropic, l = 0).
bool mean_los(const baorec_ctx* c, double l[3]);
// r = f - A v with the finest level's exact operator (difference form, FP32).
int operator_residual(baorec_ctx* ctx, const float* v, const float* f, float* r);
int start_residual(baorec_ctx* ctx, const float* f, int start, double* rel);
// capture-safe device forms of the iterative reconstruction and the read-out (api.cu)
int reconstruct_iterative_device(baorec_ctx* ctx, float* x, float* y, float* z, const float* w, int64_t n);
int positions_device(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n, int field,
                     float* ox, float* oy, float* oz);
// learned initial guess (guess_net.cu)
int guess_apply(baorec_ctx* ctx, const float* f, float* phi0);
// guess_apply on this mesh, or on its first restriction when guess_level is 1
int guess_dispatch_apply(baorec_ctx* ctx, const float* f, float* phi0);
void guess_free(baorec_ctx* ctx);
int sum_mesh(baorec_ctx* ctx, const float* m, size_t N, double* out);
int sumsq_mesh(baorec_ctx* ctx, const float* m, size_t N, double* out);
int smooth_pair(baorec_ctx* ctx, float* a, float* b);   // b == a + N uses one batched transform pair
// mg.cu
int mg_setup(baorec_ctx* ctx);
int mg_update_tables(baorec_ctx* ctx);
int xvec_update(baorec_ctx* ctx);
int mg_jacobi(baorec_ctx* ctx, float* v, const float* f, const int nl[3], int niter, float* tmp);
int mg_residual(baorec_ctx* ctx, float* r, const float* v, const float* f, const int nl[3]);
int mg_reduce(baorec_ctx* ctx, float* coarse, const float* fine, const int nl[3]);
int mg_prolong(baorec_ctx* ctx, float* fine, const float* coarse, const int nl[3], int add);
int mg_vcycle_ref(baorec_ctx* ctx, int lvl, float* v, const float* f);
int mg_fmg(baorec_ctx* ctx, const float* f, float* phi);
// fpart (optional): kFsumBlocks per-block (Σf, Σf²) pairs of f already on the device
int mg_solve(baorec_ctx* ctx, const float* f, float* phi, const float* phi0, baorec_solve_stats* st,
             const double* fpart = nullptr);
// readout.cu
// mode 0: shifts, 1: shifted positions, 2: one plain mesh; with p0 set a
// second field (field2) of the same gather goes to p0..p2
int readout(baorec_ctx* ctx, const float* psi3, const float* x, const float* y, const float* z,
            int64_t n, int field, int mode, float* o0, float* o1, float* o2, int field2 = 0,
            float* p0 = nullptr, float* p1 = nullptr, float* p2 = nullptr);

}  // namespace baorec
