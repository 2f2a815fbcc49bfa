// C ABI: context lifetime, staging, error reporting and the reconstruction
// drivers (run!, setup_overdensity!, read_shifts, ...) of src/recon.jl.
#include <atomic>
#include <math.h>
#include <stdarg.h>

#include <algorithm>
#include <initializer_list>
#include <new>

#include "common.cuh"

namespace baorec {

int set_error(baorec_ctx* c, int code, const char* fmt, ...) {
  if (!c) return code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(c->msg, sizeof(c->msg), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(baorec_ctx* c, cudaError_t e, const char* what) {
  cudaGetLastError();
  return set_error(c, e == cudaErrorMemoryAllocation ? BAOREC_ERR_NOMEM : BAOREC_ERR_CUDA, "%s: %s", what,
                   cudaGetErrorString(e));
}

int cufft_fail(baorec_ctx* c, cufftResult e, const char* what) {
  return set_error(c, BAOREC_ERR_CUFFT, "%s: cufftResult %d", what, (int)e);
}

int ensure(baorec_ctx* ctx, DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return BAOREC_OK;
  if (b.p) CK(cudaFree(b.p));
  b.p = nullptr;
  b.bytes = 0;
  size_t want = bytes + bytes / 8 + 256;
  CK(cudaMalloc(&b.p, want));
  b.bytes = want;
  return BAOREC_OK;
}

int finish(baorec_ctx* ctx, uint32_t flags) {
  if (flags & BAOREC_ASYNC) return BAOREC_OK;
  CK(cudaMemcpyAsync(ctx->herr, ctx->derr, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  unsigned e = *ctx->herr;
  if (e) {
    CK(cudaMemsetAsync(ctx->derr, 0, sizeof(unsigned), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (e & kErrOOB)
      return set_error(ctx, BAOREC_ERR_OOB, "particle outside the mesh (the reference raises BoundsError)");
    if (e & kErrTimeout)
      return set_error(ctx, BAOREC_ERR_CUDA, "a device-side wait timed out (TMA-fed pipeline)");
  }
  return BAOREC_OK;
}

// Page-locked host memory (cudaHostAlloc, cudaHostRegister) is mapped into
// the device's address space: kernels read and write it over the host link
// directly, so a host array in such memory is used in place instead of being
// copied through a staging buffer (the bytes still cross the link once, but
// the transfer overlaps the kernel that consumes it).  Returns the device
// address of p, or null for pageable memory.
static const float* host_alias(const float* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<const float*>(a.devicePointer) : nullptr;
}

int stage_in(baorec_ctx* ctx, int slot, const float* p, int64_t n, uint32_t flags, const float** out) {
  if (!(flags & BAOREC_HOST) || !p || n <= 0) { *out = p; return BAOREC_OK; }
  if (const float* d = host_alias(p)) { *out = d; return BAOREC_OK; }
  CKS(ensure(ctx, ctx->stage[slot], (size_t)n * 4));
  CK(cudaMemcpyAsync(ctx->stage[slot].p, p, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  *out = (const float*)ctx->stage[slot].p;
  return BAOREC_OK;
}

int stage_out_alloc(baorec_ctx* ctx, int slot, int64_t n, uint32_t flags, float* user, float** dev) {
  if (!(flags & BAOREC_HOST)) { *dev = user; return BAOREC_OK; }
  if (user && n > 0)
    if (const float* d = host_alias(user)) { *dev = const_cast<float*>(d); return BAOREC_OK; }
  CKS(ensure(ctx, ctx->stage[slot], (size_t)(n > 0 ? n : 1) * 4));
  *dev = (float*)ctx->stage[slot].p;
  return BAOREC_OK;
}

int stage_out_copy(baorec_ctx* ctx, float* user, const float* dev, int64_t n, uint32_t flags) {
  if (!(flags & BAOREC_HOST) || n <= 0) return BAOREC_OK;
  if (dev == user || dev == host_alias(user)) return BAOREC_OK;   // written in place
  CK(cudaMemcpyAsync(user, dev, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  return BAOREC_OK;
}

// interleave4: C2R of `batch` spectra into one mesh of 4-float cells
// (component b of cell i at 4 i + b), the layout of the read-out.
static int make_plan(baorec_ctx* ctx, cufftHandle* p, cufftType t, int batch, size_t* maxw, bool interleave4 = false) {
  long long dims[3] = {ctx->n3, ctx->n2, ctx->n1};
  size_t w = 0;
  CKFFT(cufftCreate(p));
  CKFFT(cufftSetAutoAllocation(*p, 0));
  long long idist = t == CUFFT_R2C ? (long long)ctx->N : (long long)ctx->Nk;
  long long odist = t == CUFFT_R2C ? (long long)ctx->Nk : (long long)ctx->N;
  if (interleave4) {
    long long inembed[3] = {ctx->n3, ctx->n2, ctx->n1h};
    long long onembed[3] = {ctx->n3, ctx->n2, ctx->n1};
    CKFFT(cufftMakePlanMany64(*p, 3, dims, inembed, 1, (long long)ctx->Nk, onembed, 4, 1, t, batch, &w));
  } else {
    CKFFT(cufftMakePlanMany64(*p, 3, dims, nullptr, 1, idist, nullptr, 1, odist, t, batch, &w));
  }
  CKFFT(cufftSetStream(*p, ctx->stream));
  if (w > *maxw) *maxw = w;
  return BAOREC_OK;
}

static int validate(baorec_ctx* ctx, const baorec_config* c) {
  for (int a = 0; a < 3; ++a) {
    if (c->n[a] < 2 || c->n[a] > 4096) return set_error(ctx, BAOREC_ERR_ARG, "mesh size n[%d]=%d out of range", a, c->n[a]);
  }
  if (c->n[0] % 2) return set_error(ctx, BAOREC_ERR_ARG, "n[0] must be even (real-to-complex layout)");
  if ((double)c->n[0] * c->n[1] * c->n[2] >= 2147483648.0)
    return set_error(ctx, BAOREC_ERR_ARG, "mesh of %d x %d x %d cells exceeds 2^31 cells", c->n[0], c->n[1], c->n[2]);
  for (int a = 0; a < 3; ++a)
    if (!(c->box_size[a] > 0.0f)) return set_error(ctx, BAOREC_ERR_ARG, "box_size[%d] must be positive", a);
  if (!(c->bias != 0.0f)) return set_error(ctx, BAOREC_ERR_ARG, "bias must be non-zero");
  if (c->method != BAOREC_ITERATIVE && c->method != BAOREC_MULTIGRID)
    return set_error(ctx, BAOREC_ERR_ARG, "unknown method %d", c->method);
  if (c->los_mode != BAOREC_LOS_LOCAL && c->los_mode != BAOREC_LOS_GLOBAL)
    return set_error(ctx, BAOREC_ERR_ARG, "unknown los_mode %d", c->los_mode);
  if (c->mas != BAOREC_MAS_CIC && c->mas != BAOREC_MAS_TSC) return set_error(ctx, BAOREC_ERR_ARG, "unknown mas %d", c->mas);
  if (c->n_iter < 0 || c->jacobi_niterations < 0 || c->vcycle_niterations < 0 || c->nu1 < 0 || c->nu2 < 0)
    return set_error(ctx, BAOREC_ERR_ARG, "negative iteration count");
  if (c->mg_start < BAOREC_START_ZERO || c->mg_start > BAOREC_START_LEARNED)
    return set_error(ctx, BAOREC_ERR_ARG, "unknown mg_start %d", c->mg_start);
  if (c->mg_start != BAOREC_START_ZERO && !(c->start_rate > 0.0f && c->start_rate <= 1.0f))
    return set_error(ctx, BAOREC_ERR_ARG, "start_rate %g outside (0, 1]", (double)c->start_rate);
  return BAOREC_OK;
}

}  // namespace baorec

using namespace baorec;

extern "C" void baorec_config_default(baorec_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->method = BAOREC_ITERATIVE;
  c->n[0] = c->n[1] = c->n[2] = 128;
  c->box_size[0] = c->box_size[1] = c->box_size[2] = 1000.0f;
  c->los_mode = BAOREC_LOS_LOCAL;
  c->bias = 2.0f;
  c->f = 0.8f;
  c->smoothing_radius = 15.0f;
  c->beta = 0.0f;
  c->n_iter = 3;
  c->jacobi_damping_factor = 0.4f;
  c->jacobi_niterations = 5;
  c->vcycle_niterations = 6;
  c->ran_min = 0.01f;
  c->mas = BAOREC_MAS_CIC;
  c->mg_mode = BAOREC_MG_REFERENCE;
  c->nu1 = 2;
  c->nu2 = 2;
  c->rtol = 1e-6f;
  c->max_cycles = 50;
  c->mg_start = BAOREC_START_ZERO;
  c->start_rate = 0.5f;
}

static_assert(sizeof(baorec_config) == 4 * 31, "baorec_config layout is part of the ABI");
static_assert(sizeof(baorec_solve_stats) == 32, "baorec_solve_stats layout is part of the ABI");

static thread_local char g_create_msg[512];

// error of a call made without a context (baorec_last_error(NULL) reads it)
int baorec::set_error_noctx(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_create_msg, sizeof(g_create_msg), fmt, ap);
  va_end(ap);
  return code;
}

extern "C" int baorec_create(const baorec_config* cfg, baorec_ctx** out) {
  if (!cfg || !out) return BAOREC_ERR_ARG;
  *out = nullptr;
  baorec_ctx* ctx = new (std::nothrow) baorec_ctx();
  if (!ctx) return BAOREC_ERR_NOMEM;
  ctx->cfg = *cfg;
  ctx->msg[0] = 0;
  memset(&ctx->last_stats, 0, sizeof(ctx->last_stats));
  int st = validate(ctx, cfg);
  if (st != BAOREC_OK) {
    snprintf(g_create_msg, sizeof(g_create_msg), "%s", ctx->msg);
    delete ctx;
    return st;
  }
  // recon.β defaults to f / bias (src/recon.jl:11, 29)
  if (!(ctx->cfg.beta > 0.0f)) ctx->cfg.beta = ctx->cfg.f / ctx->cfg.bias;
  if (ctx->cfg.los_mode == BAOREC_LOS_LOCAL) ctx->cfg.los[0] = ctx->cfg.los[1] = ctx->cfg.los[2] = 0.0f;
  ctx->n1 = cfg->n[0]; ctx->n2 = cfg->n[1]; ctx->n3 = cfg->n[2];
  ctx->n1h = ctx->n1 / 2 + 1;
  ctx->N = (size_t)ctx->n1 * ctx->n2 * ctx->n3;
  ctx->Nk = (size_t)ctx->n1h * ctx->n2 * ctx->n3;
  auto fail = [&](int s) {
    snprintf(g_create_msg, sizeof(g_create_msg), "%s", ctx->msg);
    baorec_destroy(ctx);
    return s;
  };
#define CKC(call)                                   \
  do {                                              \
    cudaError_t _e = (call);                        \
    if (_e != cudaSuccess) return fail(cuda_fail(ctx, _e, #call)); \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CKC(cudaMalloc(&ctx->mesh3, ctx->N * 4 * 3));
  ctx->result = ctx->mesh3;
  CKC(cudaMalloc(&ctx->psi, ctx->N * 4 * 7));   // 6 iterative parts, or interleaved Ψ (4N) + its planes (3N)
  CKC(cudaMalloc(&ctx->ck, ctx->Nk * sizeof(cufftComplex) * 6));
  for (int a = 0; a < 3; ++a) CKC(cudaMalloc(&ctx->xvec[a], (size_t)cfg->n[a] * 4));
  CKC(cudaMalloc(&ctx->dred, kRedCapacity * sizeof(double)));
  CKC(cudaMalloc(&ctx->dfsum, 2 * kFsumBlocks * sizeof(double)));
  CKC(cudaMallocHost(&ctx->hred, kRedCapacity * sizeof(double)));
  CKC(cudaMalloc(&ctx->derr, sizeof(unsigned)));
  CKC(cudaMallocHost(&ctx->herr, sizeof(unsigned)));
  CKC(cudaMemset(ctx->derr, 0, sizeof(unsigned)));
  size_t maxw = 0;
  if ((st = make_plan(ctx, &ctx->plan_r2c, CUFFT_R2C, 1, &maxw)) ||
      (st = make_plan(ctx, &ctx->plan_r2c2, CUFFT_R2C, 2, &maxw)) ||
      (st = make_plan(ctx, &ctx->plan_c2r, CUFFT_C2R, 1, &maxw)) ||
      (st = make_plan(ctx, &ctx->plan_c2r2, CUFFT_C2R, 2, &maxw)) ||
      (st = make_plan(ctx, &ctx->plan_c2r3, CUFFT_C2R, 3, &maxw)) ||
      (st = make_plan(ctx, &ctx->plan_c2r6, CUFFT_C2R, 6, &maxw)))
    return fail(st);
  CKC(cudaMalloc(&ctx->fft_work, maxw > 0 ? maxw : 256));
  ctx->fft_work_bytes = maxw > 0 ? maxw : 256;
  cufftHandle plans[6] = {ctx->plan_r2c, ctx->plan_r2c2, ctx->plan_c2r, ctx->plan_c2r2, ctx->plan_c2r3, ctx->plan_c2r6};
  for (cufftHandle p : plans)
    if (cufftSetWorkArea(p, ctx->fft_work) != CUFFT_SUCCESS) return fail(set_error(ctx, BAOREC_ERR_CUFFT, "cufftSetWorkArea"));
  if ((st = zpass_prepare(ctx))) return fail(st);
  if ((st = xvec_update(ctx))) return fail(st);
  if (cfg->method == BAOREC_MULTIGRID && (st = mg_setup(ctx))) return fail(st);
#undef CKC
  *out = ctx;
  return BAOREC_OK;
}

extern "C" int baorec_destroy(baorec_ctx* ctx) {
  if (!ctx) return BAOREC_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cufftHandle plans[6] = {ctx->plan_r2c, ctx->plan_r2c2, ctx->plan_c2r, ctx->plan_c2r2, ctx->plan_c2r3, ctx->plan_c2r6};
  for (cufftHandle p : plans)
    if (p) cufftDestroy(p);
  if (ctx->plan_c2r_spec) cufftDestroy(ctx->plan_c2r_spec);
  if (ctx->plan_r2c_xy) cufftDestroy(ctx->plan_r2c_xy);
  if (ctx->plan_c2r_xy) cufftDestroy(ctx->plan_c2r_xy);
  cudaFree(ctx->xy_work);
  cudaFree(ctx->spec_work);
  cudaFree(ctx->spec_cb);
  cudaFree(ctx->fft_work);
  cudaFree(ctx->mesh3);
  cudaFree(ctx->psi);
  cudaFree(ctx->ck);
  for (int a = 0; a < 3; ++a) cudaFree(ctx->xvec[a]);
  cudaFree(ctx->phi_lo);
  cudaFree(ctx->coarse_M);
  cudaFree(ctx->stab);
  guess_free(ctx);
  if (ctx->guess_child) baorec_destroy(ctx->guess_child);
  for (cudaEvent_t e : ctx->ev_guess)
    if (e) cudaEventDestroy(e);
  for (int l = 0; l < ctx->nlev; ++l) {
    cudaFree(ctx->lev[l].f);
    for (int a = 0; a < 3; ++a) cudaFree(ctx->lev[l].ax[a]);
  }
  cudaFree(ctx->dred);
  cudaFree(ctx->dfsum);
  cudaFreeHost(ctx->hred);
  cudaFree(ctx->derr);
  cudaFreeHost(ctx->herr);
  for (auto& b : ctx->stage) cudaFree(b.p);
  for (DevBuf* b : {&ctx->sort_keys, &ctx->sort_perm, &ctx->sort_tiles, &ctx->fix_mesh, &ctx->bin_parts,
                    &ctx->pw_mesh, &ctx->pw_spec, &ctx->pw_part, &ctx->pw_nz})
    cudaFree(b->p);
  if (ctx->ev_red) cudaEventDestroy(ctx->ev_red);
  for (int s = 0; s < 2; ++s)
    for (cudaEvent_t e : {ctx->ev_in[s], ctx->ev_k[s], ctx->ev_out[s]})
      if (e) cudaEventDestroy(e);
  if (ctx->ev_begin) cudaEventDestroy(ctx->ev_begin);
  if (ctx->ev_done) cudaEventDestroy(ctx->ev_done);
  if (ctx->s_in) cudaStreamDestroy(ctx->s_in);
  if (ctx->s_out) cudaStreamDestroy(ctx->s_out);
  cudaFree(ctx->pipe_buf.p);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BAOREC_OK;
}

extern "C" const char* baorec_last_error(const baorec_ctx* ctx) { return ctx ? ctx->msg : g_create_msg; }

extern "C" void* baorec_stream(baorec_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int64_t baorec_kernel_launches(const baorec_ctx* ctx) { return ctx ? ctx->launches : 0; }

namespace baorec {
static std::atomic<int64_t> g_kernel_launches{0};
int64_t count_launch() { return g_kernel_launches.fetch_add(1, std::memory_order_relaxed) + 1; }
}  // namespace baorec

extern "C" int64_t baorec_total_kernel_launches(void) {
  return baorec::g_kernel_launches.load(std::memory_order_relaxed);
}

extern "C" float* baorec_result_ptr(baorec_ctx* ctx) { return ctx && ctx->has_result ? ctx->result : nullptr; }

extern "C" int baorec_set_box(baorec_ctx* ctx, const float box_size[3], const float box_min[3]) {
  if (!ctx || !box_size || !box_min) return BAOREC_ERR_ARG;
  for (int a = 0; a < 3; ++a)
    if (!(box_size[a] > 0.0f)) return set_error(ctx, BAOREC_ERR_ARG, "box_size[%d] must be positive", a);
  for (int a = 0; a < 3; ++a) { ctx->cfg.box_size[a] = box_size[a]; ctx->cfg.box_min[a] = box_min[a]; }
  ctx->psi_valid = false;
  CKS(xvec_update(ctx));
  if (ctx->nlev > 0) CKS(mg_update_tables(ctx));
  return BAOREC_OK;
}

extern "C" int baorec_get_box(const baorec_ctx* ctx, float box_size[3], float box_min[3]) {
  if (!ctx) return BAOREC_ERR_ARG;
  for (int a = 0; a < 3; ++a) { box_size[a] = ctx->cfg.box_size[a]; box_min[a] = ctx->cfg.box_min[a]; }
  return BAOREC_OK;
}

extern "C" int baorec_setup_box(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                                float pad, uint32_t flags, float box_size_out[3], float box_min_out[3]) {
  if (!ctx || !x || !y || !z || n <= 0 || !box_size_out || !box_min_out)
    return set_error(ctx, BAOREC_ERR_ARG, "setup_box: empty or missing particle arrays");
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float mn[3], mx[3];
  CKS(minmax3(ctx, dx, dy, dz, n, mn, mx));
  // src/utils.jl:103-105, FP32 arithmetic
  float half = pad / 2.0f;
  float side = -INFINITY;
  for (int a = 0; a < 3; ++a) {
    box_min_out[a] = mn[a] - half;
    float bmax = mx[a] + half;
    side = fmaxf(side, bmax - box_min_out[a]);
  }
  for (int a = 0; a < 3; ++a) box_size_out[a] = side;
  return BAOREC_OK;
}

static int paint_api(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n,
                     int wrap, uint32_t flags, int mas) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!mesh || n < 0 || (n > 0 && (!x || !y || !z || !w)))
    return set_error(ctx, BAOREC_ERR_ARG, "paint: missing mesh or particle arrays");
  const float *dx, *dy, *dz, *dw;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  CKS(stage_in(ctx, 3, w, n, flags, &dw));
  CKS(paint(ctx, mesh, (float*)dx, (float*)dy, (float*)dz, dw, n, wrap, mas, flags));
  if ((flags & BAOREC_HOST) && (flags & BAOREC_WRITEBACK) && wrap && n > 0) {
    CKS(stage_out_copy(ctx, x, dx, n, flags));
    CKS(stage_out_copy(ctx, y, dy, n, flags));
    CKS(stage_out_copy(ctx, z, dz, n, flags));
  }
  ctx->psi_valid = false;
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

extern "C" int baorec_cic(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n,
                          int wrap, uint32_t flags) {
  return paint_api(ctx, mesh, x, y, z, w, n, wrap, flags, BAOREC_MAS_CIC);
}

extern "C" int baorec_tsc(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n,
                          int wrap, uint32_t flags) {
  return paint_api(ctx, mesh, x, y, z, w, n, wrap, flags, BAOREC_MAS_TSC);
}

// setup_overdensity!, data only (src/recon.jl:42-57), on staged device arrays.
static int overdensity_data(baorec_ctx* ctx, float* delta, float* x, float* y, float* z, const float* w,
                            int64_t n, int wrap, uint32_t flags) {
  CKS(paint(ctx, delta, x, y, z, w, n, wrap, ctx->cfg.mas, flags));
  CKS(smooth(ctx, delta));
  return normalize_data(ctx, delta);
}

// setup_overdensity! with randoms (src/recon.jl:60-91); `ran` is a scratch mesh.
static int overdensity_randoms(baorec_ctx* ctx, float* delta, float* ran, const float* x, const float* y,
                               const float* z, const float* w, int64_t n, const float* rx, const float* ry,
                               const float* rz, const float* rw, int64_t nr, uint32_t flags,
                               double* fpart = nullptr) {
  CK(cudaMemsetAsync(ran, 0, ctx->N * 4, ctx->stream));
  CKS(paint(ctx, delta, (float*)x, (float*)y, (float*)z, w, n, 0, ctx->cfg.mas, flags & ~BAOREC_WRITEBACK));
  CKS(paint(ctx, ran, (float*)rx, (float*)ry, (float*)rz, rw, nr, 0, ctx->cfg.mas, flags & ~BAOREC_WRITEBACK));
  CKS(smooth_pair(ctx, delta, ran));
  return normalize_randoms(ctx, delta, ran, nr, fpart);
}

struct Staged {
  const float *x, *y, *z, *w, *rx, *ry, *rz, *rw;
};

static int ensure_psi(baorec_ctx* ctx);

static int stage_catalogs(baorec_ctx* ctx, const float* x, const float* y, const float* z, const float* w, int64_t n,
                          const float* rx, const float* ry, const float* rz, const float* rw, int64_t nr,
                          uint32_t flags, Staged* s) {
  CKS(stage_in(ctx, 0, x, n, flags, &s->x));
  CKS(stage_in(ctx, 1, y, n, flags, &s->y));
  CKS(stage_in(ctx, 2, z, n, flags, &s->z));
  CKS(stage_in(ctx, 3, w, n, flags, &s->w));
  s->rx = s->ry = s->rz = s->rw = nullptr;
  if (rx) {
    CKS(stage_in(ctx, 4, rx, nr, flags, &s->rx));
    CKS(stage_in(ctx, 5, ry, nr, flags, &s->ry));
    CKS(stage_in(ctx, 6, rz, nr, flags, &s->rz));
    CKS(stage_in(ctx, 7, rw, nr, flags, &s->rw));
  }
  return BAOREC_OK;
}

static int check_catalogs(baorec_ctx* ctx, const float* x, const float* y, const float* z, const float* w, int64_t n,
                          const float* rx, const float* ry, const float* rz, const float* rw, int64_t nr) {
  if (n < 0 || (n > 0 && (!x || !y || !z || !w))) return set_error(ctx, BAOREC_ERR_ARG, "missing data arrays");
  if (rx || ry || rz || rw) {
    if (!rx || !ry || !rz || !rw || nr <= 0) return set_error(ctx, BAOREC_ERR_ARG, "incomplete or empty randoms");
  }
  return BAOREC_OK;
}

extern "C" int baorec_setup_overdensity(baorec_ctx* ctx, float* delta, float* x, float* y, float* z,
                                        const float* w, int64_t n, int wrap, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!delta) return set_error(ctx, BAOREC_ERR_ARG, "setup_overdensity: missing mesh");
  CKS(check_catalogs(ctx, x, y, z, w, n, nullptr, nullptr, nullptr, nullptr, 0));
  Staged s;
  CKS(stage_catalogs(ctx, x, y, z, w, n, nullptr, nullptr, nullptr, nullptr, 0, flags, &s));
  CKS(overdensity_data(ctx, delta, (float*)s.x, (float*)s.y, (float*)s.z, s.w, n, wrap, flags));
  if ((flags & BAOREC_HOST) && (flags & BAOREC_WRITEBACK) && wrap) {
    CKS(stage_out_copy(ctx, x, s.x, n, flags));
    CKS(stage_out_copy(ctx, y, s.y, n, flags));
    CKS(stage_out_copy(ctx, z, s.z, n, flags));
  }
  ctx->psi_valid = false;
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

extern "C" int baorec_setup_overdensity_randoms(baorec_ctx* ctx, float* delta, const float* x, const float* y,
                                                const float* z, const float* w, int64_t n, const float* rx,
                                                const float* ry, const float* rz, const float* rw, int64_t nr,
                                                uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!delta) return set_error(ctx, BAOREC_ERR_ARG, "setup_overdensity: missing mesh");
  if (!rx) return set_error(ctx, BAOREC_ERR_ARG, "setup_overdensity: missing randoms");
  CKS(check_catalogs(ctx, x, y, z, w, n, rx, ry, rz, rw, nr));
  Staged s;
  CKS(stage_catalogs(ctx, x, y, z, w, n, rx, ry, rz, rw, nr, flags, &s));
  // the randoms mesh must not alias delta; use the context mesh after delta when adjacent
  float* ran = (delta == ctx->mesh3 || delta == ctx->mesh3 + ctx->N) ? delta + ctx->N : ctx->psi;
  CKS(overdensity_randoms(ctx, delta, ran, s.x, s.y, s.z, s.w, n, s.rx, s.ry, s.rz, s.rw, nr, flags));
  ctx->psi_valid = false;
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

extern "C" int baorec_iterate(baorec_ctx* ctx, float* delta_r, const float* delta_s, int iter) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!delta_r || !delta_s || iter < 1) return set_error(ctx, BAOREC_ERR_ARG, "iterate: bad arguments");
  CKS(iterate(ctx, delta_r, delta_s, iter));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_jacobi(baorec_ctx* ctx, float* v, const float* f, const int32_t nl[3], int niter) {
  if (!ctx) return BAOREC_ERR_ARG;
  CKS(mg_setup(ctx));
  int l = -1;
  for (int q = 0; q < ctx->nlev; ++q)
    if (ctx->lev[q].n[0] == nl[0] && ctx->lev[q].n[1] == nl[1] && ctx->lev[q].n[2] == nl[2]) l = q;
  if (l < 0) return set_error(ctx, BAOREC_ERR_ARG, "jacobi: not a level of this mesh");
  const int n3[3] = {nl[0], nl[1], nl[2]};
  CKS(mg_jacobi(ctx, v, f, n3, niter, ctx->lev[l].r + ctx->lev[l].N));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_residual(baorec_ctx* ctx, float* r, const float* v, const float* f, const int32_t nl[3]) {
  if (!ctx) return BAOREC_ERR_ARG;
  CKS(mg_setup(ctx));
  const int n3[3] = {nl[0], nl[1], nl[2]};
  CKS(mg_residual(ctx, r, v, f, n3));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_reduce(baorec_ctx* ctx, float* coarse, const float* fine, const int32_t nl[3]) {
  if (!ctx) return BAOREC_ERR_ARG;
  const int n3[3] = {nl[0], nl[1], nl[2]};
  CKS(mg_reduce(ctx, coarse, fine, n3));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_prolong(baorec_ctx* ctx, float* fine, const float* coarse, const int32_t nl[3]) {
  if (!ctx) return BAOREC_ERR_ARG;
  const int n3[3] = {nl[0], nl[1], nl[2]};
  CKS(mg_prolong(ctx, fine, coarse, n3, 0));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_vcycle(baorec_ctx* ctx, float* v, const float* f, const int32_t nl[3]) {
  if (!ctx) return BAOREC_ERR_ARG;
  CKS(mg_setup(ctx));
  int l = -1;
  for (int q = 0; q < ctx->nlev; ++q)
    if (ctx->lev[q].n[0] == nl[0] && ctx->lev[q].n[1] == nl[1] && ctx->lev[q].n[2] == nl[2]) l = q;
  if (l < 0) return set_error(ctx, BAOREC_ERR_ARG, "vcycle: not a level of this mesh");
  CKS(mg_vcycle_ref(ctx, l, v, f));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_fmg(baorec_ctx* ctx, const float* f, float* phi) {
  if (!ctx || !f || !phi) return set_error(ctx, BAOREC_ERR_ARG, "fmg: missing mesh");
  CKS(mg_fmg(ctx, f, phi));
  return finish(ctx, 0);
}

extern "C" int baorec_mg_solve(baorec_ctx* ctx, const float* f, float* phi, const float* phi0,
                               baorec_solve_stats* stats) {
  if (!ctx || !f || !phi) return set_error(ctx, BAOREC_ERR_ARG, "mg_solve: missing mesh");
  int st = mg_solve(ctx, f, phi, phi0, stats);
  int st2 = finish(ctx, 0);
  return st != BAOREC_OK ? st : st2;
}

extern "C" int baorec_last_solve_stats(const baorec_ctx* ctx, baorec_solve_stats* stats) {
  if (!ctx || !stats) return BAOREC_ERR_ARG;
  *stats = ctx->last_stats;
  return BAOREC_OK;
}

extern "C" int baorec_start_residual(baorec_ctx* ctx, const float* f, int start, double* rel_residual) {
  if (!ctx || !f || !rel_residual || start < BAOREC_START_ZERO || start > BAOREC_START_LEARNED)
    return set_error(ctx, BAOREC_ERR_ARG, "start_residual: bad arguments");
  CKS(start_residual(ctx, f, start, rel_residual));
  return finish(ctx, 0);
}

extern "C" int baorec_solve_history(const baorec_ctx* ctx, double* rho, int32_t* kind, int cap) {
  if (!ctx || cap < 0 || (cap > 0 && (!rho || !kind))) return -BAOREC_ERR_ARG;
  const int n = (int)ctx->hist_rho.size();
  for (int i = 0; i < n && i < cap; ++i) {
    rho[i] = ctx->hist_rho[i];
    kind[i] = ctx->hist_kind[i];
  }
  return n;
}

// reconstructed_overdensity! (src/recon.jl:93-132) into ctx->result.
static int recon_iterative(baorec_ctx* ctx, const Staged& s, int64_t n, int64_t nr, uint32_t flags) {
  float* A = ctx->mesh3;          // δ_r = result
  float* B = A + ctx->N;          // randoms
  float* C = B + ctx->N;          // δ_s
  CK(cudaMemsetAsync(A, 0, ctx->N * 4, ctx->stream));
  if (s.rx) CKS(overdensity_randoms(ctx, A, B, s.x, s.y, s.z, s.w, n, s.rx, s.ry, s.rz, s.rw, nr, flags));
  else CKS(overdensity_data(ctx, A, (float*)s.x, (float*)s.y, (float*)s.z, s.w, n, 1, flags));
  CK(cudaMemcpyAsync(C, A, ctx->N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  for (int it = 1; it <= ctx->cfg.n_iter; ++it) CKS(iterate(ctx, A, C, it));
  ctx->has_result = true;
  ctx->psi_valid = false;
  return BAOREC_OK;
}

// Device-pointer, host-sync-free forms for graph capture (batch.cu): the
// data-only iterative reconstruction and the shifted positions.
int baorec::reconstruct_iterative_device(baorec_ctx* ctx, float* x, float* y, float* z, const float* w, int64_t n) {
  Staged s = {x, y, z, w, nullptr, nullptr, nullptr, nullptr};
  return recon_iterative(ctx, s, n, 0, BAOREC_ASYNC);
}

int baorec::positions_device(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n, int field,
                             float* ox, float* oy, float* oz) {
  CKS(ensure_psi(ctx));
  return readout(ctx, ctx->psi, x, y, z, n, field, 1, ox, oy, oz);
}

// reconstructed_potential! (src/recon.jl:184-212) into ctx->result.
static int recon_multigrid(baorec_ctx* ctx, const Staged& s, int64_t n, int64_t nr, uint32_t flags) {
  CKS(mg_setup(ctx));
  float* A = ctx->mesh3;          // φ = result
  float* B = A + ctx->N;          // δ
  float* C = B + ctx->N;          // randoms
  CK(cudaMemsetAsync(B, 0, ctx->N * 4, ctx->stream));
  // the normalisation pass also sums δ and δ² for the solve that follows
  const bool sums = s.rx && ctx->cfg.mg_mode == BAOREC_MG_CONVERGENT;
  if (s.rx)
    CKS(overdensity_randoms(ctx, B, C, s.x, s.y, s.z, s.w, n, s.rx, s.ry, s.rz, s.rw, nr, flags,
                            sums ? ctx->dfsum : nullptr));
  else CKS(overdensity_data(ctx, B, (float*)s.x, (float*)s.y, (float*)s.z, s.w, n, 1, flags));
  int st = BAOREC_OK;
  ctx->psi_ahead = false;
  if (ctx->cfg.mg_mode == BAOREC_MG_CONVERGENT) {
    ctx->want_psi_ahead = true;
    st = mg_solve(ctx, B, A, nullptr, nullptr, sums ? ctx->dfsum : nullptr);
    ctx->want_psi_ahead = false;
  } else {
    st = mg_fmg(ctx, B, A);
  }
  ctx->has_result = true;
  // the solve's last step computed the displacement of the returned solution
  ctx->psi_valid = st == BAOREC_OK && ctx->psi_ahead;
  ctx->psi_ahead = false;
  return st;
}

static int recon_common(baorec_ctx* ctx, int method, float* x, float* y, float* z, const float* w, int64_t n,
                        const float* rx, const float* ry, const float* rz, const float* rw, int64_t nr,
                        uint32_t flags, bool setup_box_from_randoms) {
  if (!ctx) return BAOREC_ERR_ARG;
  CKS(check_catalogs(ctx, x, y, z, w, n, rx, ry, rz, rw, nr));
  if (method != ctx->cfg.method)
    return set_error(ctx, BAOREC_ERR_ARG, "context was created for the other reconstruction method");
  if (setup_box_from_randoms && rx) {
    // run! with randoms: recon.box_size, recon.box_min = setup_box(randoms, 500) (src/recon.jl:172, 253)
    float bs[3], bm[3];
    CKS(baorec_setup_box(ctx, rx, ry, rz, nr, 500.0f, flags & ~BAOREC_ASYNC, bs, bm));
    CKS(baorec_set_box(ctx, bs, bm));
  }
  Staged s;
  CKS(stage_catalogs(ctx, x, y, z, w, n, rx, ry, rz, rw, nr, flags, &s));
  int st = method == BAOREC_ITERATIVE ? recon_iterative(ctx, s, n, nr, flags) : recon_multigrid(ctx, s, n, nr, flags);
  if (st != BAOREC_OK && st != BAOREC_ERR_NOT_CONVERGED) return st;
  if (!s.rx && (flags & BAOREC_HOST) && (flags & BAOREC_WRITEBACK)) {
    CKS(stage_out_copy(ctx, x, s.x, n, flags));
    CKS(stage_out_copy(ctx, y, s.y, n, flags));
    CKS(stage_out_copy(ctx, z, s.z, n, flags));
  }
  int st2 = finish(ctx, (flags & BAOREC_HOST) && (flags & BAOREC_WRITEBACK) ? (flags & ~BAOREC_ASYNC) : flags);
  return st != BAOREC_OK ? st : st2;
}

extern "C" int baorec_reconstructed_overdensity(baorec_ctx* ctx, float* x, float* y, float* z, const float* w,
                                                int64_t n, const float* rx, const float* ry, const float* rz,
                                                const float* rw, int64_t nr, uint32_t flags) {
  return recon_common(ctx, BAOREC_ITERATIVE, x, y, z, w, n, rx, ry, rz, rw, nr, flags, false);
}

extern "C" int baorec_reconstructed_potential(baorec_ctx* ctx, float* x, float* y, float* z, const float* w,
                                              int64_t n, const float* rx, const float* ry, const float* rz,
                                              const float* rw, int64_t nr, uint32_t flags) {
  return recon_common(ctx, BAOREC_MULTIGRID, x, y, z, w, n, rx, ry, rz, rw, nr, flags, false);
}

extern "C" int baorec_run(baorec_ctx* ctx, float* x, float* y, float* z, const float* w, int64_t n, const float* rx,
                          const float* ry, const float* rz, const float* rw, int64_t nr, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  return recon_common(ctx, ctx->cfg.method, x, y, z, w, n, rx, ry, rz, rw, nr, flags, true);
}

extern "C" int baorec_get_result(baorec_ctx* ctx, float* out, uint32_t flags) {
  if (!ctx || !out) return set_error(ctx, BAOREC_ERR_ARG, "get_result: missing output");
  if (!ctx->has_result) return set_error(ctx, BAOREC_ERR_STATE, "no reconstruction result yet (run! first)");
  CK(cudaMemcpyAsync(out, ctx->result, ctx->N * 4,
                     (flags & BAOREC_HOST) ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, ctx->stream));
  return finish(ctx, (flags & BAOREC_HOST) ? 0 : flags);
}

extern "C" int baorec_set_result(baorec_ctx* ctx, const float* in, uint32_t flags) {
  if (!ctx || !in) return set_error(ctx, BAOREC_ERR_ARG, "set_result: missing input");
  if (in != ctx->result)
    CK(cudaMemcpyAsync(ctx->result, in, ctx->N * 4,
                       (flags & BAOREC_HOST) ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->has_result = true;
  ctx->psi_valid = false;
  return finish(ctx, (flags & BAOREC_HOST) ? 0 : flags);
}

static int ensure_psi(baorec_ctx* ctx) {
  if (!ctx->has_result) return set_error(ctx, BAOREC_ERR_STATE, "no reconstruction result yet (run! first)");
  if (ctx->psi_valid) return BAOREC_OK;
  CKS(displacement_meshes(ctx, ctx->result, ctx->psi));
  ctx->psi_valid = true;
  return BAOREC_OK;
}

extern "C" int baorec_set_gradient(baorec_ctx* ctx, int32_t mode) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (mode != BAOREC_GRADIENT_FFT && mode != BAOREC_GRADIENT_FD)
    return set_error(ctx, BAOREC_ERR_ARG, "set_gradient: mode must be BAOREC_GRADIENT_FFT or BAOREC_GRADIENT_FD");
  if (mode == BAOREC_GRADIENT_FD && ctx->cfg.method != BAOREC_MULTIGRID)
    return set_error(ctx, BAOREC_ERR_ARG, "set_gradient: the finite-difference gradient is for multigrid contexts");
  if (mode != ctx->grad_mode) {
    ctx->grad_mode = mode;
    ctx->psi_valid = false;
  }
  return BAOREC_OK;
}

extern "C" int baorec_displacement_meshes(baorec_ctx* ctx, float* px, float* py, float* pz) {
  if (!ctx || !px || !py || !pz) return set_error(ctx, BAOREC_ERR_ARG, "displacement_meshes: missing output");
  CKS(ensure_psi(ctx));
  // the context keeps Ψ interleaved (4 floats per cell); copy out one component per mesh
  float* out[3] = {px, py, pz};
  for (int a = 0; a < 3; ++a)
    CK(cudaMemcpy2DAsync(out[a], sizeof(float), ctx->psi + a, 4 * sizeof(float), sizeof(float), ctx->N,
                         cudaMemcpyDeviceToDevice, ctx->stream));
  return finish(ctx, 0);
}

extern "C" int baorec_read_cic(baorec_ctx* ctx, const float* mesh, const float* x, const float* y, const float* z,
                               int64_t n, float* out, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!mesh || !out || n < 0 || (n > 0 && (!x || !y || !z))) return set_error(ctx, BAOREC_ERR_ARG, "read_cic: bad arguments");
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float* dout;
  CKS(stage_out_alloc(ctx, 4, n, flags, out, &dout));
  CKS(readout(ctx, mesh, dx, dy, dz, n, 0, 2, dout, nullptr, nullptr));
  CKS(stage_out_copy(ctx, out, dout, n, flags));
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

// Read-out of host particles to host outputs in chunks of kPipeChunk: the
// copy-in of chunk c+1 (stream s_in), the read-out of chunk c (the context
// stream) and the copy-out of chunk c-1 (s_out) overlap, on two staging
// slots guarded by events.  The same kernel on the same particles: results
// are those of the unchunked call.
static constexpr int64_t kPipeChunk = (int64_t)1 << 20;

// Every array page-locked: the read-out kernel reads the positions and writes
// the results in place over the host link, with no staging or chunking.
static bool all_host_alias(std::initializer_list<const float*> ps) {
  for (const float* p : ps)
    if (!host_alias(p)) return false;
  return true;
}

static int readout_pipelined(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n, int field,
                             int mode, float* const outs[6], int nout, int field2) {
  if (!ctx->s_in) {
    CK(cudaStreamCreateWithFlags(&ctx->s_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking));
    for (int s = 0; s < 2; ++s) {
      CK(cudaEventCreateWithFlags(&ctx->ev_in[s], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->ev_k[s], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->ev_out[s], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&ctx->ev_begin, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->ev_done, cudaEventDisableTiming));
  }
  constexpr int kPer = 9;   // 3 inputs + up to 6 outputs per slot
  CKS(ensure(ctx, ctx->pipe_buf, (size_t)2 * kPer * kPipeChunk * sizeof(float)));
  float* base = (float*)ctx->pipe_buf.p;
  auto buf = [&](int s, int k) { return base + ((size_t)s * kPer + k) * kPipeChunk; };
  // nothing of this call starts before the work already on the context stream
  CK(cudaEventRecord(ctx->ev_begin, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->s_in, ctx->ev_begin, 0));
  CK(cudaStreamWaitEvent(ctx->s_out, ctx->ev_begin, 0));
  const float* X[3] = {x, y, z};
  const int64_t nch = (n + kPipeChunk - 1) / kPipeChunk;
  for (int64_t c = 0; c < nch; ++c) {
    const int s = (int)(c & 1);
    const int64_t off = c * kPipeChunk, m = std::min(kPipeChunk, n - off);
    if (c >= 2) CK(cudaStreamWaitEvent(ctx->s_in, ctx->ev_k[s], 0));   // chunk c-2 has read its inputs
    for (int a = 0; a < 3; ++a)
      CK(cudaMemcpyAsync(buf(s, a), X[a] + off, (size_t)m * 4, cudaMemcpyHostToDevice, ctx->s_in));
    CK(cudaEventRecord(ctx->ev_in[s], ctx->s_in));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_in[s], 0));
    if (c >= 2) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_out[s], 0));   // chunk c-2's outputs are out
    CKS(readout(ctx, ctx->psi, buf(s, 0), buf(s, 1), buf(s, 2), m, field, mode, buf(s, 3), buf(s, 4), buf(s, 5),
                field2, nout == 6 ? buf(s, 6) : nullptr, nout == 6 ? buf(s, 7) : nullptr,
                nout == 6 ? buf(s, 8) : nullptr));
    CK(cudaEventRecord(ctx->ev_k[s], ctx->stream));
    CK(cudaStreamWaitEvent(ctx->s_out, ctx->ev_k[s], 0));
    for (int k = 0; k < nout; ++k)
      CK(cudaMemcpyAsync(outs[k] + off, buf(s, 3 + k), (size_t)m * 4, cudaMemcpyDeviceToHost, ctx->s_out));
    CK(cudaEventRecord(ctx->ev_out[s], ctx->s_out));
  }
  // the context stream (and so the caller's synchronisation) covers the copies
  CK(cudaEventRecord(ctx->ev_done, ctx->s_out));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_done, 0));
  CK(cudaEventRecord(ctx->ev_done, ctx->s_in));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_done, 0));
  return BAOREC_OK;
}

static int shifts_common(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n, int field,
                         float* o0, float* o1, float* o2, uint32_t flags, int mode) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || (n > 0 && (!x || !y || !z || !o0 || !o1 || !o2)))
    return set_error(ctx, BAOREC_ERR_ARG, "read_shifts: bad arguments");
  if (field < BAOREC_FIELD_DISP || field > BAOREC_FIELD_SUM) return set_error(ctx, BAOREC_ERR_ARG, "unknown field %d", field);
  CKS(ensure_psi(ctx));
  if ((flags & BAOREC_HOST) && n > 2 * kPipeChunk && !all_host_alias({x, y, z, o0, o1, o2})) {
    float* const outs[6] = {o0, o1, o2, nullptr, nullptr, nullptr};
    CKS(readout_pipelined(ctx, x, y, z, n, field, mode, outs, 3, 0));
    return finish(ctx, flags & ~BAOREC_ASYNC);
  }
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float *d0, *d1, *d2;
  CKS(stage_out_alloc(ctx, 4, n, flags, o0, &d0));
  CKS(stage_out_alloc(ctx, 5, n, flags, o1, &d1));
  CKS(stage_out_alloc(ctx, 6, n, flags, o2, &d2));
  CKS(readout(ctx, ctx->psi, dx, dy, dz, n, field, mode, d0, d1, d2));
  CKS(stage_out_copy(ctx, o0, d0, n, flags));
  CKS(stage_out_copy(ctx, o1, d1, n, flags));
  CKS(stage_out_copy(ctx, o2, d2, n, flags));
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

extern "C" int baorec_reconstructed_positions2(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                                               int64_t n, int field_a, float* oxa, float* oya, float* oza,
                                               int field_b, float* oxb, float* oyb, float* ozb, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || (n > 0 && (!x || !y || !z || !oxa || !oya || !oza || !oxb || !oyb || !ozb)))
    return set_error(ctx, BAOREC_ERR_ARG, "reconstructed_positions2: bad arguments");
  for (int fl : {field_a, field_b})
    if (fl < BAOREC_FIELD_DISP || fl > BAOREC_FIELD_SUM) return set_error(ctx, BAOREC_ERR_ARG, "unknown field %d", fl);
  CKS(ensure_psi(ctx));
  if ((flags & BAOREC_HOST) && n > 2 * kPipeChunk && !all_host_alias({x, y, z, oxa, oya, oza, oxb, oyb, ozb})) {
    float* const po[6] = {oxa, oya, oza, oxb, oyb, ozb};
    CKS(readout_pipelined(ctx, x, y, z, n, field_a, 1, po, 6, field_b));
    return finish(ctx, flags & ~BAOREC_ASYNC);
  }
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float* outs[6] = {oxa, oya, oza, oxb, oyb, ozb};
  const int slots[6] = {4, 5, 6, 8, 9, 10};
  float* dev[6];
  for (int k = 0; k < 6; ++k) CKS(stage_out_alloc(ctx, slots[k], n, flags, outs[k], &dev[k]));
  CKS(readout(ctx, ctx->psi, dx, dy, dz, n, field_a, 1, dev[0], dev[1], dev[2], field_b, dev[3], dev[4], dev[5]));
  for (int k = 0; k < 6; ++k) CKS(stage_out_copy(ctx, outs[k], dev[k], n, flags));
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}

extern "C" int baorec_read_shifts(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                                  int field, float* sx, float* sy, float* sz, uint32_t flags) {
  return shifts_common(ctx, x, y, z, n, field, sx, sy, sz, flags, 0);
}

extern "C" int baorec_reconstructed_positions(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                                              int64_t n, int field, float* ox, float* oy, float* oz, uint32_t flags) {
  return shifts_common(ctx, x, y, z, n, field, ox, oy, oz, flags, 1);
}
