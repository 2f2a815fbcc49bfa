// Autotuner (no reference counterpart): picks launch shapes by timing the
// candidates on the context's own meshes with CUDA events.
//   stencil: per multigrid level, 32x8x8 or 32x16x16 tiles for the tile
//            kernels (sweep; at the finest level also the accurate and the
//            running residual), where both are valid; at the finest level
//            also the streaming against the tiled residual kernels and the
//            running residual with two z-cells per thread against one, and
//            (n3 = 256) the FFT preconditioner's xy transforms + z pass
//            against its 3-D transforms, and (256 x 256 planes) the fused xy
//            kernels against cuFFT's;
//   paint:   the tile edge (4, 8 or 16 cells) of the deterministic paint,
//            on 2^21 uniform particles in the box.
// Choices live in ctx->tune and apply to every later launch of the context.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "mg_common.cuh"

namespace baorec {

int level_count(const baorec_ctx* ctx);
LG level_geom_public(const baorec_ctx* ctx, int l, float clamp);

namespace {

__global__ void uniform_particles_kernel(float* __restrict__ p, int64_t n, float3 lo, float3 span, uint32_t seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    // 32-bit integer hash per (particle, axis), kept below the box's upper edge
    float u[3];
    for (int a = 0; a < 3; ++a) {
      uint32_t h = (uint32_t)i * 2654435761u ^ (seed + 0x9E3779B9u * (uint32_t)(a + 1));
      h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
      u[a] = (float)(h >> 8) * (1.0f / 16777216.0f) * 0.999f;
    }
    p[i] = lo.x + span.x * u[0];
    p[n + i] = lo.y + span.y * u[1];
    p[2 * n + i] = lo.z + span.z * u[2];
    p[3 * n + i] = 1.0f;
  }
}

template <typename F>
int time_ms(baorec_ctx* ctx, F launch, int reps, float* ms) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int st = launch();   // warm-up
  if (st == BAOREC_OK) {
    CK(cudaEventRecord(a, ctx->stream));
    for (int r = 0; r < reps && st == BAOREC_OK; ++r) st = launch();
    CK(cudaEventRecord(b, ctx->stream));
    CK(cudaEventSynchronize(b));
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, a, b));
    *ms = t / reps;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return st;
}

constexpr int kTuneRounds = 3;   // interleaved timing rounds per candidate set

int tune_stencils(baorec_ctx* ctx) {
  CKS(mg_setup(ctx));
  const int nl = level_count(ctx);
  for (int l = 0; l < nl && l < 16; ++l) {
    Level& L = ctx->lev[l];
    if (!tile_ok(L.n) || L.n[1] % 16 || L.n[2] % 16) continue;
    CK(cudaMemsetAsync(L.f, 0, L.N * 4 * 4, ctx->stream));   // f, v, r, t
    float best = 1e30f;
    int pick = -1;
    for (int choice = 0; choice < 2; ++choice) {
      ctx->tune.big_tiles[l] = choice;
      const LG Gc = level_geom_public(ctx, l, kClamp);
      const LG G0 = level_geom_public(ctx, l, 0.0f);
      float* t = L.r + L.N;
      auto launch = [&]() -> int {
        CK(launch_rb_sweep(ctx->stream, L.v, t, L.f, Gc, 0.0f, L.needs_clamp));
        if (l == 0) {
          int np = 0;
          CK(launch_resid_acc(ctx->stream, L.v, ctx->phi_lo, nullptr, L.f, ctx->phi_hi2, ctx->phi_lo2, L.r, G0, 0.0f,
                              ctx->dred, &np));
          CK(launch_resid_diff(ctx->stream, L.v, L.f, t, G0, L.r));
        }
        return BAOREC_OK;
      };
      CK(cudaMemsetAsync(ctx->phi_lo, 0, L.N * 4 * 3, ctx->stream));
      float ms = 0.0f;
      CKS(time_ms(ctx, launch, 5, &ms));
      ctx->launches += 6 * (l == 0 ? 3 : 1);
      if (ms < best) { best = ms; pick = choice; }
    }
    ctx->tune.big_tiles[l] = pick;
  }
  // finest level: the streaming residual kernels against the tiled ones
  Level& L0 = ctx->lev[0];
  if (nl > 0 && tile_ok(L0.n) && stream_ok(L0.n)) {
    const LG G0 = level_geom_public(ctx, 0, 0.0f);
    float* t = L0.r + L0.N;
    float ms[2] = {0.0f, 0.0f};
    for (int form = 0; form < 2; ++form) {
      auto launch = [&]() -> int {
        int np = 0;
        if (form == 1) {
          CK(launch_resid_acc_stream(ctx->stream, L0.v, ctx->phi_lo, nullptr, L0.f, ctx->phi_hi2, ctx->phi_lo2, L0.r,
                                     G0, 0.0f, ctx->dred, &np));
          CK(launch_resid_diff_stream(ctx->stream, L0.v, L0.f, t, G0, L0.r));
        } else {
          CK(launch_resid_acc(ctx->stream, L0.v, ctx->phi_lo, nullptr, L0.f, ctx->phi_hi2, ctx->phi_lo2, L0.r, G0,
                              0.0f, ctx->dred, &np));
          CK(launch_resid_diff(ctx->stream, L0.v, L0.f, t, G0, L0.r));
        }
        return BAOREC_OK;
      };
      CKS(time_ms(ctx, launch, 5, &ms[form]));
      ctx->launches += 12;
    }
    ctx->tune.stream0 = ms[1] <= ms[0] ? 1 : 0;
  }
  // finest level: the tiled running residual with two z-adjacent cells per
  // thread (packed FP32x2) against one cell per thread, the packed form with
  // its window streamed in z (blocks of 16 and 32 planes), and the form with
  // TMA-staged operands and x-adjacent cell pairs (blocks of 32 and 16 planes)
  // Each candidate is timed in kTuneRounds interleaved rounds and keeps its
  // fastest: a candidate is not lost to one noisy measurement.
  if (nl > 0 && tile_ok(L0.n)) {
    float* t = L0.r + L0.N;
    float ms[7] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    const bool packed = L0.n[1] % 16 == 0 && L0.n[2] % 16 == 0;
    for (int round = 0; round < kTuneRounds; ++round)
      for (int form = 0; form < 7; ++form) {
        if (form >= 2 && form < 4 && !packed) continue;
        if (form == 6 && (L0.n[1] % 8 || L0.n[2] % 16)) continue;
        ctx->tune.pairs = form;
        const LG G0 = level_geom_public(ctx, 0, 0.0f);
        if (form >= 4 && !resid_tma_ok(G0, form == 4 ? 32 : 16)) continue;
        auto launch = [&]() -> int {
          CK(launch_resid_diff(ctx->stream, L0.v, L0.f, t, G0, L0.r));
          return BAOREC_OK;
        };
        float m = 0.0f;
        CKS(time_ms(ctx, launch, 10, &m));
        ms[form] = std::min(ms[form], m);
        ctx->launches += 11;
      }
    int best = 0;
    for (int form = 1; form < 7; ++form)
      if (ms[form] < ms[best]) best = form;
    ctx->tune.pairs = best;
  }
  // finest level: the accurate residual on 512-thread blocks (the level's
  // tiles) against 256-thread blocks on 32x8x8 and 32x8x16 tiles
  if (nl > 0 && tile_ok(L0.n)) {
    float ms[3] = {1e30f, 1e30f, 1e30f};
    for (int round = 0; round < kTuneRounds; ++round)
      for (int form = 0; form < 3; ++form) {
        ctx->tune.acc = form;
        const LG G0 = level_geom_public(ctx, 0, 0.0f);
        if (form > 0 && (size_t)tile_blocks(G0) > kRedCapacity / 2) continue;
        auto launch = [&]() -> int {
          int np = 0;
          CK(launch_resid_acc(ctx->stream, L0.v, ctx->phi_lo, nullptr, L0.f, ctx->phi_hi2, ctx->phi_lo2, L0.r, G0,
                              0.0f, ctx->dred, &np));
          return BAOREC_OK;
        };
        float m = 0.0f;
        CKS(time_ms(ctx, launch, 10, &m));
        ms[form] = std::min(ms[form], m);
        ctx->launches += 11;
      }
    int best = 0;
    for (int form = 1; form < 3; ++form)
      if (ms[form] < ms[best]) best = form;
    ctx->tune.acc = best;
  }
  // FFT preconditioner: batched xy transforms around the fused z pass (two
  // register forms; xy transforms by cuFFT or, for 256 x 256 planes, by the
  // fused kernels) against 3-D transforms with a separate multiply (n3 = 256)
  if (nl > 0 && ctx->n3 == 256) {
    const int cand[5][2] = {{0, 0}, {1, 0}, {2, 0}, {1, 1}, {2, 1}};
    const int ncand = xy_fused_ok(ctx) ? 5 : 3;
    float ms[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    for (int round = 0; round < kTuneRounds; ++round)
      for (int c = 0; c < ncand; ++c) {
        ctx->tune.zpass = cand[c][0];
        ctx->tune.xy = cand[c][1];
        auto launch = [&]() -> int { return spectral_correction(ctx, L0.f, L0.v); };
        float m = 0.0f;
        CKS(time_ms(ctx, launch, 5, &m));
        ms[c] = std::min(ms[c], m);
        ctx->launches += 6;
      }
    int pick = 1;
    for (int c = 0; c < ncand; ++c)
      if (ms[c] < ms[pick]) pick = c;
    ctx->tune.zpass = cand[pick][0];
    ctx->tune.xy = cand[pick][1];
  }
  return BAOREC_OK;
}

int tune_paint(baorec_ctx* ctx) {
  const int64_t n = 1 << 21;
  float* p = nullptr;
  CK(cudaMalloc(&p, (size_t)n * 4 * sizeof(float)));
  float3 lo = make_float3(ctx->cfg.box_min[0], ctx->cfg.box_min[1], ctx->cfg.box_min[2]);
  float3 span = make_float3(ctx->cfg.box_size[0], ctx->cfg.box_size[1], ctx->cfg.box_size[2]);
  (uniform_particles_kernel<<<8 * kNumSMs, 256, 0, ctx->stream>>>(p, n, lo, span, 12345u), ::baorec::count_launch());
  int st = cudaGetLastError() == cudaSuccess ? BAOREC_OK : set_error(ctx, BAOREC_ERR_CUDA, "autotune: particle kernel");
  float* mesh = ctx->psi;   // scratch
  ctx->psi_valid = false;
  const int cand[3] = {4, 8, 16};
  float best = 1e30f;
  int pick = ctx->tune.paint_tile;
  for (int c = 0; c < 3 && st == BAOREC_OK; ++c) {
    ctx->tune.paint_tile = cand[c];
    auto launch = [&]() -> int {
      return paint_sorted(ctx, mesh, p, p + n, p + 2 * n, p + 3 * n, n, 1, ctx->cfg.mas, BAOREC_ASYNC);
    };
    float ms = 0.0f;
    st = time_ms(ctx, launch, 3, &ms);
    if (st == BAOREC_OK && ms < best) { best = ms; pick = cand[c]; }
  }
  ctx->tune.paint_tile = pick;
  // the FP32 paint: global float atomics against the binned paint
  float ms_mode[2] = {1e30f, 1e30f};
  const int keep = ctx->tune.binned;
  for (int mode = 0; mode < 2 && st == BAOREC_OK; ++mode) {
    ctx->tune.binned = mode;
    auto launch = [&]() -> int { return paint(ctx, mesh, p, p + n, p + 2 * n, p + 3 * n, n, 1, ctx->cfg.mas, 0); };
    st = time_ms(ctx, launch, 3, &ms_mode[mode]);
  }
  ctx->tune.binned = st == BAOREC_OK ? (ms_mode[1] <= ms_mode[0] ? 1 : 0) : keep;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(p);
  return st;
}

}  // namespace
}  // namespace baorec

using namespace baorec;

extern "C" int baorec_tune_stream(const baorec_ctx* ctx) { return ctx ? ctx->tune.stream0 : -1; }

extern "C" int baorec_set_tune_stream(baorec_ctx* ctx, int stream) {
  if (!ctx || stream < -1 || stream > 1) return BAOREC_ERR_ARG;
  ctx->tune.stream0 = stream;
  return BAOREC_OK;
}

extern "C" int baorec_tune_pairs(const baorec_ctx* ctx) { return ctx ? ctx->tune.pairs : -1; }

extern "C" int baorec_set_tune_pairs(baorec_ctx* ctx, int pairs) {
  if (!ctx || pairs < 0 || pairs > 6) return BAOREC_ERR_ARG;
  ctx->tune.pairs = pairs;
  return BAOREC_OK;
}

extern "C" int baorec_tune_binned(const baorec_ctx* ctx) { return ctx ? ctx->tune.binned : -1; }

extern "C" int baorec_set_tune_binned(baorec_ctx* ctx, int binned) {
  if (!ctx || binned < 0 || binned > 1) return BAOREC_ERR_ARG;
  ctx->tune.binned = binned;
  return BAOREC_OK;
}

extern "C" int baorec_tune_acc(const baorec_ctx* ctx) { return ctx ? ctx->tune.acc : -1; }

extern "C" int baorec_set_tune_acc(baorec_ctx* ctx, int acc) {
  if (!ctx || acc < 0 || acc > 2) return BAOREC_ERR_ARG;
  ctx->tune.acc = acc;
  return BAOREC_OK;
}

extern "C" int baorec_tune_zpass(const baorec_ctx* ctx) { return ctx ? ctx->tune.zpass : -1; }

extern "C" int baorec_set_tune_zpass(baorec_ctx* ctx, int zpass) {
  if (!ctx || zpass < 0 || zpass > 2) return BAOREC_ERR_ARG;
  ctx->tune.zpass = zpass;
  return BAOREC_OK;
}

extern "C" int baorec_tune_xy(const baorec_ctx* ctx) { return ctx ? ctx->tune.xy : -1; }

extern "C" int baorec_set_tune_xy(baorec_ctx* ctx, int xy) {
  if (!ctx || xy < 0 || xy > 1) return BAOREC_ERR_ARG;
  ctx->tune.xy = xy;
  return BAOREC_OK;
}

extern "C" int baorec_autotune(baorec_ctx* ctx, uint32_t what, int32_t* paint_tile, int32_t* big_tiles) {
  if (!ctx) return BAOREC_ERR_ARG;
  if ((what & BAOREC_TUNE_STENCIL) && ctx->cfg.method == BAOREC_MULTIGRID) CKS(tune_stencils(ctx));
  if (what & BAOREC_TUNE_PAINT) CKS(tune_paint(ctx));
  ctx->tune.tuned = true;
  if (paint_tile) *paint_tile = ctx->tune.paint_tile;
  if (big_tiles)
    for (int l = 0; l < 16; ++l) big_tiles[l] = ctx->tune.big_tiles[l];
  return finish(ctx, 0);
}

extern "C" int baorec_set_tune(baorec_ctx* ctx, int32_t paint_tile, const int32_t* big_tiles) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (paint_tile < 1 || paint_tile > 16) return set_error(ctx, BAOREC_ERR_ARG, "paint tile %d outside [1, 16]", paint_tile);
  if (big_tiles)
    for (int l = 0; l < 16; ++l)
      if (big_tiles[l] < -1 || big_tiles[l] > 1) return set_error(ctx, BAOREC_ERR_ARG, "tile choice %d", big_tiles[l]);
  ctx->tune.paint_tile = paint_tile;
  if (big_tiles)
    for (int l = 0; l < 16; ++l) ctx->tune.big_tiles[l] = big_tiles[l];
  return BAOREC_OK;
}
