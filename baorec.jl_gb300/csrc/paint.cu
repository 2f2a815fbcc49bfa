// Mass assignment: CIC / TSC painting, cell binning, bounding box.
//
// Index arithmetic follows src/mas.jl:7-35 (BAOrec.jl) operation by
// operation with IEEE round-to-nearest intrinsics and no FMA contraction, so
// cell indices and fractional weights are bit-identical to the reference's
// FP32 CPU path.
#include "paint_common.cuh"

namespace baorec {
namespace {

// Adds a to cell x0 and b to cell x1 of the mesh row starting at `row`.  With
// VEC (16-byte aligned rows) a pair x1 = x0 + 1 inside one aligned group of
// four cells is one 16-byte vector reduction (the other two lanes add +0,
// which leaves every cell unchanged): 5 reductions per particle on average
// instead of 8.
template <bool VEC>
__device__ __forceinline__ void red_pair(float* __restrict__ row, int x0, int x1, float a, float b) {
  const int k = x0 & 3;
  if (VEC && x1 == x0 + 1 && k != 3) {
    float4 v;
    v.x = k == 0 ? a : 0.0f;
    v.y = k == 0 ? b : (k == 1 ? a : 0.0f);
    v.z = k == 1 ? b : (k == 2 ? a : 0.0f);
    v.w = k == 2 ? b : 0.0f;
    atomicAdd(reinterpret_cast<float4*>(row + (x0 - k)), v);
  } else {
    atomicAdd(row + x0, a);
    atomicAdd(row + x1, b);
  }
}

template <bool VEC>
__global__ void cic_paint_kernel(float* __restrict__ mesh, float* __restrict__ x, float* __restrict__ y,
                                 float* __restrict__ z, const float* __restrict__ w, int64_t n,
                                 PaintGeom g, int writeback, unsigned* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) {
      px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g);
      if (writeback) { x[i] = px; y[i] = py; z[i] = pz; }
    }
    int x0, x1, y0, y1, z0, z1;
    float wx1, wy1, wz1;
    bool ok = cic_axis(cic_coord(px, g.bmin[0], g.fn[0], g.L[0]), g.n[0], g.wrap, x0, x1, wx1);
    ok &= cic_axis(cic_coord(py, g.bmin[1], g.fn[1], g.L[1]), g.n[1], g.wrap, y0, y1, wy1);
    ok &= cic_axis(cic_coord(pz, g.bmin[2], g.fn[2], g.L[2]), g.n[2], g.wrap, z0, z1, wz1);
    if (!ok) { atomicOr(err, kErrOOB); continue; }
    float wt = w[i];
    float wx0 = __fmul_rn(__fsub_rn(1.0f, wx1), wt);
    wx1 = __fmul_rn(wx1, wt);
    float wy0 = __fsub_rn(1.0f, wy1), wz0 = __fsub_rn(1.0f, wz1);
    x0--; x1--; y0--; y1--; z0--; z1--;
    red_pair<VEC>(mesh + lin(0, y0, z0, g), x0, x1, __fmul_rn(__fmul_rn(wx0, wy0), wz0),
                  __fmul_rn(__fmul_rn(wx1, wy0), wz0));
    red_pair<VEC>(mesh + lin(0, y1, z0, g), x0, x1, __fmul_rn(__fmul_rn(wx0, wy1), wz0),
                  __fmul_rn(__fmul_rn(wx1, wy1), wz0));
    red_pair<VEC>(mesh + lin(0, y0, z1, g), x0, x1, __fmul_rn(__fmul_rn(wx0, wy0), wz1),
                  __fmul_rn(__fmul_rn(wx1, wy0), wz1));
    red_pair<VEC>(mesh + lin(0, y1, z1, g), x0, x1, __fmul_rn(__fmul_rn(wx0, wy1), wz1),
                  __fmul_rn(__fmul_rn(wx1, wy1), wz1));
  }
}

__global__ void tsc_paint_kernel(float* __restrict__ mesh, float* __restrict__ x, float* __restrict__ y,
                                 float* __restrict__ z, const float* __restrict__ w, int64_t n,
                                 PaintGeom g, int writeback, unsigned* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) {
      px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g);
      if (writeback) { x[i] = px; y[i] = py; z[i] = pz; }
    }
    int ix[3], iy[3], iz[3];
    float wx[3], wy[3], wz[3];
    bool ok = tsc_axis(px, g.bmin[0], g.fn[0], g.L[0], g.n[0], g.wrap, ix, wx);
    ok &= tsc_axis(py, g.bmin[1], g.fn[1], g.L[1], g.n[1], g.wrap, iy, wy);
    ok &= tsc_axis(pz, g.bmin[2], g.fn[2], g.L[2], g.n[2], g.wrap, iz, wz);
    if (!ok) { atomicOr(err, kErrOOB); continue; }
    float wt = w[i];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int a = 0; a < 3; ++a)
          atomicAdd(mesh + lin(ix[a], iy[b], iz[c], g),
                    __fmul_rn(__fmul_rn(__fmul_rn(wt, wx[a]), wy[b]), wz[c]));
  }
}

__global__ void cell_bins_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                 const float* __restrict__ z, int64_t n, PaintGeom g,
                                 int32_t* __restrict__ keys, int32_t* __restrict__ counts,
                                 unsigned* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) { px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g); }
    int x0, x1, y0, y1, z0, z1;
    float t;
    bool ok = cic_axis(cic_coord(px, g.bmin[0], g.fn[0], g.L[0]), g.n[0], g.wrap, x0, x1, t);
    ok &= cic_axis(cic_coord(py, g.bmin[1], g.fn[1], g.L[1]), g.n[1], g.wrap, y0, y1, t);
    ok &= cic_axis(cic_coord(pz, g.bmin[2], g.fn[2], g.L[2]), g.n[2], g.wrap, z0, z1, t);
    // the count mesh only needs the lower cell in range
    bool lo_ok = x0 >= 1 && x0 <= g.n[0] && y0 >= 1 && y0 <= g.n[1] && z0 >= 1 && z0 <= g.n[2];
    int32_t key = lo_ok ? (int32_t)lin(x0 - 1, y0 - 1, z0 - 1, g) : -1;
    (void)ok;
    if (!lo_ok) atomicOr(err, kErrOOB);
    if (keys) keys[i] = key;
    if (counts && lo_ok) atomicAdd(counts + key, 1);
  }
}

__global__ void minmax_partial_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                      const float* __restrict__ z, int64_t n, float* __restrict__ part) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int a = 0; a < 3; ++a) { mn[a] = fminf(mn[a], v[a]); mx[a] = fmaxf(mx[a], v[a]); }
  }
  __shared__ float s[6][32];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int a = 0; a < 3; ++a) { s[a][wid] = mn[a]; s[3 + a][wid] = mx[a]; }
  __syncthreads();
  if (threadIdx.x < 6) {
    int a = threadIdx.x;
    float r = s[a][0];
    for (int k = 1; k < nw; ++k) r = a < 3 ? fminf(r, s[a][k]) : fmaxf(r, s[a][k]);
    part[blockIdx.x * 6 + a] = r;
  }
}

}  // namespace

int paint(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w,
          int64_t n, int wrap, int mas, uint32_t flags) {
  if (n <= 0) return BAOREC_OK;
  if (flags & BAOREC_DETERMINISTIC) return paint_sorted(ctx, mesh, x, y, z, w, n, wrap, mas, flags);
  if (ctx->tune.binned && paint_binned_ok(ctx, n)) return paint_binned(ctx, mesh, x, y, z, w, n, wrap, mas, flags);
  PaintGeom g = paint_geom(ctx, wrap);
  unsigned grid = grid_for((size_t)n, 256);
  if (grid > 64u * kNumSMs) grid = 64u * kNumSMs;
  int wb = (flags & BAOREC_WRITEBACK) ? 1 : 0;
  if (mas == BAOREC_MAS_TSC)
    (tsc_paint_kernel<<<grid, 256, 0, ctx->stream>>>(mesh, x, y, z, w, n, g, wb, ctx->derr), ::baorec::count_launch());
  else if (g.n[0] % 4 == 0 && (uintptr_t)mesh % 16 == 0)
    (cic_paint_kernel<true><<<grid, 256, 0, ctx->stream>>>(mesh, x, y, z, w, n, g, wb, ctx->derr), ::baorec::count_launch());
  else
    (cic_paint_kernel<false><<<grid, 256, 0, ctx->stream>>>(mesh, x, y, z, w, n, g, wb, ctx->derr), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int minmax3(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
            float mn[3], float mx[3]) {
  const unsigned blocks = 2 * kNumSMs;   // 6 floats per block fit the FP64 partials buffer
  (minmax_partial_kernel<<<blocks, 256, 0, ctx->stream>>>(x, y, z, n, (float*)ctx->dred), ::baorec::count_launch());
  CKLAUNCH();
  float* h = (float*)ctx->hred;
  CK(cudaMemcpyAsync(h, ctx->dred, blocks * 6 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int a = 0; a < 3; ++a) { mn[a] = INFINITY; mx[a] = -INFINITY; }
  for (unsigned k = 0; k < blocks; ++k)
    for (int a = 0; a < 3; ++a) {
      mn[a] = fminf(mn[a], h[k * 6 + a]);
      mx[a] = fmaxf(mx[a], h[k * 6 + 3 + a]);
    }
  return BAOREC_OK;
}

}  // namespace baorec

using namespace baorec;

extern "C" int baorec_cell_bins(baorec_ctx* ctx, const float* x, const float* y, const float* z,
                                int64_t n, int wrap, uint32_t flags, int32_t* keys_out,
                                int32_t* counts_out) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || !x || !y || !z) return set_error(ctx, BAOREC_ERR_ARG, "cell_bins: bad particle arrays");
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  int32_t* dkeys = keys_out;
  int32_t* dcounts = counts_out;
  DevBuf kb, cb;
  if (flags & BAOREC_HOST) {
    if (keys_out) { CKS(ensure(ctx, kb, (size_t)n * 4)); dkeys = (int32_t*)kb.p; }
    if (counts_out) { CKS(ensure(ctx, cb, ctx->N * 4)); dcounts = (int32_t*)cb.p; }
  }
  if (dcounts) CK(cudaMemsetAsync(dcounts, 0, ctx->N * 4, ctx->stream));
  PaintGeom g = paint_geom(ctx, wrap);
  if (n > 0) {
    unsigned grid = grid_for((size_t)n, 256);
    if (grid > 64u * kNumSMs) grid = 64u * kNumSMs;
    (cell_bins_kernel<<<grid, 256, 0, ctx->stream>>>(dx, dy, dz, n, g, dkeys, dcounts, ctx->derr), ::baorec::count_launch());
    CKLAUNCH();
  }
  int st = BAOREC_OK;
  if (flags & BAOREC_HOST) {
    if (keys_out) CK(cudaMemcpyAsync(keys_out, dkeys, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (counts_out) CK(cudaMemcpyAsync(counts_out, dcounts, ctx->N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    st = finish(ctx, flags & ~BAOREC_ASYNC);
    if (kb.p) cudaFree(kb.p);
    if (cb.p) cudaFree(cb.p);
    return st;
  }
  return finish(ctx, flags);
}
