// Deterministic mass assignment (BAOREC_DETERMINISTIC; no reference
// counterpart — the reference paints serially on the CPU and with float
// atomics on the GPU, whose sums depend on thread order).
//
// Particles are bucketed by mesh tile (T^3 cells, tile of the particle's
// base cell) with an integer counting sort: tile keys and counts, an
// exclusive scan, a scatter of particle indices.  One block per tile then
// accumulates its particles' CIC (2^3) or TSC (3^3) weights in shared memory
// as 64-bit fixed-point integers (units of 2^-32) over the tile plus a
// one-cell halo, and adds the nonzero cells to a fixed-point mesh with
// integer atomics; a last pass converts to FP32 and adds to the caller's
// mesh.  Integer addition is associative, so the painted mesh is the same
// bits on every run.  The cell indices and the per-particle FP32 weights are
// those of the atomic paint (shared arithmetic in paint_common.cuh).
#include "paint_common.cuh"

namespace baorec {
namespace {

constexpr float kFix = 4294967296.0f;   // 2^32: fixed-point scale of one contribution

struct TileGeom {
  int T;            // tile edge (cells)
  int nt[3];        // tiles per axis
  int ntiles;
};

// Base cell (0-based, in the mesh) of a particle: the lower CIC cell or the
// nearest TSC node; false for a particle the reference rejects.
template <int MAS>
__device__ __forceinline__ bool base_cell(float px, float py, float pz, const PaintGeom& g, int b[3]) {
  if (MAS == BAOREC_MAS_TSC) {
    int ix[3], iy[3], iz[3];
    float wx[3], wy[3], wz[3];
    bool ok = tsc_axis(px, g.bmin[0], g.fn[0], g.L[0], g.n[0], g.wrap, ix, wx);
    ok &= tsc_axis(py, g.bmin[1], g.fn[1], g.L[1], g.n[1], g.wrap, iy, wy);
    ok &= tsc_axis(pz, g.bmin[2], g.fn[2], g.L[2], g.n[2], g.wrap, iz, wz);
    b[0] = ix[1]; b[1] = iy[1]; b[2] = iz[1];
    return ok;
  }
  int x0, x1, y0, y1, z0, z1;
  float t;
  bool ok = cic_axis(cic_coord(px, g.bmin[0], g.fn[0], g.L[0]), g.n[0], g.wrap, x0, x1, t);
  ok &= cic_axis(cic_coord(py, g.bmin[1], g.fn[1], g.L[1]), g.n[1], g.wrap, y0, y1, t);
  ok &= cic_axis(cic_coord(pz, g.bmin[2], g.fn[2], g.L[2]), g.n[2], g.wrap, z0, z1, t);
  b[0] = x0 - 1; b[1] = y0 - 1; b[2] = z0 - 1;
  return ok;
}

template <int MAS>
__global__ void tile_keys_kernel(float* __restrict__ x, float* __restrict__ y, float* __restrict__ z, int64_t n,
                                 PaintGeom g, TileGeom tg, int writeback, int32_t* __restrict__ keys,
                                 int32_t* __restrict__ counts, unsigned* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) {
      px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g);
      if (writeback) { x[i] = px; y[i] = py; z[i] = pz; }
    }
    int b[3];
    int32_t key = -1;
    if (base_cell<MAS>(px, py, pz, g, b)) {
      key = (b[0] / tg.T) + tg.nt[0] * ((b[1] / tg.T) + tg.nt[1] * (b[2] / tg.T));
      atomicAdd(counts + key, 1);
    } else {
      atomicOr(err, kErrOOB);
    }
    keys[i] = key;
  }
}

// Exclusive scan of the tile counts (one block, chunks of blockDim with a carry).
__global__ void tile_scan_kernel(const int32_t* __restrict__ counts, int32_t* __restrict__ offsets,
                                 int32_t* __restrict__ cursor, int ntiles) {
  __shared__ int32_t warp_sum[32];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < ntiles; base += blockDim.x) {
    const int t = base + threadIdx.x;
    const int v = t < ntiles ? counts[t] : 0;
    int s = v;   // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    if (lane == 31) warp_sum[warp] = s;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? warp_sum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += u;
      }
      if (lane < nw) warp_sum[lane] = w;   // inclusive sums of warps
    }
    __syncthreads();
    const int excl = carry + (warp > 0 ? warp_sum[warp - 1] : 0) + s - v;
    if (t < ntiles) { offsets[t] = excl; cursor[t] = excl; }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[ntiles] = carry;
}

__global__ void tile_scatter_kernel(const int32_t* __restrict__ keys, int64_t n, int32_t* __restrict__ cursor,
                                    int32_t* __restrict__ perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = keys[i];
    if (k >= 0) perm[atomicAdd(cursor + k, 1)] = (int32_t)i;
  }
}

__device__ __forceinline__ void fix_add(unsigned long long* acc, int local, float v) {
  atomicAdd(acc + local, (unsigned long long)__float2ll_rn(v * kFix));
}

// One block per tile: shared fixed-point accumulators over the tile plus a
// one-cell halo on each side ((T+2)^3 cells), then integer atomics into the
// fixed-point mesh.
template <int MAS>
__global__ void tile_accum_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                  const float* __restrict__ z, const float* __restrict__ w,
                                  const int32_t* __restrict__ offsets, const int32_t* __restrict__ perm,
                                  PaintGeom g, TileGeom tg, unsigned long long* __restrict__ fix) {
  extern __shared__ unsigned long long acc[];
  const int S = tg.T + 2, S3 = S * S * S;
  const int tile = blockIdx.x;
  const int begin = offsets[tile], end = offsets[tile + 1];
  if (begin == end) return;   // block-uniform: no particle in this tile
  const int tx = tile % tg.nt[0], ty = (tile / tg.nt[0]) % tg.nt[1], tz = tile / (tg.nt[0] * tg.nt[1]);
  const int o[3] = {tx * tg.T - 1, ty * tg.T - 1, tz * tg.T - 1};   // mesh cell of local 0
  for (int c = threadIdx.x; c < S3; c += blockDim.x) acc[c] = 0ull;
  __syncthreads();
  for (int p = begin + threadIdx.x; p < end; p += blockDim.x) {
    const int i = perm[p];
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) { px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g); }
    const float wt = w[i];
    if (MAS == BAOREC_MAS_TSC) {
      int ix[3], iy[3], iz[3];
      float wx[3], wy[3], wz[3];
      tsc_axis(px, g.bmin[0], g.fn[0], g.L[0], g.n[0], g.wrap, ix, wx);
      tsc_axis(py, g.bmin[1], g.fn[1], g.L[1], g.n[1], g.wrap, iy, wy);
      tsc_axis(pz, g.bmin[2], g.fn[2], g.L[2], g.n[2], g.wrap, iz, wz);
      // local coordinates from the (wrapped) centre node, offsets -1, 0, +1
      const int lx = ix[1] - o[0] - 1, ly = iy[1] - o[1] - 1, lz = iz[1] - o[2] - 1;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int a = 0; a < 3; ++a)
            fix_add(acc, (lx + a) + S * ((ly + b) + S * (lz + c)),
                    __fmul_rn(__fmul_rn(__fmul_rn(wt, wx[a]), wy[b]), wz[c]));
    } else {
      int x0, x1, y0, y1, z0, z1;
      float wx1, wy1, wz1;
      cic_axis(cic_coord(px, g.bmin[0], g.fn[0], g.L[0]), g.n[0], g.wrap, x0, x1, wx1);
      cic_axis(cic_coord(py, g.bmin[1], g.fn[1], g.L[1]), g.n[1], g.wrap, y0, y1, wy1);
      cic_axis(cic_coord(pz, g.bmin[2], g.fn[2], g.L[2]), g.n[2], g.wrap, z0, z1, wz1);
      const float wx0 = __fmul_rn(__fsub_rn(1.0f, wx1), wt);
      wx1 = __fmul_rn(wx1, wt);
      const float wy0 = __fsub_rn(1.0f, wy1), wz0 = __fsub_rn(1.0f, wz1);
      // lower cell x0-1 (0-based) at local x0-1-o; the upper one is the next local cell
      const int l0 = (x0 - 1 - o[0]) + S * ((y0 - 1 - o[1]) + S * (z0 - 1 - o[2]));
      fix_add(acc, l0, __fmul_rn(__fmul_rn(wx0, wy0), wz0));
      fix_add(acc, l0 + 1, __fmul_rn(__fmul_rn(wx1, wy0), wz0));
      fix_add(acc, l0 + S, __fmul_rn(__fmul_rn(wx0, wy1), wz0));
      fix_add(acc, l0 + S * S, __fmul_rn(__fmul_rn(wx0, wy0), wz1));
      fix_add(acc, l0 + 1 + S, __fmul_rn(__fmul_rn(wx1, wy1), wz0));
      fix_add(acc, l0 + 1 + S * S, __fmul_rn(__fmul_rn(wx1, wy0), wz1));
      fix_add(acc, l0 + S + S * S, __fmul_rn(__fmul_rn(wx0, wy1), wz1));
      fix_add(acc, l0 + 1 + S + S * S, __fmul_rn(__fmul_rn(wx1, wy1), wz1));
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < S3; c += blockDim.x) {
    const unsigned long long v = acc[c];
    if (!v) continue;
    int m[3] = {o[0] + c % S, o[1] + (c / S) % S, o[2] + c / (S * S)};
    bool in = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (m[a] < 0) m[a] += g.n[a];
      else if (m[a] >= g.n[a]) m[a] -= g.n[a];
      in &= m[a] >= 0 && m[a] < g.n[a];
    }
    if (in) atomicAdd(fix + lin(m[0], m[1], m[2], g), v);
  }
}

__global__ void fix_to_mesh_kernel(const unsigned long long* __restrict__ fix, float* __restrict__ mesh, size_t N) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    const long long v = (long long)fix[e];
    if (v) mesh[e] += (float)((double)v * (1.0 / 4294967296.0));
  }
}

}  // namespace

int paint_sorted(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n, int wrap,
                 int mas, uint32_t flags) {
  if (n <= 0) return BAOREC_OK;
  if (n > (int64_t)INT32_MAX) return set_error(ctx, BAOREC_ERR_ARG, "deterministic paint: more than 2^31 particles");
  PaintGeom g = paint_geom(ctx, wrap);
  TileGeom tg;
  tg.T = ctx->tune.paint_tile;
  for (int a = 0; a < 3; ++a) tg.nt[a] = (g.n[a] + tg.T - 1) / tg.T;
  tg.ntiles = tg.nt[0] * tg.nt[1] * tg.nt[2];
  CKS(ensure(ctx, ctx->sort_keys, (size_t)n * 4));
  CKS(ensure(ctx, ctx->sort_perm, (size_t)n * 4));
  CKS(ensure(ctx, ctx->sort_tiles, (size_t)(3 * tg.ntiles + 1) * 4));
  CKS(ensure(ctx, ctx->fix_mesh, ctx->N * 8));
  int32_t* keys = (int32_t*)ctx->sort_keys.p;
  int32_t* perm = (int32_t*)ctx->sort_perm.p;
  int32_t* counts = (int32_t*)ctx->sort_tiles.p;
  int32_t* offsets = counts + tg.ntiles;        // ntiles + 1
  int32_t* cursor = offsets + tg.ntiles + 1;
  unsigned long long* fix = (unsigned long long*)ctx->fix_mesh.p;
  CK(cudaMemsetAsync(counts, 0, (size_t)tg.ntiles * 4, ctx->stream));
  CK(cudaMemsetAsync(fix, 0, ctx->N * 8, ctx->stream));
  unsigned grid = grid_for((size_t)n, 256);
  if (grid > 64u * kNumSMs) grid = 64u * kNumSMs;
  const int wb = (flags & BAOREC_WRITEBACK) ? 1 : 0;
  if (mas == BAOREC_MAS_TSC)
    tile_keys_kernel<BAOREC_MAS_TSC><<<grid, 256, 0, ctx->stream>>>(x, y, z, n, g, tg, wb, keys, counts, ctx->derr);
  else
    tile_keys_kernel<BAOREC_MAS_CIC><<<grid, 256, 0, ctx->stream>>>(x, y, z, n, g, tg, wb, keys, counts, ctx->derr);
  CKLAUNCH();
  tile_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts, offsets, cursor, tg.ntiles);
  CKLAUNCH();
  tile_scatter_kernel<<<grid, 256, 0, ctx->stream>>>(keys, n, cursor, perm);
  CKLAUNCH();
  const int S = tg.T + 2;
  const size_t smem = (size_t)S * S * S * sizeof(unsigned long long);
  if (mas == BAOREC_MAS_TSC) {
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(tile_accum_kernel<BAOREC_MAS_TSC>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tile_accum_kernel<BAOREC_MAS_TSC><<<tg.ntiles, 256, smem, ctx->stream>>>(x, y, z, w, offsets, perm, g, tg, fix);
  } else {
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(tile_accum_kernel<BAOREC_MAS_CIC>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tile_accum_kernel<BAOREC_MAS_CIC><<<tg.ntiles, 256, smem, ctx->stream>>>(x, y, z, w, offsets, perm, g, tg, fix);
  }
  CKLAUNCH();
  fix_to_mesh_kernel<<<grid_for(ctx->N, 256) < 16u * kNumSMs ? grid_for(ctx->N, 256) : 16u * kNumSMs, 256, 0,
                       ctx->stream>>>(fix, mesh, ctx->N);
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec
