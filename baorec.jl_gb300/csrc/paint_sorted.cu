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
//
// Binned FP32 paint (baorec_set_tune_binned; the reference's CIC kernel at
// src/mas.jl:53-99, like this library's default paint, adds every weight to
// the mesh with a float atomic): particles are bucketed by mesh tile with an
// integer counting sort — per-block shared-memory histograms flushed to
// global tile counts, an exclusive scan, and a scatter that reserves each
// block's range of every tile with one atomic and writes the particles as
// (x, y, z, w) records in tile order.  One block per tile then adds its
// particles' weights in shared memory (FP32 atomics on shared memory) over
// the tile plus its halo and writes the tile once: cells that only this
// tile's particles reach with a plain read-add-store, the shared faces with
// global atomics.  The per-particle weights are the atomic paint's; only the
// order of the FP32 additions differs, as between two runs of the atomic
// paint.
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

// ---- binned FP32 paint ------------------------------------------------------

constexpr int kBinChunk = 4096;   // particles per block of the count and scatter passes
constexpr int kMaxBins = 4096;    // tiles: shared histogram of the count and scatter passes
constexpr int kBinThreads = 256;
static_assert(kBinChunk <= 4096 && kMaxBins <= (1 << 19), "key and rank packed in 31 bits");

struct BinGeom {
  int T, shift;   // tile edge (a power of two) and its log2
  int nt[3];
  int ntiles;
};

template <int MAS>
__device__ __forceinline__ int bin_of(float px, float py, float pz, const PaintGeom& g, const BinGeom& bg) {
  int b[3];
  if (!base_cell<MAS>(px, py, pz, g, b)) return -1;
  return (b[0] >> bg.shift) + bg.nt[0] * ((b[1] >> bg.shift) + bg.nt[1] * (b[2] >> bg.shift));
}

// Tile counts: a shared histogram per block of kBinChunk particles, flushed
// with one global atomic per nonempty tile.  Wraps (and writes back) the
// positions as the atomic paint does.
template <int MAS>
__global__ void __launch_bounds__(kBinThreads) bin_count_kernel(float* __restrict__ x, float* __restrict__ y,
                                                                float* __restrict__ z, int64_t n, PaintGeom g,
                                                                BinGeom bg, int writeback,
                                                                int32_t* __restrict__ counts, unsigned* err) {
  __shared__ int h[kMaxBins];
  for (int b = threadIdx.x; b < bg.ntiles; b += kBinThreads) h[b] = 0;
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * kBinChunk;
  const int64_t i1 = n < i0 + kBinChunk ? n : i0 + kBinChunk;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kBinThreads) {
    float px = x[i], py = y[i], pz = z[i];
    if (g.wrap) {
      px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g);
      if (writeback) { x[i] = px; y[i] = py; z[i] = pz; }
    }
    const int k = bin_of<MAS>(px, py, pz, g, bg);
    if (k < 0) atomicOr(err, kErrOOB);
    else atomicAdd(&h[k], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < bg.ntiles; b += kBinThreads)
    if (h[b]) atomicAdd(counts + b, h[b]);
}

// Scatter: each particle's rank within its block and tile from a shared
// atomic, one global atomic per (block, nonempty tile) to reserve the
// block's range of the tile, then (x, y, z, w) to its place.
template <int MAS>
__global__ void __launch_bounds__(kBinThreads) bin_scatter_kernel(const float* __restrict__ x,
                                                                  const float* __restrict__ y,
                                                                  const float* __restrict__ z,
                                                                  const float* __restrict__ w, int64_t n,
                                                                  PaintGeom g, BinGeom bg,
                                                                  int32_t* __restrict__ cursor,
                                                                  float4* __restrict__ parts) {
  __shared__ int h[kMaxBins];          // counts, then the block's base in each tile
  __shared__ int kr[kBinChunk];        // tile << 12 | rank, -1 outside the mesh
  for (int b = threadIdx.x; b < bg.ntiles; b += kBinThreads) h[b] = 0;
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * kBinChunk;
  const int m = (int)((n < i0 + kBinChunk ? n : i0 + kBinChunk) - i0);
  for (int j = threadIdx.x; j < m; j += kBinThreads) {
    float px = x[i0 + j], py = y[i0 + j], pz = z[i0 + j];
    if (g.wrap) { px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g); }
    const int k = bin_of<MAS>(px, py, pz, g, bg);
    kr[j] = k < 0 ? -1 : (k << 12) | atomicAdd(&h[k], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < bg.ntiles; b += kBinThreads)
    if (h[b]) h[b] = atomicAdd(cursor + b, h[b]);
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += kBinThreads) {
    const int v = kr[j];
    if (v < 0) continue;
    float px = x[i0 + j], py = y[i0 + j], pz = z[i0 + j];
    if (g.wrap) { px = wrap_pos(px, g); py = wrap_pos(py, g); pz = wrap_pos(pz, g); }
    parts[h[v >> 12] + (v & 4095)] = make_float4(px, py, pz, w[i0 + j]);
  }
}

// One block per tile: the tile's particles into shared FP32 accumulators
// over cells t0-1 .. t0+T per axis (local 0 .. T+1), then each nonzero cell
// once into the mesh.  A cell that no other tile's particles reach (CIC:
// t0+1 .. t0+T-1, TSC: t0+1 .. t0+T-2, short of the mesh's last cell or two
// where a wrapped neighbour tile reaches) gets a plain read-add-store; the
// shared faces get global atomics.
template <int MAS>
__global__ void __launch_bounds__(kBinThreads) bin_paint_kernel(const float4* __restrict__ parts,
                                                                const int32_t* __restrict__ offsets, PaintGeom g,
                                                                BinGeom bg, float* __restrict__ mesh) {
  extern __shared__ float acc_f[];
  const int T = bg.T, S = T + 2, S3 = S * S * S;
  const int tile = blockIdx.x;
  const int begin = offsets[tile], end = offsets[tile + 1];
  if (begin == end) return;   // block-uniform
  const int tx = tile % bg.nt[0], ty = (tile / bg.nt[0]) % bg.nt[1], tz = tile / (bg.nt[0] * bg.nt[1]);
  const int t0[3] = {tx * T, ty * T, tz * T};
  const int o[3] = {t0[0] - 1, t0[1] - 1, t0[2] - 1};   // mesh cell of local 0
  for (int c = threadIdx.x; c < S3; c += kBinThreads) acc_f[c] = 0.0f;
  __syncthreads();
  for (int p = begin + threadIdx.x; p < end; p += kBinThreads) {
    const float4 q = parts[p];
    if (MAS == BAOREC_MAS_TSC) {
      int ix[3], iy[3], iz[3];
      float wx[3], wy[3], wz[3];
      tsc_axis(q.x, g.bmin[0], g.fn[0], g.L[0], g.n[0], g.wrap, ix, wx);
      tsc_axis(q.y, g.bmin[1], g.fn[1], g.L[1], g.n[1], g.wrap, iy, wy);
      tsc_axis(q.z, g.bmin[2], g.fn[2], g.L[2], g.n[2], g.wrap, iz, wz);
      const int lx = ix[1] - o[0] - 1, ly = iy[1] - o[1] - 1, lz = iz[1] - o[2] - 1;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int a = 0; a < 3; ++a)
            atomicAdd(acc_f + (lx + a) + S * ((ly + b) + S * (lz + c)),
                      __fmul_rn(__fmul_rn(__fmul_rn(q.w, wx[a]), wy[b]), wz[c]));
    } else {
      int x0, x1, y0, y1, z0, z1;
      float wx1, wy1, wz1;
      cic_axis(cic_coord(q.x, g.bmin[0], g.fn[0], g.L[0]), g.n[0], g.wrap, x0, x1, wx1);
      cic_axis(cic_coord(q.y, g.bmin[1], g.fn[1], g.L[1]), g.n[1], g.wrap, y0, y1, wy1);
      cic_axis(cic_coord(q.z, g.bmin[2], g.fn[2], g.L[2]), g.n[2], g.wrap, z0, z1, wz1);
      const float wx0 = __fmul_rn(__fsub_rn(1.0f, wx1), q.w);
      wx1 = __fmul_rn(wx1, q.w);
      const float wy0 = __fsub_rn(1.0f, wy1), wz0 = __fsub_rn(1.0f, wz1);
      const int l0 = (x0 - 1 - o[0]) + S * ((y0 - 1 - o[1]) + S * (z0 - 1 - o[2]));
      atomicAdd(acc_f + l0, __fmul_rn(__fmul_rn(wx0, wy0), wz0));
      atomicAdd(acc_f + l0 + 1, __fmul_rn(__fmul_rn(wx1, wy0), wz0));
      atomicAdd(acc_f + l0 + S, __fmul_rn(__fmul_rn(wx0, wy1), wz0));
      atomicAdd(acc_f + l0 + S * S, __fmul_rn(__fmul_rn(wx0, wy0), wz1));
      atomicAdd(acc_f + l0 + 1 + S, __fmul_rn(__fmul_rn(wx1, wy1), wz0));
      atomicAdd(acc_f + l0 + 1 + S * S, __fmul_rn(__fmul_rn(wx1, wy0), wz1));
      atomicAdd(acc_f + l0 + S + S * S, __fmul_rn(__fmul_rn(wx0, wy1), wz1));
      atomicAdd(acc_f + l0 + 1 + S + S * S, __fmul_rn(__fmul_rn(wx1, wy1), wz1));
    }
  }
  __syncthreads();
  const int reach = MAS == BAOREC_MAS_TSC ? 1 : 0;   // how far above a particle's tile its weights land, minus one
  for (int c = threadIdx.x; c < S3; c += kBinThreads) {
    const float v = acc_f[c];
    if (v == 0.0f) continue;
    const int l[3] = {c % S, (c / S) % S, c / (S * S)};
    int m[3];
    bool in = true, own = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int u = o[a] + l[a];   // unwrapped mesh cell
      const int hi = min(t0[a] + T - 1, g.n[a] - 1) - reach;
      own &= u >= t0[a] + 1 && u <= hi;
      m[a] = u < 0 ? u + g.n[a] : (u >= g.n[a] ? u - g.n[a] : u);
      in &= m[a] >= 0 && m[a] < g.n[a];
    }
    if (!in) continue;
    float* cell = mesh + lin(m[0], m[1], m[2], g);
    if (own) *cell = __fadd_rn(*cell, v);
    else atomicAdd(cell, v);
  }
}

}  // namespace

// Tile edge of the binned paint: the smallest power of two >= 16 with at
// most kMaxBins tiles; 0 when none fits the shared accumulators.
static int bin_tile(const int n[3]) {
  for (int T = 16; T <= 32; T *= 2) {
    const long long nt = (long long)((n[0] + T - 1) / T) * ((n[1] + T - 1) / T) * ((n[2] + T - 1) / T);
    if (nt <= kMaxBins) return T;
  }
  return 0;
}

bool paint_binned_ok(const baorec_ctx* ctx, int64_t n) {
  const int nn[3] = {ctx->n1, ctx->n2, ctx->n3};
  return n > 0 && n <= (int64_t)INT32_MAX && bin_tile(nn) > 0;
}

int paint_binned(baorec_ctx* ctx, float* mesh, float* x, float* y, float* z, const float* w, int64_t n, int wrap,
                 int mas, uint32_t flags) {
  if (n <= 0) return BAOREC_OK;
  if (!paint_binned_ok(ctx, n)) return set_error(ctx, BAOREC_ERR_ARG, "binned paint: mesh or catalogue too large");
  PaintGeom g = paint_geom(ctx, wrap);
  BinGeom bg;
  const int nn[3] = {ctx->n1, ctx->n2, ctx->n3};
  bg.T = bin_tile(nn);
  bg.shift = bg.T == 16 ? 4 : 5;
  for (int a = 0; a < 3; ++a) bg.nt[a] = (g.n[a] + bg.T - 1) / bg.T;
  bg.ntiles = bg.nt[0] * bg.nt[1] * bg.nt[2];
  CKS(ensure(ctx, ctx->bin_parts, (size_t)n * sizeof(float4)));
  CKS(ensure(ctx, ctx->sort_tiles, (size_t)(3 * bg.ntiles + 1) * 4));
  int32_t* counts = (int32_t*)ctx->sort_tiles.p;
  int32_t* offsets = counts + bg.ntiles;   // ntiles + 1
  int32_t* cursor = offsets + bg.ntiles + 1;
  float4* parts = (float4*)ctx->bin_parts.p;
  CK(cudaMemsetAsync(counts, 0, (size_t)bg.ntiles * 4, ctx->stream));
  const unsigned blocks = (unsigned)((n + kBinChunk - 1) / kBinChunk);
  const int wb = (flags & BAOREC_WRITEBACK) ? 1 : 0;
  const int S = bg.T + 2;
  const size_t smem = (size_t)S * S * S * sizeof(float);
  if (mas == BAOREC_MAS_TSC) {
    (bin_count_kernel<BAOREC_MAS_TSC><<<blocks, kBinThreads, 0, ctx->stream>>>(x, y, z, n, g, bg, wb, counts, ctx->derr), ::baorec::count_launch());
    CKLAUNCH();
    (tile_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts, offsets, cursor, bg.ntiles), ::baorec::count_launch());
    CKLAUNCH();
    (bin_scatter_kernel<BAOREC_MAS_TSC><<<blocks, kBinThreads, 0, ctx->stream>>>(x, y, z, w, n, g, bg, cursor, parts), ::baorec::count_launch());
    CKLAUNCH();
    if (smem > 48 * 1024)
      CK(cudaFuncSetAttribute(bin_paint_kernel<BAOREC_MAS_TSC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    (bin_paint_kernel<BAOREC_MAS_TSC><<<bg.ntiles, kBinThreads, smem, ctx->stream>>>(parts, offsets, g, bg, mesh), ::baorec::count_launch());
  } else {
    (bin_count_kernel<BAOREC_MAS_CIC><<<blocks, kBinThreads, 0, ctx->stream>>>(x, y, z, n, g, bg, wb, counts, ctx->derr), ::baorec::count_launch());
    CKLAUNCH();
    (tile_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts, offsets, cursor, bg.ntiles), ::baorec::count_launch());
    CKLAUNCH();
    (bin_scatter_kernel<BAOREC_MAS_CIC><<<blocks, kBinThreads, 0, ctx->stream>>>(x, y, z, w, n, g, bg, cursor, parts), ::baorec::count_launch());
    CKLAUNCH();
    if (smem > 48 * 1024)
      CK(cudaFuncSetAttribute(bin_paint_kernel<BAOREC_MAS_CIC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    (bin_paint_kernel<BAOREC_MAS_CIC><<<bg.ntiles, kBinThreads, smem, ctx->stream>>>(parts, offsets, g, bg, mesh), ::baorec::count_launch());
  }
  CKLAUNCH();
  return BAOREC_OK;
}

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
    (tile_keys_kernel<BAOREC_MAS_TSC><<<grid, 256, 0, ctx->stream>>>(x, y, z, n, g, tg, wb, keys, counts, ctx->derr), ::baorec::count_launch());
  else
    (tile_keys_kernel<BAOREC_MAS_CIC><<<grid, 256, 0, ctx->stream>>>(x, y, z, n, g, tg, wb, keys, counts, ctx->derr), ::baorec::count_launch());
  CKLAUNCH();
  (tile_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts, offsets, cursor, tg.ntiles), ::baorec::count_launch());
  CKLAUNCH();
  (tile_scatter_kernel<<<grid, 256, 0, ctx->stream>>>(keys, n, cursor, perm), ::baorec::count_launch());
  CKLAUNCH();
  const int S = tg.T + 2;
  const size_t smem = (size_t)S * S * S * sizeof(unsigned long long);
  if (mas == BAOREC_MAS_TSC) {
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(tile_accum_kernel<BAOREC_MAS_TSC>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    (tile_accum_kernel<BAOREC_MAS_TSC><<<tg.ntiles, 256, smem, ctx->stream>>>(x, y, z, w, offsets, perm, g, tg, fix), ::baorec::count_launch());
  } else {
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(tile_accum_kernel<BAOREC_MAS_CIC>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    (tile_accum_kernel<BAOREC_MAS_CIC><<<tg.ntiles, 256, smem, ctx->stream>>>(x, y, z, w, offsets, perm, g, tg, fix), ::baorec::count_launch());
  }
  CKLAUNCH();
  (fix_to_mesh_kernel<<<grid_for(ctx->N, 256) < 16u * kNumSMs ? grid_for(ctx->N, 256) : 16u * kNumSMs, 256, 0,
                       ctx->stream>>>(fix, mesh, ctx->N), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec
