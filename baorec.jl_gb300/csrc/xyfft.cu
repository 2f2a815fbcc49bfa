// Fused 2-D real transforms of 256 x 256 xy planes (the x and y passes of the
// FFT preconditioner's, the smoothing's and the displacement's transforms),
// one kernel per direction instead of cuFFT's two passes: each plane is read
// once and written once.
//
// A plane runs on a cluster of four CTAs (two CTAs per SM): the row
// transforms of the space side and the column transforms of the spectrum
// side are split between the four, and the transposition between them is
// a push of every value into the owning CTA's shared memory through the
// cluster's distributed shared memory, so no CTA repeats another's row
// transforms and no intermediate leaves the chip.
//   rows: the 256 reals of a row packed as 128 complex values, a four-step
//         128 = 16 x 8 (16-point DFT in registers, twiddles, an exchange in
//         shared memory, 8-point DFTs) and the real-to-half-spectrum unpack
//         X[k] = (Z[k] + Z*[128-k])/2 - i/2 e^{-2πik/256} (Z[k] - Z*[128-k]);
//   columns: a four-step 256 = 16 x 16 per column.
// The inverse mirrors it.  The index algebra was checked against numpy's
// FFT by an emulation of both kernels' thread mappings.
#include "common.cuh"

namespace baorec {
namespace {

constexpr int kXN = 256;         // points along x and y
constexpr int kXH = kXN / 2;     // packed complex points of a row
constexpr int kXC = kXN / 2 + 1; // half-spectrum length (129)

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {   // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 addf2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 subf2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

template <bool INV>
__device__ __forceinline__ void dft4x(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = addf2(a0, a2), t1 = subf2(a0, a2), t2 = addf2(a1, a3), d = subf2(a1, a3);
  const float2 t3 = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  a0 = addf2(t0, t2);
  a2 = subf2(t0, t2);
  a1 = addf2(t1, t3);
  a3 = subf2(t1, t3);
}

template <bool INV>
__device__ __forceinline__ float2 w16x(int m) {
  constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f, h = 0.70710678118654752f;
  float c = 1.0f, sn = 0.0f;
  switch (m) {
    case 1: c = c1; sn = s1; break;
    case 2: c = h; sn = h; break;
    case 3: c = s1; sn = c1; break;
    case 4: c = 0.0f; sn = 1.0f; break;
    case 6: c = -h; sn = h; break;
    case 9: c = -c1; sn = -s1; break;
    default: break;
  }
  return make_float2(c, INV ? sn : -sn);
}

// 16-point DFT in registers, natural order in and out.
template <bool INV>
__device__ __forceinline__ void dft16x(float2 (&v)[16]) {
#pragma unroll
  for (int b = 0; b < 4; ++b) dft4x<INV>(v[b], v[4 + b], v[8 + b], v[12 + b]);
#pragma unroll
  for (int b = 1; b < 4; ++b)
#pragma unroll
    for (int c = 1; c < 4; ++c) v[4 * c + b] = cmul(v[4 * c + b], w16x<INV>(b * c));
#pragma unroll
  for (int c = 0; c < 4; ++c) dft4x<INV>(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int d = c + 1; d < 4; ++d) {
      const float2 q = v[4 * c + d];
      v[4 * c + d] = v[4 * d + c];
      v[4 * d + c] = q;
    }
}

// 8-point DFT in registers, natural order: n = 2a + b, k = c + 4d.
template <bool INV>
__device__ __forceinline__ void dft8x(float2 (&v)[8]) {
  float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4x<INV>(e[0], e[1], e[2], e[3]);
  dft4x<INV>(o[0], o[1], o[2], o[3]);
  constexpr float h = 0.70710678118654752f;
  // e^{∓2πi c/8}, c = 1..3
  o[1] = cmul(o[1], make_float2(h, INV ? h : -h));
  o[2] = cmul(o[2], make_float2(0.0f, INV ? 1.0f : -1.0f));
  o[3] = cmul(o[3], make_float2(-h, INV ? h : -h));
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    v[c] = addf2(e[c], o[c]);
    v[c + 4] = subf2(e[c], o[c]);
  }
}

// ---- cluster plumbing -------------------------------------------------------
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// store v in cluster CTA `rank` at the position of this CTA's shared-memory address `local`
__device__ __forceinline__ void st_peer(uint32_t local, unsigned rank, float2 v) {
  uint32_t a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(local), "r"(rank));
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

// ---- layout ---------------------------------------------------------------------
// A plane's 256 x 256 transform runs on a cluster of kCl CTAs.  The packed
// half spectrum of a row has 128 complex slots: slot 0 holds the two real
// values (X[0], X[128]), slots 1..127 the complex X[1..127].  CTA q owns
// rows [64q, 64q + 64) of the space side and packed columns [32q, 32q + 32)
// of the spectrum side; the rows <-> columns exchange is a push of each
// value into its owner's shared memory (distributed shared memory), fenced
// by one cluster barrier.
constexpr int kCl = 4;                  // CTAs per plane
constexpr int kCT = 256;                // threads per CTA
constexpr int kRows = kXN / kCl;        // 64 space rows per CTA
constexpr int kCols = kXH / kCl;        // 32 packed columns per CTA
constexpr int kXP = 136;                // float2 pitch of a row buffer: 1088 B, a 16-bank shift between rows
static_assert(kCT == kXN, "one twiddle per thread");

// Slot of value (c, bb) of a row's 16 x 8 four-step exchange: rotated so
// that neither the writes (fixed c, 8 bb) nor the reads (8 c, fixed bb) of
// the two rows sharing a half-warp meet in a bank.
__device__ __forceinline__ int xslot(int c, int bb, int rot) { return 8 * c + ((bb + (c >> 1) + rot) & 7); }

// Twiddles in shared memory: W256^m at [m], then the row transform's
// W128^{bc} = W256^{2bc} at [256 + 8c + b] (eight consecutive entries per c,
// so the eight lanes of a row read distinct banks).
constexpr int kTw = kXN + 128;
__device__ __forceinline__ void load_twiddles(float2* w, const float2* __restrict__ tw, int t) {
  w[t] = __ldg(tw + t);
  if (t < 128) w[kXN + t] = __ldg(tw + ((2 * (t & 7) * (t >> 3)) & (kXN - 1)));
}

// Spectrum-side column buffer of the forward kernel: [256 rows][32 columns],
// column index XOR 8 on odd rows (two rows of one half-warp's pushes land
// in disjoint banks).
__device__ __forceinline__ int ycell(int y, int lc) { return y * kCols + (lc ^ ((y & 1) << 3)); }

__device__ __forceinline__ float2 r2c_unpack(float2 zk, float2 p, float2 wk) {   // p = Z[128 - k]
  const float2 zm = conjf2(p);
  const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
  const float2 dd = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y - zm.y));
  return addf2(e, cmul(make_float2(dd.y, -dd.x), wk));   // e - i dd W^k
}

// Forward: real planes [plane][y][x] -> half spectra [plane][ky][kx], row
// length 129, as cuFFT's batched 2-D R2C.
//   x: 8 threads per row; the row's 256 reals as 128 packed complex values
//      z[8a + b] (thread b holds a = 0..15), a 16-point DFT over a, twiddles,
//      an exchange through the row buffer, an 8-point DFT over b: Z[c + 16 d]
//      for c in {b, b + 8}.  The partner Z[128 - k] of the unpack is in lane
//      (8 - b) & 7 of the row (shuffles).  X[k] is pushed to CTA k / 32.
//   y: 16 threads per column; four-step 256 = 16 x 16 in place in the column
//      buffer; the packed column 0 (X[0] + i X[128], both real) is separated
//      into the spectra of kx = 0 and kx = 128 with W[256 - ky].
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kCT, 2)
    xy_r2c_kernel(const float* __restrict__ in, float2* __restrict__ out, const float2* __restrict__ tw) {
  extern __shared__ __align__(16) float2 xsm[];
  float2* ys = xsm;                          // [256][32] (ycell)
  float2* xb = ys + kXN * kCols;             // [32 rows][kXP]; later the separation buffer
  float2* w = xb + 32 * kXP;                 // e^{-2πi m/256}
  const int t = threadIdx.x;
  const unsigned rank = cluster_rank();
  const size_t plane = blockIdx.y;
  cluster_arrive_relaxed();                  // matched below, before the first push
  load_twiddles(w, tw, t);
  const int rl = t >> 3, b = t & 7, rot = 4 * (rl & 1);
  const float2* src = reinterpret_cast<const float2*>(in + plane * (size_t)(kXN * kXN));
  const int y0 = kRows * (int)rank + rl;
  float2 va[16], vb[16];
#pragma unroll
  for (int a = 0; a < 16; ++a) va[a] = __ldg(src + (size_t)y0 * kXH + 8 * a + b);
#pragma unroll
  for (int a = 0; a < 16; ++a) vb[a] = __ldg(src + (size_t)(y0 + 32) * kXH + 8 * a + b);
  __syncthreads();
  const uint32_t ys0 = smem_addr(ys);
  const float2* twx = w + kXN;
  float2* rb = xb + rl * kXP;
  const unsigned lane = t & 31, partner = (lane & ~7u) | ((8u - b) & 7u);
#pragma unroll
  for (int round = 0; round < 2; ++round) {
    float2(&v)[16] = round ? vb : va;
    const int y = y0 + 32 * round;
    dft16x<false>(v);
#pragma unroll
    for (int c = 0; c < 16; ++c) rb[xslot(c, b, rot)] = cmul(v[c], twx[8 * c + b]);   // W128^{bc}
    __syncwarp();
    float2 o[2][8];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = b + 8 * q;
#pragma unroll
      for (int bb = 0; bb < 8; ++bb) o[q][bb] = rb[xslot(c, bb, rot)];
      dft8x<false>(o[q]);                    // o[q][d] = Z[c + 16 d]
    }
    __syncwarp();                            // the row buffer is free for the next round
    const int ysw = (y & 1) << 3;
    if (round == 0) cluster_wait();          // every CTA of the cluster runs: pushes may start
    {   // c = b: partner Z[128 - k] = lane (8 - b)'s o[1][7 - d]; b = 0: own o[0][8 - d]
      float2 p[8];
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        const float2 s = o[1][7 - d];
        p[d] = make_float2(__shfl_sync(0xffffffffu, s.x, partner), __shfl_sync(0xffffffffu, s.y, partner));
      }
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        const int k = b + 16 * d;
        float2 x = r2c_unpack(o[0][d], b == 0 ? o[0][(8 - d) & 7] : p[d], w[k]);
        if (d == 0 && b == 0) x = make_float2(o[0][0].x + o[0][0].y, o[0][0].x - o[0][0].y);   // (X[0], X[128])
        st_peer(ys0 + 8u * (uint32_t)(y * kCols + ((k & 31) ^ ysw)), (unsigned)(k >> 5), x);
      }
    }
    {   // c = b + 8: partner = lane (8 - b)'s o[0][7 - d]; b = 0 (c = 8): own o[1][7 - d]
      float2 p[8];
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        const float2 s = o[0][7 - d];
        p[d] = make_float2(__shfl_sync(0xffffffffu, s.x, partner), __shfl_sync(0xffffffffu, s.y, partner));
      }
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        const int k = b + 8 + 16 * d;
        const float2 x = r2c_unpack(o[1][d], b == 0 ? o[1][7 - d] : p[d], w[k]);
        st_peer(ys0 + 8u * (uint32_t)(y * kCols + ((k & 31) ^ ysw)), (unsigned)(k >> 5), x);
      }
    }
  }
  cluster_arrive_release();
  cluster_wait_acquire();                    // the CTA's 32 columns are complete
  float2* dst = out + plane * (size_t)(kXC * kXN);
  float2* sep = xb;                          // W of the packed column (rank 0)
  const int col = t & 15, r = t >> 4;
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    const int lc = 16 * g + col;
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) v[n1] = ys[ycell(16 * n1 + r, lc)];
    dft16x<false>(v);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) ys[ycell(16 * k1 + r, lc)] = cmul(v[k1], w[r * k1]);
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = ys[ycell(16 * r + n2, lc)];
    dft16x<false>(v);                        // v[k2] = Y[ky = r + 16 k2]
    const int kx = kCols * (int)rank + lc;
    if (kx == 0) {
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2) sep[r + 16 * k2] = v[k2];
    } else {
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2) dst[(size_t)(r + 16 * k2) * kXC + kx] = v[k2];
    }
  }
  if (rank == 0) {                           // block-uniform
    __syncthreads();
    const float2 W = sep[t], Wm = conjf2(sep[(kXN - t) & (kXN - 1)]);
    const float2 s = addf2(W, Wm), d = subf2(W, Wm);
    dst[(size_t)t * kXC] = make_float2(0.5f * s.x, 0.5f * s.y);                 // Y0 = (W + W*[-ky]) / 2
    dst[(size_t)t * kXC + kXH] = make_float2(0.5f * d.y, -0.5f * d.x);          // Y128 = (W - W*[-ky]) / 2i
  }
}

// Inverse: half spectra [plane][ky][kx] -> real planes [plane][y][x],
// unnormalised as cuFFT's C2R.
//   y: 16 threads per column; column kx = 0 is packed with kx = 128 as
//      Y[0] + i Y[128], whose inverse is the packed slot (X[0], X[128]) of
//      the rows directly (both real for Hermitian columns); four-step 256
//      through a column exchange buffer; each value pushed to the CTA that
//      owns its row.
//   x: 8 threads per row; Z[k] = (X[k] + X*[128-k]) + i (X[k] - X*[128-k])
//      e^{2πik/256} from the row buffer, an inverse four-step 128 with the
//      exchange in the row buffer itself, x[2n] = Re z[n], x[2n+1] = Im z[n].
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kCT, 2)
    xy_c2r_kernel(const float2* __restrict__ in, float* __restrict__ out, const float2* __restrict__ tw) {
  extern __shared__ __align__(16) float2 xsm[];
  float2* xr = xsm;                          // [64 rows][kXP]
  float2* eb = xr + kRows * kXP;             // [256][16] column exchange
  float2* w = eb + kXN * 16;
  const int t = threadIdx.x;
  const unsigned rank = cluster_rank();
  const size_t plane = blockIdx.y;
  cluster_arrive_relaxed();
  load_twiddles(w, tw, t);
  const int col = t & 15, r = t >> 4;
  const float2* src = in + plane * (size_t)(kXC * kXN);
  float2 va[16], vb[16];
  {
    const int kx0 = kCols * (int)rank + col;
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const float2* row = src + (size_t)(16 * n1 + r) * kXC;
      float2 a = __ldg(row + kx0);
      if (kx0 == 0) {                         // Y[0] + i Y[128]
        const float2 h = __ldg(row + kXH);
        a = make_float2(a.x - h.y, a.y + h.x);
      }
      va[n1] = a;
      vb[n1] = __ldg(row + kx0 + 16);
    }
  }
  __syncthreads();
  const uint32_t xr0 = smem_addr(xr);
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    float2(&v)[16] = g ? vb : va;
    dft16x<true>(v);
    if (g) __syncthreads();                  // the previous round's reads of eb are done
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) eb[(16 * k1 + r) * 16 + col] = cmulc(v[k1], w[r * k1]);
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = eb[(16 * r + n2) * 16 + col];
    dft16x<true>(v);                         // v[k2] = X_kx[y = r + 16 k2]
    const int kx = kCols * (int)rank + 16 * g + col;
    if (g == 0) cluster_wait();              // every CTA of the cluster runs: pushes may start
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      const int y = r + 16 * k2;
      st_peer(xr0 + 8u * (uint32_t)((y & (kRows - 1)) * kXP + kx), (unsigned)(y >> 6), v[k2]);
    }
  }
  cluster_arrive_release();
  cluster_wait_acquire();                    // the CTA's 64 rows are complete
  const int rl = t >> 3, b = t & 7, rot = 4 * (rl & 1);
  float* dst = out + plane * (size_t)(kXN * kXN);
#pragma unroll
  for (int round = 0; round < 2; ++round) {
    const int row = 32 * round + rl;
    float2* xrow = xr + row * kXP;
    float2 v[16];
#pragma unroll
    for (int a = 0; a < 16; ++a) {
      const int k = 8 * a + b;
      const float2 xk = xrow[k];
      if (a == 0 && b == 0) {
        v[0] = make_float2(xk.x + xk.y, xk.x - xk.y);   // (X[0] + X[128]) + i (X[0] - X[128])
      } else {
        const float2 xm = conjf2(xrow[kXH - k]);
        const float2 sdf = cmulc(subf2(xk, xm), w[k]);
        v[a] = make_float2(xk.x + xm.x - sdf.y, xk.y + xm.y + sdf.x);
      }
    }
    __syncwarp();                            // the row's reads are done: it becomes the exchange
    dft16x<true>(v);
#pragma unroll
    for (int c = 0; c < 16; ++c) xrow[xslot(c, b, rot)] = cmulc(v[c], w[kXN + 8 * c + b]);
    __syncwarp();
    float2* xo = reinterpret_cast<float2*>(dst + (size_t)(kRows * (int)rank + row) * kXN);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = b + 8 * q;
      float2 o[8];
#pragma unroll
      for (int bb = 0; bb < 8; ++bb) o[bb] = xrow[xslot(c, bb, rot)];
      dft8x<true>(o);                        // o[d] = z[c + 16 d]
#pragma unroll
      for (int d = 0; d < 8; ++d) xo[c + 16 * d] = o[d];   // (x[2n], x[2n+1])
    }
  }
}

constexpr size_t kR2CSmem = sizeof(float2) * (kXN * kCols + 32 * kXP + kTw);
constexpr size_t kC2RSmem = sizeof(float2) * (kRows * kXP + kXN * 16 + kTw);
static_assert(kR2CSmem <= 113 * 1024 && kC2RSmem <= 113 * 1024, "two CTAs per SM");

}  // namespace

bool xy_fused_ok(const baorec_ctx* ctx) { return ctx->n1 == kXN && ctx->n2 == kXN && ctx->stab != nullptr; }

int xy_fused_prepare(baorec_ctx* ctx) {
  CK(cudaFuncSetAttribute(xy_r2c_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kR2CSmem));
  CK(cudaFuncSetAttribute(xy_c2r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kC2RSmem));
  return BAOREC_OK;
}

static const float2* w256_of(const baorec_ctx* ctx) {
  return reinterpret_cast<const float2*>(ctx->stab + 2 * (ctx->n1h + ctx->n2 + ctx->n3));
}

int xy_r2c(baorec_ctx* ctx, const float* in, cufftComplex* out, int planes) {
  (xy_r2c_kernel<<<dim3(kCl, planes), kCT, kR2CSmem, ctx->stream>>>(in, reinterpret_cast<float2*>(out), w256_of(ctx)),
   ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int xy_c2r(baorec_ctx* ctx, const cufftComplex* in, float* out, int planes) {
  (xy_c2r_kernel<<<dim3(kCl, planes), kCT, kC2RSmem, ctx->stream>>>(reinterpret_cast<const float2*>(in), out,
                                                                    w256_of(ctx)),
   ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec
