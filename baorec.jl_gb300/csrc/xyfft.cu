// Fused 2-D real transforms of 256 x 256 xy planes (the x and y passes of the
// FFT preconditioner's, the smoothing's and the displacement's transforms),
// one kernel per direction instead of cuFFT's two passes.
//
// Forward (R2C), two blocks per plane, block h keeping kx in [65h, 65h + 65 - h):
//   x: each row of 256 reals is packed as 128 complex z[n] = x[2n] + i x[2n+1],
//      transformed with a four-step 128 = 16 x 8 (a 16-point DFT in registers,
//      the 128-point twiddles, an exchange in shared memory, two 8-point
//      DFTs), and unpacked: X[k] = (Z[k] + Z*[128-k])/2
//      - i/2 e^{-2πik/256} (Z[k] - Z*[128-k]), k = 0..128;
//   y: each kept column (256 rows, in shared memory) is transformed with the
//      four-step 256 = 16 x 16 of the z pass, in place, and written to the
//      spectrum [plane][ky][kx] (row length 129) as cuFFT's batched 2-D R2C does.
// Both blocks of a plane read the whole plane; the second read hits L2.
// Inverse (C2R), two blocks per plane, block h producing rows [128h, 128h+128):
//   y: every column is inverse-transformed (four-step, exchange in shared
//      memory) and the block keeps its 128 rows;
//   x: each kept row is packed, Z[k] = (X[k] + X*[128-k]) + i (X[k] - X*[128-k])
//      e^{2πik/256}, inverse-transformed (four-step 128) and unpacked,
//      x[2n] = Re z[n], x[2n+1] = Im z[n]; unnormalised like cuFFT's C2R.
// The index algebra of both kernels was checked against numpy's FFT.  On a
// GB300 one 256-plane transform takes 108.6 us forward and 104.2 us inverse
// (one 200 KB block per SM, 16 warps, the row and column phases serialised
// by barriers) against about 60 us for cuFFT's two passes, so the autotuner
// keeps cuFFT; the kernels stay a timed candidate.
#include "common.cuh"

namespace baorec {
namespace {

constexpr int kXN = 256;         // points along x and y
constexpr int kXH = kXN / 2;     // packed complex points of a row
constexpr int kXC = kXN / 2 + 1; // half-spectrum length (129)
constexpr int kXT = 512;         // threads per block
constexpr int kXRows = kXT / 8;  // rows of one x-transform group (8 threads per row)
constexpr int kYCols = kXT / 16; // columns of one y-transform round (16 threads per column)

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

// Four-step 128-point transform of one packed row held by 8 threads (b =
// lane-in-row): input values in[8a + b], a = 0..15 (already in registers v);
// rb is the row's 128-value exchange buffer.  On return the thread holds
// outputs k = c + 16 d for c in {b, b + 8} (d = 0..7) in o[2][8].
template <bool INV>
__device__ __forceinline__ void fft128_row(float2 (&v)[16], float2* __restrict__ rb, int b,
                                           const float2* __restrict__ w256, float2 (&o)[2][8]) {
  dft16x<INV>(v);   // over a: v[c]
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float2 w = w256[2 * ((b * c) & 127)];   // e^{-2πi bc/128}
    rb[8 * c + b] = INV ? cmulc(v[c], w) : cmul(v[c], w);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int c = b + 8 * q;
#pragma unroll
    for (int bb = 0; bb < 8; ++bb) o[q][bb] = rb[8 * c + bb];
    dft8x<INV>(o[q]);   // over b: o[q][d] = out[c + 16 d]
  }
}

__global__ void __launch_bounds__(kXT, 1) xy_r2c_kernel(const float* __restrict__ in, cufftComplex* __restrict__ out,
                                                       const float2* __restrict__ tw) {
  extern __shared__ __align__(16) float2 xsm[];
  constexpr int HW = 65;                        // kept columns (block 1: 64)
  float2* hs = xsm;                             // [256 rows][HW]
  float2* rbuf = xsm + kXN * HW;                // [kXRows rows][128]
  float2* w256 = rbuf + kXRows * kXH;           // e^{-2πi m/256}
  const int t = threadIdx.x;
  const int h = blockIdx.x, k0 = 65 * h, ncol = HW - h;
  const size_t plane = blockIdx.y;
  const float* src = in + plane * (size_t)(kXN * kXN);
  float2* dst = reinterpret_cast<float2*>(out) + plane * (size_t)(kXC * kXN);
  if (t < kXN) w256[t] = __ldg(tw + t);
  __syncthreads();
  const int rl = t >> 3, b = t & 7;             // row within the group, lane within the row
  float2* rb = rbuf + rl * kXH;
  for (int g = 0; g < kXN / kXRows; ++g) {
    const int row = g * kXRows + rl;
    float2 v[16];
    const float2* xr = reinterpret_cast<const float2*>(src + (size_t)row * kXN);
#pragma unroll
    for (int a = 0; a < 16; ++a) v[a] = __ldg(xr + 8 * a + b);   // z[8a + b] = (x[16a+2b], x[16a+2b+1])
    float2 o[2][8];
    fft128_row<false>(v, rb, b, w256, o);
    __syncthreads();   // every thread of the row has read the exchange buffer
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int d = 0; d < 8; ++d) rb[b + 8 * q + 16 * d] = o[q][d];   // Z in natural order
    __syncthreads();
    // unpack X[k] = (Z[k] + Z*[128-k])/2 - i/2 W256^k (Z[k] - Z*[128-k]) for the kept k
    for (int j = b; j < ncol; j += 8) {
      const int k = k0 + j;
      const float2 zk = rb[k & (kXH - 1)], zm = conjf2(rb[(kXH - k) & (kXH - 1)]);
      const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
      const float2 dd = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y - zm.y));
      const float2 od = cmul(make_float2(dd.y, -dd.x), w256[k & (kXN - 1)]);   // -i dd W^k
      hs[row * HW + j] = addf2(e, od);
    }
    __syncthreads();   // the exchange buffer is free for the next group
  }
  // y: four-step 256 = 16 x 16 per kept column, in place in hs, then out
  const int cl = t & (kYCols - 1), r = t >> 5;
  for (int c0 = 0; c0 < ncol; c0 += kYCols) {
    const int col = c0 + cl;
    const bool ok = col < ncol;
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) v[n1] = ok ? hs[(16 * n1 + r) * HW + col] : make_float2(0.0f, 0.0f);
    dft16x<false>(v);
    if (ok) {
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) hs[(16 * k1 + r) * HW + col] = cmul(v[k1], w256[r * k1]);
    }
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = ok ? hs[(16 * r + n2) * HW + col] : make_float2(0.0f, 0.0f);
    dft16x<false>(v);   // v[k2] = X[ky = r + 16 k2]
    if (ok) {
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2) dst[(size_t)(r + 16 * k2) * kXC + k0 + col] = v[k2];
    }
  }
}

__global__ void __launch_bounds__(kXT, 1) xy_c2r_kernel(const cufftComplex* __restrict__ in, float* __restrict__ out,
                                                       const float2* __restrict__ tw) {
  extern __shared__ __align__(16) float2 xsm[];
  constexpr int HP = kXC;                       // row length of the kept rows
  constexpr int SP = kXN + 1;                   // padded column of the y exchange
  float2* hr = xsm;                             // [128 rows][129]
  float2* rbuf = xsm + kXH * HP;                // y exchange [kYCols][257], then x rows [kXRows][128]
  float2* w256 = rbuf + kYCols * SP;
  const int t = threadIdx.x;
  const int h = blockIdx.x, y0 = kXH * h;
  const size_t plane = blockIdx.y;
  const float2* src = reinterpret_cast<const float2*>(in) + plane * (size_t)(kXC * kXN);
  float* dst = out + plane * (size_t)(kXN * kXN);
  if (t < kXN) w256[t] = __ldg(tw + t);
  __syncthreads();
  // y: inverse four-step per column, the block's rows kept
  const int cl = t & (kYCols - 1), r = t >> 5;
  for (int c0 = 0; c0 < kXC; c0 += kYCols) {
    const int col = c0 + cl;
    const bool ok = col < kXC;
    float2* s = rbuf + cl * SP;
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) v[n1] = ok ? __ldg(src + (size_t)(16 * n1 + r) * kXC + col) : make_float2(0.0f, 0.0f);
    dft16x<true>(v);
    __syncthreads();   // the previous round's reads of the exchange are done
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) s[16 * k1 + r] = cmulc(v[k1], w256[r * k1]);
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = s[16 * r + n2];
    dft16x<true>(v);   // v[k2] = y[r + 16 k2]
    if (ok) {
#pragma unroll
      for (int k2 = 0; k2 < 8; ++k2) hr[(r + 16 * (k2 + 8 * h) - y0) * HP + col] = v[k2 + 8 * h];
    }
  }
  __syncthreads();
  // x: pack, inverse four-step 128, unpack, per kept row
  const int rl = t >> 3, b = t & 7;
  float2* rb = rbuf + rl * kXH;
  for (int g = 0; g < kXH / kXRows; ++g) {
    const int row = g * kXRows + rl;
    const float2* xr = hr + row * HP;
    float2 v[16];
#pragma unroll
    for (int a = 0; a < 16; ++a) {
      const int k = 8 * a + b;   // packed index; Z[k] = (X[k] + X*[128-k]) + i (X[k] - X*[128-k]) W256^{-k}
      const float2 xk = xr[k], xm = conjf2(xr[kXH - k]);
      const float2 sdf = cmulc(subf2(xk, xm), w256[k]);
      v[a] = make_float2(xk.x + xm.x - sdf.y, xk.y + xm.y + sdf.x);
    }
    float2 o[2][8];
    fft128_row<true>(v, rb, b, w256, o);
    float2* xo = reinterpret_cast<float2*>(dst + (size_t)(y0 + row) * kXN);
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int d = 0; d < 8; ++d) xo[b + 8 * q + 16 * d] = o[q][d];   // (x[2n], x[2n+1]), n = c + 16 d
    __syncthreads();   // the exchange buffer is free for the next group
  }
}

constexpr size_t kR2CSmem = sizeof(float2) * (kXN * 65 + kXRows * kXH + kXN);
constexpr size_t kC2RSmem = sizeof(float2) * (kXH * kXC + kYCols * (kXN + 1) + kXN);
static_assert(kXRows * kXH <= kYCols * (kXN + 1), "the x rows fit the y exchange region");

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
  (xy_r2c_kernel<<<dim3(2, planes), kXT, kR2CSmem, ctx->stream>>>(in, out, w256_of(ctx)), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int xy_c2r(baorec_ctx* ctx, const cufftComplex* in, float* out, int planes) {
  (xy_c2r_kernel<<<dim3(2, planes), kXT, kC2RSmem, ctx->stream>>>(in, out, w256_of(ctx)), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec
