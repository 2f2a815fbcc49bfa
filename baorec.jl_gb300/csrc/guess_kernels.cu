// Tensor-core implicit-GEMM kernels of the learned initial guess: the gather
// convolution (forward and backward-data) and its weight gradient.  BF16
// operands, FP32 accumulation, warp-level mma.sync (m16n8k16; m16n8k8 for
// the 8-channel input layer).
#include <cuda_runtime.h>

#include "common.cuh"
#include "guess.cuh"

namespace baorec {
namespace guess {
namespace {

constexpr int kWarps = 8;   // warps per block
constexpr int kMT = 2;      // 16-voxel M tiles per warp in the forward kernel
constexpr int kG = 4;       // weight-gradient tiles held per warp at a time

__device__ __forceinline__ void mma16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                      uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma8(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ size_t vox(int n, int x, int y, int z) { return ((size_t)z * n + y) * n + x; }

// K order of the m16n8k16 operands.  A lane (q = lane & 3) holds the K
// indices 2q, 2q+1, 8+2q, 9+2q of a k-step; the sum over K does not care
// which input channel each index stands for, as long as the A loads and the
// weight fragments agree.  The channels are assigned so that a lane's A
// values are contiguous in the voxel's channel vector: with 16 input channels
// lane q holds channels 4q .. 4q+3 (one 8-byte load), with 32 or more the
// k-steps go in pairs and lane q holds channels 32p + 8q .. 8q+7 of pair p
// (one 16-byte load feeding two k-steps).  K index j of k-step ks is channel
// kchan(ks, j, KS).
__host__ __device__ __forceinline__ int kchan(int ks, int j, int KS) {
  const int q = (j & 7) >> 1, hi = j >= 8 ? 2 : 0, e = j & 1;
  if (KS == 1) return 4 * q + hi + e;
  return 32 * (ks >> 1) + 8 * q + 4 * (ks & 1) + hi + e;
}

// Source voxel of output voxel (x, y, z) through tap t; false when it falls
// in the zero padding.  For UP the tap is the output's parity (checked by the
// caller) and (x, y, z) are the coarse coordinates.
template <int KIND>
__device__ __forceinline__ bool src_of(int t, int x, int y, int z, int n_in, int& xs, int& ys, int& zs) {
  if (KIND == C3) {
    xs = x + t % 3 - 1; ys = y + (t / 3) % 3 - 1; zs = z + t / 9 - 1;
  } else if (KIND == DN) {
    xs = 2 * x + (t & 1); ys = 2 * y + ((t >> 1) & 1); zs = 2 * z + (t >> 2);
  } else {
    xs = x; ys = y; zs = z;
  }
  return xs >= 0 && xs < n_in && ys >= 0 && ys < n_in && zs >= 0 && zs < n_in;
}

// One warp = one task: kMT*16 consecutive x of one output row (for UP: of
// one coarse row and one output parity), all output channels.
template <int KIND, int CIN, int COUT, int WB = kWarps>
__global__ void __launch_bounds__(WB * 32) conv_fwd_kernel(ConvArgs a) {
  constexpr int NB = COUT / 8;
  constexpr bool K8 = CIN == 8;
  constexpr int KS = K8 ? 1 : CIN / 16;
  constexpr int T = KIND == C3 ? 27 : 8;
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  const int nx = KIND == UP ? a.n_in : a.n_out;   // grid the tasks walk
  const int chunks = (nx + 16 * kMT - 1) / (16 * kMT);
  const long long task = (long long)blockIdx.x * WB + (threadIdx.x >> 5);
  const long long ntask = (long long)chunks * nx * nx * (KIND == UP ? 8 : 1);
  if (task >= ntask) return;
  const int cx = (int)(task % chunks);
  long long r = task / chunks;
  const int y = (int)(r % nx);
  r /= nx;
  const int z = (int)(r % nx);
  const int par = KIND == UP ? (int)(r / nx) : 0;
  const int x0 = cx * 16 * kMT;

  float acc[kMT][NB][4];
#pragma unroll
  for (int m = 0; m < kMT; ++m)
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[m][b][e] = 0.0f;

  // 3x3x3 layers with 32+ input and at most 32 output channels: a software
  // pipeline over (tap, pair of k-steps) loads the next step's operands into
  // registers while this step's MMAs run (the operand order is that of the
  // pair branch below, see kchan)
  constexpr bool PIPE = KIND == C3 && !K8 && KS % 2 == 0 && NB <= 4;
  if constexpr (PIPE) {
    constexpr int KP = KS / 2, NSTEP = 27 * KP;
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    uint4 ca0[kMT], ca1[kMT], na0[kMT], na1[kMT];
    uint2 cb0[NB], cb1[NB], nb0[NB], nb1[NB];
    auto fetch = [&](int st, uint4(&A0)[kMT], uint4(&A1)[kMT], uint2(&B0)[NB], uint2(&B1)[NB]) {
      const int t = st / KP, kp = st - KP * t;
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {
        B0[nb] = __ldg(a.w + ((size_t)(t * KS + 2 * kp) * NB + nb) * 32 + lane);
        B1[nb] = __ldg(a.w + ((size_t)(t * KS + 2 * kp + 1) * NB + nb) * 32 + lane);
      }
#pragma unroll
      for (int m = 0; m < kMT; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int x = x0 + 16 * m + g + 8 * h;
          int xs, ys, zs;
          const bool ok = x < nx && src_of<C3>(t, x, y, z, a.n_in, xs, ys, zs);
          const uint4 v =
              ok ? __ldg(reinterpret_cast<const uint4*>(a.in + vox(a.n_in, xs, ys, zs) * a.in_cs) + 4 * kp + q) : z4;
          if (h == 0) A0[m] = v;
          else A1[m] = v;
        }
    };
    fetch(0, ca0, ca1, cb0, cb1);
#pragma unroll 1
    for (int st = 0; st < NSTEP; ++st) {
      if (st + 1 < NSTEP) fetch(st + 1, na0, na1, nb0, nb1);
#pragma unroll
      for (int m = 0; m < kMT; ++m)
#pragma unroll
        for (int nb = 0; nb < NB; ++nb) {
          mma16(acc[m][nb], ca0[m].x, ca1[m].x, ca0[m].y, ca1[m].y, cb0[nb].x, cb0[nb].y);
          mma16(acc[m][nb], ca0[m].z, ca1[m].z, ca0[m].w, ca1[m].w, cb1[nb].x, cb1[nb].y);
        }
#pragma unroll
      for (int m = 0; m < kMT; ++m) { ca0[m] = na0[m]; ca1[m] = na1[m]; }
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) { cb0[nb] = nb0[nb]; cb1[nb] = nb1[nb]; }
    }
  } else {
    for (int t = 0; t < T; ++t) {
      if (KIND == UP && t != par) continue;
      const uint32_t* rows[kMT][2];
  #pragma unroll
      for (int m = 0; m < kMT; ++m)
  #pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int x = x0 + 16 * m + g + 8 * h;
          int xs, ys, zs;
          const bool ok = x < nx && src_of<KIND>(t, x, y, z, a.n_in, xs, ys, zs);
          rows[m][h] = ok ? reinterpret_cast<const uint32_t*>(a.in + vox(a.n_in, xs, ys, zs) * a.in_cs) : nullptr;
        }
      if (K8) {
        uint2 b[NB];
  #pragma unroll
        for (int nb = 0; nb < NB; ++nb) b[nb] = __ldg(a.w + ((size_t)t * NB + nb) * 32 + lane);
  #pragma unroll
        for (int m = 0; m < kMT; ++m) {
          const uint32_t a0 = rows[m][0] ? __ldg(rows[m][0] + q) : 0u;
          const uint32_t a1 = rows[m][1] ? __ldg(rows[m][1] + q) : 0u;
  #pragma unroll
          for (int nb = 0; nb < NB; ++nb) mma8(acc[m][nb], a0, a1, b[nb].x);
        }
      } else if (KS == 1) {
        // channels 4q .. 4q+3 of the row: (a0, a2) for row g, (a1, a3) for row g+8 (kchan)
        uint2 b[NB];
  #pragma unroll
        for (int nb = 0; nb < NB; ++nb) b[nb] = __ldg(a.w + ((size_t)t * NB + nb) * 32 + lane);
  #pragma unroll
        for (int m = 0; m < kMT; ++m) {
          const uint2 u0 = rows[m][0] ? __ldg(reinterpret_cast<const uint2*>(rows[m][0]) + q) : make_uint2(0u, 0u);
          const uint2 u1 = rows[m][1] ? __ldg(reinterpret_cast<const uint2*>(rows[m][1]) + q) : make_uint2(0u, 0u);
  #pragma unroll
          for (int nb = 0; nb < NB; ++nb) mma16(acc[m][nb], u0.x, u1.x, u0.y, u1.y, b[nb].x, b[nb].y);
        }
      } else {
        // k-steps in pairs: channels 32p + 8q .. 8q+7 of the row feed k-steps 2p and 2p+1 (kchan)
  #pragma unroll
        for (int kp = 0; kp < KS / 2; ++kp) {
          uint2 b0[NB], b1[NB];
  #pragma unroll
          for (int nb = 0; nb < NB; ++nb) {
            b0[nb] = __ldg(a.w + ((size_t)(t * KS + 2 * kp) * NB + nb) * 32 + lane);
            b1[nb] = __ldg(a.w + ((size_t)(t * KS + 2 * kp + 1) * NB + nb) * 32 + lane);
          }
  #pragma unroll
          for (int m = 0; m < kMT; ++m) {
            const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
            const uint4 u0 = rows[m][0] ? __ldg(reinterpret_cast<const uint4*>(rows[m][0]) + 4 * kp + q) : z4;
            const uint4 u1 = rows[m][1] ? __ldg(reinterpret_cast<const uint4*>(rows[m][1]) + 4 * kp + q) : z4;
  #pragma unroll
            for (int nb = 0; nb < NB; ++nb) {
              mma16(acc[m][nb], u0.x, u1.x, u0.y, u1.y, b0[nb].x, b0[nb].y);
              mma16(acc[m][nb], u0.z, u1.z, u0.w, u1.w, b1[nb].x, b1[nb].y);
            }
          }
        }
      }
    }
  }
  // epilogue: bias, addend, ReLU, BF16.  C3 and DN: the warp's 32 output
  // voxels are consecutive in x, so they are staged in shared memory and
  // written as 16-byte vectors (a voxel's COUT channels are contiguous); UP
  // (its own kernel in the network) keeps per-thread stores.
  __shared__ __align__(16) __nv_bfloat16 stile[KIND == UP ? 1 : WB][KIND == UP ? 8 : 16 * kMT * COUT];
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < kMT; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int x = x0 + 16 * m + g + 8 * h;
      size_t vo;
      if (KIND == UP)
        vo = vox(a.n_out, 2 * x + (par & 1), 2 * y + ((par >> 1) & 1), 2 * z + (par >> 2));
      else
        vo = vox(a.n_out, x, y, z);
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {
        const int n = 8 * nb + 2 * q;
        float v0 = acc[m][nb][2 * h], v1 = acc[m][nb][2 * h + 1];
        if (a.bias) { v0 += __ldg(a.bias + n); v1 += __ldg(a.bias + n + 1); }
        if (a.add && x < nx) {
          const __nv_bfloat162 ad = *reinterpret_cast<const __nv_bfloat162*>(a.add + vo * a.add_cs + n);
          v0 += __bfloat162float(ad.x);
          v1 += __bfloat162float(ad.y);
        }
        if (a.relu) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
        if (KIND == UP) {
          if (x < nx) *reinterpret_cast<__nv_bfloat162*>(a.out + vo * a.out_cs + n) = __floats2bfloat162_rn(v0, v1);
        } else {
          *reinterpret_cast<__nv_bfloat162*>(&stile[warp][(16 * m + g + 8 * h) * COUT + n]) =
              __floats2bfloat162_rn(v0, v1);
        }
      }
    }
  if (KIND != UP) {
    constexpr int VPV = COUT / 8;   // 16-byte vectors per voxel
    __syncwarp();
    const uint4* sv = reinterpret_cast<const uint4*>(stile[warp]);
    const size_t row0 = vox(a.n_out, x0, y, z);
#pragma unroll
    for (int k = 0; k < kMT * VPV / 2; ++k) {
      const int vi = lane + 32 * k;   // 16 kMT voxels x VPV vectors
      const int j = vi / VPV, part = vi - VPV * j;
      if (x0 + j < nx) *reinterpret_cast<uint4*>(a.out + (row0 + j) * a.out_cs + 8 * part) = sv[vi];
    }
  }
}

// Weight gradient dW[t][ci][co] = Σ_v x[src(v,t)][ci] dy[v][co]: an MMA with
// M = input channels, N = output channels, K = 16 voxels of one output row.
// Each block walks a contiguous range of 16-voxel rows; each warp holds kG
// (tap, ci tile, co block) accumulators at a time and flushes them with FP32
// atomics at the end.
template <int KIND, int CIN, int COUT>
__global__ void __launch_bounds__(kWarps * 32) wgrad_kernel(WgradArgs a, int rows_per_block) {
  constexpr int NB = COUT / 8;
  constexpr int CIT = (CIN + 15) / 16;
  constexpr int T = KIND == C3 ? 27 : 8;
  constexpr int ITEMS = T * CIT * NB;
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3, warp = threadIdx.x >> 5;
  const int nx = KIND == UP ? a.n_in : a.n_out;
  const int chunks = (nx + 15) / 16;
  const long long nrows = (long long)chunks * nx * nx;
  const long long r0 = (long long)blockIdx.x * rows_per_block;
  const long long r1 = r0 + rows_per_block < nrows ? r0 + rows_per_block : nrows;
  for (int i0 = warp; i0 < ITEMS; i0 += kWarps * kG) {
    float acc[kG][4];
#pragma unroll
    for (int j = 0; j < kG; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[j][e] = 0.0f;
    for (long long rr = r0; rr < r1; ++rr) {
      const int cx = (int)(rr % chunks);
      const long long s = rr / chunks;
      const int y = (int)(s % nx), z = (int)(s / nx);
      const int x0 = 16 * cx;
#pragma unroll
      for (int j = 0; j < kG; ++j) {
        const int item = i0 + j * kWarps;
        if (item >= ITEMS) break;
        const int t = item / (CIT * NB);
        const int rem = item - t * CIT * NB;
        const int cit = rem / NB, nb = rem - cit * NB;
        const int c0 = 16 * cit, n0 = 8 * nb;
        // the four K columns of this lane: 2q, 2q+1, 2q+8, 2q+9
        __nv_bfloat16 xa[4], xb[4], dv[4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const int k = 2 * q + (kk & 1) + 8 * (kk >> 1);
          const int x = x0 + k;
          xa[kk] = xb[kk] = dv[kk] = __float2bfloat16(0.0f);
          if (x >= nx) continue;
          size_t vo;
          int xs, ys, zs;
          bool ok;
          if (KIND == UP) {
            vo = vox(a.n_out, 2 * x + (t & 1), 2 * y + ((t >> 1) & 1), 2 * z + (t >> 2));
            ok = true;
            xs = x; ys = y; zs = z;
          } else {
            vo = vox(a.n_out, x, y, z);
            ok = src_of<KIND>(t, x, y, z, a.n_in, xs, ys, zs);
          }
          dv[kk] = a.dy[vo * a.dy_cs + n0 + g];
          if (ok) {
            const __nv_bfloat16* xp = a.in + vox(a.n_in, xs, ys, zs) * a.in_cs + c0 + g;
            xa[kk] = xp[0];
            if (c0 + g + 8 < CIN) xb[kk] = xp[8];
          }
        }
        mma16(acc[j], pack2(xa[0], xa[1]), pack2(xb[0], xb[1]), pack2(xa[2], xa[3]), pack2(xb[2], xb[3]),
              pack2(dv[0], dv[1]), pack2(dv[2], dv[3]));
      }
    }
#pragma unroll
    for (int j = 0; j < kG; ++j) {
      const int item = i0 + j * kWarps;
      if (item >= ITEMS) break;
      const int t = item / (CIT * NB);
      const int rem = item - t * CIT * NB;
      const int cit = rem / NB, nb = rem - cit * NB;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int ci = 16 * cit + g + 8 * h;
        if (ci >= CIN) continue;
        const int co = 8 * nb + 2 * q;
        float* d = a.dw + ((size_t)t * CIN + ci) * COUT + co;
        atomicAdd(d, acc[j][2 * h]);
        atomicAdd(d + 1, acc[j][2 * h + 1]);
      }
    }
  }
}

__global__ void frag_kernel(int kind, int cin, int cout, const float* __restrict__ w, uint2* __restrict__ frag,
                            int backward) {
  // the convolution these fragments feed: (kind', cin', cout')
  const int k2 = backward ? (kind == DN ? UP : kind == UP ? DN : C3) : kind;
  const int ci2 = backward ? cout : cin, co2 = backward ? cin : cout;
  const int T = k2 == C3 ? 27 : 8;
  const int KS = ci2 >= 16 ? ci2 / 16 : 1, NB = co2 / 8;
  const size_t total = (size_t)T * KS * NB * 32;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int lane = (int)(e % 32);
    size_t r = e / 32;
    const int nb = (int)(r % NB);
    r /= NB;
    const int ks = (int)(r % KS);
    const int t = (int)(r / KS);
    const int g = lane >> 2, q = lane & 3;
    const int n = 8 * nb + g;
    auto W = [&](int k) -> __nv_bfloat16 {
      if (k >= ci2) return __float2bfloat16(0.0f);
      // forward: W[t][k][n]; backward: W[flip t][n][k] (k: original output channel)
      float v = backward ? w[((size_t)(kind == C3 ? 26 - t : t) * cin + n) * cout + k]
                         : w[((size_t)t * cin + k) * cout + n];
      return __float2bfloat16(v);
    };
    uint2 f;
    if (ci2 >= 16) {   // K index j of k-step ks stands for input channel kchan(ks, j, KS)
      f.x = pack2(W(kchan(ks, 2 * q, KS)), W(kchan(ks, 2 * q + 1, KS)));
      f.y = pack2(W(kchan(ks, 8 + 2 * q, KS)), W(kchan(ks, 9 + 2 * q, KS)));
    } else {           // 8 input channels: m16n8k8, K index j is channel j
      f.x = pack2(W(2 * q), W(2 * q + 1));
      f.y = 0u;
    }
    frag[e] = f;
  }
}

// UP (2x2x2 transposed, stride 2) with coalesced stores: one warp takes 32
// consecutive coarse voxels of a coarse row and one (py, pz) parity pair, and
// computes both x parities, so the 64 fine voxels it produces are adjacent in
// the fine row (2y + py, 2z + pz).  They are staged in shared memory and
// written as 16-byte vectors (a voxel's COUT channels are contiguous).
template <int CIN, int COUT>
__global__ void __launch_bounds__(kWarps * 32) up_kernel(ConvArgs a) {
  constexpr int NB = COUT / 8, KS = CIN / 16, VPV = COUT / 8;   // 16-byte vectors per fine voxel
  __shared__ __align__(16) __nv_bfloat16 stile[kWarps][64 * COUT];
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3, warp = threadIdx.x >> 5;
  const int nx = a.n_in;
  const int chunks = (nx + 31) / 32;
  const long long task = (long long)blockIdx.x * kWarps + warp;
  if (task >= (long long)chunks * nx * nx * 4) return;   // warp-uniform; no block barrier below
  const int cx = (int)(task % chunks);
  long long r = task / chunks;
  const int y = (int)(r % nx);
  r /= nx;
  const int z = (int)(r % nx);
  const int pyz = (int)(r / nx), py = pyz & 1, pz = pyz >> 1;
  const int x0 = 32 * cx;
  float acc[2][2][NB][4];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int px = 0; px < 2; ++px)
#pragma unroll
      for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[m][px][b][e] = 0.0f;
  const uint32_t* rows[2][2];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int x = x0 + 16 * m + g + 8 * h;
      rows[m][h] = x < nx ? reinterpret_cast<const uint32_t*>(a.in + vox(nx, x, y, z) * a.in_cs) : nullptr;
    }
  static_assert(KS % 2 == 0, "the up-sampling layers have 32 or 64 input channels: k-steps in pairs");
#pragma unroll
  for (int ks = 0; ks < KS; ++ks) {
    // channels 32p + 8q .. 8q+7 of the row feed k-steps 2p and 2p+1 (kchan)
    uint32_t av[2][4];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
      const uint4 u0 = rows[m][0] ? __ldg(reinterpret_cast<const uint4*>(rows[m][0]) + 4 * (ks >> 1) + q) : z4;
      const uint4 u1 = rows[m][1] ? __ldg(reinterpret_cast<const uint4*>(rows[m][1]) + 4 * (ks >> 1) + q) : z4;
      av[m][0] = (ks & 1) ? u0.z : u0.x;
      av[m][1] = (ks & 1) ? u1.z : u1.x;
      av[m][2] = (ks & 1) ? u0.w : u0.y;
      av[m][3] = (ks & 1) ? u1.w : u1.y;
    }
#pragma unroll
    for (int px = 0; px < 2; ++px) {
      const int t = px + 2 * py + 4 * pz;
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {
        const uint2 b = __ldg(a.w + ((size_t)(t * KS + ks) * NB + nb) * 32 + lane);
#pragma unroll
        for (int m = 0; m < 2; ++m) mma16(acc[m][px][nb], av[m][0], av[m][1], av[m][2], av[m][3], b.x, b.y);
      }
    }
  }
  // epilogue into the staging tile: fine-local voxel j = 2 (16 m + g + 8 h) + px
  const int fy = 2 * y + py, fz = 2 * z + pz, nf = a.n_out;
  __nv_bfloat16* st = stile[warp];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int px = 0; px < 2; ++px) {
        const int j = 2 * (16 * m + g + 8 * h) + px;
        const int fx = 2 * x0 + j;
#pragma unroll
        for (int nb = 0; nb < NB; ++nb) {
          const int n = 8 * nb + 2 * q;
          float v0 = acc[m][px][nb][2 * h], v1 = acc[m][px][nb][2 * h + 1];
          if (a.bias) { v0 += __ldg(a.bias + n); v1 += __ldg(a.bias + n + 1); }
          if (a.add && fx < nf) {
            const __nv_bfloat162 ad =
                *reinterpret_cast<const __nv_bfloat162*>(a.add + vox(nf, fx, fy, fz) * a.add_cs + n);
            v0 += __bfloat162float(ad.x);
            v1 += __bfloat162float(ad.y);
          }
          if (a.relu) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
          *reinterpret_cast<__nv_bfloat162*>(st + j * COUT + n) = __floats2bfloat162_rn(v0, v1);
        }
      }
  __syncwarp();
  const uint4* sv = reinterpret_cast<const uint4*>(st);
  const size_t row0 = vox(nf, 2 * x0, fy, fz);
#pragma unroll
  for (int k = 0; k < 2 * VPV; ++k) {
    const int vi = lane + 32 * k;            // 64 voxels x VPV vectors
    const int j = vi / VPV, part = vi - VPV * j;
    if (2 * x0 + j < nf)
      *reinterpret_cast<uint4*>(a.out + (row0 + j) * a.out_cs + 8 * part) = sv[vi];
  }
}

template <int CIN, int COUT>
cudaError_t up_t(cudaStream_t s, const ConvArgs& a) {
  const int nx = a.n_in;
  const long long ntask = (long long)((nx + 31) / 32) * nx * nx * 4;
  const unsigned blocks = (unsigned)((ntask + kWarps - 1) / kWarps);
  (up_kernel<CIN, COUT><<<blocks, kWarps * 32, 0, s>>>(a), ::baorec::count_launch());
  return cudaGetLastError();
}

template <int KIND, int CIN, int COUT>
cudaError_t fwd_t(cudaStream_t s, const ConvArgs& a) {
  const int nx = KIND == UP ? a.n_in : a.n_out;
  const long long ntask = (long long)((nx + 16 * kMT - 1) / (16 * kMT)) * nx * nx * (KIND == UP ? 8 : 1);
  const unsigned blocks = (unsigned)((ntask + kWarps - 1) / kWarps);
  if (blocks < 2u * kNumSMs) {
    // a small grid (the network's n/4 level): blocks of 2 warps spread it over every SM
    constexpr int kSmall = 2;
    (conv_fwd_kernel<KIND, CIN, COUT, kSmall><<<(unsigned)((ntask + kSmall - 1) / kSmall), kSmall * 32, 0, s>>>(a), ::baorec::count_launch());
  } else {
    (conv_fwd_kernel<KIND, CIN, COUT><<<blocks, kWarps * 32, 0, s>>>(a), ::baorec::count_launch());
  }
  return cudaGetLastError();
}

template <int KIND, int CIN, int COUT>
cudaError_t wgrad_t(cudaStream_t s, const WgradArgs& a) {
  const int nx = KIND == UP ? a.n_in : a.n_out;
  const long long nrows = (long long)((nx + 15) / 16) * nx * nx;
  const int target = 2 * 152;   // two blocks per SM
  int per = (int)((nrows + target - 1) / target);
  if (per < 1) per = 1;
  const unsigned blocks = (unsigned)((nrows + per - 1) / per);
  (wgrad_kernel<KIND, CIN, COUT><<<blocks, kWarps * 32, 0, s>>>(a, per), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace

cudaError_t conv_forward(cudaStream_t s, int kind, int cin, int cout, const ConvArgs& a) {
  if (a.wimg && a.n_in == a.n_out && tc_supported(kind, cin, cout, a.n_out)) return conv_forward_tc(s, cin, cout, a);
  if (kind == UP && cin == 32 && cout == 16) return up_t<32, 16>(s, a);
  if (kind == UP && cin == 64 && cout == 32) return up_t<64, 32>(s, a);
#define X(K, I, O) \
  if (kind == K && cin == I && cout == O) return fwd_t<K, I, O>(s, a);
  BAOREC_GUESS_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t conv_wgrad(cudaStream_t s, int kind, int cin, int cout, const WgradArgs& a) {
#define X(K, I, O) \
  if (kind == K && cin == I && cout == O) return wgrad_t<K, I, O>(s, a);
  BAOREC_GUESS_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t weight_frags(cudaStream_t s, int kind, int cin, int cout, const float* w, uint2* frag, bool backward) {
  (frag_kernel<<<64, 256, 0, s>>>(kind, cin, cout, w, frag, backward ? 1 : 0), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace guess
}  // namespace baorec
