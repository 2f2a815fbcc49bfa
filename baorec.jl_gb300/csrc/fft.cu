// k-space operators around cuFFT: Gaussian smoothing, overdensity
// normalisation (FP64 reductions), the iterative-FFT step and the
// displacement / gradient meshes.
//
// Spectra are the halved R2C layout of an x-fastest mesh: element (i, j, k)
// with i < n1/2+1 at i + (n1/2+1)*(j + n2*k); the halved axis is x as in
// rfftfreq(dims[1]) (src/utils.jl:6).  The 1/N of the inverse transform is
// folded into the k-space multiply that precedes every C2R.
#include <algorithm>
#include <cmath>

#include <cufftXt.h>

#include "common.cuh"

// LTO IR of lto/spectral_cb.cu, embedded at build time (sm_103a and sm_103 targets)
extern "C" const unsigned char baorec_lto_spectral_cb_a[];
extern "C" const size_t baorec_lto_spectral_cb_a_size;
extern "C" const unsigned char baorec_lto_spectral_cb_p[];
extern "C" const size_t baorec_lto_spectral_cb_p_size;

namespace baorec {
namespace {

struct KGeom {
  int n1h, n2, n3;
  int nyq[3];      // index of the Nyquist mode per axis (n/2), -1 for odd n
  float mult[3];   // T(fs/n), fs = T(2π n / L) — the k-axis step of k_vec (src/utils.jl:3-10)
  float invN;
};

KGeom kgeom_of(const baorec_ctx* c) {
  KGeom g;
  g.n1h = c->n1h; g.n2 = c->n2; g.n3 = c->n3;
  const int n[3] = {c->n1, c->n2, c->n3};
  for (int a = 0; a < 3; ++a) {
    float fs = (float)(2.0 * 3.14159265358979323846 * (double)n[a] / (double)c->cfg.box_size[a]);
    g.mult[a] = fs / (float)n[a];
    g.nyq[a] = n[a] % 2 == 0 ? n[a] / 2 : -1;
  }
  g.invN = (float)(1.0 / (double)c->N);
  return g;
}

// Hermitian part of a spectral product in the planes a C2R reads as Hermitian.
//
// A real field's half-complex spectrum F satisfies F(partner) = conj F, where
// inside the kx = 0 and kx = n1/2 planes the partner of (ky, kz) is
// (-ky, -kz) and the Nyquist indices n/2 are their own partners (their k value
// is the same -k_nyq on both sides; the kx = n1/2 plane is its own partner in
// x).  A factor odd in k_a flips sign between partners except where the
// a-index is its own partner, so on those entries i k_a F (a derivative) or
// k_a k_b F with exactly one self-partnered index (a mixed Hessian term) is
// anti-Hermitian.  FFTW's c2r (the reference's plan_rfft inverse) and
// pocketfft read only the Hermitian part of these two planes; cuFFT resolves
// the rest differently.  The kernels below therefore write the Hermitian part,
// zero on those entries, so every correct C2R gives the reference's field.
__device__ __forceinline__ bool in_real_plane(const KGeom& g, int i) { return i == 0 || i == g.nyq[0]; }

// index along axis a is its own partner (x: always, inside the two planes)
__device__ __forceinline__ bool self_partner(const KGeom& g, int a, int j, int k) {
  return a == 0 ? true : (a == 1 ? j == g.nyq[1] : k == g.nyq[2]);
}

// entry (i, j, k) of (odd factor in a) x F is anti-Hermitian: drop it
__device__ __forceinline__ bool drop_odd(const KGeom& g, int a, int i, int j, int k) {
  return in_real_plane(g, i) && self_partner(g, a, j, k);
}

// entry of (odd in a) x (odd in b) x F, a != b, is anti-Hermitian: drop it
__device__ __forceinline__ bool drop_odd2(const KGeom& g, int a, int b, int i, int j, int k) {
  return in_real_plane(g, i) && (self_partner(g, a, j, k) != self_partner(g, b, j, k));
}

// k axes of k_vec: rfftfreq for x, fftfreq (negative half from -n/2) for y, z.
__device__ __forceinline__ void kvals(const KGeom& g, int i, int j, int k, float& kx, float& ky, float& kz) {
  int jj = j < (g.n2 + 1) / 2 ? j : j - g.n2;
  int kk = k < (g.n3 + 1) / 2 ? k : k - g.n3;
  kx = __fmul_rn((float)i, g.mult[0]);
  ky = __fmul_rn((float)jj, g.mult[1]);
  kz = __fmul_rn((float)kk, g.mult[2]);
}

__device__ __forceinline__ float ksq(float kx, float ky, float kz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
}

__device__ __forceinline__ void decompose(size_t e, const KGeom& g, int& i, int& j, int& k) {
  i = (int)(e % g.n1h);
  size_t r = e / g.n1h;
  j = (int)(r % g.n2);
  k = (int)(r / g.n2);
}

// smooth!: δ_k *= exp(-0.5 R² k²) (src/utils.jl:50-53), times 1/N.
__global__ void gauss_kernel(cufftComplex* __restrict__ a, size_t nk, int batch, size_t stride,
                             KGeom g, float R2) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; decompose(e, g, i, j, k);
    float kx, ky, kz; kvals(g, i, j, k, kx, ky, kz);
    float fac = expf(-0.5f * R2 * ksq(kx, ky, kz)) * g.invN;
    for (int b = 0; b < batch; ++b) {
      cufftComplex v = a[e + b * stride];
      v.x *= fac; v.y *= fac;
      a[e + b * stride] = v;
    }
  }
}

// iterate!, first half (src/iterative.jl:8-14, 26-28, 52-54): δ_k/k² (DC → 0)
// and the products handed to the inverse transforms.
//  local LOS: out[m] = k_i k_j δ_k/k² for (i,j) in (11,12,13,22,23,33)
//  global LOS: out[m] = k_i² r̂_i δ_k/k² for each axis with r̂_i != 0.
__global__ void hessian_kernel(const cufftComplex* __restrict__ dk, cufftComplex* __restrict__ out,
                               size_t nk, KGeom g, int local, float3 los, int nprod, int axes_mask) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; decompose(e, g, i, j, k);
    float kv[3]; kvals(g, i, j, k, kv[0], kv[1], kv[2]);
    float k2 = ksq(kv[0], kv[1], kv[2]);
    cufftComplex d = dk[e];
    if (k2 == 0.0f) { d.x = 0.0f; d.y = 0.0f; }
    else { d.x = __fdiv_rn(d.x, k2); d.y = __fdiv_rn(d.y, k2); }
    d.x *= g.invN; d.y *= g.invN;
    if (local) {
      int m = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = a; b < 3; ++b) {
          float s = __fmul_rn(kv[a], kv[b]);
          if (a != b && drop_odd2(g, a, b, i, j, k)) s = 0.0f;
          out[e + (size_t)m * nk] = make_float2(__fmul_rn(s, d.x), __fmul_rn(s, d.y));
          ++m;
        }
    } else {
      const float r[3] = {los.x, los.y, los.z};
      int m = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (!((axes_mask >> a) & 1)) continue;
        float s = __fmul_rn(__fmul_rn(kv[a], kv[a]), r[a]);
        out[e + (size_t)m * nk] = make_float2(__fmul_rn(s, d.x), __fmul_rn(s, d.y));
        ++m;
      }
    }
  }
}

// iterate!, second half (src/iterative.jl:17, 32-35, 58-60): δ_r = δ_s then
// the terms subtracted in the reference's (i, j) order.
__global__ void iterate_update_kernel(float* __restrict__ dr, const float* __restrict__ ds,
                                      const float* __restrict__ parts, size_t N, int n1, int n2,
                                      const float* __restrict__ ax, const float* __restrict__ ay,
                                      const float* __restrict__ az, int local, int nprod,
                                      float fac_diag, float fac_off) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    float v = ds[e];
    if (local) {
      int i = (int)(e % n1);
      size_t r = e / n1;
      int j = (int)(r % n2);
      int k = (int)(r / n2);
      float xv[3] = {ax[i], ay[j], az[k]};
      float x2 = __fadd_rn(__fadd_rn(__fmul_rn(xv[0], xv[0]), __fmul_rn(xv[1], xv[1])), __fmul_rn(xv[2], xv[2]));
      int m = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = a; b < 3; ++b) {
          float fac = (a == b) ? fac_diag : fac_off;
          float t = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(fac, parts[e + (size_t)m * N]), xv[a]), xv[b]), x2);
          v = x2 > 0.0f ? __fsub_rn(v, t) : 0.0f;
          ++m;
        }
    } else {
      for (int m = 0; m < nprod; ++m) v = __fsub_rn(v, __fmul_rn(fac_diag, parts[e + (size_t)m * N]));
    }
    dr[e] = v;
  }
}

// compute_displacements, iterative (src/iterative.jl:265-270): Ψ_i = i k_i δ_k / k²
// (mode == 0); multigrid (src/multigrid.jl:765-768): ∂_i φ = i k_i φ_k (mode == 1).
__global__ void grad_kernel(const cufftComplex* __restrict__ src, cufftComplex* __restrict__ out,
                            size_t nk, KGeom g, int inv_lap) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; decompose(e, g, i, j, k);
    float kv[3]; kvals(g, i, j, k, kv[0], kv[1], kv[2]);
    float k2 = ksq(kv[0], kv[1], kv[2]);
    cufftComplex d = src[e];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      // (i k) * (re + i im) = (-k im, k re)
      const float ka = drop_odd(g, a, i, j, k) ? 0.0f : kv[a];
      float re = -__fmul_rn(ka, d.y), im = __fmul_rn(ka, d.x);
      if (inv_lap) {
        if (k2 > 0.0f) { re = __fdiv_rn(re, k2); im = __fdiv_rn(im, k2); }
        else { re = 0.0f; im = 0.0f; }
      }
      out[e + (size_t)a * nk] = make_float2(re * g.invN, im * g.invN);
    }
  }
}

// FP64 block partial sums of up to two meshes (deterministic two-stage
// reduction).  Each group of 4 consecutive cells is added in FP32 before it
// joins the FP64 accumulator: FP64 arithmetic is slow on this GPU, and a
// 4-term FP32 sum carries at most 3 roundings.
__global__ void sum2_partial_kernel(const float* __restrict__ a, const float* __restrict__ b, size_t N,
                                    double* __restrict__ part) {
  double sa = 0.0, sb = 0.0;
  // vector path only for 16-byte aligned meshes (sub-meshes of a batch may not be)
  const bool vec = ((uintptr_t)a % 16 == 0) && (!b || (uintptr_t)b % 16 == 0);
  const size_t N4 = vec ? N / 4 : 0;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  const float4* b4 = reinterpret_cast<const float4*>(b);
  // four 16-byte loads per array in flight per thread before their sums join
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e0 < N4; e0 += 4 * stride) {
    float4 u[4], w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const size_t e = e0 + k * stride;
      u[k] = e < N4 ? a4[e] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      w[k] = (b && e < N4) ? b4[e] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      sa += (double)((u[k].x + u[k].y) + (u[k].z + u[k].w));
      sb += (double)((w[k].x + w[k].y) + (w[k].z + w[k].w));
    }
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += stride) {
    sa += (double)a[e];
    if (b) sb += (double)b[e];
  }
  for (int o = 16; o > 0; o >>= 1) {
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  __shared__ double s[2][32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s[0][wid] = sa; s[1][wid] = sb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { ta += s[0][k]; tb += s[1][k]; }
    part[2 * blockIdx.x] = ta;
    part[2 * blockIdx.x + 1] = tb;
  }
}

// Block-cooperative total of the nb two-component FP64 partials; the result
// is valid in thread 0.  Summation order is fixed, so it is deterministic.
__device__ __forceinline__ void total2(const double* part, int nb, double& ta, double& tb) {
  ta = 0.0; tb = 0.0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) { ta += part[2 * k]; tb += part[2 * k + 1]; }
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_xor_sync(0xffffffffu, ta, o);
    tb += __shfl_xor_sync(0xffffffffu, tb, o);
  }
  __shared__ double s[2][32];
  if ((threadIdx.x & 31) == 0) { s[0][threadIdx.x >> 5] = ta; s[1][threadIdx.x >> 5] = tb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    ta = 0.0; tb = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { ta += s[0][k]; tb += s[1][k]; }
  }
}

constexpr unsigned kElemBlocks = 8 * kNumSMs;   // grid of the element-wise passes

// setup_overdensity! data only (src/recon.jl:54-55): δ = (δ/mean - 1)/b.
__global__ void norm_data_kernel(float* __restrict__ d, size_t N, const double* __restrict__ part, int nb,
                                 float bias) {
  __shared__ float mean_s;
  double ta, tb;
  total2(part, nb, ta, tb);
  if (threadIdx.x == 0) mean_s = (float)(ta / (double)N);
  __syncthreads();
  const float mean = mean_s;
  auto norm = [&](float v) { return __fdiv_rn(__fsub_rn(__fdiv_rn(v, mean), 1.0f), bias); };
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t N4 = (uintptr_t)d % 16 == 0 ? N / 4 : 0;   // four cells per 16-byte access
  float4* d4 = reinterpret_cast<float4*>(d);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N4; e += stride) {
    const float4 v = d4[e];
    d4[e] = make_float4(norm(v.x), norm(v.y), norm(v.z), norm(v.w));
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += stride) d[e] = norm(d[e]);
}

// setup_overdensity! with randoms (src/recon.jl:78-85).
// With fpart, also the block's (Σδ, Σδ²) of the written mesh in FP64 (the
// norm and the mean the residual-driven solve needs next, without a pass of
// its own).
__global__ void norm_randoms_kernel(float* __restrict__ d, const float* __restrict__ r, size_t N,
                                    const double* __restrict__ part, int nb, float bias, float ran_min,
                                    float nrand, double* __restrict__ fpart) {
  __shared__ float al_s, thr_s;
  double ta, tb;
  total2(part, nb, ta, tb);
  if (threadIdx.x == 0) {
    al_s = (float)(ta / tb);
    thr_s = __fdiv_rn(__fmul_rn(ran_min, (float)tb), nrand);
  }
  __syncthreads();
  const float al = al_s, thr = thr_s;
  const float bal = __fmul_rn(bias, al);
  auto norm = [&](float dv0, float rv) {
    const float dv = __fsub_rn(dv0, __fmul_rn(al, rv));
    return rv > thr ? __fdiv_rn(dv, __fmul_rn(bal, rv)) : 0.0f;
  };
  // four cells per step (16-byte accesses); their sums in FP32, then FP64
  double s1 = 0.0, s2 = 0.0;
  const size_t N4 = ((uintptr_t)d % 16 == 0 && (uintptr_t)r % 16 == 0) ? N / 4 : 0;
  float4* d4 = reinterpret_cast<float4*>(d);
  const float4* r4 = reinterpret_cast<const float4*>(r);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N4; e += (size_t)gridDim.x * blockDim.x) {
    const float4 dv = d4[e], rv = r4[e];
    const float4 o = make_float4(norm(dv.x, rv.x), norm(dv.y, rv.y), norm(dv.z, rv.z), norm(dv.w, rv.w));
    d4[e] = o;
    if (fpart) {
      s1 += (double)((o.x + o.y) + (o.z + o.w));
      s2 += (double)((o.x * o.x + o.y * o.y) + (o.z * o.z + o.w * o.w));
    }
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    const float out = norm(d[e], r[e]);
    d[e] = out;
    s1 += (double)out;
    s2 += (double)out * (double)out;
  }
  if (!fpart) return;   // grid-uniform
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double red[2][32];
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = s1; red[1][threadIdx.x >> 5] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0.0, t2 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { t1 += red[0][k]; t2 += red[1][k]; }
    fpart[2 * blockIdx.x] = t1;
    fpart[2 * blockIdx.x + 1] = t2;
  }
}

constexpr int kRedBlocks = 2 * kNumSMs;

}  // namespace

int sum_mesh(baorec_ctx* ctx, const float* m, size_t N, double* out) {
  (sum2_partial_kernel<<<kRedBlocks, 256, 0, ctx->stream>>>(m, nullptr, N, ctx->dred), ::baorec::count_launch());
  CKLAUNCH();
  CK(cudaMemcpyAsync(ctx->hred, ctx->dred, 2 * kRedBlocks * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) s += ctx->hred[2 * k];
  *out = s;
  return BAOREC_OK;
}

__global__ void sumsq_partial_kernel(const float* __restrict__ a, size_t N, double* __restrict__ part) {
  double s = 0.0;
  const size_t N4 = ((uintptr_t)a % 16 == 0) ? N / 4 : 0;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N4; e += (size_t)gridDim.x * blockDim.x) {
    const float4 u = a4[e];
    s += (double)((u.x * u.x + u.y * u.y) + (u.z * u.z + u.w * u.w));
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    s += (double)a[e] * (double)a[e];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    part[blockIdx.x] = t;
  }
}

int sumsq_mesh(baorec_ctx* ctx, const float* m, size_t N, double* out) {
  (sumsq_partial_kernel<<<kRedBlocks, 256, 0, ctx->stream>>>(m, N, ctx->dred), ::baorec::count_launch());
  CKLAUNCH();
  CK(cudaMemcpyAsync(ctx->hred, ctx->dred, kRedBlocks * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) s += ctx->hred[k];
  *out = s;
  return BAOREC_OK;
}

namespace {
bool use_zpass(const baorec_ctx* ctx);
int smooth_zpass(baorec_ctx* ctx, float* mesh, int batch);
int zgrad_launch(baorec_ctx* ctx, const cufftComplex* src, int inv_lap);

// Batched 2-D transforms of `meshes` adjacent meshes' xy planes: the fused
// kernels of xyfft.cu for 256 x 256 planes (unless the autotuner chose
// cuFFT), else the cuFFT plans (which overwrite a C2R input).
int xy_forward(baorec_ctx* ctx, const float* in, cufftComplex* out, int meshes) {
  if (ctx->tune.xy && xy_fused_ok(ctx)) return xy_r2c(ctx, in, out, meshes * ctx->n3);
  for (int b = 0; b < meshes; ++b)
    CKFFT(cufftExecR2C(ctx->plan_r2c_xy, (cufftReal*)(in + (size_t)b * ctx->N), out + (size_t)b * ctx->Nk));
  return BAOREC_OK;
}
int xy_inverse(baorec_ctx* ctx, cufftComplex* in, float* out, int meshes) {
  if (ctx->tune.xy && xy_fused_ok(ctx)) return xy_c2r(ctx, in, out, meshes * ctx->n3);
  for (int b = 0; b < meshes; ++b)
    CKFFT(cufftExecC2R(ctx->plan_c2r_xy, in + (size_t)b * ctx->Nk, out + (size_t)b * ctx->N));
  return BAOREC_OK;
}
}  // namespace

int smooth(baorec_ctx* ctx, float* mesh) {
  if (use_zpass(ctx)) return smooth_zpass(ctx, mesh, 1);
  KGeom g = kgeom_of(ctx);
  float R = ctx->cfg.smoothing_radius;
  CKFFT(cufftExecR2C(ctx->plan_r2c, mesh, ctx->ck));
  (gauss_kernel<<<grid_for(ctx->Nk, 256), 256, 0, ctx->stream>>>(ctx->ck, ctx->Nk, 1, ctx->Nk, g, R * R), ::baorec::count_launch());
  CKLAUNCH();
  CKFFT(cufftExecC2R(ctx->plan_c2r, ctx->ck, mesh));
  return BAOREC_OK;
}

// Smooth the data and randoms meshes with one batched transform pair.
int smooth_pair(baorec_ctx* ctx, float* a, float* b) {
  if (b != a + ctx->N) {   // batched plans need the two meshes adjacent
    CKS(smooth(ctx, a));
    return smooth(ctx, b);
  }
  if (use_zpass(ctx)) return smooth_zpass(ctx, a, 2);
  KGeom g = kgeom_of(ctx);
  float R = ctx->cfg.smoothing_radius;
  CKFFT(cufftExecR2C(ctx->plan_r2c2, a, ctx->ck));
  (gauss_kernel<<<grid_for(ctx->Nk, 256), 256, 0, ctx->stream>>>(ctx->ck, ctx->Nk, 2, ctx->Nk, g, R * R), ::baorec::count_launch());
  CKLAUNCH();
  CKFFT(cufftExecC2R(ctx->plan_c2r2, ctx->ck, a));
  return BAOREC_OK;
}

int normalize_data(baorec_ctx* ctx, float* delta) {
  (sum2_partial_kernel<<<kRedBlocks, 256, 0, ctx->stream>>>(delta, nullptr, ctx->N, ctx->dred), ::baorec::count_launch());
  CKLAUNCH();
  (norm_data_kernel<<<kElemBlocks, 256, 0, ctx->stream>>>(delta, ctx->N, ctx->dred, kRedBlocks, ctx->cfg.bias), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int normalize_randoms(baorec_ctx* ctx, float* delta, const float* ran, int64_t nr, double* fpart) {
  static_assert(kElemBlocks == (unsigned)kFsumBlocks, "one (Σδ, Σδ²) pair per block of the normalisation");
  (sum2_partial_kernel<<<kRedBlocks, 256, 0, ctx->stream>>>(delta, ran, ctx->N, ctx->dred), ::baorec::count_launch());
  CKLAUNCH();
  (norm_randoms_kernel<<<kElemBlocks, 256, 0, ctx->stream>>>(
      delta, ran, ctx->N, ctx->dred, kRedBlocks, ctx->cfg.bias, ctx->cfg.ran_min, (float)nr, fpart), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int iterate(baorec_ctx* ctx, float* delta_r, const float* delta_s, int iter) {
  KGeom g = kgeom_of(ctx);
  const bool local = ctx->cfg.los_mode == BAOREC_LOS_LOCAL;
  float beta = ctx->cfg.beta;
  // factor = (1 + [i != j]) β, divided by (1 + β) on the first iteration
  float fac_diag = beta, fac_off = 2.0f * beta;
  if (iter == 1) { fac_diag = fac_diag / (1.0f + beta); fac_off = fac_off / (1.0f + beta); }
  int mask = 0, nprod = 6;
  float3 los = make_float3(ctx->cfg.los[0], ctx->cfg.los[1], ctx->cfg.los[2]);
  if (!local) {
    nprod = 0;
    for (int a = 0; a < 3; ++a)
      if (ctx->cfg.los[a] != 0.0f) { mask |= 1 << a; ++nprod; }
  }
  CKFFT(cufftExecR2C(ctx->plan_r2c, delta_r, ctx->ck));
  (hessian_kernel<<<grid_for(ctx->Nk, 256), 256, 0, ctx->stream>>>(ctx->ck, ctx->ck, ctx->Nk, g, local ? 1 : 0,
                                                                  los, nprod, mask), ::baorec::count_launch());
  CKLAUNCH();
  if (nprod == 6) {
    CKFFT(cufftExecC2R(ctx->plan_c2r6, ctx->ck, ctx->psi));
  } else {
    for (int m = 0; m < nprod; ++m)
      CKFFT(cufftExecC2R(ctx->plan_c2r, ctx->ck + (size_t)m * ctx->Nk, ctx->psi + (size_t)m * ctx->N));
  }
  (iterate_update_kernel<<<grid_for(ctx->N, 256), 256, 0, ctx->stream>>>(
      delta_r, delta_s, ctx->psi, ctx->N, ctx->n1, ctx->n2, ctx->xvec[0], ctx->xvec[1], ctx->xvec[2],
      local ? 1 : 0, nprod, fac_diag, fac_off), ::baorec::count_launch());
  CKLAUNCH();
  ctx->psi_valid = false;
  return BAOREC_OK;
}

// (x, y, z) planes -> one mesh of 4-float cells (x, y, z, 0), the read-out layout.
__global__ void interleave3_kernel(const float* __restrict__ p, float4* __restrict__ out, size_t N) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    out[e] = make_float4(p[e], p[e + N], p[e + 2 * N], 0.0f);
}

// Finite-difference gradient of φ (the reference's read_grad_cic,
// src/mas.jl:388-466, as a mesh): Ψ_a = (φ[c + e_a] - φ[c - e_a]) / cell2_a
// with periodic neighbours and cell2_a = T(2 L_a) / n_a as the reference
// spells it.  CIC-reading this mesh at a particle gives the reference's
// weighted sum of node differences divided by cell2 (up to FP32 rounding
// order).  One pass: read φ (neighbours from L1/L2), write 16 B per cell.
__global__ void fd_grad_kernel(const float* __restrict__ phi, float4* __restrict__ out, int n1, int n2, int n3,
                               float c2x, float c2y, float c2z) {
  const size_t N = (size_t)n1 * n2 * n3;
  const size_t plane = (size_t)n1 * n2;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % n1);
    const size_t r = e / n1;
    const int j = (int)(r % n2), k = (int)(r / n2);
    const size_t xp = i + 1 < n1 ? e + 1 : e + 1 - n1, xm = i > 0 ? e - 1 : e + n1 - 1;
    const size_t yp = j + 1 < n2 ? e + n1 : e + n1 - plane, ym = j > 0 ? e - n1 : e + plane - n1;
    const size_t zp = k + 1 < n3 ? e + plane : e + plane - N, zm = k > 0 ? e - plane : e + N - plane;
    out[e] = make_float4(__fdiv_rn(__fsub_rn(__ldg(phi + xp), __ldg(phi + xm)), c2x),
                         __fdiv_rn(__fsub_rn(__ldg(phi + yp), __ldg(phi + ym)), c2y),
                         __fdiv_rn(__fsub_rn(__ldg(phi + zp), __ldg(phi + zm)), c2z), 0.0f);
  }
}

// Ψ (iterative: i k δ_k / k²; multigrid: i k φ_k, or its finite-difference
// form) as an interleaved mesh at psi4[0, 4N); psi4[4N, 7N) holds the three
// planes on the way.
int displacement_meshes(baorec_ctx* ctx, const float* field, float* psi4) {
  if (ctx->cfg.method == BAOREC_MULTIGRID && ctx->grad_mode == BAOREC_GRADIENT_FD) {
    const int n[3] = {ctx->n1, ctx->n2, ctx->n3};
    float c2[3];
    for (int a = 0; a < 3; ++a) c2[a] = (2.0f * ctx->cfg.box_size[a]) / (float)n[a];   // FP32, as T(2L)/n
    (fd_grad_kernel<<<kElemBlocks, 256, 0, ctx->stream>>>(field, reinterpret_cast<float4*>(psi4), n[0], n[1], n[2],
                                                         c2[0], c2[1], c2[2]), ::baorec::count_launch());
    CKLAUNCH();
    return BAOREC_OK;
  }
  float* planes = psi4 + 4 * ctx->N;
  const int inv_lap = ctx->cfg.method == BAOREC_ITERATIVE ? 1 : 0;
  if (use_zpass(ctx)) {
    CKS(xy_forward(ctx, field, ctx->ck + 3 * ctx->Nk, 1));
    CKS(zgrad_launch(ctx, ctx->ck + 3 * ctx->Nk, inv_lap));
    CKS(xy_inverse(ctx, ctx->ck, planes, 3));
    (interleave3_kernel<<<kElemBlocks, 256, 0, ctx->stream>>>(planes, reinterpret_cast<float4*>(psi4), ctx->N), ::baorec::count_launch());
    CKLAUNCH();
    return BAOREC_OK;
  }
  KGeom g = kgeom_of(ctx);
  // cuFFT's R2C reads but does not modify its input
  CKFFT(cufftExecR2C(ctx->plan_r2c, (cufftReal*)field, ctx->ck + 3 * ctx->Nk));
  (grad_kernel<<<grid_for(ctx->Nk, 256), 256, 0, ctx->stream>>>(ctx->ck + 3 * ctx->Nk, ctx->ck, ctx->Nk, g, inv_lap), ::baorec::count_launch());
  CKLAUNCH();
  CKFFT(cufftExecC2R(ctx->plan_c2r3, ctx->ck, planes));
  (interleave3_kernel<<<kElemBlocks, 256, 0, ctx->stream>>>(planes, reinterpret_cast<float4*>(psi4), ctx->N), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

// ---- FFT preconditioner of the multigrid operator ------------------------
//
// With one line of sight l for the whole mesh the 19-point operator of the
// multigrid (src/multigrid.jl:14-135, first-derivative terms dropped) is a
// convolution, diagonal in Fourier space.  Per axis a with cell c_a and grid
// angle θ_a = 2π m_a / n_a:
//   A(k) = Σ_a (1 + β l_a²)/c_a² · 4 sin²(θ_a/2)
//        + Σ_{a<b} 2 β l_a l_b / (c_a c_b) · sin θ_a sin θ_b,
// positive except at k = 0.  For a fixed line of sight this is the exact
// inverse; for a radial one, l is the direction of the box centre (or the
// isotropic average l_a l_b -> δ_ab/3 when the observer sits inside the box).
bool mean_los(const baorec_ctx* c, double l[3]) {
  double Lmax = 0.0;
  for (int a = 0; a < 3; ++a) Lmax = std::max(Lmax, (double)c->cfg.box_size[a]);
  for (int a = 0; a < 3; ++a)
    l[a] = c->cfg.los_mode == BAOREC_LOS_GLOBAL ? (double)c->cfg.los[a]
                                                : (double)c->cfg.box_min[a] + 0.5 * (double)c->cfg.box_size[a];
  const double nl = sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
  const bool iso = !(nl > 0.0) || (c->cfg.los_mode == BAOREC_LOS_LOCAL && nl < 0.25 * Lmax);
  for (int a = 0; a < 3; ++a) l[a] = iso ? 0.0 : l[a] / nl;
  return !iso;
}

namespace {

struct SGeom {
  int n1, n2, n3, n1h;
  float diag[3];   // (1 + β l_a²) / c_a², times 4
  float cross[3];  // 2 β l_a l_b / (c_a c_b) for ab = xy, xz, yz
  float invN;
};

SGeom sgeom_of(const baorec_ctx* c) {
  SGeom g;
  g.n1 = c->n1; g.n2 = c->n2; g.n3 = c->n3; g.n1h = c->n1h;
  const int n[3] = {c->n1, c->n2, c->n3};
  double cell[3], l[3];
  for (int a = 0; a < 3; ++a) cell[a] = (double)(c->cfg.box_size[a] / (float)n[a]);
  const double beta = c->cfg.beta;
  const bool iso = !mean_los(c, l);
  for (int a = 0; a < 3; ++a) {
    const double lp = iso ? 1.0 / 3.0 : l[a] * l[a];
    g.diag[a] = (float)(4.0 * (1.0 + beta * lp) / (cell[a] * cell[a]));
  }
  g.cross[0] = (float)(2.0 * beta * l[0] * l[1] / (cell[0] * cell[1]));
  g.cross[1] = (float)(2.0 * beta * l[0] * l[2] / (cell[0] * cell[2]));
  g.cross[2] = (float)(2.0 * beta * l[1] * l[2] / (cell[1] * cell[2]));
  g.invN = (float)(1.0 / (double)c->N);
  return g;
}

// Per-axis tables sin²(π m/n) and sin(2π m/n) (m the signed frequency):
// tab = hx2[n1h] | sx[n1h] | hy2[n2] | sy[n2] | hz2[n3] | sz[n3].  Each block
// holds `rpb` k-space rows (fixed j, k) of n1h threads each, x along the threads.
__global__ void spectral_inverse_kernel(cufftComplex* __restrict__ a, SGeom g, const float* __restrict__ tab,
                                        int rpb) {
  const float* hx2 = tab;
  const float* sx = hx2 + g.n1h;
  const float* hy2 = sx + g.n1h;
  const float* sy = hy2 + g.n2;
  const float* hz2 = sy + g.n2;
  const float* sz = hz2 + g.n3;
  const int rows = g.n2 * g.n3;   // 32-bit row arithmetic (n2 n3 < 2^31)
  const int slot = (int)threadIdx.x / g.n1h, i = (int)threadIdx.x - slot * g.n1h;
  if (slot >= rpb) return;
  const float hxi = __ldg(hx2 + i), sxi = __ldg(sx + i);
  for (int row = (int)blockIdx.x * rpb + slot; row < rows; row += (int)gridDim.x * rpb) {
    const int k = row / g.n2, j = row - k * g.n2;
    const float syj = __ldg(sy + j), szk = __ldg(sz + k);
    const float A = g.diag[1] * __ldg(hy2 + j) + g.diag[2] * __ldg(hz2 + k) + g.cross[2] * syj * szk +
                    g.diag[0] * hxi + (g.cross[0] * syj + g.cross[1] * szk) * sxi;
    // one reciprocal per mode (a preconditioner); the k = 0 mode is dropped
    const float s = (row == 0 && i == 0) ? 0.0f : g.invN * __frcp_rn(A);
    cufftComplex* e = a + (size_t)row * g.n1h + i;
    cufftComplex v = *e;
    v.x *= s; v.y *= s;
    *e = v;
  }
}

// ---- the preconditioner's z pass (n3 = 256) --------------------------------
// After batched 2-D R2C transforms of the xy planes, a column (kx, ky) of the
// spectrum holds its 256 z planes at a stride of one plane.  One kernel
// transforms each column along z (four-step: 256 = 16 x 16, two 16-point
// DFTs in registers with the 256-point twiddles between them, one shared-
// memory exchange), multiplies by the preconditioner S⁻¹(k) and transforms
// back the same way, so the multiply costs no pass of its own and the 3-D
// transforms' z passes are replaced by one read and one write of the spectrum.
constexpr int kZLen = 256;   // z planes the z pass transforms (16 x 16)
constexpr int kZCols = 16;   // columns per block; thread (column c, row r) = (t & 15, t >> 4)

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulf_conj(float2 a, float2 b) {   // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// 4-point DFT in place, natural order; INV uses e^{+2πi/4}.
template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = make_float2(a0.x + a2.x, a0.y + a2.y), t1 = make_float2(a0.x - a2.x, a0.y - a2.y);
  const float2 t2 = make_float2(a1.x + a3.x, a1.y + a3.y), d = make_float2(a1.x - a3.x, a1.y - a3.y);
  const float2 t3 = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);   // d · (±i)
  a0 = make_float2(t0.x + t2.x, t0.y + t2.y);
  a2 = make_float2(t0.x - t2.x, t0.y - t2.y);
  a1 = make_float2(t1.x + t3.x, t1.y + t3.y);
  a3 = make_float2(t1.x - t3.x, t1.y - t3.y);
}

// e^{∓2πi m/16} for the products m = b c (b, c in 1..3) of the 4 x 4 split.
template <bool INV>
__device__ __forceinline__ float2 w16(int m) {
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

// 16-point DFT in registers, natural order in and out:
// v[k] <- Σ_n v[n] e^{∓2πi nk/16}; n = 4a + b, k = c + 4d.
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&v)[16]) {
#pragma unroll
  for (int b = 0; b < 4; ++b) dft4<INV>(v[b], v[4 + b], v[8 + b], v[12 + b]);   // v[4c + b] = y_b[c]
#pragma unroll
  for (int b = 1; b < 4; ++b)
#pragma unroll
    for (int c = 1; c < 4; ++c) v[4 * c + b] = cmulf(v[4 * c + b], w16<INV>(b * c));
#pragma unroll
  for (int c = 0; c < 4; ++c) dft4<INV>(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);   // v[4c + d] = X[c + 4d]
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int d = c + 1; d < 4; ++d) {
      const float2 q = v[4 * c + d];
      v[4 * c + d] = v[4 * d + c];
      v[4 * d + c] = q;
    }
}

// a: n3 = 256 planes of ncols = n1h * n2 modes (column i + n1h j), transformed
// over x and y; tw: e^{-2πi m/256}.  In place: a <- IFFT_z(S⁻¹ FFT_z(a)), with
// S⁻¹ and the 1/N of the unnormalised transforms as spectral_inverse_kernel.
// Per-mode multipliers of the z pass.  setup(kzt, t) fills the block's
// per-kz table (t = kz), column(col) the per-column terms, factor(kzt, k)
// gives the multiplier of mode (column, kz = k).
struct PrecondMul {   // S⁻¹(k)/N of the FFT preconditioner (spectral_inverse_kernel)
  SGeom g;
  const float* tab;
  float c0, c1;
  int cc;
  __device__ __forceinline__ void setup(float2* kzt, int t) const {
    const float* hz2 = tab + 2 * g.n1h + 2 * g.n2;
    kzt[t] = make_float2(g.diag[2] * __ldg(hz2 + t), __ldg(hz2 + g.n3 + t));   // diag_z sin²(θz/2), sin θz
  }
  // S(k) = c0 + diag_z sin²(θz/2) + c1 sin θz with the column's x and y terms in c0, c1
  __device__ __forceinline__ void column(int col) {
    cc = col;
    const int j = col / g.n1h, i = col - j * g.n1h;
    const float* sx = tab + g.n1h;
    const float* hy2 = sx + g.n1h;
    const float* sy = hy2 + g.n2;
    const float hxi = __ldg(tab + i), sxi = __ldg(sx + i), hyj = __ldg(hy2 + j), syj = __ldg(sy + j);
    c0 = g.diag[1] * hyj + g.diag[0] * hxi + g.cross[0] * syj * sxi;
    c1 = g.cross[2] * syj + g.cross[1] * sxi;
  }
  // one approximate reciprocal per mode (a preconditioner); the k = 0 mode is dropped
  __device__ __forceinline__ float factor(const float2* kzt, int k) const {
    const float2 z = kzt[k];
    return (k == 0 && cc == 0) ? 0.0f : __fdividef(g.invN, c0 + fmaf(z.y, c1, z.x));
  }
};

struct GaussMul {   // smooth!: exp(-0.5 R² k²)/N, k² and the factor as gauss_kernel evaluates them
  KGeom g;
  float R2;
  float c0;
  __device__ __forceinline__ void setup(float2* kzt, int t) const {
    float kx, ky, kz;
    kvals(g, 0, 0, t, kx, ky, kz);
    kzt[t] = make_float2(__fmul_rn(kz, kz), 0.0f);
  }
  __device__ __forceinline__ void column(int col) {
    const int j = col / g.n1h, i = col - j * g.n1h;
    float kx, ky, kz;
    kvals(g, i, j, 0, kx, ky, kz);
    c0 = __fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky));
  }
  __device__ __forceinline__ float factor(const float2* kzt, int k) const {
    return expf(-0.5f * R2 * __fadd_rn(c0, kzt[k].x)) * g.invN;
  }
};

// a (+ blockIdx.y spectra of n3 = 256 planes each): planes of ncols = n1h n2
// modes (column i + n1h j), transformed over x and y; tw: e^{-2πi m/256}.
// In place: a <- IFFT_z(M(k) FFT_z(a)) for the multiplier M.
template <int MINB, class M>
__global__ void __launch_bounds__(256, MINB) zpass_kernel(cufftComplex* __restrict__ a, M m,
                                                          const float2* __restrict__ tw, int ncols) {
  __shared__ float2 s[kZCols][kZLen + 1];
  __shared__ float2 w[kZLen];
  __shared__ float2 kzt[kZLen];
  const int t = threadIdx.x, cl = t & (kZCols - 1), r = t >> 4;
  const int col = (int)blockIdx.x * kZCols + cl;
  const bool ok = col < ncols;
  w[t] = __ldg(tw + t);
  m.setup(kzt, t);
  const size_t plane = (size_t)ncols;
  float2* base = reinterpret_cast<float2*>(a) + (size_t)blockIdx.y * plane * kZLen + (ok ? col : 0);
  float2 v[16];
  // x[16 n1 + r], n1 = 0..15 -> Σ_n1 x[16 n1 + r] W16^{n1 k1}, times W256^{r k1}
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) v[n1] = ok ? base[(size_t)(16 * n1 + r) * plane] : make_float2(0.0f, 0.0f);
  dft16<false>(v);
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) s[cl][16 * k1 + r] = cmulf(v[k1], w[r * k1]);
  __syncthreads();
  // row k1 = r: X[r + 16 k2] = Σ_n2 Y[r][n2] W16^{n2 k2}
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) v[n2] = s[cl][16 * r + n2];
  dft16<false>(v);
  m.column(ok ? col : 0);
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    const float sc = m.factor(kzt, r + 16 * k2);
    v[k2].x *= sc;
    v[k2].y *= sc;
  }
  // inverse: Z[r][n2] = W256^{-n2 r} Σ_k2 X[r + 16 k2] W16^{-n2 k2}
  dft16<true>(v);
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) s[cl][16 * r + n2] = cmulf_conj(v[n2], w[n2 * r]);
  __syncthreads();
  // x[16 n1 + r] = Σ_k1 Z[k1][r] W16^{-n1 k1}
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) v[k1] = s[cl][16 * k1 + r];
  dft16<true>(v);
  if (ok) {
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) base[(size_t)(16 * n1 + r) * plane] = v[n1];
  }
}

// Displacement spectra through the z pass: one xy-transformed spectrum in
// (a, 256 planes), three out (out + c Nk, c = 0..2): forward z transform,
// then per component the multiply of grad_kernel (i k_c / N, over k² for the
// iterative method) and the inverse z transform.  The forward spectrum stays
// in shared memory (each thread reads back its own values) between components;
// dynamic shared memory: exchange 16 x 257, spectrum 256 x 16, twiddles, kz.
constexpr size_t kZGradSmem = sizeof(float2) * (kZCols * (kZLen + 1) + kZLen * kZCols + kZLen) + sizeof(float) * kZLen;

template <int MINB>
__global__ void __launch_bounds__(256, MINB) zgrad_kernel(const cufftComplex* __restrict__ a,
                                                          cufftComplex* __restrict__ out, KGeom g, int inv_lap,
                                                          const float2* __restrict__ tw, int ncols) {
  extern __shared__ __align__(16) float2 zg_smem[];
  float2 (*s)[kZLen + 1] = reinterpret_cast<float2 (*)[kZLen + 1]>(zg_smem);
  float2 (*xs)[kZCols] = reinterpret_cast<float2 (*)[kZCols]>(zg_smem + kZCols * (kZLen + 1));   // [kz][column]
  float2* w = zg_smem + kZCols * (kZLen + 1) + kZLen * kZCols;
  float* kzt = reinterpret_cast<float*>(w + kZLen);
  const int t = threadIdx.x, cl = t & (kZCols - 1), r = t >> 4;
  const int col = (int)blockIdx.x * kZCols + cl;
  const bool ok = col < ncols;
  w[t] = __ldg(tw + t);
  {
    float kx, ky, kz;
    kvals(g, 0, 0, t, kx, ky, kz);
    kzt[t] = kz;
  }
  const size_t plane = (size_t)ncols, nk = plane * kZLen;
  const float2* src = reinterpret_cast<const float2*>(a) + (ok ? col : 0);
  float2 v[16];
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) v[n1] = ok ? src[(size_t)(16 * n1 + r) * plane] : make_float2(0.0f, 0.0f);
  dft16<false>(v);
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) s[cl][16 * k1 + r] = cmulf(v[k1], w[r * k1]);
  __syncthreads();
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) v[n2] = s[cl][16 * r + n2];
  dft16<false>(v);   // v[k2] = X[kz = r + 16 k2]
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) xs[16 * r + k2][cl] = v[k2];
  float kxy[2];
  bool real_plane, jnyq;   // column in the kx = 0 / n1/2 planes; ky index Nyquist
  {
    const int cc = ok ? col : 0;
    const int j = cc / g.n1h, i = cc - j * g.n1h;
    float kz;
    kvals(g, i, j, 0, kxy[0], kxy[1], kz);
    real_plane = in_real_plane(g, i);
    jnyq = j == g.nyq[1];
  }
  const float c0 = __fadd_rn(__fmul_rn(kxy[0], kxy[0]), __fmul_rn(kxy[1], kxy[1]));
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      const float kz = kzt[r + 16 * k2];
      float kc = c == 0 ? kxy[0] : (c == 1 ? kxy[1] : kz);
      // the Hermitian part in the kx = 0 / n1/2 planes (see drop_odd)
      if (real_plane && (c == 0 || (c == 1 && jnyq) || (c == 2 && r + 16 * k2 == g.nyq[2]))) kc = 0.0f;
      const float2 d = xs[16 * r + k2][cl];
      // (i k) (re + i im) = (-k im, k re), as grad_kernel
      float re = -__fmul_rn(kc, d.y), im = __fmul_rn(kc, d.x);
      if (inv_lap) {
        const float k2v = __fadd_rn(c0, __fmul_rn(kz, kz));
        if (k2v > 0.0f) { re = __fdiv_rn(re, k2v); im = __fdiv_rn(im, k2v); }
        else { re = 0.0f; im = 0.0f; }
      }
      v[k2] = make_float2(re * g.invN, im * g.invN);
    }
    dft16<true>(v);
    __syncthreads();   // the previous component's reads of s are done
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) s[cl][16 * r + n2] = cmulf_conj(v[n2], w[n2 * r]);
    __syncthreads();
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) v[k1] = s[cl][16 * k1 + r];
    dft16<true>(v);
    if (ok) {
      float2* dst = reinterpret_cast<float2*>(out) + (size_t)c * nk + col;
#pragma unroll
      for (int n1 = 0; n1 < 16; ++n1) dst[(size_t)(16 * n1 + r) * plane] = v[n1];
    }
  }
}

// Batched 2-D transforms of the n3 xy planes (R2C and C2R) for the z pass,
// built at the first correction; any failure leaves the 3-D transforms in use.
bool xy_plans(baorec_ctx* ctx) {
  if (ctx->xy_state != 0) return ctx->xy_state == 1;
  ctx->xy_state = -1;
  long long dims[2] = {ctx->n2, ctx->n1};
  const long long nr = (long long)ctx->n1 * ctx->n2, nc = (long long)ctx->n1h * ctx->n2;
  cufftHandle p[2] = {0, 0};
  size_t w[2] = {0, 0};
  bool ok = cufftCreate(&p[0]) == CUFFT_SUCCESS && cufftCreate(&p[1]) == CUFFT_SUCCESS &&
            cufftSetAutoAllocation(p[0], 0) == CUFFT_SUCCESS && cufftSetAutoAllocation(p[1], 0) == CUFFT_SUCCESS &&
            cufftMakePlanMany64(p[0], 2, dims, nullptr, 1, nr, nullptr, 1, nc, CUFFT_R2C, ctx->n3, &w[0]) ==
                CUFFT_SUCCESS &&
            cufftMakePlanMany64(p[1], 2, dims, nullptr, 1, nc, nullptr, 1, nr, CUFFT_C2R, ctx->n3, &w[1]) ==
                CUFFT_SUCCESS;
  const size_t need = std::max(w[0], w[1]);
  if (ok && need > ctx->fft_work_bytes) {
    ok = cudaMalloc(&ctx->xy_work, need) == cudaSuccess;
    if (!ok) cudaGetLastError();
  }
  void* work = ctx->xy_work ? ctx->xy_work : ctx->fft_work;
  for (int q = 0; q < 2 && ok; ++q)
    ok = cufftSetWorkArea(p[q], work) == CUFFT_SUCCESS && cufftSetStream(p[q], ctx->stream) == CUFFT_SUCCESS;
  if (!ok) {
    for (int q = 0; q < 2; ++q)
      if (p[q]) cufftDestroy(p[q]);
    return false;
  }
  ctx->plan_r2c_xy = p[0];
  ctx->plan_c2r_xy = p[1];
  ctx->xy_state = 1;
  return true;
}

int spectral_tables(baorec_ctx* ctx);
}  // namespace

// One batched xy transform of the finest mesh (the measurement hook): r ->
// the spectrum buffer, or (inverse) the spectrum buffer -> out, by the
// autotuner's current choice between the fused kernels and cuFFT.
int xy_profile(baorec_ctx* ctx, int inverse, const float* r, float* out) {
  if (ctx->n3 != kZLen || !ctx->ck || !xy_plans(ctx))
    return set_error(ctx, BAOREC_ERR_ARG, "profile_kernel: no batched xy transforms for this mesh");
  return inverse ? xy_inverse(ctx, ctx->ck, out, 1) : xy_forward(ctx, r, ctx->ck, 1);
}

namespace {
// z pass over `batch` spectra of n3 = 256 planes at a, multiplier m; form 2
// caps the registers for three resident blocks per SM instead of two.
template <class M>
int zpass_launch(baorec_ctx* ctx, cufftComplex* a, const M& m, int batch) {
  CKS(spectral_tables(ctx));
  const int ncols = ctx->n1h * ctx->n2;
  const float2* tw = reinterpret_cast<const float2*>(ctx->stab + 2 * (ctx->n1h + ctx->n2 + ctx->n3));
  auto k = ctx->tune.zpass == 2 ? zpass_kernel<3, M> : zpass_kernel<1, M>;
  (k<<<dim3((ncols + kZCols - 1) / kZCols, batch), 256, 0, ctx->stream>>>(a, m, tw, ncols), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

// True when smoothing and the preconditioner go through xy transforms and the
// z pass: 256 z planes, the form enabled, and the plans built (eagerly at
// context creation, so a graph capture never builds them).
bool use_zpass(const baorec_ctx* ctx) { return ctx->n3 == kZLen && ctx->tune.zpass != 0 && ctx->xy_state == 1; }

// smooth! of `batch` adjacent meshes through the z pass.
int smooth_zpass(baorec_ctx* ctx, float* mesh, int batch) {
  GaussMul m;
  m.g = kgeom_of(ctx);
  m.R2 = ctx->cfg.smoothing_radius * ctx->cfg.smoothing_radius;
  CKS(xy_forward(ctx, mesh, ctx->ck, batch));
  CKS(zpass_launch(ctx, ctx->ck, m, batch));
  CKS(xy_inverse(ctx, ctx->ck, mesh, batch));
  return BAOREC_OK;
}

// Ψ spectra (three, at ctx->ck) of the xy-transformed field spectrum at src.
int zgrad_launch(baorec_ctx* ctx, const cufftComplex* src, int inv_lap) {
  const int ncols = ctx->n1h * ctx->n2;
  const float2* tw = reinterpret_cast<const float2*>(ctx->stab + 2 * (ctx->n1h + ctx->n2 + ctx->n3));
  auto k = ctx->tune.zpass == 2 ? zgrad_kernel<3> : zgrad_kernel<1>;
  (k<<<(ncols + kZCols - 1) / kZCols, 256, kZGradSmem, ctx->stream>>>(src, ctx->ck, kgeom_of(ctx), inv_lap, tw, ncols), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int spectral_tables(baorec_ctx* ctx) {
  if (ctx->stab) return BAOREC_OK;
  const int n[3] = {ctx->n1, ctx->n2, ctx->n3};
  const int len[3] = {ctx->n1h, ctx->n2, ctx->n3};
  std::vector<float> t;
  for (int a = 0; a < 3; ++a) {
    std::vector<float> h(len[a]), sn(len[a]);
    for (int m = 0; m < len[a]; ++m) {
      const int f = (a == 0 || m < (n[a] + 1) / 2) ? m : m - n[a];
      const double th = 2.0 * 3.14159265358979323846 * (double)f / (double)n[a];
      const double hh = sin(0.5 * th);
      h[m] = (float)(hh * hh);
      sn[m] = (float)sin(th);
    }
    t.insert(t.end(), h.begin(), h.end());
    t.insert(t.end(), sn.begin(), sn.end());
  }
  // e^{-2πi m/256}, m = 0..255, for the four-step z transform (8-byte aligned:
  // the per-axis tables above hold an even number of floats)
  for (int m = 0; m < kZLen; ++m) {
    const double th = 2.0 * 3.14159265358979323846 * (double)m / (double)kZLen;
    t.push_back((float)cos(th));
    t.push_back((float)-sin(th));
  }
  CK(cudaMalloc(&ctx->stab, t.size() * sizeof(float)));
  CK(cudaMemcpy(ctx->stab, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice));
  return BAOREC_OK;
}

// Parameters of the LTO load callback (the same layout as in lto/spectral_cb.cu).
struct SpecCallbackInfo {
  const float* tab;
  unsigned long long nk;
  int n1h, n2, n3;
  float diag[3], cross[3];
  float invN;
};

// written by a kernel, so the update is ordered on the stream like the transforms
__global__ void set_callback_info_kernel(SpecCallbackInfo* dst, SpecCallbackInfo v) { *dst = v; }

// The inverse transform of the preconditioner with the k-space multiply as a
// cuFFT load callback.  Any failure (a cuFFT without LTO callbacks, a JIT
// link error) leaves the separate multiply kernel in use and notes why.
// one attempt with one IR target; on failure *stage/*res say where
bool try_callback_plan(baorec_ctx* ctx, const char* symbol, const unsigned char* ir, size_t ir_size, cufftHandle* out,
                       size_t* work, const char** stage, cufftResult* res) {
  cufftHandle p = 0;
  long long dims[3] = {ctx->n3, ctx->n2, ctx->n1};
  void* info[1] = {ctx->spec_cb};
  *res = CUFFT_SUCCESS;
  *stage = "cufftCreate";
  if ((*res = cufftCreate(&p)) != CUFFT_SUCCESS) return false;
  *stage = "cufftXtSetJITCallback";
  if ((*res = cufftXtSetJITCallback(p, symbol, ir, ir_size, CUFFT_CB_LD_COMPLEX, info)) == CUFFT_SUCCESS) {
    *stage = "cufftSetAutoAllocation";
    if ((*res = cufftSetAutoAllocation(p, 0)) == CUFFT_SUCCESS) {
      // 32-bit plan interface (the sizes of one spectrum fit)
      int n[3] = {(int)dims[0], (int)dims[1], (int)dims[2]};
      *stage = "cufftMakePlanMany";
      if ((*res = cufftMakePlanMany(p, 3, n, nullptr, 1, (int)ctx->Nk, nullptr, 1, (int)ctx->N, CUFFT_C2R, 1,
                                    work)) == CUFFT_SUCCESS) {
        *out = p;
        return true;
      }
    }
  }
  cufftDestroy(p);
  return false;
}

// The inverse transform of the preconditioner with the k-space multiply as a
// cuFFT load callback.  Any failure (a cuFFT without LTO callbacks, a JIT
// link error) leaves the separate multiply kernel in use and notes why.
void spectral_callback_plan(baorec_ctx* ctx) {
  ctx->spec_cb_state = -1;
  if (ctx->Nk >= (1ull << 32)) {
    snprintf(ctx->spec_cb_note, sizeof(ctx->spec_cb_note), "spectrum above 2^32 modes");
    return;
  }
  if (!ctx->spec_cb && cudaMalloc(&ctx->spec_cb, sizeof(SpecCallbackInfo)) != cudaSuccess) {
    cudaGetLastError();
    snprintf(ctx->spec_cb_note, sizeof(ctx->spec_cb_note), "callback parameters: cudaMalloc failed");
    return;
  }
  const unsigned char* irs[2] = {baorec_lto_spectral_cb_a, baorec_lto_spectral_cb_p};
  const size_t sizes[2] = {baorec_lto_spectral_cb_a_size, baorec_lto_spectral_cb_p_size};
  const char* names[2] = {"sm_103a", "sm_103"};
  const char* symbols[2] = {"baorec_spectral_load", "_Z21baorec_spectral_load2PvyS_S_"};
  char why[4][48] = {{0}, {0}, {0}, {0}};
  for (int t = 0; t < 4; ++t) {
    const int v = t / 2, sy = t % 2;
    cufftHandle p = 0;
    size_t w = 0;
    const char* stage = "";
    cufftResult r = CUFFT_SUCCESS;
    if (!try_callback_plan(ctx, symbols[sy], irs[v], sizes[v], &p, &w, &stage, &r)) {
      snprintf(why[t], sizeof(why[t]), "%s/%d: %s %d", names[v], sy, stage + 4, (int)r);
      continue;
    }
    if (w > ctx->fft_work_bytes && !ctx->spec_work && cudaMalloc(&ctx->spec_work, w) != cudaSuccess) {
      cudaGetLastError();
      cufftDestroy(p);
      snprintf(why[t], sizeof(why[t]), "%s: work area", names[v]);
      continue;
    }
    if (cufftSetWorkArea(p, ctx->spec_work ? ctx->spec_work : ctx->fft_work) != CUFFT_SUCCESS ||
        cufftSetStream(p, ctx->stream) != CUFFT_SUCCESS) {
      cufftDestroy(p);
      snprintf(why[t], sizeof(why[t]), "%s: work area / stream", names[v]);
      continue;
    }
    ctx->plan_c2r_spec = p;
    ctx->spec_cb_state = 1;
    snprintf(ctx->spec_cb_note, sizeof(ctx->spec_cb_note), "k-space multiply fused as a cuFFT LTO load callback (%s IR)",
             names[v]);
    return;
  }
  snprintf(ctx->spec_cb_note, sizeof(ctx->spec_cb_note), "callback plan unavailable (%s; %s; %s; %s)", why[0], why[1],
           why[2], why[3]);
}

}  // namespace

// The z pass's batched xy plans and tables for meshes of 256 z planes, built
// when the context is created (a plan failure leaves the 3-D transforms in use).
int zpass_prepare(baorec_ctx* ctx) {
  if (ctx->n3 != kZLen) return BAOREC_OK;
  CKS(spectral_tables(ctx));   // the twiddles and sine tables, before any graph capture
  xy_plans(ctx);
  CKS(xy_fused_prepare(ctx));
  CK(cudaFuncSetAttribute(zgrad_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZGradSmem));
  CK(cudaFuncSetAttribute(zgrad_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZGradSmem));
  return BAOREC_OK;
}

// e = S⁻¹ r (zero mean), S the operator with the box's mean line of sight.
// r is read only; e may not alias r.
int spectral_correction(baorec_ctx* ctx, const float* r, float* e) {
  SGeom g = sgeom_of(ctx);
  CKS(spectral_tables(ctx));
  if (ctx->spec_cb_state == 0) spectral_callback_plan(ctx);
  if (ctx->spec_cb_state != 1 && use_zpass(ctx)) {
    const int ncols = ctx->n1h * ctx->n2;
    CKS(xy_forward(ctx, r, ctx->ck, 1));
    PrecondMul m;
    m.g = g;
    m.tab = ctx->stab;
    CKS(zpass_launch(ctx, ctx->ck, m, 1));
    CKS(xy_inverse(ctx, ctx->ck, e, 1));
    return BAOREC_OK;
  }
  CKFFT(cufftExecR2C(ctx->plan_r2c, (cufftReal*)r, ctx->ck));
  if (ctx->spec_cb_state == 1) {
    SpecCallbackInfo info;
    info.tab = ctx->stab;
    info.nk = ctx->Nk;
    info.n1h = g.n1h; info.n2 = g.n2; info.n3 = g.n3;
    for (int a = 0; a < 3; ++a) { info.diag[a] = g.diag[a]; info.cross[a] = g.cross[a]; }
    info.invN = g.invN;
    (set_callback_info_kernel<<<1, 1, 0, ctx->stream>>>((SpecCallbackInfo*)ctx->spec_cb, info), ::baorec::count_launch());
    CKLAUNCH();
    CKFFT(cufftExecC2R(ctx->plan_c2r_spec, ctx->ck, e));
    return BAOREC_OK;
  }
  // rows of n1h threads per block (n1h <= 1024, as the mesh-size limit guarantees up to n1 = 2046)
  if (ctx->n1h > 1024) return set_error(ctx, BAOREC_ERR_ARG, "FFT start: n1 above 2046");
  const int rpb = std::max(1, 1024 / ctx->n1h);
  const size_t rows = (size_t)ctx->n2 * ctx->n3;
  const unsigned blocks = (unsigned)std::min<size_t>((rows + rpb - 1) / rpb, 16 * kNumSMs);
  (spectral_inverse_kernel<<<blocks, rpb * ctx->n1h, 0, ctx->stream>>>(ctx->ck, g, ctx->stab, rpb), ::baorec::count_launch());
  CKLAUNCH();
  CKFFT(cufftExecC2R(ctx->plan_c2r, ctx->ck, e));
  return BAOREC_OK;
}

}  // namespace baorec

extern "C" int baorec_smooth(baorec_ctx* ctx, float* mesh) {
  if (!ctx || !mesh) return BAOREC_ERR_ARG;
  CKS(baorec::smooth(ctx, mesh));
  return baorec::finish(ctx, 0);
}

extern "C" int baorec_fft_callbacks(const baorec_ctx* ctx, const char** note) {
  if (!ctx) return -1;
  if (note) *note = ctx->spec_cb_note;
  return ctx->spec_cb_state;
}

extern "C" int baorec_set_fft_callbacks(baorec_ctx* ctx, int enable) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!enable) {
    ctx->spec_cb_state = -1;
    snprintf(ctx->spec_cb_note, sizeof(ctx->spec_cb_note), "callbacks disabled by the caller");
  } else if (ctx->plan_c2r_spec) {
    ctx->spec_cb_state = 1;
  } else {
    ctx->spec_cb_state = 0;   // build the callback plan at the next correction
  }
  return BAOREC_OK;
}
