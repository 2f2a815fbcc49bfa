// Learned initial guess for the multigrid solve (no reference counterpart).
//
// The network predicts the error of the FFT start: with S the operator for
// the box's mean line of sight, φ_s = S⁻¹ f, the converged potential is
// φ ≈ φ_s + s·net(features), s = rms(φ_s).  Features per cell (BF16, 8
// channels): f c²/s, φ_s/s, (f - A φ_s) c²/s, r̂ - l (3), 0, 0; r̂ is the
// radial direction of the cell centre, l the mean line of sight.
//
// The network is a 3-level U-Net (levels n, n/2, n/4 with 16/32/64 channels,
// 3x3x3 convolutions, strided 2x2x2 down/up-sampling, skip connections by
// channel concatenation, ReLU, a 1x1x1 linear head; 431,969 parameters).
// Training runs on the device: synthetic lognormal fields in the survey
// window of random sub-boxes, targets from the residual-driven solver, the
// mean squared error of the potential or of its 7-point Laplacian as loss,
// Adam.  Parameters are FP32 masters; the convolutions read BF16
// copies in tensor-core fragment order.
#include <math.h>

#include <algorithm>
#include <new>
#include <random>
#include <vector>

#include "common.cuh"
#include "guess.cuh"

namespace baorec {

using guess::C3;
using guess::DN;
using guess::UP;
typedef __nv_bfloat16 bf16;

namespace {

enum TId { T_X, T_A0, T_CAT0, T_B0, T_C0, T_A1, T_B1, T_CAT1, T_D1, T_E1, T_A2, T_B2, T_C2, T_COUNT };
struct TensorDef { int level, ch; };
const TensorDef kTensors[T_COUNT] = {{0, 8},  {0, 16}, {0, 32}, {0, 16}, {0, 16}, {1, 32}, {1, 32},
                                     {1, 64}, {1, 32}, {1, 32}, {2, 64}, {2, 64}, {2, 64}};

struct LayerDef {
  int kind, cin, cout;
  int in_t, in_off, out_t, out_off;
  bool acc_grad;   // the backward-data output adds to a gradient written earlier
};
constexpr int kLayers = 14;
const LayerDef kNet[kLayers] = {
    {C3, 8, 16, T_X, 0, T_A0, 0, false},       {C3, 16, 16, T_A0, 0, T_CAT0, 16, false},
    {DN, 16, 32, T_CAT0, 16, T_A1, 0, true},   {C3, 32, 32, T_A1, 0, T_B1, 0, false},
    {C3, 32, 32, T_B1, 0, T_CAT1, 32, false},  {DN, 32, 64, T_CAT1, 32, T_A2, 0, true},
    {C3, 64, 64, T_A2, 0, T_B2, 0, false},     {C3, 64, 64, T_B2, 0, T_C2, 0, false},
    {UP, 64, 32, T_C2, 0, T_CAT1, 0, false},   {C3, 64, 32, T_CAT1, 0, T_D1, 0, false},
    {C3, 32, 32, T_D1, 0, T_E1, 0, false},     {UP, 32, 16, T_E1, 0, T_CAT0, 0, false},
    {C3, 32, 16, T_CAT0, 0, T_B0, 0, false},   {C3, 16, 16, T_B0, 0, T_C0, 0, false}};
constexpr int kHeadIn = 16;
constexpr int kFeat = 8;

struct ParamLayout {
  size_t w[kLayers + 1], b[kLayers + 1], total;
  ParamLayout() {
    size_t o = 0;
    for (int l = 0; l < kLayers; ++l) {
      w[l] = o;
      o += (size_t)guess::taps_of(kNet[l].kind) * kNet[l].cin * kNet[l].cout;
      b[l] = o;
      o += kNet[l].cout;
    }
    w[kLayers] = o;
    o += kHeadIn;
    b[kLayers] = o;
    o += 1;
    total = o;
  }
};
const ParamLayout kP;

constexpr int kRedBlocksG = 2 * kNumSMs;

// ---- elementwise and reduction kernels ------------------------------------

__device__ __forceinline__ size_t gstride() { return (size_t)gridDim.x * blockDim.x; }
__device__ __forceinline__ size_t gtid() { return blockIdx.x * (size_t)blockDim.x + threadIdx.x; }

// out[v] = b + Σ_c W[c] x[v][c]
__global__ void head_fwd_kernel(const bf16* __restrict__ x, const float* __restrict__ w, float* __restrict__ out,
                                size_t nv) {
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const uint4* p = reinterpret_cast<const uint4*>(x + v * kHeadIn);
    float s = __ldg(w + kHeadIn);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint4 u = __ldg(p + h);
      const uint32_t wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const __nv_bfloat162 b2 = *reinterpret_cast<const __nv_bfloat162*>(&wd[j]);
        s += __ldg(w + 8 * h + 2 * j) * __bfloat162float(b2.x) + __ldg(w + 8 * h + 2 * j + 1) * __bfloat162float(b2.y);
      }
    }
    out[v] = s;
  }
}

// MSE loss: dout = 2 (out - tgt) / N, per-block FP64 partial of Σ (out - tgt)^2
__global__ void loss_kernel(const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ dout,
                            size_t nv, double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  const float sc = 2.0f / (float)nv;
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const float d = out[v] - tgt[v];
    dout[v] = sc * d;
    s += (double)(d * d);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// head backward: dx[v][c] = W[c] dout[v]; dW[c] += Σ_v x[v][c] dout[v]; db += Σ dout
__global__ void head_bwd_kernel(const bf16* __restrict__ x, const float* __restrict__ w, const float* __restrict__ dout,
                                bf16* __restrict__ dx, float* __restrict__ dw, size_t nv) {
  __shared__ float sh[kHeadIn + 1][32];
  float acc[kHeadIn + 1];
#pragma unroll
  for (int c = 0; c <= kHeadIn; ++c) acc[c] = 0.0f;
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const float d = dout[v];
#pragma unroll
    for (int c = 0; c < kHeadIn; c += 2) {
      const __nv_bfloat162 xv = *reinterpret_cast<const __nv_bfloat162*>(x + v * kHeadIn + c);
      acc[c] += __bfloat162float(xv.x) * d;
      acc[c + 1] += __bfloat162float(xv.y) * d;
      *reinterpret_cast<__nv_bfloat162*>(dx + v * kHeadIn + c) = __floats2bfloat162_rn(__ldg(w + c) * d, __ldg(w + c + 1) * d);
    }
    acc[kHeadIn] += d;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c <= kHeadIn; ++c) {
    float s = acc[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sh[c][warp] = s;
  }
  __syncthreads();
  if ((int)threadIdx.x <= kHeadIn) {
    float s = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[threadIdx.x][k];
    atomicAdd(dw + threadIdx.x, s);   // dw[0..15] = weights, dw[16] = bias
  }
}

// dy[v][c] = 0 where the forward output y[v][c] <= 0 (ReLU), C channels at
// offset (pointers pre-offset), channel stride cs.
__global__ void relu_bwd_kernel(bf16* __restrict__ dy, const bf16* __restrict__ y, int cs, int C, size_t nv) {
  const int cp = C / 2;
  for (size_t e = gtid(); e < nv * cp; e += gstride()) {
    const size_t v = e / cp;
    const int c = 2 * (int)(e - v * cp);
    __nv_bfloat162* d = reinterpret_cast<__nv_bfloat162*>(dy + v * cs + c);
    const __nv_bfloat162 yy = *reinterpret_cast<const __nv_bfloat162*>(y + v * cs + c);
    __nv_bfloat162 dd = *d;
    if (!(__bfloat162float(yy.x) > 0.0f)) dd.x = __float2bfloat16(0.0f);
    if (!(__bfloat162float(yy.y) > 0.0f)) dd.y = __float2bfloat16(0.0f);
    *d = dd;
  }
}

// db[c] += Σ_v dy[v][c]
__global__ void bias_grad_kernel(const bf16* __restrict__ dy, int cs, int C, size_t nv, float* __restrict__ db) {
  __shared__ float sh[256];
  // thread -> channel c = tid % C, voxel lane = tid / C (C divides 256)
  const int c = threadIdx.x % C, lanes = blockDim.x / C, vl = threadIdx.x / C;
  float s = 0.0f;
  for (size_t v = blockIdx.x * (size_t)lanes + vl; v < nv; v += (size_t)gridDim.x * lanes)
    s += __bfloat162float(dy[v * cs + c]);
  sh[threadIdx.x] = s;
  __syncthreads();
  if ((int)threadIdx.x < C) {
    float t = 0.0f;
    for (int k = 0; k < lanes; ++k) t += sh[threadIdx.x + k * C];
    atomicAdd(db + threadIdx.x, t);
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, size_t n, float lr, float gscale, float b1, float b2, float c1,
                            float c2, float eps) {
  for (size_t i = gtid(); i < n; i += gstride()) {
    const float gr = g[i] * gscale;
    const float mi = b1 * m[i] + (1.0f - b1) * gr;
    const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

struct FeatGeom {
  int n1, n2;
  float c2s;      // cell² / s
  float is;       // 1 / s
  float l[3];     // mean line of sight (0 when isotropic or global)
  int local;
};

// X[v] = (f c²/s, φ_s/s, r_s c²/s, r̂ - l, 0, 0)
__global__ void features_kernel(const float* __restrict__ f, const float* __restrict__ phs,
                                const float* __restrict__ rs, const float* __restrict__ ax,
                                const float* __restrict__ ay, const float* __restrict__ az, FeatGeom G,
                                bf16* __restrict__ X, size_t nv) {
  for (size_t v = gtid(); v < nv; v += gstride()) {
    float d[3] = {0.0f, 0.0f, 0.0f};
    if (G.local) {
      const int i = (int)(v % G.n1);
      const size_t r = v / G.n1;
      const int j = (int)(r % G.n2), k = (int)(r / G.n2);
      const float x = ax[i], y = ay[j], z = az[k];
      const float rn = sqrtf(x * x + y * y + z * z);
      const float ir = rn > 0.0f ? 1.0f / rn : 0.0f;
      d[0] = x * ir - G.l[0];
      d[1] = y * ir - G.l[1];
      d[2] = z * ir - G.l[2];
    }
    __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(X + v * kFeat);
    o[0] = __floats2bfloat162_rn(f[v] * G.c2s, phs[v] * G.is);
    o[1] = __floats2bfloat162_rn(rs[v] * G.c2s, d[0]);
    o[2] = __floats2bfloat162_rn(d[1], d[2]);
    o[3] = __floats2bfloat162_rn(0.0f, 0.0f);
  }
}

// Laplacian of d = out - tgt (7-point, periodic, cell units): q = Δd, and
// per-block FP64 partials of Σ q².
__global__ void lap_loss_kernel(const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ q,
                                int n, double* __restrict__ part) {
  __shared__ double sh[256];
  const size_t nv = (size_t)n * n * n;
  double s = 0.0;
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
    auto D = [&](int a, int b, int c) {
      a = a < 0 ? a + n : a >= n ? a - n : a;
      b = b < 0 ? b + n : b >= n ? b - n : b;
      c = c < 0 ? c + n : c >= n ? c - n : c;
      const size_t w = ((size_t)c * n + b) * n + a;
      return out[w] - tgt[w];
    };
    const float lap = D(i + 1, j, k) + D(i - 1, j, k) + D(i, j + 1, k) + D(i, j - 1, k) + D(i, j, k + 1) +
                      D(i, j, k - 1) - 6.0f * D(i, j, k);
    q[v] = lap;
    s += (double)lap * lap;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// dout = (2/N) Δq (the Laplacian is symmetric on the periodic mesh)
__global__ void lap_grad_kernel(const float* __restrict__ q, float* __restrict__ dout, int n) {
  const size_t nv = (size_t)n * n * n;
  const float sc = 2.0f / (float)nv;
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
    auto Q = [&](int a, int b, int c) {
      a = a < 0 ? a + n : a >= n ? a - n : a;
      b = b < 0 ? b + n : b >= n ? b - n : b;
      c = c < 0 ? c + n : c >= n ? c - n : c;
      return q[((size_t)c * n + b) * n + a];
    };
    dout[v] = sc * (Q(i + 1, j, k) + Q(i - 1, j, k) + Q(i, j + 1, k) + Q(i, j - 1, k) + Q(i, j, k + 1) +
                    Q(i, j, k - 1) - 6.0f * Q(i, j, k));
  }
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, size_t n) {
  for (size_t i = gtid(); i < n; i += gstride()) b[i] = __float2bfloat16(a[i]);
}

// phi0 = φ_s + s out
__global__ void axpy_kernel(float* __restrict__ y, const float* __restrict__ x, float s, size_t n) {
  for (size_t i = gtid(); i < n; i += gstride()) y[i] += s * x[i];
}

// target = ((φ - mean φ) - φ_s) / s
__global__ void target_kernel(const float* __restrict__ phi, const float* __restrict__ phs, float mean, float is,
                              float* __restrict__ t, size_t n) {
  for (size_t i = gtid(); i < n; i += gstride()) t[i] = ((phi[i] - mean) - phs[i]) * is;
}

// ---- synthetic fields ------------------------------------------------------

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {   // SplitMix64 finaliser
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float u01(uint64_t h) { return ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f); }

struct NoiseGeom {
  int n1, n2, n3, n1h;
  float kf[3];     // 2π / L per axis
  float slope2;    // P(k) ∝ k^slope: amplitude ∝ k^(slope/2)
  float R2h;       // R² / 2 (Gaussian smoothing)
  uint64_t seed;
};

// Gaussian random modes: (N1 + i N2) k^(slope/2) exp(-R²k²/2), DC = 0.
__global__ void noise_kernel(cufftComplex* __restrict__ ck, size_t nk, NoiseGeom G) {
  for (size_t e = gtid(); e < nk; e += gstride()) {
    const int i = (int)(e % G.n1h);
    const size_t r = e / G.n1h;
    const int j = (int)(r % G.n2), k = (int)(r / G.n2);
    const int mj = j < (G.n2 + 1) / 2 ? j : j - G.n2;
    const int mk = k < (G.n3 + 1) / 2 ? k : k - G.n3;
    const float kx = G.kf[0] * i, ky = G.kf[1] * mj, kz = G.kf[2] * mk;
    const float k2 = kx * kx + ky * ky + kz * kz;
    cufftComplex c = make_float2(0.0f, 0.0f);
    if (k2 > 0.0f) {
      const uint64_t h1 = mix64(G.seed ^ (2 * e)), h2 = mix64(G.seed ^ (2 * e + 1));
      // Box-Muller
      const float rad = sqrtf(-2.0f * logf(u01(h1)));
      float sn, cs;
      sincospif(2.0f * u01(h2), &sn, &cs);
      const float amp = powf(k2, 0.5f * G.slope2) * expf(-G.R2h * k2);
      c = make_float2(amp * rad * cs, amp * rad * sn);
    }
    ck[e] = c;
  }
}

struct WindowGeom {
  int n1, n2;
  float r2min, r2max;
  float ra0, ra1, dec0, dec1;   // radians
  float sig_rms;                // σ_G / rms(G)
  float half_var;               // σ_G² / 2
  float ib;                     // 1 / bias
};

// f = W(x) (exp(σ G/rms - σ²/2) - 1) / b with W the survey window at the cell centre
__global__ void lognormal_window_kernel(const float* __restrict__ G, const float* __restrict__ ax,
                                        const float* __restrict__ ay, const float* __restrict__ az,
                                        WindowGeom W, float* __restrict__ f, size_t nv) {
  for (size_t v = gtid(); v < nv; v += gstride()) {
    const int i = (int)(v % W.n1);
    const size_t r = v / W.n1;
    const int j = (int)(r % W.n2), k = (int)(r / W.n2);
    const float x = ax[i], y = ay[j], z = az[k];
    const float r2 = x * x + y * y + z * z;
    bool in = r2 >= W.r2min && r2 <= W.r2max;
    if (in) {
      const float ra = atan2f(y, x);
      const float dec = asinf(z * rsqrtf(r2));
      in = ra >= W.ra0 && ra <= W.ra1 && dec >= W.dec0 && dec <= W.dec1;
    }
    f[v] = in ? (expf(W.sig_rms * G[v] - W.half_var) - 1.0f) * W.ib : 0.0f;
  }
}

unsigned eblocks(size_t n) {
  size_t b = (n + 255) / 256;
  return (unsigned)std::min<size_t>(b, 8 * kNumSMs);
}

}  // namespace

// ---- the network object ----------------------------------------------------

struct GuessNet {
  int n = 0;
  bool has_params = false, frags_ok = false, train_ready = false;
  float* params = nullptr;   // kP.total
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int64_t adam_t = 0;
  uint2* ffrag[kLayers] = {};
  uint2* bfrag[kLayers] = {};
  void* frag_mem = nullptr;
  // tcgen05 weight images of the layers whose shape has a tensor-core kernel
  bf16* fimg[kLayers] = {};
  bf16* bimg[kLayers] = {};
  void* img_mem = nullptr;
  bool use_tc = true;
  int tc_layers = 0;         // convolutions of the last forward that ran on tcgen05
  bf16* act[T_COUNT] = {};
  bf16* grad[T_COUNT] = {};
  void* act_mem = nullptr;
  void* grad_mem = nullptr;
  float* out = nullptr;      // head output (N)
  float* dout = nullptr;
  float* tgt = nullptr;
  double* part = nullptr;    // loss partials
  double* hpart = nullptr;   // pinned
};

namespace {

size_t nvox(const GuessNet* g, int level) {
  const size_t m = (size_t)(g->n >> level);
  return m * m * m;
}

int net_alloc(baorec_ctx* ctx) {
  if (ctx->net) return BAOREC_OK;
  if (!(ctx->n1 == ctx->n2 && ctx->n2 == ctx->n3) || ctx->n1 % 4 != 0)
    return set_error(ctx, BAOREC_ERR_ARG, "learned guess: needs a cubic mesh with n divisible by 4 (got %d x %d x %d)",
                     ctx->n1, ctx->n2, ctx->n3);
  GuessNet* g = new (std::nothrow) GuessNet();
  if (!g) return set_error(ctx, BAOREC_ERR_NOMEM, "learned guess: host allocation");
  ctx->net = g;
  g->n = ctx->n1;
  CK(cudaMalloc(&g->params, kP.total * sizeof(float)));
  CK(cudaMemsetAsync(g->params, 0, kP.total * sizeof(float), ctx->stream));
  size_t nf = 0;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    nf += guess::frag_count(L.kind, L.cin, L.cout);
    const int k2 = L.kind == DN ? UP : L.kind == UP ? DN : C3;
    nf += guess::frag_count(k2, L.cout, L.cin);
  }
  CK(cudaMalloc(&g->frag_mem, nf * sizeof(uint2)));
  uint2* fp = (uint2*)g->frag_mem;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    g->ffrag[l] = fp;
    fp += guess::frag_count(L.kind, L.cin, L.cout);
    const int k2 = L.kind == DN ? UP : L.kind == UP ? DN : C3;
    g->bfrag[l] = fp;
    fp += guess::frag_count(k2, L.cout, L.cin);
  }
  // weight images, 256-byte aligned each
  size_t ni = 0;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    const int nl = g->n >> kTensors[L.out_t].level;
    if (guess::tc_supported(L.kind, L.cin, L.cout, nl)) ni += (guess::image_count(L.cin, L.cout) * 2 + 255) / 256;
    if (l > 0 && guess::tc_supported(L.kind, L.cout, L.cin, nl)) ni += (guess::image_count(L.cout, L.cin) * 2 + 255) / 256;
  }
  if (ni) {
    CK(cudaMalloc(&g->img_mem, ni * 256));
    char* ip = (char*)g->img_mem;
    for (int l = 0; l < kLayers; ++l) {
      const LayerDef& L = kNet[l];
      const int nl = g->n >> kTensors[L.out_t].level;
      if (guess::tc_supported(L.kind, L.cin, L.cout, nl)) {
        g->fimg[l] = (bf16*)ip;
        ip += (guess::image_count(L.cin, L.cout) * 2 + 255) / 256 * 256;
      }
      if (l > 0 && guess::tc_supported(L.kind, L.cout, L.cin, nl)) {
        g->bimg[l] = (bf16*)ip;
        ip += (guess::image_count(L.cout, L.cin) * 2 + 255) / 256 * 256;
      }
    }
  }
  size_t na = 0;
  for (int t = 0; t < T_COUNT; ++t) na += nvox(g, kTensors[t].level) * kTensors[t].ch;
  CK(cudaMalloc(&g->act_mem, na * sizeof(bf16)));
  bf16* ap = (bf16*)g->act_mem;
  for (int t = 0; t < T_COUNT; ++t) {
    g->act[t] = ap;
    ap += nvox(g, kTensors[t].level) * kTensors[t].ch;
  }
  const size_t N = nvox(g, 0);
  CK(cudaMalloc(&g->out, N * sizeof(float)));
  CK(cudaMalloc(&g->part, kRedBlocksG * sizeof(double)));
  CK(cudaMallocHost(&g->hpart, kRedBlocksG * sizeof(double)));
  return BAOREC_OK;
}

int net_train_alloc(baorec_ctx* ctx) {
  GuessNet* g = ctx->net;
  if (g->train_ready) return BAOREC_OK;
  CK(cudaMalloc(&g->grads, kP.total * sizeof(float)));
  CK(cudaMalloc(&g->adam_m, kP.total * sizeof(float)));
  CK(cudaMalloc(&g->adam_v, kP.total * sizeof(float)));
  CK(cudaMemsetAsync(g->adam_m, 0, kP.total * sizeof(float), ctx->stream));
  CK(cudaMemsetAsync(g->adam_v, 0, kP.total * sizeof(float), ctx->stream));
  size_t na = 0;
  for (int t = 0; t < T_COUNT; ++t) na += nvox(g, kTensors[t].level) * kTensors[t].ch;
  CK(cudaMalloc(&g->grad_mem, na * sizeof(bf16)));
  bf16* ap = (bf16*)g->grad_mem;
  for (int t = 0; t < T_COUNT; ++t) {
    g->grad[t] = ap;
    ap += nvox(g, kTensors[t].level) * kTensors[t].ch;
  }
  const size_t N = nvox(g, 0);
  CK(cudaMalloc(&g->dout, N * sizeof(float)));
  CK(cudaMalloc(&g->tgt, N * sizeof(float)));
  g->adam_t = 0;
  g->train_ready = true;
  return BAOREC_OK;
}

int net_frags(baorec_ctx* ctx) {
  GuessNet* g = ctx->net;
  if (g->frags_ok) return BAOREC_OK;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    CK(guess::weight_frags(ctx->stream, L.kind, L.cin, L.cout, g->params + kP.w[l], g->ffrag[l], false));
    ctx->launches++;
    if (l > 0) {
      CK(guess::weight_frags(ctx->stream, L.kind, L.cin, L.cout, g->params + kP.w[l], g->bfrag[l], true));
      ctx->launches++;
    }
    if (g->fimg[l]) {
      CK(guess::weight_image(ctx->stream, L.cin, L.cout, g->params + kP.w[l], g->fimg[l], false));
      ctx->launches++;
    }
    if (g->bimg[l]) {
      CK(guess::weight_image(ctx->stream, L.cin, L.cout, g->params + kP.w[l], g->bimg[l], true));
      ctx->launches++;
    }
  }
  g->frags_ok = true;
  return BAOREC_OK;
}

// act[T_X] holds the features; the head output goes to g->out.
int net_forward(baorec_ctx* ctx) {
  GuessNet* g = ctx->net;
  CKS(net_frags(ctx));
  g->tc_layers = 0;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    guess::ConvArgs a;
    a.in = g->act[L.in_t] + L.in_off;
    a.in_cs = kTensors[L.in_t].ch;
    a.out = g->act[L.out_t] + L.out_off;
    a.out_cs = kTensors[L.out_t].ch;
    a.add = nullptr;
    a.add_cs = 0;
    a.w = g->ffrag[l];
    a.bias = g->params + kP.b[l];
    a.relu = 1;
    a.n_in = g->n >> kTensors[L.in_t].level;
    a.n_out = g->n >> kTensors[L.out_t].level;
    a.wimg = g->use_tc ? g->fimg[l] : nullptr;
    a.err = ctx->derr;
    if (a.wimg) g->tc_layers++;
    CK(guess::conv_forward(ctx->stream, L.kind, L.cin, L.cout, a));
    ctx->launches++;
  }
  (head_fwd_kernel<<<eblocks(nvox(g, 0)), 256, 0, ctx->stream>>>(g->act[T_C0], g->params + kP.w[kLayers], g->out,
                                                                 nvox(g, 0)), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

// loss and dout from g->out and g->tgt: kind 0 the mean squared error of the
// potential, kind 1 that of its Laplacian (weights the error by k^4, as the
// residual of the solve sees it); *loss gets the value
int net_loss(baorec_ctx* ctx, int kind, double* loss) {
  GuessNet* g = ctx->net;
  const size_t N = nvox(g, 0);
  if (kind == 1) {
    float* q = ctx->lev[0].r + N;   // scratch mesh
    (lap_loss_kernel<<<kRedBlocksG, 256, 0, ctx->stream>>>(g->out, g->tgt, q, g->n, g->part), ::baorec::count_launch());
    CKLAUNCH();
    (lap_grad_kernel<<<eblocks(N), 256, 0, ctx->stream>>>(q, g->dout, g->n), ::baorec::count_launch());
    CKLAUNCH();
  } else {
    (loss_kernel<<<kRedBlocksG, 256, 0, ctx->stream>>>(g->out, g->tgt, g->dout, N, g->part), ::baorec::count_launch());
    CKLAUNCH();
  }
  if (loss) {
    CK(cudaMemcpyAsync(g->hpart, g->part, kRedBlocksG * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (int b = 0; b < kRedBlocksG; ++b) s += g->hpart[b];
    *loss = s / (double)N;
  }
  return BAOREC_OK;
}

// accumulates parameter gradients into g->grads from g->dout
int net_backward(baorec_ctx* ctx) {
  GuessNet* g = ctx->net;
  const size_t N = nvox(g, 0);
  (head_bwd_kernel<<<kRedBlocksG, 256, 0, ctx->stream>>>(g->act[T_C0], g->params + kP.w[kLayers], g->dout,
                                                         g->grad[T_C0], g->grads + kP.w[kLayers], N), ::baorec::count_launch());
  CKLAUNCH();
  for (int l = kLayers - 1; l >= 0; --l) {
    const LayerDef& L = kNet[l];
    const int ocs = kTensors[L.out_t].ch, ics = kTensors[L.in_t].ch;
    const size_t nvo = nvox(g, kTensors[L.out_t].level);
    bf16* dy = g->grad[L.out_t] + L.out_off;
    (relu_bwd_kernel<<<eblocks(nvo * L.cout / 2), 256, 0, ctx->stream>>>(dy, g->act[L.out_t] + L.out_off, ocs, L.cout, nvo), ::baorec::count_launch());
    CKLAUNCH();
    guess::WgradArgs w;
    w.in = g->act[L.in_t] + L.in_off;
    w.in_cs = ics;
    w.dy = dy;
    w.dy_cs = ocs;
    w.dw = g->grads + kP.w[l];
    w.n_in = g->n >> kTensors[L.in_t].level;
    w.n_out = g->n >> kTensors[L.out_t].level;
    CK(guess::conv_wgrad(ctx->stream, L.kind, L.cin, L.cout, w));
    ctx->launches++;
    (bias_grad_kernel<<<kRedBlocksG, 256, 0, ctx->stream>>>(dy, ocs, L.cout, nvo, g->grads + kP.b[l]), ::baorec::count_launch());
    CKLAUNCH();
    if (l == 0) break;
    guess::ConvArgs a;
    a.in = dy;
    a.in_cs = ocs;
    a.out = g->grad[L.in_t] + L.in_off;
    a.out_cs = ics;
    a.add = L.acc_grad ? a.out : nullptr;
    a.add_cs = ics;
    a.w = g->bfrag[l];
    a.bias = nullptr;
    a.relu = 0;
    a.n_in = w.n_out;
    a.n_out = w.n_in;
    a.wimg = g->use_tc ? g->bimg[l] : nullptr;
    a.err = ctx->derr;
    const int k2 = L.kind == DN ? UP : L.kind == UP ? DN : C3;
    CK(guess::conv_forward(ctx->stream, k2, L.cout, L.cin, a));
    ctx->launches++;
  }
  return BAOREC_OK;
}

// Features of the rhs f into act[T_X]; φ_s = S⁻¹ f into phs; returns s = rms(φ_s).
int net_features(baorec_ctx* ctx, const float* f, float* phs, float* rs, float* s_out) {
  GuessNet* g = ctx->net;
  const size_t N = ctx->N;
  CKS(spectral_correction(ctx, f, phs));
  CKS(operator_residual(ctx, phs, f, rs));
  double ss = 0.0;
  CKS(sumsq_mesh(ctx, phs, N, &ss));
  const double rms = sqrt(ss / (double)N);
  const float s = rms > 0.0 ? (float)rms : 1.0f;
  FeatGeom G;
  G.n1 = ctx->n1;
  G.n2 = ctx->n2;
  const double cell = (double)ctx->cfg.box_size[0] / ctx->n1;
  G.c2s = (float)(cell * cell / s);
  G.is = 1.0f / s;
  double l[3];
  mean_los(ctx, l);
  G.local = ctx->cfg.los_mode == BAOREC_LOS_LOCAL ? 1 : 0;
  for (int a = 0; a < 3; ++a) G.l[a] = (float)l[a];
  (features_kernel<<<eblocks(N), 256, 0, ctx->stream>>>(f, phs, rs, ctx->xvec[0], ctx->xvec[1], ctx->xvec[2], G,
                                                       g->act[T_X], N), ::baorec::count_launch());
  CKLAUNCH();
  *s_out = s;
  return BAOREC_OK;
}

int net_adam(baorec_ctx* ctx, float lr, float gscale) {
  GuessNet* g = ctx->net;
  g->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = (float)(1.0 - pow((double)b1, (double)g->adam_t));
  const float c2 = (float)(1.0 - pow((double)b2, (double)g->adam_t));
  (adam_kernel<<<eblocks(kP.total), 256, 0, ctx->stream>>>(g->params, g->grads, g->adam_m, g->adam_v, kP.total, lr,
                                                          gscale, b1, b2, c1, c2, 1e-8f), ::baorec::count_launch());
  CKLAUNCH();
  g->frags_ok = false;
  return BAOREC_OK;
}

int need_params(baorec_ctx* ctx) {
  if (!ctx->net || !ctx->net->has_params)
    return set_error(ctx, BAOREC_ERR_ARG, "learned guess: no network parameters (init, set or train them first)");
  return BAOREC_OK;
}

// One training pair on this context's mesh: a sub-box at a random origin of
// the region, lognormal field in the survey window as f, the converged φ.
int make_sample(baorec_ctx* ctx, const baorec_guess_train_config* tc, uint64_t index, float* f, float* phi) {
  std::mt19937_64 rng(((uint64_t)tc->seed << 32) ^ (index * 0x9E3779B97F4A7C15ull));
  std::uniform_real_distribution<double> U(0.0, 1.0);
  float bmin[3];
  for (int a = 0; a < 3; ++a) {
    const double span = std::max(0.0, (double)tc->region_size[a] - (double)ctx->cfg.box_size[a]);
    bmin[a] = (float)(tc->region_min[a] + span * U(rng));
  }
  CKS(baorec_set_box(ctx, ctx->cfg.box_size, bmin));
  NoiseGeom NG;
  NG.n1 = ctx->n1; NG.n2 = ctx->n2; NG.n3 = ctx->n3; NG.n1h = ctx->n1h;
  for (int a = 0; a < 3; ++a) NG.kf[a] = (float)(2.0 * M_PI / ctx->cfg.box_size[a]);
  NG.slope2 = 0.5f * tc->pk_slope;
  NG.R2h = 0.5f * ctx->cfg.smoothing_radius * ctx->cfg.smoothing_radius;
  NG.seed = mix64(((uint64_t)tc->seed << 20) + index);
  (noise_kernel<<<eblocks(ctx->Nk), 256, 0, ctx->stream>>>(ctx->ck, ctx->Nk, NG), ::baorec::count_launch());
  CKLAUNCH();
  float* G = ctx->psi;   // scratch
  CKFFT(cufftExecC2R(ctx->plan_c2r, ctx->ck, G));
  double ss = 0.0;
  CKS(sumsq_mesh(ctx, G, ctx->N, &ss));
  const double rms = sqrt(ss / (double)ctx->N);
  WindowGeom W;
  W.n1 = ctx->n1; W.n2 = ctx->n2;
  W.r2min = tc->r_min * tc->r_min;
  W.r2max = tc->r_max * tc->r_max;
  const double d2r = M_PI / 180.0;
  W.ra0 = (float)(tc->ra_min * d2r); W.ra1 = (float)(tc->ra_max * d2r);
  W.dec0 = (float)(tc->dec_min * d2r); W.dec1 = (float)(tc->dec_max * d2r);
  W.sig_rms = rms > 0.0 ? (float)(tc->sigma_g / rms) : 0.0f;
  W.half_var = 0.5f * tc->sigma_g * tc->sigma_g;
  W.ib = 1.0f / ctx->cfg.bias;
  (lognormal_window_kernel<<<eblocks(ctx->N), 256, 0, ctx->stream>>>(G, ctx->xvec[0], ctx->xvec[1], ctx->xvec[2], W, f,
                                                                    ctx->N), ::baorec::count_launch());
  CKLAUNCH();
  const baorec_config saved = ctx->cfg;
  ctx->cfg.mg_start = BAOREC_START_SPECTRAL;
  ctx->cfg.rtol = tc->rtol;
  const int st = mg_solve(ctx, f, phi, nullptr, nullptr);
  ctx->cfg = saved;
  // a target a little short of rtol (the double-float floor) is still a target
  if (st == BAOREC_ERR_NOT_CONVERGED && ctx->last_stats.rel_residual <= 10.0 * (double)tc->rtol) return BAOREC_OK;
  return st;
}

}  // namespace

void guess_free(baorec_ctx* ctx) {
  GuessNet* g = ctx->net;
  if (!g) return;
  cudaFree(g->params);
  cudaFree(g->grads);
  cudaFree(g->adam_m);
  cudaFree(g->adam_v);
  cudaFree(g->frag_mem);
  cudaFree(g->img_mem);
  cudaFree(g->act_mem);
  cudaFree(g->grad_mem);
  cudaFree(g->out);
  cudaFree(g->dout);
  cudaFree(g->tgt);
  cudaFree(g->part);
  cudaFreeHost(g->hpart);
  delete g;
  ctx->net = nullptr;
}

// φ0 = φ_s + s net(features(f)) into phi0 (device meshes of the context's size)
int guess_apply(baorec_ctx* ctx, const float* f, float* phi0) {
  CKS(need_params(ctx));
  CKS(mg_setup(ctx));
  float s = 1.0f;
  CKS(net_features(ctx, f, phi0, ctx->lev[0].r, &s));
  CKS(net_forward(ctx));
  (axpy_kernel<<<eblocks(ctx->N), 256, 0, ctx->stream>>>(phi0, ctx->net->out, s, ctx->N), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec

using namespace baorec;

static_assert(sizeof(baorec_guess_train_config) == 4 * 20, "baorec_guess_train_config layout is part of the ABI");

extern "C" int64_t baorec_guess_num_params(void) { return (int64_t)kP.total; }

static int guess_init_impl(baorec_ctx* ctx, uint32_t seed) {
  CKS(net_alloc(ctx));
  std::mt19937_64 rng(seed);
  std::vector<float> p(kP.total, 0.0f);
  for (int l = 0; l < kLayers; ++l) {
    const LayerDef& L = kNet[l];
    const int fan_in = guess::taps_of(L.kind) * L.cin;
    std::normal_distribution<double> nd(0.0, sqrt(2.0 / fan_in));   // He initialisation
    const size_t nw = (size_t)guess::taps_of(L.kind) * L.cin * L.cout;
    for (size_t i = 0; i < nw; ++i) p[kP.w[l] + i] = (float)nd(rng);
  }
  // a small head: the untrained network starts close to the FFT start
  std::normal_distribution<double> nh(0.0, 1e-3);
  for (int c = 0; c < kHeadIn; ++c) p[kP.w[kLayers] + c] = (float)nh(rng);
  CK(cudaMemcpyAsync(ctx->net->params, p.data(), p.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->net->has_params = true;
  ctx->net->frags_ok = false;
  ctx->net->adam_t = 0;
  if (ctx->net->train_ready) {
    CK(cudaMemsetAsync(ctx->net->adam_m, 0, kP.total * 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->net->adam_v, 0, kP.total * 4, ctx->stream));
  }
  return BAOREC_OK;
}

static int guess_set_params_impl(baorec_ctx* ctx, const float* params, int64_t n) {
  if (n != (int64_t)kP.total)
    return set_error(ctx, BAOREC_ERR_ARG, "guess_set_params: %lld values, the network has %zu", (long long)n, kP.total);
  CKS(net_alloc(ctx));
  CK(cudaMemcpyAsync(ctx->net->params, params, kP.total * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->net->has_params = true;
  ctx->net->frags_ok = false;
  return BAOREC_OK;
}

static int guess_get_params_impl(baorec_ctx* ctx, float* params, int64_t n) {
  CKS(need_params(ctx));
  if (n != (int64_t)kP.total)
    return set_error(ctx, BAOREC_ERR_ARG, "guess_get_params: room for %lld values, the network has %zu", (long long)n,
                     kP.total);
  CK(cudaMemcpyAsync(params, ctx->net->params, kP.total * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return BAOREC_OK;
}

static int guess_eval_impl(baorec_ctx* ctx, const float* features, const float* target, float* out, float* grads,
                           double* loss, int loss_kind) {
  CKS(need_params(ctx));
  CKS(mg_setup(ctx));
  GuessNet* g = ctx->net;
  const size_t N = ctx->N;
  (f32_to_bf16_kernel<<<eblocks(N * kFeat), 256, 0, ctx->stream>>>(features, g->act[T_X], N * kFeat), ::baorec::count_launch());
  CKLAUNCH();
  CKS(net_forward(ctx));
  CK(cudaMemcpyAsync(out, g->out, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  if (target) {
    CKS(net_train_alloc(ctx));
    CK(cudaMemcpyAsync(g->tgt, target, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    double l = 0.0;
    CKS(net_loss(ctx, loss_kind, &l));
    if (loss) *loss = l;
    if (grads) {
      CK(cudaMemsetAsync(g->grads, 0, kP.total * 4, ctx->stream));
      CKS(net_backward(ctx));
      CK(cudaMemcpyAsync(grads, g->grads, kP.total * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  return finish(ctx, 0);
}

static int guess_sample_impl(baorec_ctx* ctx, const baorec_guess_train_config* tc, int64_t index, float* f,
                             float* phi) {
  CKS(mg_setup(ctx));
  CKS(make_sample(ctx, tc, (uint64_t)index, f, phi));
  return finish(ctx, 0);
}

static int guess_train_impl(baorec_ctx* ctx, const baorec_guess_train_config* tc, float* loss_history) {
  CKS(need_params(ctx));
  CKS(net_train_alloc(ctx));
  CKS(mg_setup(ctx));
  GuessNet* g = ctx->net;
  const size_t N = ctx->N;
  float* f = ctx->mesh3 + N;       // B
  float* phi = ctx->mesh3;         // A
  float* phs = ctx->mesh3 + 2 * N; // C
  const float saved_box[3] = {ctx->cfg.box_min[0], ctx->cfg.box_min[1], ctx->cfg.box_min[2]};
  uint64_t index = 0;
  for (int step = 0; step < tc->steps; ++step) {
    CK(cudaMemsetAsync(g->grads, 0, kP.total * 4, ctx->stream));
    double lsum = 0.0;
    for (int b = 0; b < tc->batch; ++b) {
      CKS(make_sample(ctx, tc, index++, f, phi));
      float s = 1.0f;
      CKS(net_features(ctx, f, phs, ctx->lev[0].r, &s));
      double mphi = 0.0;
      CKS(sum_mesh(ctx, phi, N, &mphi));
      (target_kernel<<<eblocks(N), 256, 0, ctx->stream>>>(phi, phs, (float)(mphi / (double)N), 1.0f / s, g->tgt, N), ::baorec::count_launch());
      CKLAUNCH();
      CKS(net_forward(ctx));
      double l = 0.0;
      CKS(net_loss(ctx, tc->loss, loss_history ? &l : nullptr));
      lsum += l;
      CKS(net_backward(ctx));
    }
    CKS(net_adam(ctx, tc->lr, 1.0f / (float)tc->batch));
    if (loss_history) loss_history[step] = (float)(lsum / tc->batch);
  }
  CKS(baorec_set_box(ctx, ctx->cfg.box_size, saved_box));
  ctx->has_result = false;
  return finish(ctx, 0);
}

static int guess_set_conv_path_impl(baorec_ctx* ctx, int32_t tensor_core) {
  CKS(net_alloc(ctx));
  ctx->net->use_tc = tensor_core != 0;
  return BAOREC_OK;
}


// ---- the network on this mesh or on its first restriction -----------------
//
// guess_level 0: the network runs on the context's own mesh.  guess_level 1:
// it runs on a child context at n/2 per axis over the same box (the first
// restriction of the multigrid), which owns the network; every
// baorec_guess_* call is routed to the context that owns it, and its error
// message is copied back.

namespace baorec {
namespace {

baorec_ctx* net_ctx(baorec_ctx* ctx) { return ctx->guess_level == 1 && ctx->guess_child ? ctx->guess_child : ctx; }

int routed(baorec_ctx* ctx, baorec_ctx* c, int st) {
  if (st != BAOREC_OK && c != ctx) {
    snprintf(ctx->msg, sizeof(ctx->msg), "%s", c->msg);
    ctx->launches += 0;
  }
  return st;
}

int sync_child_box(baorec_ctx* ctx) {
  baorec_ctx* c = ctx->guess_child;
  bool same = true;
  for (int a = 0; a < 3; ++a)
    same = same && c->cfg.box_size[a] == ctx->cfg.box_size[a] && c->cfg.box_min[a] == ctx->cfg.box_min[a];
  if (same) return BAOREC_OK;
  return routed(ctx, c, baorec_set_box(c, ctx->cfg.box_size, ctx->cfg.box_min));
}

__global__ void scale_kernel(float* __restrict__ a, float s, size_t n) {
  for (size_t i = gtid(); i < n; i += gstride()) a[i] *= s;
}

// φ0 = S⁻¹ f + P (s_c net_c(features of R f)): the FFT start on this mesh plus
// the network's correction computed on the child from the full-weighting
// restriction R f (src/multigrid.jl:520-584) and brought back by the
// trilinear prolongation P (src/multigrid.jl:398-453), added in place.
int guess_apply_coarse(baorec_ctx* ctx, const float* f, float* phi0) {
  baorec_ctx* c = ctx->guess_child;
  if (!c->net || !c->net->has_params)
    return set_error(ctx, BAOREC_ERR_ARG, "learned guess: no network parameters (init, set or train them first)");
  CKS(sync_child_box(ctx));
  CKS(mg_setup(ctx));
  CKS(routed(ctx, c, mg_setup(c)));
  for (cudaEvent_t* e : {&ctx->ev_guess[0], &ctx->ev_guess[1]})
    if (!*e) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  const int nl[3] = {ctx->n1, ctx->n2, ctx->n3};
  float* fc = c->mesh3;            // R f
  float* phs = c->mesh3 + c->N;    // the child's FFT start of R f (a feature)
  const int64_t l0 = c->launches;
  // the child starts as soon as R f exists; this mesh's FFT start, which
  // does not depend on the network, runs on this context's stream meanwhile
  CKS(mg_reduce(ctx, fc, f, nl));
  CK(cudaEventRecord(ctx->ev_guess[0], ctx->stream));
  CK(cudaStreamWaitEvent(c->stream, ctx->ev_guess[0], 0));
  CKS(spectral_correction(ctx, f, phi0));
  float s = 1.0f;
  CKS(routed(ctx, c, net_features(c, fc, phs, c->lev[0].r, &s)));
  CKS(routed(ctx, c, net_forward(c)));
  (scale_kernel<<<eblocks(c->N), 256, 0, c->stream>>>(c->net->out, s, c->N), ::baorec::count_launch());
  CK(cudaGetLastError());
  c->launches++;
  CK(cudaEventRecord(ctx->ev_guess[1], c->stream));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_guess[1], 0));
  ctx->launches += c->launches - l0;
  return mg_prolong(ctx, phi0, c->net->out, nl, 1);
}

// move the parameters of the network owned by `from` into `to` (allocating its network)
int move_params(baorec_ctx* ctx, baorec_ctx* from, baorec_ctx* to) {
  if (!from->net || !from->net->has_params) return BAOREC_OK;
  CKS(routed(ctx, to, net_alloc(to)));
  CK(cudaStreamSynchronize(from->stream));
  CK(cudaMemcpyAsync(to->net->params, from->net->params, kP.total * 4, cudaMemcpyDeviceToDevice, to->stream));
  CK(cudaStreamSynchronize(to->stream));
  to->net->has_params = true;
  to->net->frags_ok = false;
  to->net->use_tc = from->net->use_tc;
  return BAOREC_OK;
}

}  // namespace

int guess_dispatch_apply(baorec_ctx* ctx, const float* f, float* phi0) {
  // With one line of sight for the whole box the operator is a convolution
  // and the FFT start S⁻¹f is its exact inverse: the error the network
  // predicts is zero (and the network only ever saw the radial line of
  // sight), so the learned start is the FFT start.
  if (ctx->cfg.los_mode == BAOREC_LOS_GLOBAL) return spectral_correction(ctx, f, phi0);
  return ctx->guess_level == 1 && ctx->guess_child ? guess_apply_coarse(ctx, f, phi0) : guess_apply(ctx, f, phi0);
}

}  // namespace baorec

extern "C" int baorec_guess_set_level(baorec_ctx* ctx, int32_t level) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (level != 0 && level != 1) return set_error(ctx, BAOREC_ERR_ARG, "guess_set_level: level must be 0 or 1");
  if (level == ctx->guess_level) return BAOREC_OK;
  if (level == 1) {
    const int n = ctx->n1;
    if (!(ctx->n1 == ctx->n2 && ctx->n2 == ctx->n3) || n % 8 != 0)
      return set_error(ctx, BAOREC_ERR_ARG, "guess_set_level: the restriction needs a cubic mesh with n divisible by 8");
    if (!ctx->guess_child) {
      baorec_config cc = ctx->cfg;
      for (int a = 0; a < 3; ++a) cc.n[a] = n / 2;
      cc.method = BAOREC_MULTIGRID;
      cc.mg_mode = BAOREC_MG_CONVERGENT;
      cc.mg_start = BAOREC_START_SPECTRAL;
      baorec_ctx* c = nullptr;
      const int st = baorec_create(&cc, &c);
      if (st != BAOREC_OK) {
        set_error(ctx, st, "guess_set_level: %s", baorec_last_error(c));
        if (c) baorec_destroy(c);
        return st;
      }
      ctx->guess_child = c;
    }
    CKS(move_params(ctx, ctx, ctx->guess_child));
    guess_free(ctx);
  } else {
    CKS(move_params(ctx, ctx->guess_child, ctx));
    baorec_destroy(ctx->guess_child);
    ctx->guess_child = nullptr;
  }
  ctx->guess_level = level;
  return BAOREC_OK;
}

extern "C" int32_t baorec_guess_level(const baorec_ctx* ctx) { return ctx ? ctx->guess_level : -1; }

extern "C" int baorec_guess_init(baorec_ctx* ctx, uint32_t seed) {
  if (!ctx) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_init_impl(c, seed));
}

extern "C" int baorec_guess_set_params(baorec_ctx* ctx, const float* params, int64_t n) {
  if (!ctx || !params) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_set_params_impl(c, params, n));
}

extern "C" int baorec_guess_get_params(baorec_ctx* ctx, float* params, int64_t n) {
  if (!ctx || !params) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_get_params_impl(c, params, n));
}

extern "C" int baorec_guess_eval(baorec_ctx* ctx, const float* features, const float* target, float* out,
                                 float* grads, double* loss, int loss_kind) {
  if (!ctx || !features || !out || loss_kind < 0 || loss_kind > 1) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_eval_impl(c, features, target, out, grads, loss, loss_kind));
}

extern "C" int baorec_guess_apply(baorec_ctx* ctx, const float* f, float* phi0) {
  if (!ctx || !f || !phi0) return BAOREC_ERR_ARG;
  CKS(guess_dispatch_apply(ctx, f, phi0));
  return finish(ctx, 0);
}

extern "C" int baorec_guess_sample(baorec_ctx* ctx, const baorec_guess_train_config* tc, int64_t index, float* f,
                                   float* phi) {
  if (!ctx || !tc || !f || !phi) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_sample_impl(c, tc, index, f, phi));
}

extern "C" int baorec_guess_train(baorec_ctx* ctx, const baorec_guess_train_config* tc, float* loss_history) {
  if (!ctx || !tc || tc->steps < 0 || tc->batch < 1 || tc->loss < 0 || tc->loss > 1)
    return set_error(ctx, BAOREC_ERR_ARG, "guess_train: bad config");
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_train_impl(c, tc, loss_history));
}

extern "C" int baorec_guess_set_conv_path(baorec_ctx* ctx, int32_t tensor_core) {
  if (!ctx || tensor_core < 0 || tensor_core > 1) return BAOREC_ERR_ARG;
  baorec_ctx* c = net_ctx(ctx);
  return routed(ctx, c, guess_set_conv_path_impl(c, tensor_core));
}

extern "C" int32_t baorec_guess_tc_layers(baorec_ctx* ctx) {
  if (!ctx) return -1;
  baorec_ctx* c = net_ctx(ctx);
  return c->net ? c->net->tc_layers : -1;
}

extern "C" int baorec_guess_conv3(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n, const void* x,
                                  const float* w, const float* bias, const void* add, void* y, int32_t relu,
                                  int32_t path) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!x || !w || !y || n < 1 || path < 0 || path > 2)
    return set_error(ctx, BAOREC_ERR_ARG, "guess_conv3: bad arguments");
  bool known = false;
#define X(K, I, O) \
  if (K == C3 && cin == I && cout == O) known = true;
  BAOREC_GUESS_SHAPES(X)
#undef X
  if (!known) return set_error(ctx, BAOREC_ERR_ARG, "guess_conv3: no kernel for %d -> %d channels", cin, cout);
  if (path >= 1 && !guess::tc_supported(C3, cin, cout, n))
    return set_error(ctx, BAOREC_ERR_ARG, "guess_conv3: no tcgen05 kernel for %d -> %d channels at n = %d", cin, cout, n);
  uint2* frag = nullptr;
  bf16* img = nullptr;
  int rc = BAOREC_OK;
  cudaError_t e = cudaMalloc(&frag, guess::frag_count(C3, cin, cout) * sizeof(uint2));
  if (e == cudaSuccess && path >= 1) e = cudaMalloc(&img, guess::image_count(cin, cout) * sizeof(bf16));
  if (e == cudaSuccess) e = guess::weight_frags(ctx->stream, C3, cin, cout, w, frag, false);
  if (e == cudaSuccess && img) e = guess::weight_image(ctx->stream, cin, cout, w, img, false);
  if (e == cudaSuccess) {
    guess::ConvArgs a;
    a.in = (const bf16*)x;
    a.in_cs = cin;
    a.out = (bf16*)y;
    a.out_cs = cout;
    a.add = (const bf16*)add;
    a.add_cs = cout;
    a.w = frag;
    a.bias = bias;
    a.relu = relu ? 1 : 0;
    a.n_in = a.n_out = n;
    a.wimg = img;
    a.err = ctx->derr;
    a.tc_loader = path == 2 ? 1 : 0;   // 1: TMA boxes, 2: cp.async warps
    e = guess::conv_forward(ctx->stream, C3, cin, cout, a);
    ctx->launches++;
  }
  if (e != cudaSuccess) rc = set_error(ctx, BAOREC_ERR_CUDA, "guess_conv3: %s", cudaGetErrorString(e));
  else rc = finish(ctx, 0);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(frag);
  cudaFree(img);
  return rc;
}

extern "C" int baorec_guess_conv3_held_back(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n,
                                            int64_t wait_ns) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (wait_ns < 1 || !guess::tc_supported(C3, cin, cout, n))
    return set_error(ctx, BAOREC_ERR_ARG, "guess_conv3_held_back: no tcgen05 kernel for %d -> %d at n = %d", cin, cout,
                     n);
  const size_t nv = (size_t)n * n * n;
  bf16 *x = nullptr, *y = nullptr, *img = nullptr;
  float* w = nullptr;
  uint2* frag = nullptr;
  cudaError_t e = cudaMalloc(&x, nv * cin * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&y, nv * cout * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&w, (size_t)27 * cin * cout * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&frag, guess::frag_count(C3, cin, cout) * sizeof(uint2));
  if (e == cudaSuccess) e = cudaMalloc(&img, guess::image_count(cin, cout) * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMemsetAsync(x, 0, nv * cin * sizeof(bf16), ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, (size_t)27 * cin * cout * sizeof(float), ctx->stream);
  if (e == cudaSuccess) e = guess::weight_frags(ctx->stream, C3, cin, cout, w, frag, false);
  if (e == cudaSuccess) e = guess::weight_image(ctx->stream, cin, cout, w, img, false);
  if (e == cudaSuccess) {
    guess::ConvArgs a;
    a.in = x;
    a.in_cs = cin;
    a.out = y;
    a.out_cs = cout;
    a.add = nullptr;
    a.add_cs = 0;
    a.w = frag;
    a.bias = nullptr;
    a.relu = 0;
    a.n_in = a.n_out = n;
    a.wimg = img;
    a.err = ctx->derr;
    a.tc_loader = 0;            // TMA boxes
    a.wait_ns = (unsigned long long)wait_ns;
    a.hold_back = 1;            // no slab is ever loaded: the MMA issuer's first wait expires
    e = guess::conv_forward(ctx->stream, C3, cin, cout, a);
    ctx->launches++;
  }
  int rc = e != cudaSuccess ? set_error(ctx, BAOREC_ERR_CUDA, "guess_conv3_held_back: %s", cudaGetErrorString(e))
                            : finish(ctx, 0);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(x);
  cudaFree(y);
  cudaFree(w);
  cudaFree(frag);
  cudaFree(img);
  return rc;
}

extern "C" int baorec_guess_profile_conv(baorec_ctx* ctx, int32_t cin, int32_t cout, int32_t n, int32_t path,
                                         int32_t reps, float* avg_ms, double* flops) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 1 || reps < 1 || path < 0 || path > 2 || !avg_ms || !flops)
    return set_error(ctx, BAOREC_ERR_ARG, "guess_profile_conv: bad arguments");
  if (path >= 1 && !guess::tc_supported(C3, cin, cout, n))
    return set_error(ctx, BAOREC_ERR_ARG, "guess_profile_conv: no tcgen05 kernel for %d -> %d at n = %d", cin, cout, n);
  const size_t nv = (size_t)n * n * n;
  bf16 *x = nullptr, *y = nullptr, *img = nullptr;
  float *w = nullptr, *b = nullptr;
  uint2* frag = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = BAOREC_OK;
  cudaError_t e = cudaMalloc(&x, nv * cin * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&y, nv * cout * sizeof(bf16));
  if (e == cudaSuccess) e = cudaMalloc(&w, (size_t)27 * cin * cout * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&b, (size_t)cout * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&frag, guess::frag_count(C3, cin, cout) * sizeof(uint2));
  if (e == cudaSuccess && path >= 1) e = cudaMalloc(&img, guess::image_count(cin, cout) * sizeof(bf16));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMemsetAsync(x, 0x3c, nv * cin * sizeof(bf16), ctx->stream);   // finite BF16 values
  if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, (size_t)27 * cin * cout * sizeof(float), ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b, 0, (size_t)cout * sizeof(float), ctx->stream);
  if (e == cudaSuccess) e = guess::weight_frags(ctx->stream, C3, cin, cout, w, frag, false);
  if (e == cudaSuccess && img) e = guess::weight_image(ctx->stream, cin, cout, w, img, false);
  guess::ConvArgs a;
  a.in = x;
  a.in_cs = cin;
  a.out = y;
  a.out_cs = cout;
  a.add = nullptr;
  a.add_cs = 0;
  a.w = frag;
  a.bias = b;
  a.relu = 1;
  a.n_in = a.n_out = n;
  a.wimg = img;
  a.err = ctx->derr;
  a.tc_loader = path == 2 ? 1 : 0;
  if (e == cudaSuccess) e = guess::conv_forward(ctx->stream, C3, cin, cout, a);   // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) e = guess::conv_forward(ctx->stream, C3, cin, cout, a);
  if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  ctx->launches += reps + 1;
  if (e != cudaSuccess) rc = set_error(ctx, BAOREC_ERR_CUDA, "guess_profile_conv: %s", cudaGetErrorString(e));
  else rc = finish(ctx, 0);
  *avg_ms = ms / (float)reps;
  *flops = 2.0 * 27.0 * cin * cout * (double)nv;
  cudaStreamSynchronize(ctx->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  cudaFree(w);
  cudaFree(b);
  cudaFree(frag);
  cudaFree(img);
  return rc;
}
