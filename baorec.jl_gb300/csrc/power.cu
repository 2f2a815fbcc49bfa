// Power-spectrum multipoles of a catalog (or catalog minus randoms) on the
// context's mesh: the science check of the reference's test helpers
// (test_helpers/simulation.py:40-55, test_helpers/lightcone.py:48-75), which
// call the external pypowspec.  Restated from the published estimators:
// the periodic-box estimator with a fixed line of sight, and the FFT form of
// the Yamamoto estimator with a local line of sight (Bianchi et al. 2015,
// Scoccimarro 2015): A_0 = FFT[F], A_2 = Σ k̂_i k̂_j FFT[r̂_i r̂_j F],
// A_4 = Σ k̂_i k̂_j k̂_k k̂_l FFT[r̂_i r̂_j r̂_k r̂_l F].
//
// Device work: one paint of F = Σ w_d - α Σ w_r (CIC or TSC, nodes at
// box_min + i L/n, periodic), 1 (box; 2 interlaced) or 22 (survey) R2C
// transforms, element-wise r̂ products and k̂ accumulations, and one binning
// pass that applies the window compensation and the Legendre weights with
// FP64 per-block shell sums.
#include <math.h>

#include <vector>

#include "common.cuh"

namespace baorec {
namespace {

struct PwGeom {
  int n[3];
  float bmin[3];
  float cell[3];       // L / n
  float inv_cell[3];   // n / L
};

PwGeom pw_geom(const baorec_ctx* c) {
  PwGeom g;
  const int n[3] = {c->n1, c->n2, c->n3};
  for (int a = 0; a < 3; ++a) {
    g.n[a] = n[a];
    g.bmin[a] = c->cfg.box_min[a];
    g.cell[a] = c->cfg.box_size[a] / (float)n[a];
    g.inv_cell[a] = (float)n[a] / c->cfg.box_size[a];
  }
  return g;
}

__device__ __forceinline__ int pw_wrap(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// Paint w * scale (w = 1 when null) at the grid coordinate
// (p - box_min) / cell + shift; out-of-box particles set kErrOOB when
// `survey` and are wrapped either way (memory stays in bounds).
template <int MAS>
__global__ void pw_paint_kernel(float* __restrict__ mesh, const float* __restrict__ x, const float* __restrict__ y,
                                const float* __restrict__ z, const float* __restrict__ w, int64_t n, PwGeom g,
                                float shift, float scale, int survey, unsigned* err) {
  constexpr int K = MAS == BAOREC_MAS_TSC ? 3 : 2;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const float p[3] = {x[q], y[q], z[q]};
    const float wt = (w ? w[q] : 1.0f) * scale;
    int idx[3][K];
    float wts[3][K];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float u = (p[a] - g.bmin[a]) * g.inv_cell[a] + shift;
      if (survey && !(u >= 0.0f && u < (float)g.n[a])) atomicOr(err, kErrOOB);
      if (MAS == BAOREC_MAS_TSC) {
        const float c = floorf(u + 0.5f);
        const float d = u - c;
        const int ic = (int)c;
        wts[a][0] = 0.5f * (0.5f - d) * (0.5f - d);
        wts[a][1] = 0.75f - d * d;
        wts[a][K - 1] = 0.5f * (0.5f + d) * (0.5f + d);
        idx[a][0] = pw_wrap(ic - 1, g.n[a]);
        idx[a][1] = pw_wrap(ic, g.n[a]);
        idx[a][K - 1] = pw_wrap(ic + 1, g.n[a]);
      } else {
        const float c = floorf(u);
        const float f = u - c;
        const int i0 = (int)c;
        wts[a][0] = 1.0f - f;
        wts[a][K - 1] = f;
        idx[a][0] = pw_wrap(i0, g.n[a]);
        idx[a][K - 1] = pw_wrap(i0 + 1, g.n[a]);
      }
    }
#pragma unroll
    for (int c = 0; c < K; ++c)
#pragma unroll
      for (int b = 0; b < K; ++b)
#pragma unroll
        for (int a = 0; a < K; ++a)
          atomicAdd(mesh + ((size_t)idx[2][c] * g.n[1] + idx[1][b]) * g.n[0] + idx[0][a],
                    wt * wts[0][a] * wts[1][b] * wts[2][c]);
  }
}

// FP64 block partials of Σw, Σw², Σ nz w² (w = 1 when null; nz optional)
__global__ void pw_sums_kernel(const float* __restrict__ w, const float* __restrict__ nz, int64_t n,
                               double* __restrict__ part) {
  __shared__ double sh[3][256];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const double v = w ? (double)w[q] : 1.0;
    s0 += v;
    s1 += v * v;
    if (nz) s2 += (double)nz[q] * v * v;
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 3) part[3 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// out = F * Π_q r̂_{ax[q]} (q < na) with r̂ the unit vector of the node
// position box_min + i cell (zero at the origin)
__global__ void pw_rhat_kernel(const float* __restrict__ F, float* __restrict__ out, PwGeom g, int na, int a0, int a1,
                               int a2, int a3) {
  const size_t N = (size_t)g.n[0] * g.n[1] * g.n[2];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.n[0]);
    const size_t r = e / g.n[0];
    const int j = (int)(r % g.n[1]), k = (int)(r / g.n[1]);
    const float p[3] = {g.bmin[0] + i * g.cell[0], g.bmin[1] + j * g.cell[1], g.bmin[2] + k * g.cell[2]};
    const float d = sqrtf(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    const float inv = d > 0.0f ? 1.0f / d : 0.0f;
    const int ax[4] = {a0, a1, a2, a3};
    float prod = 1.0f;
    for (int q = 0; q < na; ++q) prod *= p[ax[q]] * inv;
    out[e] = F[e] * prod;
  }
}

struct PwK {
  int n1h, n[3];
  float kf[3];     // 2π / L
  float cell[3];
};

// wave vector and half-spectrum multiplicity of mode e (x is the halved axis)
__device__ __forceinline__ void pw_mode(size_t e, const PwK& g, float kv[3], int& mult) {
  const int i = (int)(e % g.n1h);
  const size_t r = e / g.n1h;
  const int j = (int)(r % g.n[1]), k = (int)(r / g.n[1]);
  const int jj = j <= g.n[1] / 2 ? j : j - g.n[1];
  const int kk = k <= g.n[2] / 2 ? k : k - g.n[2];
  kv[0] = i * g.kf[0];
  kv[1] = jj * g.kf[1];
  kv[2] = kk * g.kf[2];
  mult = (i == 0 || (g.n[0] % 2 == 0 && i == g.n[0] / 2)) ? 1 : 2;
}

// A += c Π_q k̂_{ax[q]} S (the k = 0 mode contributes nothing)
__global__ void pw_accum_kernel(const cufftComplex* __restrict__ S, cufftComplex* __restrict__ A, PwK g, size_t nk,
                                int na, int a0, int a1, int a2, int a3, float c) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    float kv[3];
    int m;
    pw_mode(e, g, kv, m);
    const float kk = sqrtf(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
    if (!(kk > 0.0f)) continue;
    const int ax[4] = {a0, a1, a2, a3};
    float f = c;
    for (int q = 0; q < na; ++q) f *= kv[ax[q]] / kk;
    const cufftComplex s = S[e];
    cufftComplex a = A[e];
    a.x += f * s.x;
    a.y += f * s.y;
    A[e] = a;
  }
}

// interlacing: S1 = (S1 + S2 e^{i k·h}) / 2, h = half a cell on every axis
// (S2 painted at positions shifted by +h)
__global__ void pw_interlace_kernel(cufftComplex* __restrict__ S1, const cufftComplex* __restrict__ S2, PwK g,
                                    size_t nk) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    float kv[3];
    int m;
    pw_mode(e, g, kv, m);
    const float ph = 0.5f * (kv[0] * g.cell[0] + kv[1] * g.cell[1] + kv[2] * g.cell[2]);
    float sn, cs;
    sincosf(ph, &sn, &cs);
    const cufftComplex a = S1[e], b = S2[e];
    S1[e] = make_float2(0.5f * (a.x + cs * b.x - sn * b.y), 0.5f * (a.y + cs * b.y + sn * b.x));
  }
}

__device__ __forceinline__ double pw_sinc(double v) { return fabs(v) < 1e-8 ? 1.0 : sin(v) / v; }

// Shell sums per block: [k sum, modes, P0, P2, P4] x nbins FP64 in shared
// memory, written to part[block][5][nbins].  Box: P = |A0|²/I/W², μ = k̂·los.
// Survey: a_l = A_l / W, Yamamoto combinations.  Shot noise off P0.
__global__ void pw_bin_kernel(const cufftComplex* __restrict__ A0, const cufftComplex* __restrict__ A2,
                              const cufftComplex* __restrict__ A4, PwK g, size_t nk, int survey, float lx, float ly,
                              float lz, int wpow, float kmin, float dk, int nbins, double inv_norm, double shot,
                              double* __restrict__ part) {
  extern __shared__ double sb[];
  for (int q = threadIdx.x; q < 5 * nbins; q += blockDim.x) sb[q] = 0.0;
  __syncthreads();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nk; e += (size_t)gridDim.x * blockDim.x) {
    float kv[3];
    int m;
    pw_mode(e, g, kv, m);
    const double kx = kv[0], ky = kv[1], kz = kv[2];
    const double kk = sqrt(kx * kx + ky * ky + kz * kz);
    if (!(kk > 0.0)) continue;
    const int b = (int)floor((kk - (double)kmin) / (double)dk);
    if (b < 0 || b >= nbins) continue;
    double W = pw_sinc(0.5 * kx * g.cell[0]) * pw_sinc(0.5 * ky * g.cell[1]) * pw_sinc(0.5 * kz * g.cell[2]);
    W = wpow == 3 ? W * W * W : W * W;
    const double iw2 = 1.0 / (W * W);
    const cufftComplex a0 = A0[e];
    const double p00 = ((double)a0.x * a0.x + (double)a0.y * a0.y) * iw2 * inv_norm;
    double c0, c2, c4;
    if (!survey) {
      const double mu = (kx * lx + ky * ly + kz * lz) / kk, mu2 = mu * mu;
      c0 = p00 - shot;
      c2 = 5.0 * p00 * 0.5 * (3.0 * mu2 - 1.0);
      c4 = 9.0 * p00 * 0.125 * (35.0 * mu2 * mu2 - 30.0 * mu2 + 3.0);
    } else {
      const cufftComplex a2 = A2[e], a4 = A4[e];
      // Re[a0 conj(z)] = a0.x z.x + a0.y z.y
      const double z2x = 3.0 * a2.x - a0.x, z2y = 3.0 * a2.y - a0.y;
      const double z4x = 35.0 * a4.x - 30.0 * a2.x + 3.0 * a0.x, z4y = 35.0 * a4.y - 30.0 * a2.y + 3.0 * a0.y;
      c0 = p00 - shot;
      c2 = 2.5 * ((double)a0.x * z2x + (double)a0.y * z2y) * iw2 * inv_norm;
      c4 = 1.125 * ((double)a0.x * z4x + (double)a0.y * z4y) * iw2 * inv_norm;
    }
    atomicAdd(&sb[b], (double)m * kk);
    atomicAdd(&sb[nbins + b], (double)m);
    atomicAdd(&sb[2 * nbins + b], (double)m * c0);
    atomicAdd(&sb[3 * nbins + b], (double)m * c2);
    atomicAdd(&sb[4 * nbins + b], (double)m * c4);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < 5 * nbins; q += blockDim.x) part[(size_t)blockIdx.x * 5 * nbins + q] = sb[q];
}

constexpr unsigned kPwBlocks = 2 * kNumSMs;

}  // namespace
}  // namespace baorec

using namespace baorec;

extern "C" int baorec_power_multipoles(baorec_ctx* ctx, const baorec_power_config* pc, const float* x, const float* y,
                                       const float* z, const float* w, int64_t n, const float* rx, const float* ry,
                                       const float* rz, const float* rw, const float* rnz, int64_t nr, double* k_mean,
                                       double* p0, double* p2, double* p4, int64_t* nmodes, double* shot_out,
                                       double* norm_out, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (!pc || !k_mean || !p0 || !p2 || !p4 || !nmodes) return set_error(ctx, BAOREC_ERR_ARG, "power: missing argument");
  const bool survey = pc->geometry == BAOREC_POWER_SURVEY;
  if (pc->geometry != BAOREC_POWER_BOX && !survey) return set_error(ctx, BAOREC_ERR_ARG, "power: unknown geometry");
  if (pc->mas != BAOREC_MAS_CIC && pc->mas != BAOREC_MAS_TSC) return set_error(ctx, BAOREC_ERR_ARG, "power: unknown mas");
  if (pc->nbins < 1 || pc->nbins > 1024 || !(pc->dk > 0.0f) || !(pc->kmin >= 0.0f))
    return set_error(ctx, BAOREC_ERR_ARG, "power: need 1 <= nbins <= 1024, dk > 0, kmin >= 0");
  if (n < 1 || !x || !y || !z) return set_error(ctx, BAOREC_ERR_ARG, "power: empty or missing data catalog");
  if (nr < 0 || (nr > 0 && (!rx || !ry || !rz))) return set_error(ctx, BAOREC_ERR_ARG, "power: bad randoms");
  if (survey && (nr == 0 || !rnz)) return set_error(ctx, BAOREC_ERR_ARG, "power: the survey geometry needs randoms and their n(z)");
  if (survey && pc->interlace) return set_error(ctx, BAOREC_ERR_ARG, "power: interlacing is for the box geometry");
  double lv[3] = {pc->los[0], pc->los[1], pc->los[2]};
  const double ln = sqrt(lv[0] * lv[0] + lv[1] * lv[1] + lv[2] * lv[2]);
  if (!survey && !(ln > 0.0)) return set_error(ctx, BAOREC_ERR_ARG, "power: the box geometry needs a line of sight");
  if (!survey)
    for (double& v : lv) v /= ln;

  // particles on the device (slots 0-3 data, 4-7 randoms; n(z) in its own buffer)
  const float *dx, *dy, *dz, *dw = nullptr, *ex = nullptr, *ey = nullptr, *ez = nullptr, *ew = nullptr, *enz = nullptr;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  if (w) CKS(stage_in(ctx, 3, w, n, flags, &dw));
  if (nr > 0) {
    CKS(stage_in(ctx, 4, rx, nr, flags, &ex));
    CKS(stage_in(ctx, 5, ry, nr, flags, &ey));
    CKS(stage_in(ctx, 6, rz, nr, flags, &ez));
    if (rw) CKS(stage_in(ctx, 7, rw, nr, flags, &ew));
    if (rnz) {
      if (flags & BAOREC_HOST) {
        CKS(ensure(ctx, ctx->pw_nz, (size_t)nr * 4));
        CK(cudaMemcpyAsync(ctx->pw_nz.p, rnz, (size_t)nr * 4, cudaMemcpyHostToDevice, ctx->stream));
        enz = (const float*)ctx->pw_nz.p;
      } else {
        enz = rnz;
      }
    }
  }

  // FP64 sums: data Σw, Σw²; randoms Σw, Σw², Σ n(z) w²
  CKS(ensure(ctx, ctx->pw_part, (size_t)kPwBlocks * 5 * 1024 * sizeof(double)));
  double* part = (double*)ctx->pw_part.p;
  double sd[3] = {0, 0, 0}, sr[3] = {0, 0, 0};
  {
    std::vector<double> h(6 * kPwBlocks);
    (pw_sums_kernel<<<kPwBlocks, 256, 0, ctx->stream>>>(dw, nullptr, n, part), ::baorec::count_launch());
    CKLAUNCH();
    if (nr > 0) {
      (pw_sums_kernel<<<kPwBlocks, 256, 0, ctx->stream>>>(ew, enz, nr, part + 3 * kPwBlocks), ::baorec::count_launch());
      CKLAUNCH();
    }
    CK(cudaMemcpyAsync(h.data(), part, (nr > 0 ? 6 : 3) * kPwBlocks * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (unsigned b = 0; b < kPwBlocks; ++b)
      for (int c = 0; c < 3; ++c) {
        sd[c] += h[3 * b + c];
        if (nr > 0) sr[c] += h[3 * (kPwBlocks + b) + c];
      }
  }
  if (!(sd[0] > 0.0)) return set_error(ctx, BAOREC_ERR_ARG, "power: the data weights sum to %g", sd[0]);
  if (nr > 0 && !(sr[0] > 0.0)) return set_error(ctx, BAOREC_ERR_ARG, "power: the random weights sum to %g", sr[0]);
  const double alpha = nr > 0 ? sd[0] / sr[0] : 0.0;
  const double V = (double)ctx->cfg.box_size[0] * ctx->cfg.box_size[1] * ctx->cfg.box_size[2];
  const double norm = survey ? alpha * sr[2] : sd[0] * sd[0] / V;
  if (!(norm > 0.0)) return set_error(ctx, BAOREC_ERR_ARG, "power: normalisation %g (check the randoms' n(z))", norm);
  const double shot = (sd[1] + alpha * alpha * sr[1]) / norm;

  // scratch: two meshes, four half spectra (A0, A2, A4, S)
  const size_t N = ctx->N, Nk = ctx->Nk;
  CKS(ensure(ctx, ctx->pw_mesh, 2 * N * sizeof(float)));
  CKS(ensure(ctx, ctx->pw_spec, 4 * Nk * sizeof(cufftComplex)));
  float* F = (float*)ctx->pw_mesh.p;
  float* M2 = F + N;
  cufftComplex* A0 = (cufftComplex*)ctx->pw_spec.p;
  cufftComplex* A2 = A0 + Nk;
  cufftComplex* A4 = A2 + Nk;
  cufftComplex* S = A4 + Nk;
  const PwGeom g = pw_geom(ctx);
  PwK kg;
  kg.n1h = ctx->n1h;
  kg.n[0] = ctx->n1;
  kg.n[1] = ctx->n2;
  kg.n[2] = ctx->n3;
  for (int a = 0; a < 3; ++a) {
    kg.kf[a] = (float)(2.0 * M_PI / (double)ctx->cfg.box_size[a]);
    kg.cell[a] = g.cell[a];
  }
  const unsigned pgrid = 64u * kNumSMs;
  auto paint_all = [&](float* mesh, float shift) -> int {
    CK(cudaMemsetAsync(mesh, 0, N * sizeof(float), ctx->stream));
    if (pc->mas == BAOREC_MAS_TSC) {
      (pw_paint_kernel<BAOREC_MAS_TSC><<<pgrid, 256, 0, ctx->stream>>>(mesh, dx, dy, dz, dw, n, g, shift, 1.0f,
                                                                     survey, ctx->derr), ::baorec::count_launch());
      CKLAUNCH();
      if (nr > 0) {
        (pw_paint_kernel<BAOREC_MAS_TSC><<<pgrid, 256, 0, ctx->stream>>>(mesh, ex, ey, ez, ew, nr, g, shift,
                                                                       (float)-alpha, survey, ctx->derr), ::baorec::count_launch());
        CKLAUNCH();
      }
    } else {
      (pw_paint_kernel<BAOREC_MAS_CIC><<<pgrid, 256, 0, ctx->stream>>>(mesh, dx, dy, dz, dw, n, g, shift, 1.0f,
                                                                     survey, ctx->derr), ::baorec::count_launch());
      CKLAUNCH();
      if (nr > 0) {
        (pw_paint_kernel<BAOREC_MAS_CIC><<<pgrid, 256, 0, ctx->stream>>>(mesh, ex, ey, ez, ew, nr, g, shift,
                                                                       (float)-alpha, survey, ctx->derr), ::baorec::count_launch());
        CKLAUNCH();
      }
    }
    return BAOREC_OK;
  };
  const unsigned eg = 8u * kNumSMs;
  CKS(paint_all(F, 0.0f));
  CKFFT(cufftExecR2C(ctx->plan_r2c, F, A0));
  if (!survey && pc->interlace) {
    CKS(paint_all(M2, 0.5f));
    CKFFT(cufftExecR2C(ctx->plan_r2c, M2, S));
    (pw_interlace_kernel<<<eg, 256, 0, ctx->stream>>>(A0, S, kg, Nk), ::baorec::count_launch());
    CKLAUNCH();
  }
  if (survey) {
    CK(cudaMemsetAsync(A2, 0, 2 * Nk * sizeof(cufftComplex), ctx->stream));   // A2 and A4
    // quadrupole: the 6 index pairs i <= j, off-diagonal ones twice
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        (pw_rhat_kernel<<<eg, 256, 0, ctx->stream>>>(F, M2, g, 2, i, j, 0, 0), ::baorec::count_launch());
        CKLAUNCH();
        CKFFT(cufftExecR2C(ctx->plan_r2c, M2, S));
        (pw_accum_kernel<<<eg, 256, 0, ctx->stream>>>(S, A2, kg, Nk, 2, i, j, 0, 0, i == j ? 1.0f : 2.0f), ::baorec::count_launch());
        CKLAUNCH();
      }
    // hexadecapole: the 15 multisets i <= j <= k <= l with their 4!/(a! b! c!) orderings
    const int fact[5] = {1, 1, 2, 6, 24};
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j)
        for (int k = j; k < 3; ++k)
          for (int l = k; l < 3; ++l) {
            int cnt[3] = {0, 0, 0};
            cnt[i]++;
            cnt[j]++;
            cnt[k]++;
            cnt[l]++;
            const float c = (float)(24 / (fact[cnt[0]] * fact[cnt[1]] * fact[cnt[2]]));
            (pw_rhat_kernel<<<eg, 256, 0, ctx->stream>>>(F, M2, g, 4, i, j, k, l), ::baorec::count_launch());
            CKLAUNCH();
            CKFFT(cufftExecR2C(ctx->plan_r2c, M2, S));
            (pw_accum_kernel<<<eg, 256, 0, ctx->stream>>>(S, A4, kg, Nk, 4, i, j, k, l, c), ::baorec::count_launch());
            CKLAUNCH();
          }
  }
  const int nb = pc->nbins;
  (pw_bin_kernel<<<kPwBlocks, 256, 5 * nb * sizeof(double), ctx->stream>>>(
      A0, A2, A4, kg, Nk, survey ? 1 : 0, (float)lv[0], (float)lv[1], (float)lv[2], pc->mas == BAOREC_MAS_TSC ? 3 : 2,
      pc->kmin, pc->dk, nb, 1.0 / norm, shot, part), ::baorec::count_launch());
  CKLAUNCH();
  std::vector<double> h((size_t)kPwBlocks * 5 * nb);
  CK(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CKS(finish(ctx, 0));
  for (int b = 0; b < nb; ++b) {
    double s[5] = {0, 0, 0, 0, 0};
    for (unsigned q = 0; q < kPwBlocks; ++q)
      for (int c = 0; c < 5; ++c) s[c] += h[((size_t)q * 5 + c) * nb + b];
    const double m = s[1];
    nmodes[b] = (int64_t)llround(m);
    k_mean[b] = m > 0 ? s[0] / m : 0.0;
    p0[b] = m > 0 ? s[2] / m : 0.0;
    p2[b] = m > 0 ? s[3] / m : 0.0;
    p4[b] = m > 0 ? s[4] / m : 0.0;
  }
  if (shot_out) *shot_out = shot;
  if (norm_out) *norm_out = norm;
  return BAOREC_OK;
}
