// Multigrid for the anisotropic reconstruction operator (src/multigrid.jl).
//
// Operator on a level with cell sizes c_a and per-axis tables p_a
// (x_vec / cell for the local line of sight, los / cell for a global one):
//   g = β / Σ c_a² p_a²,  gp_a = 1/c_a² + g p_a²
//   (A v)_0 = 2 Σ gp_a v_0 − [ Σ gp_a (v_{+a} + v_{−a})
//             + g/2 Σ_{a<b} p_a p_b (v_{++} + v_{−−} − v_{−+} − v_{+−})
//             + (local only) g Σ p_a (v_{+a} − v_{−a}) ]        (periodic)
// The neighbour coefficients sum to the diagonal, so A annihilates constants:
// the periodic system is singular.
//
// Two solvers:
//  * reference schedule (src/multigrid.jl:654-752): FMG with damped Jacobi
//    (ω, ν sweeps), `vcycle_niterations` V-cycles per level, FP32;
//  * convergent (no reference counterpart): defect correction
//        r_k = f − α_k − A v_k,  α_{k+1} = α_k + mean(r_k),
//        v_{k+1} = v_k + V(r_k − mean(r_k))
//    with v held as a double-float pair (hi + lo) on the finest level and
//    r_k evaluated in difference form, so the relative residual can reach
//    1e-6 although every mesh is FP32.  The shift α converges to the value
//    that makes the singular system consistent.  V is one V-cycle with
//    red-black Gauss-Seidel smoothing on the operator whose first-derivative
//    coefficients are clamped to |g p_a| <= κ gp_a (only cells next to the
//    observer change), an FP64 shared-memory solve on the coarsest level.
#include <math.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "mg_common.cuh"

namespace baorec {
namespace {

constexpr int kCoarseSweeps = 200;   // FP64 red-black sweeps on the coarsest level (fallback)
constexpr int kCoarseMaxCells = 2048;
// ---- reference-schedule kernels -------------------------------------------

// One damped-Jacobi sweep (src/multigrid.jl:137-191, 207): out = (1-ω)v + ω jac.
__global__ void jacobi_kernel(const float* __restrict__ v, const float* __restrict__ f, float* __restrict__ out,
                              LG G, float omega, size_t N) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, G.n, i, j, k);
    Coef c = coef_at(G, i, j, k);
    Nb b = gather([&](int a, int bb, int cc) { return v[at(G.n, a, bb, cc)]; }, G.n, i, j, k);
    float jac = f[e] + offdiag(c, b, G.local);
    jac /= 2.0f * (c.gpx + c.gpy + c.gpz);
    out[e] = (1.0f - omega) * v[e] + omega * jac;
  }
}

// r = f - A v (src/multigrid.jl:328-376, 393).
__global__ void residual_kernel(const float* __restrict__ v, const float* __restrict__ f, float* __restrict__ r,
                                LG G, size_t N, float shift, float* __restrict__ acc = nullptr) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, G.n, i, j, k);
    Coef c = coef_at(G, i, j, k);
    Nb b = gather([&](int a, int bb, int cc) { return v[at(G.n, a, bb, cc)]; }, G.n, i, j, k);
    float av = 2.0f * (c.gpx + c.gpy + c.gpz) * v[e] - offdiag(c, b, G.local);
    r[e] = (f[e] - shift) - av;
    if (acc) acc[e] += v[e];
  }
}

// r = f - A v over differences v_nb - v_0 (accurate for smooth v); acc += v
__global__ void residual_diff_kernel(const float* __restrict__ v, const float* __restrict__ f, float* __restrict__ r,
                                     LG G, size_t N, float* __restrict__ acc) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, G.n, i, j, k);
    Coef c = coef_at(G, i, j, k);
    const float v0 = v[e];
    Nb b = gather([&](int a, int bb, int cc) { return v[at(G.n, a, bb, cc)] - v0; }, G.n, i, j, k);
    r[e] = f[e] + offdiag(c, b, G.local);
    if (acc) acc[e] += v0;
  }
}

__global__ void add_kernel(float* __restrict__ a, const float* __restrict__ b, size_t N) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    a[e] += b[e];
}

// Per-block (Σf, Σf²) in FP64 (four-cell FP32 partial sums) for the norm
// |f - α| and the shift α = mean f of the residual-driven solve.
__global__ void sum_sumsq_partial_kernel(const float* __restrict__ a, size_t N, double* __restrict__ part) {
  double s1 = 0.0, s2 = 0.0;
  const size_t N4 = ((uintptr_t)a % 16 == 0) ? N / 4 : 0;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N4; e += (size_t)gridDim.x * blockDim.x) {
    const float4 u = a4[e];
    s1 += (double)((u.x + u.y) + (u.z + u.w));
    s2 += (double)((u.x * u.x + u.y * u.y) + (u.z * u.z + u.w * u.w));
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    const double v = (double)a[e];
    s1 += v;
    s2 += v * v;
  }
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
    part[2 * blockIdx.x] = t1;
    part[2 * blockIdx.x + 1] = t2;
  }
}

// r = f - α with α = Σf / N from the nb partials of sum_sumsq_partial_kernel:
// the residual of a zero solution, as the accurate residual kernel would
// compute it ((f - α) + a bracket of zero differences), formed without the
// host reading the sums first.
__global__ void shift_mean_kernel(const float* __restrict__ f, float* __restrict__ r, size_t N,
                                  const double* __restrict__ part, int nb) {
  __shared__ double red[32];
  __shared__ float alpha_s;
  double t = 0.0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) t += part[2 * k];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) sum += red[k];
    alpha_s = (float)(sum / (double)N);
  }
  __syncthreads();
  const float alpha = alpha_s;
  const size_t N4 = ((uintptr_t)f % 16 == 0 && (uintptr_t)r % 16 == 0) ? N / 4 : 0;
  const float4* f4 = reinterpret_cast<const float4*>(f);
  float4* r4 = reinterpret_cast<float4*>(r);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N4; e += (size_t)gridDim.x * blockDim.x) {
    const float4 u = f4[e];
    r4[e] = make_float4(u.x - alpha, u.y - alpha, u.z - alpha, u.w - alpha);
  }
  for (size_t e = 4 * N4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x)
    r[e] = f[e] - alpha;
}

// Full-weighting restriction (src/multigrid.jl:586-640): coarse c centred on fine 2c+1.
__global__ void reduce_kernel(const float* __restrict__ fine, float* __restrict__ coarse, int3 nf, int3 nc,
                              size_t Nc) {
  const int nfa[3] = {nf.x, nf.y, nf.z};
  const int nca[3] = {nc.x, nc.y, nc.z};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < Nc; e += (size_t)gridDim.x * blockDim.x) {
    int ci, cj, ck; cell_ijk(e, nca, ci, cj, ck);
    int i = 2 * ci + 1, j = 2 * cj + 1, k = 2 * ck + 1;
    int ip = i + 1 == nf.x ? 0 : i + 1, im = i - 1;
    int jp = j + 1 == nf.y ? 0 : j + 1, jm = j - 1;
    int kp = k + 1 == nf.z ? 0 : k + 1, km = k - 1;
    auto F = [&](int a, int b, int c) { return fine[at(nfa, a, b, c)]; };
    float s = 8.0f * F(i, j, k) +
              4.0f * (F(ip, j, k) + F(im, j, k) + F(i, jp, k) + F(i, jm, k) + F(i, j, kp) + F(i, j, km)) +
              2.0f * (F(ip, jp, k) + F(im, jp, k) + F(ip, jm, k) + F(im, jm, k) + F(ip, j, kp) + F(im, j, kp) +
                      F(ip, j, km) + F(im, j, km) + F(i, jp, kp) + F(i, jm, kp) + F(i, jp, km) + F(i, jm, km)) +
              F(ip, jp, kp) + F(im, jp, kp) + F(ip, jm, kp) + F(im, jm, kp) + F(ip, jp, km) + F(im, jp, km) +
              F(ip, jm, km) + F(im, jm, km);
    coarse[e] = s / 64.0f;
  }
}

// Trilinear prolongation (src/multigrid.jl:456-509): coarse c → fine 2c+1,
// midpoints 2c+2 (periodic).  add != 0 adds into fine (v += prolong(v2h)).
__global__ void prolong_kernel(const float* __restrict__ coarse, float* __restrict__ fine, int3 nc, int3 nf,
                               size_t Nc, int add) {
  const int nfa[3] = {nf.x, nf.y, nf.z};
  const int nca[3] = {nc.x, nc.y, nc.z};
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < Nc; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, nca, i, j, k);
    int ip = i + 1 == nc.x ? 0 : i + 1, jp = j + 1 == nc.y ? 0 : j + 1, kp = k + 1 == nc.z ? 0 : k + 1;
    auto C = [&](int a, int b, int c) { return coarse[at(nca, a, b, c)]; };
    float c000 = C(i, j, k), c100 = C(ip, j, k), c010 = C(i, jp, k), c001 = C(i, j, kp);
    float c110 = C(ip, jp, k), c011 = C(i, jp, kp), c101 = C(ip, j, kp), c111 = C(ip, jp, kp);
    int x0 = 2 * i + 1, y0 = 2 * j + 1, z0 = 2 * k + 1;
    int x1 = x0 + 1 == nf.x ? 0 : x0 + 1, y1 = y0 + 1 == nf.y ? 0 : y0 + 1, z1 = z0 + 1 == nf.z ? 0 : z0 + 1;
    float v[8] = {c000,
                  (c000 + c100) / 2.0f,
                  (c000 + c010) / 2.0f,
                  (c000 + c001) / 2.0f,
                  (c000 + c100 + c010 + c110) / 4.0f,
                  (c000 + c010 + c001 + c011) / 4.0f,
                  (c000 + c100 + c001 + c101) / 4.0f,
                  (c000 + c100 + c010 + c001 + c110 + c101 + c011 + c111) / 8.0f};
    size_t o[8] = {at(nfa, x0, y0, z0), at(nfa, x1, y0, z0), at(nfa, x0, y1, z0), at(nfa, x0, y0, z1),
                   at(nfa, x1, y1, z0), at(nfa, x0, y1, z1), at(nfa, x1, y0, z1), at(nfa, x1, y1, z1)};
#pragma unroll
    for (int q = 0; q < 8; ++q) fine[o[q]] = add ? fine[o[q]] + v[q] : v[q];
  }
}

// ---- convergent-solver kernels --------------------------------------------

// Half of a red-black Gauss-Seidel sweep, out of place: cells of `colour`
// ((i+j+k) mod 2) get (rhs - shift + neighbours(in)) / diag, the others copy.
__global__ void rb_half_kernel(const float* __restrict__ in, float* __restrict__ out, const float* __restrict__ rhs,
                               LG G, size_t N, int colour, float shift) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, G.n, i, j, k);
    if (((i + j + k) & 1) != colour) { out[e] = in[e]; continue; }
    Coef c = coef_at(G, i, j, k);
    Nb b = gather([&](int a, int bb, int cc) { return in[at(G.n, a, bb, cc)]; }, G.n, i, j, k);
    out[e] = (rhs[e] - shift + offdiag(c, b, G.local)) / (2.0f * (c.gpx + c.gpy + c.gpz));
  }
}
// Accurate residual with the exact (unclamped) operator, fused with the
// solution update v' = v + e:  r = (f - α) + [neighbour bracket in differences
// D = v_nb - v_0].  Writes hi', lo', r and FP64 block partials (Σr, Σr²).
__global__ void resid_acc_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                                 const float* __restrict__ e_corr, const float* __restrict__ f,
                                 float* __restrict__ ohi, float* __restrict__ olo, float* __restrict__ r,
                                 LG G, size_t N, float alpha, double* __restrict__ part) {
  double s1 = 0.0, s2 = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k; cell_ijk(e, G.n, i, j, k);
    Coef c = coef_at(G, i, j, k);
    auto V = [&](int a, int bb, int cc, float& h, float& l) {
      size_t q = at(G.n, a, bb, cc);
      h = hi[q]; l = lo[q];
      if (e_corr) df_add(h, l, e_corr[q], h, l);
    };
    float h0, l0;
    V(i, j, k, h0, l0);
    // (h_u - h_0, l_u - l_0) of every neighbour, combined by dd_sum2 / dd_cross / dd_diff2
    auto Dh = [&](int a, int bb, int cc) {
      float h, l; V(a, bb, cc, h, l);
      return __fsub_rn(h, h0);
    };
    auto Dl = [&](int a, int bb, int cc) {
      float h, l; V(a, bb, cc, h, l);
      return __fsub_rn(l, l0);
    };
    const Nb bh = gather(Dh, G.n, i, j, k), bl = gather(Dl, G.n, i, j, k);
    auto P = [](float h, float l) { return make_float2(h, l); };
    // −A v expressed with differences (the constant terms cancel)
    float br = c.gpx * dd_sum2(P(bh.xp, bl.xp), P(bh.xm, bl.xm)) + c.gpy * dd_sum2(P(bh.yp, bl.yp), P(bh.ym, bl.ym)) +
               c.gpz * dd_sum2(P(bh.zp, bl.zp), P(bh.zm, bl.zm)) +
               c.g / 2.0f *
                   (c.pxy * dd_cross(P(bh.pp0, bl.pp0), P(bh.mm0, bl.mm0), P(bh.mp0, bl.mp0), P(bh.pm0, bl.pm0)) +
                    c.pxz * dd_cross(P(bh.p0p, bl.p0p), P(bh.m0m, bl.m0m), P(bh.m0p, bl.m0p), P(bh.p0m, bl.p0m)) +
                    c.pyz * dd_cross(P(bh._pp, bl._pp), P(bh._mm, bl._mm), P(bh._mp, bl._mp), P(bh._pm, bl._pm)));
    if (G.local)
      br += c.dx * dd_diff2(P(bh.xp, bl.xp), P(bh.xm, bl.xm)) + c.dy * dd_diff2(P(bh.yp, bl.yp), P(bh.ym, bl.ym)) +
            c.dz * dd_diff2(P(bh.zp, bl.zp), P(bh.zm, bl.zm));
    float rv = (f[e] - alpha) + br;
    ohi[e] = h0;
    olo[e] = l0;
    r[e] = rv;
    s1 += (double)rv;
    s2 += (double)rv * (double)rv;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double sh[2][32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = s1; sh[1][wid] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b2 = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += sh[0][q]; b2 += sh[1][q]; }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b2;
  }
}

// FP64 red-black solve of the coarsest level in one block (shared memory):
// mean-free right-hand side, kCoarseSweeps sweeps, mean-free solution.
__global__ void coarse_solve_kernel(const float* __restrict__ rhs, float* __restrict__ v, LG G, int sweeps) {
  extern __shared__ double sm[];
  const int N = G.n[0] * G.n[1] * G.n[2];
  double* sv = sm;
  double* sf = sm + N;
  __shared__ double red[32];
  // mean of rhs
  double loc = 0.0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) { sf[e] = rhs[e]; loc += sf[e]; sv[e] = 0.0; }
  for (int o = 16; o > 0; o >>= 1) loc += __shfl_xor_sync(0xffffffffu, loc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    red[0] = t / N;
  }
  __syncthreads();
  const double mean = red[0];
  for (int e = threadIdx.x; e < N; e += blockDim.x) sf[e] -= mean;
  __syncthreads();
  // each thread owns at most kCoarseMaxCells / blockDim cells; new values are
  // staged in registers so same-colour (edge) neighbours read pre-update values
  constexpr int kPer = kCoarseMaxCells / 256;
  for (int s = 0; s < sweeps; ++s) {
    for (int colour = 0; colour < 2; ++colour) {
      double nv[kPer];
      int q = 0;
      for (int e = threadIdx.x; e < N; e += blockDim.x, ++q) {
        int i, j, k; cell_ijk((size_t)e, G.n, i, j, k);
        nv[q] = sv[e];
        if (((i + j + k) & 1) != colour) continue;
        Coef c = coef_at(G, i, j, k);
        int ip = i + 1 == G.n[0] ? 0 : i + 1, im = i == 0 ? G.n[0] - 1 : i - 1;
        int jp = j + 1 == G.n[1] ? 0 : j + 1, jm = j == 0 ? G.n[1] - 1 : j - 1;
        int kp = k + 1 == G.n[2] ? 0 : k + 1, km = k == 0 ? G.n[2] - 1 : k - 1;
        auto S = [&](int a, int bb, int cc) { return sv[at(G.n, a, bb, cc)]; };
        double o = (double)c.gpx * (S(ip, j, k) + S(im, j, k)) + (double)c.gpy * (S(i, jp, k) + S(i, jm, k)) +
                   (double)c.gpz * (S(i, j, kp) + S(i, j, km)) +
                   (double)c.g / 2.0 *
                       ((double)c.pxy * (S(ip, jp, k) + S(im, jm, k) - S(im, jp, k) - S(ip, jm, k)) +
                        (double)c.pxz * (S(ip, j, kp) + S(im, j, km) - S(im, j, kp) - S(ip, j, km)) +
                        (double)c.pyz * (S(i, jp, kp) + S(i, jm, km) - S(i, jm, kp) - S(i, jp, km)));
        if (G.local)
          o += (double)c.dx * (S(ip, j, k) - S(im, j, k)) + (double)c.dy * (S(i, jp, k) - S(i, jm, k)) +
               (double)c.dz * (S(i, j, kp) - S(i, j, km));
        nv[q] = (sf[e] + o) / (2.0 * ((double)c.gpx + (double)c.gpy + (double)c.gpz));
      }
      __syncthreads();
      q = 0;
      for (int e = threadIdx.x; e < N; e += blockDim.x, ++q) sv[e] = nv[q];
      __syncthreads();
    }
  }
  loc = 0.0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) loc += sv[e];
  for (int o = 16; o > 0; o >>= 1) loc += __shfl_xor_sync(0xffffffffu, loc, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    red[0] = t / N;
  }
  __syncthreads();
  const double vm = red[0];
  for (int e = threadIdx.x; e < N; e += blockDim.x) v[e] = (float)(sv[e] - vm);
}

// Coarsest level: v = M rhs with M the top-left block of the inverse of the
// bordered matrix [[A, 1], [1ᵀ, 0]] (FP64, precomputed on the host), i.e. the
// mean-free solution of A v + λ1 = rhs.  M 1 = 0, so a constant shift of the
// right-hand side does not change v.
__global__ void coarse_dense_kernel(const double* __restrict__ M, const float* __restrict__ rhs, float* __restrict__ v,
                                    int N) {
  for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < N; i += blockDim.x * gridDim.x) {
    double s = 0.0;
    const double* row = M + (size_t)i * N;
    for (int j = 0; j < N; ++j) s += row[j] * (double)rhs[j];
    v[i] = (float)s;
  }
}

LG level_geom(const baorec_ctx* ctx, int l, float clamp) {
  const baorec::Level& L = ctx->lev[l];
  LG G;
  for (int a = 0; a < 3; ++a) {
    G.n[a] = L.n[a];
    float cell = ctx->cfg.box_size[a] / (float)L.n[a];
    G.cell2[a] = cell * cell;
    G.icell2[a] = 1.0f / G.cell2[a];
    G.P[a] = L.ax[a];   // the level's p tables (x_vec / cell)
    G.pg[a] = ctx->cfg.los[a] / cell;
  }
  G.beta = ctx->cfg.beta;
  G.local = ctx->cfg.los_mode == BAOREC_LOS_LOCAL ? 1 : 0;
  G.clamp = clamp;
  G.tile16 = l < 16 ? ctx->tune.big_tiles[l] : -1;
  G.pairs = ctx->tune.pairs;
  G.accf = ctx->tune.acc;
  G.err = ctx->derr;
  return G;
}

int level_of(const baorec_ctx* ctx, const int nl[3]) {
  for (int l = 0; l < ctx->nlev; ++l)
    if (ctx->lev[l].n[0] == nl[0] && ctx->lev[l].n[1] == nl[1] && ctx->lev[l].n[2] == nl[2]) return l;
  return -1;
}

bool can_recurse(const int n[3]) {
  for (int a = 0; a < 3; ++a)
    if (!(n[a] > 4 && n[a] % 2 == 0)) return false;
  return true;
}

unsigned blocks_for(size_t N) {
  unsigned g = grid_for(N, 256);
  return g > 32u * kNumSMs ? 32u * kNumSMs : g;
}

constexpr int kResBlocks = 2 * kNumSMs;
constexpr size_t kMaxPartials = kRedCapacity / 2;   // blocks whose (Σr, Σr²) fit the partials buffer
constexpr int kDenseMaxCells = 512;                  // coarsest levels up to 8^3 use the dense inverse
constexpr int kSpectralInnerMax = 6;                 // FFT corrections per accurate residual, at most
constexpr int kSpectralFirst = 4;                    // FFT corrections in the first outer step
constexpr double kSpectralRateFloor = 0.1;           // planning never assumes a faster contraction

}  // namespace

int coarse_setup(baorec_ctx* ctx);

// Allocate the level hierarchy and the per-level p tables (x_vec / cell of
// src/utils.jl:21-25 with that level's cell size, rounded to FP32).
int mg_setup(baorec_ctx* ctx) {
  if (ctx->nlev > 0) return BAOREC_OK;
  int n[3] = {ctx->n1, ctx->n2, ctx->n3};
  int l = 0;
  while (true) {
    baorec::Level& L = ctx->lev[l];
    for (int a = 0; a < 3; ++a) L.n[a] = n[a];
    L.N = (size_t)n[0] * n[1] * n[2];
    CK(cudaMalloc(&L.f, L.N * 4 * 4));   // f, v, r, t contiguous
    L.v = L.f + L.N;
    L.r = L.v + L.N;
    for (int a = 0; a < 3; ++a) CK(cudaMalloc(&L.ax[a], (size_t)n[a] * 4));
    ++l;
    if (!can_recurse(n) || l == 16) break;
    for (int a = 0; a < 3; ++a) n[a] /= 2;
  }
  ctx->nlev = l;
  const size_t N0 = ctx->lev[0].N;
  CK(cudaMalloc(&ctx->phi_lo, N0 * 4 * 3));
  ctx->phi_lo2 = ctx->phi_lo + N0;
  ctx->phi_hi2 = ctx->phi_lo2 + N0;
  return mg_update_tables(ctx);
}

int mg_update_tables(baorec_ctx* ctx) {
  for (int l = 0; l < ctx->nlev; ++l) {
    baorec::Level& L = ctx->lev[l];
    for (int a = 0; a < 3; ++a) {
      std::vector<float> t(L.n[a]);
      float cell = ctx->cfg.box_size[a] / (float)L.n[a];
      for (int i = 0; i < L.n[a]; ++i) {
        float xv = (float)((double)ctx->cfg.box_min[a] + ((double)i + 0.5) * (double)cell);
        t[i] = xv / cell;
      }
      CK(cudaMemcpy(L.ax[a], t.data(), t.size() * 4, cudaMemcpyHostToDevice));
      L.ptab[a] = t;
    }
    // Does any cell of this level need its first-derivative coefficient
    // clamped (|g p_a| > κ gp_a)?  |g p_a| <= β / (c² |p|) and κ gp_a >= κ / c²,
    // so only cells with |p| < β/κ can: search the cells near the observer.
    L.needs_clamp = false;
    if (ctx->cfg.los_mode == BAOREC_LOS_LOCAL) {
      const float lim = ctx->cfg.beta / kClamp + 1.0f;
      std::vector<int> near[3];
      for (int a = 0; a < 3; ++a)
        for (int i = 0; i < L.n[a]; ++i)
          if (fabsf(L.ptab[a][i]) < lim) near[a].push_back(i);
      float c2[3], ic2[3];
      for (int a = 0; a < 3; ++a) {
        float cell = ctx->cfg.box_size[a] / (float)L.n[a];
        c2[a] = cell * cell;
        ic2[a] = 1.0f / c2[a];
      }
      for (int i : near[0])
        for (int j : near[1])
          for (int k : near[2]) {
            const float p[3] = {L.ptab[0][i], L.ptab[1][j], L.ptab[2][k]};
            const float g = ctx->cfg.beta / (c2[0] * p[0] * p[0] + c2[1] * p[1] * p[1] + c2[2] * p[2] * p[2]);
            for (int a = 0; a < 3; ++a)
              if (fabsf(g * p[a]) > kClamp * (ic2[a] + g * p[a] * p[a])) L.needs_clamp = true;
          }
    }
  }
  // the dense inverse is built when a V-cycle first needs it (a box change
  // between spectral-only solves costs no host elimination)
  if (ctx->coarse_M) { cudaFree(ctx->coarse_M); ctx->coarse_M = nullptr; }
  ctx->coarse_dirty = true;
  return BAOREC_OK;
}

// Dense FP64 inverse for the coarsest level (the "FP64 coarsest solve"): the
// matrix of the V-cycle operator (clamped first-derivative coefficients, as
// the smoother uses), bordered by a row and a column of ones so that the
// singular periodic system becomes A v + λ1 = rhs with Σv = 0; inverted by
// Gauss-Jordan elimination with partial pivoting.  Geometry only: recomputed
// when the box changes.
int coarse_setup(baorec_ctx* ctx) {
  ctx->coarse_dirty = false;
  if (ctx->coarse_M) { cudaFree(ctx->coarse_M); ctx->coarse_M = nullptr; }
  // the first level small enough for the dense inverse ends the residual-driven V-cycles
  ctx->dense_level = -1;
  for (int l = 0; l < ctx->nlev; ++l)
    if (ctx->lev[l].N <= (size_t)kDenseMaxCells) { ctx->dense_level = l; break; }
  if (ctx->dense_level < 0) return BAOREC_OK;
  const baorec::Level& C = ctx->lev[ctx->dense_level];
  const int N = (int)C.N;
  const int n0 = C.n[0], n1 = C.n[1], n2 = C.n[2];
  const bool local = ctx->cfg.los_mode == BAOREC_LOS_LOCAL;
  float cell[3], cell2[3], icell2[3], pg[3];
  std::vector<float> P[3];
  for (int a = 0; a < 3; ++a) {
    cell[a] = ctx->cfg.box_size[a] / (float)C.n[a];
    cell2[a] = cell[a] * cell[a];
    icell2[a] = 1.0f / cell2[a];
    pg[a] = ctx->cfg.los[a] / cell[a];
    P[a].resize(C.n[a]);
    for (int i = 0; i < C.n[a]; ++i) {
      float xv = (float)((double)ctx->cfg.box_min[a] + ((double)i + 0.5) * (double)cell[a]);
      P[a][i] = xv / cell[a];
    }
  }
  const int B = N + 1;
  std::vector<double> A((size_t)B * B, 0.0), Inv((size_t)B * B, 0.0);
  auto id = [&](int i, int j, int k) {
    i = (i + n0) % n0; j = (j + n1) % n1; k = (k + n2) % n2;
    return i + n0 * (j + n1 * k);
  };
  for (int k = 0; k < n2; ++k)
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n0; ++i) {
        const int r = id(i, j, k);
        const float px = local ? P[0][i] : pg[0], py = local ? P[1][j] : pg[1], pz = local ? P[2][k] : pg[2];
        const float g = ctx->cfg.beta / (cell2[0] * px * px + cell2[1] * py * py + cell2[2] * pz * pz);
        const float gp[3] = {icell2[0] + g * px * px, icell2[1] + g * py * py, icell2[2] + g * pz * pz};
        float d[3] = {0.0f, 0.0f, 0.0f};
        if (local) {
          const float p[3] = {px, py, pz};
          for (int a = 0; a < 3; ++a) d[a] = fminf(fmaxf(g * p[a], -kClamp * gp[a]), kClamp * gp[a]);
        }
        double* row = &A[(size_t)r * B];
        row[r] += 2.0 * ((double)gp[0] + gp[1] + gp[2]);
        row[id(i + 1, j, k)] -= (double)gp[0] + d[0];
        row[id(i - 1, j, k)] -= (double)gp[0] - d[0];
        row[id(i, j + 1, k)] -= (double)gp[1] + d[1];
        row[id(i, j - 1, k)] -= (double)gp[1] - d[1];
        row[id(i, j, k + 1)] -= (double)gp[2] + d[2];
        row[id(i, j, k - 1)] -= (double)gp[2] - d[2];
        const double hxy = 0.5 * g * px * py, hxz = 0.5 * g * px * pz, hyz = 0.5 * g * py * pz;
        row[id(i + 1, j + 1, k)] -= hxy; row[id(i - 1, j - 1, k)] -= hxy;
        row[id(i - 1, j + 1, k)] += hxy; row[id(i + 1, j - 1, k)] += hxy;
        row[id(i + 1, j, k + 1)] -= hxz; row[id(i - 1, j, k - 1)] -= hxz;
        row[id(i - 1, j, k + 1)] += hxz; row[id(i + 1, j, k - 1)] += hxz;
        row[id(i, j + 1, k + 1)] -= hyz; row[id(i, j - 1, k - 1)] -= hyz;
        row[id(i, j - 1, k + 1)] += hyz; row[id(i, j + 1, k - 1)] += hyz;
        row[N] = 1.0;
        A[(size_t)N * B + r] = 1.0;
      }
  for (int i = 0; i < B; ++i) Inv[(size_t)i * B + i] = 1.0;
  for (int c = 0; c < B; ++c) {
    int piv = c;
    for (int r = c + 1; r < B; ++r)
      if (fabs(A[(size_t)r * B + c]) > fabs(A[(size_t)piv * B + c])) piv = r;
    if (fabs(A[(size_t)piv * B + c]) < 1e-300) return set_error(ctx, BAOREC_ERR_ARG, "coarsest multigrid level is singular");
    if (piv != c)
      for (int q = 0; q < B; ++q) {
        std::swap(A[(size_t)c * B + q], A[(size_t)piv * B + q]);
        std::swap(Inv[(size_t)c * B + q], Inv[(size_t)piv * B + q]);
      }
    const double inv = 1.0 / A[(size_t)c * B + c];
    for (int q = 0; q < B; ++q) { A[(size_t)c * B + q] *= inv; Inv[(size_t)c * B + q] *= inv; }
    for (int r = 0; r < B; ++r) {
      if (r == c) continue;
      const double fct = A[(size_t)r * B + c];
      if (fct == 0.0) continue;
      for (int q = 0; q < B; ++q) {
        A[(size_t)r * B + q] -= fct * A[(size_t)c * B + q];
        Inv[(size_t)r * B + q] -= fct * Inv[(size_t)c * B + q];
      }
    }
  }
  std::vector<double> M((size_t)N * N);
  for (int r = 0; r < N; ++r)
    for (int q = 0; q < N; ++q) M[(size_t)r * N + q] = Inv[(size_t)r * B + q];
  CK(cudaMalloc(&ctx->coarse_M, M.size() * sizeof(double)));
  CK(cudaMemcpy(ctx->coarse_M, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice));
  return BAOREC_OK;
}

// x_vec of the mesh (src/utils.jl:21-25) for the iterative update.
int xvec_update(baorec_ctx* ctx) {
  const int n[3] = {ctx->n1, ctx->n2, ctx->n3};
  for (int a = 0; a < 3; ++a) {
    std::vector<float> t(n[a]);
    float cell = ctx->cfg.box_size[a] / (float)n[a];
    for (int i = 0; i < n[a]; ++i) t[i] = (float)((double)ctx->cfg.box_min[a] + ((double)i + 0.5) * (double)cell);
    CK(cudaMemcpy(ctx->xvec[a], t.data(), t.size() * 4, cudaMemcpyHostToDevice));
  }
  return BAOREC_OK;
}

int mg_jacobi(baorec_ctx* ctx, float* v, const float* f, const int nl[3], int niter, float* tmp) {
  int l = level_of(ctx, nl);
  if (l < 0) return set_error(ctx, BAOREC_ERR_ARG, "jacobi: %dx%dx%d is not a level of this mesh", nl[0], nl[1], nl[2]);
  LG G = level_geom(ctx, l, 0.0f);
  size_t N = ctx->lev[l].N;
  float* a = v;
  float* b = tmp;
  const bool tiled = tile_ok(ctx->lev[l].n) && (uintptr_t)v % 16 == 0 && (uintptr_t)tmp % 16 == 0;
  for (int s = 0; s < niter; ++s) {
    if (tiled) {
      CK(launch_jacobi(ctx->stream, a, f, b, G, ctx->cfg.jacobi_damping_factor));
    } else {
      (jacobi_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(a, f, b, G, ctx->cfg.jacobi_damping_factor, N), ::baorec::count_launch());
      CKLAUNCH();
    }
    float* t = a; a = b; b = t;
  }
  if (a != v) CK(cudaMemcpyAsync(v, a, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  return BAOREC_OK;
}

int mg_residual(baorec_ctx* ctx, float* r, const float* v, const float* f, const int nl[3]) {
  int l = level_of(ctx, nl);
  if (l < 0) return set_error(ctx, BAOREC_ERR_ARG, "residual: %dx%dx%d is not a level of this mesh", nl[0], nl[1], nl[2]);
  LG G = level_geom(ctx, l, 0.0f);
  if (tile_ok(ctx->lev[l].n) && (uintptr_t)v % 16 == 0) {
    CK(launch_ref_residual(ctx->stream, v, f, r, G, 0.0f));
  } else {
    (residual_kernel<<<blocks_for(ctx->lev[l].N), 256, 0, ctx->stream>>>(v, f, r, G, ctx->lev[l].N, 0.0f), ::baorec::count_launch());
    CKLAUNCH();
  }
  return BAOREC_OK;
}

int mg_reduce(baorec_ctx* ctx, float* coarse, const float* fine, const int nl[3]) {
  if (!can_recurse(nl)) return set_error(ctx, BAOREC_ERR_ARG, "reduce: level %dx%dx%d cannot be coarsened", nl[0], nl[1], nl[2]);
  int3 nf = make_int3(nl[0], nl[1], nl[2]);
  int3 nc = make_int3(nl[0] / 2, nl[1] / 2, nl[2] / 2);
  size_t Nc = (size_t)nc.x * nc.y * nc.z;
  (reduce_kernel<<<blocks_for(Nc), 256, 0, ctx->stream>>>(fine, coarse, nf, nc, Nc), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

int mg_prolong(baorec_ctx* ctx, float* fine, const float* coarse, const int nl[3], int add) {
  if (!can_recurse(nl)) return set_error(ctx, BAOREC_ERR_ARG, "prolong: level %dx%dx%d has no coarse level", nl[0], nl[1], nl[2]);
  int3 nf = make_int3(nl[0], nl[1], nl[2]);
  int3 nc = make_int3(nl[0] / 2, nl[1] / 2, nl[2] / 2);
  size_t Nc = (size_t)nc.x * nc.y * nc.z;
  (prolong_kernel<<<blocks_for(Nc), 256, 0, ctx->stream>>>(coarse, fine, nc, nf, Nc, add), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

// vcycle! (src/multigrid.jl:689-719) on level lvl; level lvl+1 buffers are scratch.
int mg_vcycle_ref(baorec_ctx* ctx, int lvl, float* v, const float* f) {
  baorec::Level& L = ctx->lev[lvl];
  const int nu = ctx->cfg.jacobi_niterations;
  CKS(mg_jacobi(ctx, v, f, L.n, nu, L.r + L.N));
  if (lvl + 1 < ctx->nlev) {
    baorec::Level& C = ctx->lev[lvl + 1];
    CKS(mg_residual(ctx, L.r, v, f, L.n));
    CKS(mg_reduce(ctx, C.f, L.r, L.n));
    CK(cudaMemsetAsync(C.v, 0, C.N * 4, ctx->stream));
    CKS(mg_vcycle_ref(ctx, lvl + 1, C.v, C.f));
    CKS(mg_prolong(ctx, v, C.v, L.n, 1));
  }
  return mg_jacobi(ctx, v, f, L.n, nu, L.r + L.N);
}

// fmg (src/multigrid.jl:722-752) starting at level lvl.
static int fmg_level(baorec_ctx* ctx, int lvl, const float* f, float* v) {
  baorec::Level& L = ctx->lev[lvl];
  if (lvl + 1 < ctx->nlev) {
    baorec::Level& C = ctx->lev[lvl + 1];
    CKS(mg_reduce(ctx, C.f, f, L.n));
    // the coarse solution lives in C.v; the coarse V-cycles use level lvl+2 as scratch
    CKS(fmg_level(ctx, lvl + 1, C.f, C.v));
    CKS(mg_prolong(ctx, v, C.v, L.n, 0));
  } else {
    CK(cudaMemsetAsync(v, 0, L.N * 4, ctx->stream));
  }
  for (int c = 0; c < ctx->cfg.vcycle_niterations; ++c) CKS(mg_vcycle_ref(ctx, lvl, v, f));
  return BAOREC_OK;
}

int mg_fmg(baorec_ctx* ctx, const float* f, float* phi) {
  CKS(mg_setup(ctx));
  // the recursion reads C.f of every coarser level while the V-cycles of the
  // finer level overwrite it only after that level's FMG stage has finished
  return fmg_level(ctx, 0, f, phi);
}

// ---- convergent solve -------------------------------------------------------

// One correction V-cycle on level lvl: lev[lvl].v ← V(rhs), rhs = lev[lvl].f - shift.
// `nsweeps` red-black sweeps on level lvl; the result ends in L.v.
static int smooth_rb(baorec_ctx* ctx, int lvl, const LG& G, float shift, int nsweeps) {
  baorec::Level& L = ctx->lev[lvl];
  const size_t N = L.N;
  float* a = L.v;
  float* b = L.r + N;   // ping-pong partner
  for (int s = 0; s < nsweeps; ++s) {
    if (tile_ok(L.n)) {
      CK(launch_rb_sweep(ctx->stream, a, b, L.f, G, shift, L.needs_clamp));
      ctx->launches++;
      float* q = a; a = b; b = q;
    } else {
      (rb_half_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(a, b, L.f, G, N, 0, shift), ::baorec::count_launch());
      CKLAUNCH();
      (rb_half_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(b, a, L.f, G, N, 1, shift), ::baorec::count_launch());
      CKLAUNCH();
    }
  }
  if (a != L.v) CK(cudaMemcpyAsync(L.v, a, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  return BAOREC_OK;
}

static int vcycle_rb(baorec_ctx* ctx, int lvl, float shift) {
  if (ctx->coarse_dirty) CKS(coarse_setup(ctx));
  baorec::Level& L = ctx->lev[lvl];
  LG G = level_geom(ctx, lvl, kClamp);
  const size_t N = L.N;
  float* v = L.v;
  float* t = L.r + N;   // ping-pong partner
  // small levels down to the dense one: one cooperative kernel
  if (ctx->coarse_M && L.N <= (size_t)kTailMaxCells && ctx->dense_level - lvl + 1 <= kTailMaxLevels) {
    TailArgs A;
    A.nl = ctx->dense_level - lvl + 1;
    A.nu1 = ctx->cfg.nu1;
    A.nu2 = ctx->cfg.nu2;
    A.shift0 = shift;
    A.M = ctx->coarse_M;
    for (int q = 0; q < A.nl; ++q) {
      baorec::Level& T = ctx->lev[lvl + q];
      A.L[q].f = T.f;
      A.L[q].v = T.v;
      A.L[q].r = T.r;
      A.L[q].t = T.r + T.N;
      A.L[q].G = level_geom(ctx, lvl + q, kClamp);
      A.L[q].N = (int)T.N;
    }
    CK(launch_coarse_tail(ctx->stream, A));
    ctx->launches++;
    return BAOREC_OK;
  }
  if (lvl == ctx->dense_level || lvl + 1 == ctx->nlev) {
    if (ctx->coarse_M && lvl == ctx->dense_level) {
      (coarse_dense_kernel<<<(unsigned)((N + 255) / 256), 256, 0, ctx->stream>>>(ctx->coarse_M, L.f, v, (int)N), ::baorec::count_launch());
      CKLAUNCH();
      return BAOREC_OK;
    }
    if (N <= (size_t)kCoarseMaxCells) {
      // the shift only moves the mean, which the coarse solve removes
      (coarse_solve_kernel<<<1, 256, 2 * N * sizeof(double), ctx->stream>>>(L.f, v, G, kCoarseSweeps), ::baorec::count_launch());
      CKLAUNCH();
      return BAOREC_OK;
    }
    CK(cudaMemsetAsync(v, 0, N * 4, ctx->stream));
    for (int s = 0; s < 50; ++s) {
      (rb_half_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(v, t, L.f, G, N, 0, shift), ::baorec::count_launch());
      CKLAUNCH();
      (rb_half_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(t, v, L.f, G, N, 1, shift), ::baorec::count_launch());
      CKLAUNCH();
    }
    return BAOREC_OK;
  }
  CK(cudaMemsetAsync(v, 0, N * 4, ctx->stream));
  CKS(smooth_rb(ctx, lvl, G, shift, ctx->cfg.nu1));
  baorec::Level& C = ctx->lev[lvl + 1];
  if (tile_ok(L.n)) {
    CK(launch_resid(ctx->stream, v, L.f, L.r, G, shift, L.needs_clamp));
    ctx->launches++;
  } else {
    (residual_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(v, L.f, L.r, G, N, shift), ::baorec::count_launch());
    CKLAUNCH();
  }
  CKS(mg_reduce(ctx, C.f, L.r, L.n));
  CKS(vcycle_rb(ctx, lvl + 1, 0.0f));
  CKS(mg_prolong(ctx, v, C.v, L.n, 1));
  return smooth_rb(ctx, lvl, G, shift, ctx->cfg.nu2);
}

int level_count(const baorec_ctx* ctx) { return ctx->nlev; }

LG level_geom_public(const baorec_ctx* ctx, int l, float clamp) { return level_geom(ctx, l, clamp); }

int operator_residual(baorec_ctx* ctx, const float* v, const float* f, float* r) {
  CKS(mg_setup(ctx));
  const baorec::Level& L0 = ctx->lev[0];
  LG G = level_geom(ctx, 0, 0.0f);
  const bool aligned = (uintptr_t)v % 16 == 0;
  if (aligned && tile_ok(L0.n)) {
    CK(launch_resid_diff(ctx->stream, v, f, r, G, nullptr));
    ctx->launches++;
  } else {
    (residual_diff_kernel<<<blocks_for(L0.N), 256, 0, ctx->stream>>>(v, f, r, G, L0.N, nullptr), ::baorec::count_launch());
    CKLAUNCH();
  }
  return BAOREC_OK;
}

// Relative residual |r - mean r| / |f - mean f|, r = f - A φ0, of a start φ0
// for the right-hand side f: zero, the FFT start S⁻¹ f, or the learned one.
int start_residual(baorec_ctx* ctx, const float* f, int start, double* rel) {
  CKS(mg_setup(ctx));
  baorec::Level& L0 = ctx->lev[0];
  const size_t N = L0.N;
  float* v = L0.v;
  float* r = L0.r + N;
  if (start == BAOREC_START_ZERO) CK(cudaMemsetAsync(v, 0, N * 4, ctx->stream));
  else if (start == BAOREC_START_SPECTRAL) CKS(spectral_correction(ctx, f, v));
  else CKS(guess_dispatch_apply(ctx, f, v));
  CKS(operator_residual(ctx, v, f, r));
  double sf = 0.0, sf2 = 0.0, sr = 0.0, sr2 = 0.0;
  CKS(sum_mesh(ctx, f, N, &sf));
  CKS(sumsq_mesh(ctx, f, N, &sf2));
  CKS(sum_mesh(ctx, r, N, &sr));
  CKS(sumsq_mesh(ctx, r, N, &sr2));
  const double den = sf2 - sf * sf / (double)N;
  *rel = den > 0.0 ? sqrt(std::max(0.0, sr2 - sr * sr / (double)N) / den) : 0.0;
  return BAOREC_OK;
}

int mg_solve(baorec_ctx* ctx, const float* f, float* phi, const float* phi0, baorec_solve_stats* st,
             const double* fpart) {
  CKS(mg_setup(ctx));
  baorec::Level& L0 = ctx->lev[0];
  const size_t N = L0.N;
  float* hiA = phi;
  float* hiB = ctx->phi_hi2;
  float* loA = ctx->phi_lo;
  float* loB = ctx->phi_lo2;
  if (phi0 && phi0 != phi) CK(cudaMemcpyAsync(hiA, phi0, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  else if (!phi0) CK(cudaMemsetAsync(hiA, 0, N * 4, ctx->stream));
  // The first residual of a zero solution needs no stencil: r = f - α with
  // α = mean f, so Σr = 0 and |r| = |f - α| (relative residual 1), and the
  // solution pair stays zero.  The FFT start and the learned start are that
  // zero start's first correction: d_0 = S⁻¹ r (FFT start) or d_0 = S⁻¹ r +
  // the network's correction (learned start; S⁻¹ r = S⁻¹ f, the mean being
  // outside S⁻¹'s range), so neither needs an accurate residual of its own.
  const bool zero_start = !phi0;
  const bool learned = !phi0 && ctx->cfg.mg_start == BAOREC_START_LEARNED;
  CK(cudaMemsetAsync(loA, 0, N * 4, ctx->stream));
  // Σf, Σf² for |f - α| = sqrt(Σf² - 2αΣf + Nα²), in one pass (or from the
  // pass that produced f: fpart); the host reads them when it first needs
  // them (a zero start forms its first residual and queues its first FFT
  // correction on the device before that)
  constexpr int kSumBlocks = 8 * kNumSMs;
  static_assert(kSumBlocks == kFsumBlocks, "the producer's per-block sums stand in for this pass");
  const double* fsums = fpart ? fpart : ctx->dred;
  if (!fpart) {
    (sum_sumsq_partial_kernel<<<kSumBlocks, 256, 0, ctx->stream>>>(f, N, ctx->dred), ::baorec::count_launch());
    CKLAUNCH();
  }
  CK(cudaMemcpyAsync(ctx->hred, fsums, 2 * kSumBlocks * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!ctx->ev_red) CK(cudaEventCreateWithFlags(&ctx->ev_red, cudaEventDisableTiming));
  CK(cudaEventRecord(ctx->ev_red, ctx->stream));
  double sf = 0.0, sf2 = 0.0, alpha = 0.0, fn2 = 0.0;
  bool sums_read = false;
  auto read_sums = [&]() -> int {
    if (sums_read) return BAOREC_OK;
    sums_read = true;
    CK(cudaEventSynchronize(ctx->ev_red));
    for (int q = 0; q < kSumBlocks; ++q) { sf += ctx->hred[2 * q]; sf2 += ctx->hred[2 * q + 1]; }
    alpha = sf / (double)N;
    fn2 = sf2 - 2.0 * alpha * sf + (double)N * alpha * alpha;   // |f - α|² at the initial α
    return BAOREC_OK;
  };
  if (!zero_start) CKS(read_sums());
  LG G = level_geom(ctx, 0, 0.0f);
  bool have_e = false;
  int cycles = 0;
  double rho = 0.0, rho0 = 0.0;
  int status = BAOREC_ERR_NOT_CONVERGED;
  // the tile kernel reads the solution pair in 16-byte chunks
  const bool aligned = (uintptr_t)phi % 16 == 0 && (uintptr_t)ctx->phi_lo % 16 == 0 && (uintptr_t)ctx->phi_hi2 % 16 == 0 &&
                       (uintptr_t)ctx->phi_lo2 % 16 == 0;
  const bool tile0 = aligned && tile_ok(L0.n) && (size_t)tile_blocks(G) <= kMaxPartials;
  // the streaming residual kernels unless the autotuner chose the tile ones
  const bool stream0 = aligned && stream_ok(L0.n) && ctx->tune.stream0 != 0 &&
                       (size_t)stream_blocks(L0.n) <= kMaxPartials;
  int nparts = kResBlocks;
  // spectral corrections (FFT inverse of the operator with the box's mean line
  // of sight) run first, for as long as each one shrinks the residual by at
  // least start_rate; V-cycles take over after the first one that does not
  ctx->hist_rho.clear();
  ctx->hist_kind.clear();
  bool spectral = ctx->cfg.mg_start != BAOREC_START_ZERO;
  int nspec = 0, m_last = 0;
  double rho_prev = 0.0, rate = 0.0;
  const float* pending_d = nullptr;   // last FFT correction of an outer step, not yet added to e
  // An FFT or learned start from zero never forms r = f - α as a mesh: its
  // first correction transforms f itself (S⁻¹ f = S⁻¹ (f - α), the mean lying
  // outside S⁻¹'s range) and the first running residual reads f and subtracts
  // α as it loads it, the same FP32 subtraction.
  const bool first_from_f = zero_start && spectral && ctx->cfg.max_cycles > 0 && (tile0 || stream0);
  for (int it = 0;; ++it) {
    double s1 = 0.0, s2 = 0.0;
    bool speculative = false;
    if (it == 0 && zero_start) {
      if (!first_from_f) {
        (shift_mean_kernel<<<8 * kNumSMs, 256, 0, ctx->stream>>>(f, L0.f, N, fsums, kSumBlocks), ::baorec::count_launch());
        CKLAUNCH();
      }
      // the first FFT correction needs only r: queue it before waiting for the sums
      if (spectral && ctx->cfg.max_cycles > 0) {
        if (learned) {
          // the network's features reuse the partial-sum buffers that still hold Σf, Σf²
          CKS(read_sums());
          CKS(guess_dispatch_apply(ctx, f, L0.v));
        } else {
          CKS(spectral_correction(ctx, first_from_f ? f : L0.f, L0.v));
        }
        speculative = true;
      }
      CKS(read_sums());
      s2 = fn2;
    } else {
      if (stream0) {
        CK(launch_resid_acc_stream(ctx->stream, hiA, loA, have_e ? L0.v : nullptr, f, hiB, loB, L0.f, G, (float)alpha,
                                   ctx->dred, &nparts));
        ctx->launches++;
      } else if (tile0) {
        CK(launch_resid_acc(ctx->stream, hiA, loA, have_e ? L0.v : nullptr, f, hiB, loB, L0.f, G, (float)alpha,
                            ctx->dred, &nparts, have_e ? pending_d : nullptr));
        pending_d = nullptr;
        ctx->launches++;
      } else {
        (resid_acc_kernel<<<kResBlocks, 256, 0, ctx->stream>>>(hiA, loA, have_e ? L0.v : nullptr, f, hiB, loB, L0.f,
                                                              G, N, (float)alpha, ctx->dred), ::baorec::count_launch());
        CKLAUNCH();
      }
      CK(cudaMemcpyAsync(ctx->hred, ctx->dred, 2 * nparts * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      // While the host reads the partial sums, the GPU already computes the
      // first FFT correction of the next outer step, d_0 = S⁻¹ r, which needs
      // nothing the host decides (it writes only the correction lev[0].v; a
      // V-cycle zeroes that first).  Skipped when the last step's rate says
      // this residual is already below rtol.
      bool predicted_done = false;
      if (spectral && nspec < ctx->cfg.max_cycles) {
        const double predicted = m_last > 0 ? rho_prev * pow(std::max(rate, 0.0), (double)m_last) : 1.0;
        predicted_done = m_last > 0 && rate > 0.0 && predicted <= (double)ctx->cfg.rtol;
        speculative = !predicted_done;
      }
      bool psi_now = false;
      if (speculative) {
        if (!ctx->ev_red) CK(cudaEventCreateWithFlags(&ctx->ev_red, cudaEventDisableTiming));
        CK(cudaEventRecord(ctx->ev_red, ctx->stream));
        CKS(spectral_correction(ctx, L0.f, L0.v));
        CK(cudaEventSynchronize(ctx->ev_red));
      } else if (ctx->want_psi_ahead && predicted_done) {
        // predicted converged: the displacement of this iterate (the hi part
        // just written) runs while the host reads the residual; it stands if
        // the solve stops here
        if (!ctx->ev_red) CK(cudaEventCreateWithFlags(&ctx->ev_red, cudaEventDisableTiming));
        CK(cudaEventRecord(ctx->ev_red, ctx->stream));
        CKS(displacement_meshes(ctx, hiB, ctx->psi));
        CK(cudaEventSynchronize(ctx->ev_red));
        psi_now = true;
      } else {
        CK(cudaStreamSynchronize(ctx->stream));
      }
      ctx->psi_ahead = psi_now;
      for (int q = 0; q < nparts; ++q) { s1 += ctx->hred[2 * q]; s2 += ctx->hred[2 * q + 1]; }
      { float* t = hiA; hiA = hiB; hiB = t; t = loA; loA = loB; loB = t; }
    }
    const double rn2 = sf2 - 2.0 * alpha * sf + (double)N * alpha * alpha;   // |f - α|² at the current α
    rho = rn2 > 0.0 ? sqrt(s2 / rn2) : 0.0;
    if (it == 0) rho0 = rho;
    ctx->hist_rho.push_back(rho);
    ctx->hist_kind.push_back(-1);
    if (!(rho == rho)) { status = set_error(ctx, BAOREC_ERR_NOT_CONVERGED, "multigrid solve produced NaN"); break; }
    if (rho <= (double)ctx->cfg.rtol) { status = BAOREC_OK; break; }
    if (cycles >= ctx->cfg.max_cycles) {
      status = set_error(ctx, BAOREC_ERR_NOT_CONVERGED, "multigrid: relative residual %.3e after %d V-cycles (rtol %.1e)",
                         rho, cycles, (double)ctx->cfg.rtol);
      break;
    }
    double mean_r = s1 / (double)N;
    alpha += mean_r;
    if (spectral && m_last > 0) {
      // observed contraction per FFT correction of the last outer step
      rate = rho_prev > 0.0 ? pow(rho / rho_prev, 1.0 / m_last) : 0.0;
      if (!(rate <= (double)ctx->cfg.start_rate)) spectral = false;
    }
    if (spectral && nspec >= ctx->cfg.max_cycles) spectral = false;
    rho_prev = rho;
    // the correction solves A e = r - mean(r); r sits in lev[0].f
    if (spectral) {
      // m FFT corrections against an FP32 running residual, no host round trip:
      //   d_0 = S⁻¹ r_0;  r_q = r_{q-1} - A d_{q-1};  d_q = S⁻¹ r_q;  e = Σ d_q
      // with m from the observed rate, enough to reach rtol if it holds
      // The first outer step is held to kSpectralFirst corrections: its shift
      // α = mean(f) is not yet the consistent one, and the corrections cannot
      // go below that inconsistency (on the 256^3 lightcone the residual
      // stalls near 1e-3 after about four corrections; fewer leave a third
      // outer step, more are wasted against the stall).
      // With one line of sight the operator is symmetric (no first-derivative
      // term): its left null vector is constant, α = mean(f) is already the
      // consistent shift, and S⁻¹ is its exact inverse, so the first outer
      // step is the FFT start alone and the next one sizes itself from it.
      int m = ctx->cfg.los_mode == BAOREC_LOS_GLOBAL ? 1 : kSpectralFirst;
      if (m_last > 0) {
        const double r = std::min(std::max(rate, kSpectralRateFloor), 0.9);
        const double want = log((double)ctx->cfg.rtol / rho) / log(r);
        m = (int)std::min<double>(kSpectralInnerMax, std::max(1.0, ceil(want)));
      }
      float* rin = L0.f;
      float* rout = L0.r + N;
      float* d = L0.r;
      if (!speculative) CKS(spectral_correction(ctx, rin, L0.v));
      for (int q = 1; q < m; ++q) {
        const float* dprev = q == 1 ? L0.v : d;
        float* acc = q == 1 ? nullptr : L0.v;
        // the first outer step of an FFT start from zero: r_0 = f - α formed on load
        const bool from_f = first_from_f && it == 0 && q == 1;
        const float* src = from_f ? f : rin;
        const float shift = from_f ? (float)alpha : 0.0f;
        if (stream0) {
          CK(launch_resid_diff_stream(ctx->stream, dprev, src, rout, G, acc, shift));
          ctx->launches++;
        } else if (tile0) {
          CK(launch_resid_diff(ctx->stream, dprev, src, rout, G, acc, shift));
          ctx->launches++;
        } else {
          (residual_diff_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(dprev, rin, rout, G, N, acc), ::baorec::count_launch());
          CKLAUNCH();
        }
        std::swap(rin, rout);
        CKS(spectral_correction(ctx, rin, d));
      }
      if (m > 1 && tile0 && !stream0) {
        pending_d = d;   // the tiled accurate residual adds the last correction as it loads e
      } else if (m > 1) {
        (add_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(L0.v, d, N), ::baorec::count_launch());
        CKLAUNCH();
      }
      nspec += m;
      m_last = m;
      ctx->hist_kind.back() = m;
    } else {
      CKS(vcycle_rb(ctx, 0, (float)mean_r));
      ++cycles;
      ctx->hist_kind.back() = 0;
    }
    have_e = true;
  }
  if (hiA != phi) CK(cudaMemcpyAsync(phi, hiA, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  if (loA != ctx->phi_lo) CK(cudaMemcpyAsync(ctx->phi_lo, loA, N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  baorec_solve_stats s;
  s.cycles = cycles;
  s.spectral_steps = nspec;
  s.rel_residual = rho;
  s.alpha = alpha;
  s.rel_residual_initial = rho0;
  ctx->last_stats = s;
  if (st) *st = s;
  return status;
}

}  // namespace baorec

extern "C" int baorec_profile_kernel(baorec_ctx* ctx, int which, int reps, float* avg_ms, double* bytes) {
  using namespace baorec;
  if (!ctx || !avg_ms || !bytes || reps <= 0) return BAOREC_ERR_ARG;
  CKS(mg_setup(ctx));
  Level& L = ctx->lev[0];
  const size_t N = L.N;
  float* t = L.r + N;
  LG G = level_geom(ctx, 0, 0.0f);
  LG Gc = level_geom(ctx, 0, kClamp);
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int np = 0, xst = BAOREC_OK;
  auto launch = [&]() {
    if (which == 8 || which == 9)
      xst = xy_profile(ctx, which == 9, L.f, t);
    else if (which == 0 && tile_ok(L.n))
      launch_rb_sweep(ctx->stream, L.v, t, L.f, Gc, 0.0f, L.needs_clamp);
    else if (which == 0)
      (rb_half_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(L.v, t, L.f, Gc, N, 0, 0.0f), ::baorec::count_launch());
    else if (which == 1 && tile_ok(L.n))
      launch_resid_acc(ctx->stream, L.v, L.f, L.r, L.f, ctx->phi_hi2, ctx->phi_lo2, t, G, 0.0f, ctx->dred, &np);
    else if (which == 1)
      (resid_acc_kernel<<<kResBlocks, 256, 0, ctx->stream>>>(L.v, L.f, L.r, L.f, ctx->phi_hi2, ctx->phi_lo2, t, G, N,
                                                            0.0f, ctx->dred), ::baorec::count_launch());
    else if (which == 4)
      launch_resid_acc_stream(ctx->stream, L.v, L.f, L.r, L.f, ctx->phi_hi2, ctx->phi_lo2, t, G, 0.0f, ctx->dred, &np);
    else if (which == 5)
      launch_resid_diff_stream(ctx->stream, L.v, L.f, t, G, L.r);
    else if (which == 3 && tile_ok(L.n))
      launch_resid_diff(ctx->stream, L.v, L.f, t, G, L.r);
    else if (which == 3)
      (residual_diff_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(L.v, L.f, t, G, N, L.r), ::baorec::count_launch());
    else if (which == 6)
      vcycle_rb(ctx, 0, 0.0f);
    else if (which == 7)
      mg_vcycle_ref(ctx, 0, L.v, L.f);
    else if (tile_ok(L.n))
      launch_jacobi(ctx->stream, L.v, L.f, t, G, ctx->cfg.jacobi_damping_factor);
    else
      (jacobi_kernel<<<blocks_for(N), 256, 0, ctx->stream>>>(L.v, L.f, t, G, ctx->cfg.jacobi_damping_factor, N), ::baorec::count_launch());
  };
  if (which < 0 || which > 9) return set_error(ctx, BAOREC_ERR_ARG, "profile_kernel: unknown kernel %d", which);
  if ((which == 4 || which == 5) && !stream_ok(L.n))
    return set_error(ctx, BAOREC_ERR_ARG, "profile_kernel: no streaming form here");
  launch();   // warm-up
  if (xst != BAOREC_OK) {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return xst;
  }
  CK(cudaEventRecord(a, ctx->stream));
  for (int r = 0; r < reps; ++r) launch();
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  CKLAUNCH();
  ctx->launches += reps;
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *avg_ms = ms / reps;
  // algorithmic bytes: a full smoothing sweep reads v and f and writes v (12 B/cell;
  // the one-cell kernel does one colour, half of that); the accurate residual
  // reads hi, lo, e, f and writes hi, lo, r (28 B/cell); the FP32 running
  // residual of the FFT corrections reads d, r, acc and writes r, acc (20 B/cell)
  *bytes = which == 0 ? (tile_ok(L.n) ? 12.0 : 6.0) * N : (which == 1 || which == 4) ? 28.0 * N
          : (which == 3 || which == 5) ? 20.0 * N : 12.0 * N;
  if (which == 6 || which == 7) {
    // a V-cycle: on every level its sweeps (12 B/cell each: read v and f,
    // write v), the residual (12 B/cell), the restriction (4 B/cell read, 0.5
    // written) and the prolongation (read 0.5, read and write v: 8.5 B/cell);
    // the coarsest level's sweeps are counted like the others
    const double sweeps = which == 6 ? ctx->cfg.nu1 + ctx->cfg.nu2 : 2.0 * ctx->cfg.jacobi_niterations;
    double b = 0.0;
    for (int l = 0; l < ctx->nlev; ++l) b += (double)ctx->lev[l].N * (12.0 * sweeps + 12.0 + 4.5 + 8.5);
    *bytes = b;
  }
  // a batched xy transform reads the real mesh and writes the half spectrum
  // (8 + 4 B per half-spectrum cell and real cell), or the reverse
  if (which == 8 || which == 9) *bytes = 4.0 * N + 8.0 * (double)ctx->n1h * ctx->n2 * ctx->n3;
  return BAOREC_OK;
}
