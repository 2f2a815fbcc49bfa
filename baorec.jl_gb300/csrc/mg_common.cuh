// Device helpers shared by the multigrid translation units (mg.cu, mg_tiles.cu).
#pragma once

#include "common.cuh"
#include "packed_f32x2.cuh"

namespace baorec {

constexpr float kClamp = 0.5f;       // κ: |g p_a| <= κ gp_a in the V-cycle operators

struct LG {                           // level geometry passed to kernels
  int n[3];
  float cell2[3], icell2[3];
  const float* P[3];                  // p_a tables (local) — n[a] entries each
  float pg[3];                        // los / cell (global)
  float beta;
  int local;
  float clamp;                        // > 0: clamp derivative coefficients
  int tile16;                         // tile kernels: -1 heuristic, 0 = 32x8x8, 1 = 32x16x16 tiles
  int pairs;                          // form of the running residual (0-5, see baorec_set_tune_pairs)
  int accf = 0;                       // accurate residual: 0 512-thread blocks, 1 / 2 256-thread blocks (32x8x8 / 32x8x16)
  unsigned* err = nullptr;            // device error word of the context (bounded waits report here)
};

struct Coef {
  float gpx, gpy, gpz, g, pxy, pxz, pyz, dx, dy, dz;
};

__device__ __forceinline__ Coef coef_at(const LG& G, int i, int j, int k) {
  float px, py, pz;
  if (G.local) { px = G.P[0][i]; py = G.P[1][j]; pz = G.P[2][k]; }
  else { px = G.pg[0]; py = G.pg[1]; pz = G.pg[2]; }
  Coef c;
  float px2 = px * px, py2 = py * py, pz2 = pz * pz;
  c.g = G.beta / (G.cell2[0] * px2 + G.cell2[1] * py2 + G.cell2[2] * pz2);
  c.gpx = G.icell2[0] + c.g * px2;
  c.gpy = G.icell2[1] + c.g * py2;
  c.gpz = G.icell2[2] + c.g * pz2;
  c.pxy = px * py; c.pxz = px * pz; c.pyz = py * pz;
  if (G.local) {
    c.dx = c.g * px; c.dy = c.g * py; c.dz = c.g * pz;
    if (G.clamp > 0.0f) {
      c.dx = fminf(fmaxf(c.dx, -G.clamp * c.gpx), G.clamp * c.gpx);
      c.dy = fminf(fmaxf(c.dy, -G.clamp * c.gpy), G.clamp * c.gpy);
      c.dz = fminf(fmaxf(c.dz, -G.clamp * c.gpz), G.clamp * c.gpz);
    }
  } else {
    c.dx = c.dy = c.dz = 0.0f;
  }
  return c;
}

struct Nb {                           // the 18 neighbours
  float xp, xm, yp, ym, zp, zm;
  float pp0, mm0, mp0, pm0;           // xy plane: (+,+), (−,−), (−,+), (+,−)
  float p0p, m0m, m0p, p0m;           // xz
  float _pp, _mm, _mp, _pm;           // yz
};

__device__ __forceinline__ void cell_ijk(size_t e, const int n[3], int& i, int& j, int& k) {
  i = (int)(e % (unsigned)n[0]);
  size_t r = e / (unsigned)n[0];
  j = (int)(r % (unsigned)n[1]);
  k = (int)(r / (unsigned)n[1]);
}

template <typename F>
__device__ __forceinline__ Nb gather(F get, const int n[3], int i, int j, int k) {
  int ip = i + 1 == n[0] ? 0 : i + 1, im = i == 0 ? n[0] - 1 : i - 1;
  int jp = j + 1 == n[1] ? 0 : j + 1, jm = j == 0 ? n[1] - 1 : j - 1;
  int kp = k + 1 == n[2] ? 0 : k + 1, km = k == 0 ? n[2] - 1 : k - 1;
  Nb b;
  b.xp = get(ip, j, k); b.xm = get(im, j, k);
  b.yp = get(i, jp, k); b.ym = get(i, jm, k);
  b.zp = get(i, j, kp); b.zm = get(i, j, km);
  b.pp0 = get(ip, jp, k); b.mm0 = get(im, jm, k); b.mp0 = get(im, jp, k); b.pm0 = get(ip, jm, k);
  b.p0p = get(ip, j, kp); b.m0m = get(im, j, km); b.m0p = get(im, j, kp); b.p0m = get(ip, j, km);
  b._pp = get(i, jp, kp); b._mm = get(i, jm, km); b._mp = get(i, jm, kp); b._pm = get(i, jp, km);
  return b;
}

// The bracket of src/multigrid.jl:64-79 (neighbour part), reference order.
__device__ __forceinline__ float offdiag(const Coef& c, const Nb& b, int local) {
  float s = c.gpx * (b.xp + b.xm) + c.gpy * (b.yp + b.ym) + c.gpz * (b.zp + b.zm) +
            c.g / 2.0f * (c.pxy * (b.pp0 + b.mm0 - b.mp0 - b.pm0) + c.pxz * (b.p0p + b.m0m - b.m0p - b.p0m) +
                          c.pyz * (b._pp + b._mm - b._mp - b._pm));
  if (local) s += c.dx * (b.xp - b.xm) + c.dy * (b.yp - b.ym) + c.dz * (b.zp - b.zm);
  return s;
}

__device__ __forceinline__ size_t at(const int n[3], int i, int j, int k) {
  return (size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * (size_t)k);
}



__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Stencil combinations of a double-float solution in difference form.  Each
// argument is the pair (h_u - h_0, l_u - l_0) of a neighbour u of the cell.
// The hi differences of a combination are summed first — neighbouring values
// of a smooth field are within a factor of two, so these sums are exact
// (Sterbenz) — then the lo differences, and the two are added with one
// rounding, relative to the combination itself.  Rounding each first
// difference before combining would cost ε/(h k) of the second difference:
// about 1e-6 of the residual at 512^3, a floor for the solve.
__device__ __forceinline__ float dd_sum2(float2 p, float2 m) {   // p + m: second difference
  return __fadd_rn(__fadd_rn(p.x, m.x), __fadd_rn(p.y, m.y));
}
__device__ __forceinline__ float dd_diff2(float2 p, float2 m) {  // p - m: central first difference
  return __fadd_rn(__fsub_rn(p.x, m.x), __fsub_rn(p.y, m.y));
}
// (pp + mm) - (mp + pm): mixed second difference
__device__ __forceinline__ float dd_cross(float2 pp, float2 mm, float2 mp, float2 pm) {
  return __fadd_rn(__fsub_rn(__fadd_rn(pp.x, mm.x), __fadd_rn(mp.x, pm.x)),
                   __fsub_rn(__fadd_rn(pp.y, mm.y), __fadd_rn(mp.y, pm.y)));
}

// v' = (hi + lo) + e as a renormalised double-float pair.
__device__ __forceinline__ void df_add(float hi, float lo, float e, float& ohi, float& olo) {
  float s, err;
  two_sum(hi, e, s, err);
  float t = __fadd_rn(lo, err);
  ohi = __fadd_rn(s, t);
  olo = __fsub_rn(t, __fsub_rn(ohi, s));
}


// ---- shared-memory tile kernels (mg_tiles.cu) -------------------------------
// Levels whose sizes are multiples of the tile use these; the launchers
// return a cudaError_t of the launch.
bool tile_ok(const int n[3]);
// One red-black Gauss-Seidel sweep vin -> vout on rhs - shift.
cudaError_t launch_rb_sweep(cudaStream_t s, const float* vin, float* vout, const float* rhs, const LG& G, float shift,
                            bool clamp);
// r = rhs - shift - Ã e (clamped operator).
// r = rhs - A e in difference form (exact operator, no clamp), accurate for
// smooth e; with acc != nullptr also acc += e
// one damped-Jacobi sweep of the reference schedule on shared-memory tiles (tile_ok meshes)
cudaError_t launch_jacobi(cudaStream_t s, const float* v, const float* f, float* out, const LG& G, float omega);
// r = (f - shift) - A v of the reference schedule on shared-memory tiles (tile_ok meshes)
cudaError_t launch_ref_residual(cudaStream_t s, const float* v, const float* f, float* r, const LG& G, float shift);
// r = (rhs - shift) + bracket(e_nb - e_0), acc += e (optional)
cudaError_t launch_resid_diff(cudaStream_t s, const float* e, const float* rhs, float* r, const LG& G, float* acc,
                              float shift = 0.0f);
// r = rhs - shift - A e; with acc != nullptr also acc += e
cudaError_t launch_resid(cudaStream_t s, const float* e, const float* rhs, float* r, const LG& G, float shift, bool clamp,
                         float* acc = nullptr);
// Accurate residual with solution update; writes (Σr, Σr²) per block to part, returns the block count.
// The correction is e (+ ed, added in FP32 first, when both are given).
cudaError_t launch_resid_acc(cudaStream_t s, const float* hi, const float* lo, const float* e, const float* f,
                             float* ohi, float* olo, float* r, const LG& G, float alpha, double* part, int* nparts,
                             const float* ed = nullptr);
int tile_blocks(const LG& G);
__device__ __forceinline__ f2 rcp2(f2 a) {
  float x, y;
  U2(a, x, y);
  return P2(__frcp_rn(x), __frcp_rn(y));
}

// c_x^2 p_x^2 + c_y^2 p_y^2 of the fast coefficients, in one fixed rounding
// order (no contraction), so that the running-residual forms that pair
// cells differently produce the same bits.
__device__ __forceinline__ float coef_dxy(const LG& G, float px2, float py2) {
  return __fadd_rn(__fmul_rn(G.cell2[0], px2), __fmul_rn(G.cell2[1], py2));
}

// the running residual with TMA-staged operands, blocks of tz planes (mg_tma.cu)
bool resid_tma_ok(const LG& G, int tz);
cudaError_t launch_resid_diff_tma(cudaStream_t s, const float* d, const float* rin, float* rout, const LG& G,
                                  float* acc, int tz, float shift = 0.0f);

// streaming (2.5-D, cp.async-pipelined) forms of the finest-level residuals (mg_stream.cu)
bool stream_ok(const int n[3]);
int stream_blocks(const int n[3]);
cudaError_t launch_resid_acc_stream(cudaStream_t s, const float* hi, const float* lo, const float* e, const float* f,
                                    float* ohi, float* olo, float* r, const LG& G, float alpha, double* part,
                                    int* nparts);
cudaError_t launch_resid_diff_stream(cudaStream_t s, const float* d, const float* rin, float* rout, const LG& G,
                                     float* acc, float shift = 0.0f);

// ---- cooperative coarse tail (mg_tail.cu) -----------------------------------
constexpr int kTailMaxCells = 64 * 64 * 64;   // levels at most this big run in the tail kernel
constexpr int kTailMaxLevels = 8;
struct TailLevel {
  float* f;   // right-hand side
  float* v;   // correction
  float* r;   // residual scratch
  float* t;   // half-sweep partner
  LG G;       // geometry (clamped operator)
  int N;
};
struct TailArgs {
  int nl;              // levels; the last is solved with the dense inverse M
  int nu1, nu2;
  float shift0;        // subtracted from the first level's right-hand side
  const double* M;
  TailLevel L[kTailMaxLevels];
};
cudaError_t launch_coarse_tail(cudaStream_t s, const TailArgs& args);

}  // namespace baorec
