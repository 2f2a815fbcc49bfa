// Fused read-out: trilinear gather of the three displacement meshes at the
// particles (read_cic!, src/mas.jl:218-269), the RSD term (read_shifts,
// src/recon.jl:264-306) and the position shift (reconstructed_positions,
// src/recon.jl:366-380) in one pass.  Every multiply and add is an IEEE
// round-to-nearest intrinsic in the reference's evaluation order, so given
// the same meshes the outputs are bit-identical to the reference's FP32 CPU
// arithmetic.
#include "common.cuh"

namespace baorec {
namespace {

struct RGeom {
  int n[3];
  float cell[3];   // T(L/n)
  float bmin[3];
  float f;         // growth rate
  float los[3];
  int local;
};

__device__ __forceinline__ bool axis_idx(float p, float bmin, float cell, int n, int& lo, int& hi, float& d,
                                         float& u) {
  float dist = __fdiv_rn(__fsub_rn(p, bmin), cell);
  int i = (int)floorf(dist);
  u = __fsub_rn(dist, (float)i);
  d = __fsub_rn(1.0f, u);
  i += 1;
  lo = i > n ? i - n : i;          // wrap = true (the reference's callers never pass it)
  hi = lo + 1;
  hi = hi > n ? hi - n : hi;
  bool ok = lo >= 1 && lo <= n && hi >= 1 && hi <= n;
  lo -= 1; hi -= 1;
  return ok;
}

__device__ __forceinline__ float tri(const float* __restrict__ m, const size_t o[8], float dx, float dy, float dz,
                                     float ux, float uy, float uz) {
  // terms in the order of src/mas.jl:258-265, summed left to right
  float s = __fmul_rn(__fmul_rn(__fmul_rn(m[o[0]], dx), dy), dz);
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[1]], dx), dy), uz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[2]], dx), uy), dz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[3]], dx), uy), uz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[4]], ux), dy), dz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[5]], ux), dy), uz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[6]], ux), uy), dz));
  s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(m[o[7]], ux), uy), uz));
  return s;
}

// mode 0: write shifts; mode 1: write p - shift; mode 2: write the raw read of
// mesh 0 only (read_cic!).  field: 0 disp, 1 rsd, 2 sum.
__global__ void readout_kernel(const float* __restrict__ psi, size_t N, const float* __restrict__ x,
                               const float* __restrict__ y, const float* __restrict__ z, int64_t n, RGeom G,
                               int field, int mode, float* __restrict__ o0, float* __restrict__ o1,
                               float* __restrict__ o2, int field2, float* __restrict__ p0, float* __restrict__ p1,
                               float* __restrict__ p2, unsigned* err) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    float px = x[q], py = y[q], pz = z[q];
    int xl, xh, yl, yh, zl, zh;
    float dx, ux, dy, uy, dz, uz;
    bool ok = axis_idx(px, G.bmin[0], G.cell[0], G.n[0], xl, xh, dx, ux);
    ok &= axis_idx(py, G.bmin[1], G.cell[1], G.n[1], yl, yh, dy, uy);
    ok &= axis_idx(pz, G.bmin[2], G.cell[2], G.n[2], zl, zh, dz, uz);
    if (!ok) {
      atomicOr(err, kErrOOB);
      const float nan = __int_as_float(0x7fc00000);
      o0[q] = nan;
      if (mode != 2) { o1[q] = nan; o2[q] = nan; }
      if (p0) { p0[q] = nan; p1[q] = nan; p2[q] = nan; }
      continue;
    }
    const size_t n0 = (size_t)G.n[0], n01 = (size_t)G.n[0] * G.n[1];
    const size_t o[8] = {xl + n0 * yl + n01 * zl, xl + n0 * yl + n01 * zh, xl + n0 * yh + n01 * zl,
                         xl + n0 * yh + n01 * zh, xh + n0 * yl + n01 * zl, xh + n0 * yl + n01 * zh,
                         xh + n0 * yh + n01 * zl, xh + n0 * yh + n01 * zh};
    if (mode == 2) { o0[q] = tri(psi, o, dx, dy, dz, ux, uy, uz); continue; }
    // Ψ is interleaved (x, y, z, pad) per cell: one 16-byte load per corner
    const float4* p4 = reinterpret_cast<const float4*>(psi);
    const float4 c0 = __ldg(p4 + o[0]), c1 = __ldg(p4 + o[1]), c2 = __ldg(p4 + o[2]), c3 = __ldg(p4 + o[3]);
    const float4 c4 = __ldg(p4 + o[4]), c5 = __ldg(p4 + o[5]), c6 = __ldg(p4 + o[6]), c7 = __ldg(p4 + o[7]);
    float s[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      auto C = [&](const float4& v) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); };
      float t = __fmul_rn(__fmul_rn(__fmul_rn(C(c0), dx), dy), dz);
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c1), dx), dy), uz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c2), dx), uy), dz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c3), dx), uy), uz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c4), ux), dy), dz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c5), ux), dy), uz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c6), ux), uy), dz));
      t = __fadd_rn(t, __fmul_rn(__fmul_rn(__fmul_rn(C(c7), ux), uy), uz));
      s[a] = t;
    }
    (void)N;
    // one gathered Ψ, one or two fields out (the same arithmetic either way)
    auto emit = [&](int fld, float* __restrict__ a0, float* __restrict__ a1, float* __restrict__ a2) {
      float t[3] = {s[0], s[1], s[2]};
      if (fld != 0) {
        float l0, l1, l2;
        if (G.local) {
          float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)), __fmul_rn(pz, pz)));
          l0 = __fdiv_rn(px, dist); l1 = __fdiv_rn(py, dist); l2 = __fdiv_rn(pz, dist);
        } else {
          l0 = G.los[0]; l1 = G.los[1]; l2 = G.los[2];
        }
        float dot = __fadd_rn(__fadd_rn(__fmul_rn(t[0], l0), __fmul_rn(t[1], l1)), __fmul_rn(t[2], l2));
        float fd = __fmul_rn(G.f, dot);
        float r0 = __fmul_rn(fd, l0), r1 = __fmul_rn(fd, l1), r2 = __fmul_rn(fd, l2);
        if (fld == 1) { t[0] = r0; t[1] = r1; t[2] = r2; }
        else { t[0] = __fadd_rn(t[0], r0); t[1] = __fadd_rn(t[1], r1); t[2] = __fadd_rn(t[2], r2); }
      }
      if (mode == 1) { t[0] = __fsub_rn(px, t[0]); t[1] = __fsub_rn(py, t[1]); t[2] = __fsub_rn(pz, t[2]); }
      a0[q] = t[0]; a1[q] = t[1]; a2[q] = t[2];
    };
    emit(field, o0, o1, o2);
    if (p0) emit(field2, p0, p1, p2);
  }
}

}  // namespace

int readout(baorec_ctx* ctx, const float* psi3, const float* x, const float* y, const float* z, int64_t n,
            int field, int mode, float* o0, float* o1, float* o2, int field2, float* p0, float* p1, float* p2) {
  if (n <= 0) return BAOREC_OK;
  RGeom G;
  const int nn[3] = {ctx->n1, ctx->n2, ctx->n3};
  for (int a = 0; a < 3; ++a) {
    G.n[a] = nn[a];
    G.cell[a] = ctx->cfg.box_size[a] / (float)nn[a];
    G.bmin[a] = ctx->cfg.box_min[a];
    G.los[a] = ctx->cfg.los[a];
  }
  G.f = ctx->cfg.f;
  G.local = ctx->cfg.los_mode == BAOREC_LOS_LOCAL ? 1 : 0;
  unsigned grid = grid_for((size_t)n, 256);
  if (grid > 64u * kNumSMs) grid = 64u * kNumSMs;
  (readout_kernel<<<grid, 256, 0, ctx->stream>>>(psi3, ctx->N, x, y, z, n, G, field, mode, o0, o1, o2, field2, p0, p1,
                                                 p2, ctx->derr), ::baorec::count_launch());
  CKLAUNCH();
  return BAOREC_OK;
}

}  // namespace baorec
