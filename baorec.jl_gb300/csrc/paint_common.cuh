// Index arithmetic of the mass assignments shared by the atomic paint
// (paint.cu) and the sorted, deterministic one (paint_sorted.cu).
//
// It follows src/mas.jl:7-35 (BAOrec.jl) operation by operation with IEEE
// round-to-nearest intrinsics and no FMA contraction, so cell indices and
// fractional weights are bit-identical to the reference's FP32 CPU path.
#pragma once

#include "common.cuh"

namespace baorec {
namespace {

struct PaintGeom {
  int n[3];
  float fn[3];     // float(n)
  float L[3];
  float bmin[3];
  int wrap;
};

// src/mas.jl:8-10: every axis is tested against box_min[1] / box_size[1].
__device__ __forceinline__ float wrap_pos(float p, const PaintGeom& g) {
  return (__fsub_rn(p, g.bmin[0]) > g.L[0]) ? __fsub_rn(p, g.L[0]) : p;
}

// (p - box_min) * n / box_size + 1 (src/mas.jl:13-15), left to right.
__device__ __forceinline__ float cic_coord(float p, float bmin, float fn, float L) {
  return __fadd_rn(__fdiv_rn(__fmul_rn(__fsub_rn(p, bmin), fn), L), 1.0f);
}

// Lower/upper 1-based CIC cells and the fractional weight of the upper one
// (src/mas.jl:17-35).  Returns false when the reference would raise BoundsError.
__device__ __forceinline__ bool cic_axis(float gcoord, int n, int wrap, int& i0, int& i1, float& w1) {
  int c = (int)floorf(gcoord);
  w1 = __fsub_rn(gcoord, (float)c);
  if (c == n + 1) c = 1;
  int u = (c == n && wrap) ? 1 : c + 1;
  i0 = c; i1 = u;
  return c >= 1 && c <= n && u >= 1 && u <= n;
}

__device__ __forceinline__ size_t lin(int ix, int iy, int iz, const PaintGeom& g) {
  return (size_t)ix + (size_t)g.n[0] * ((size_t)iy + (size_t)g.n[1] * (size_t)iz);
}

// TSC: node i at box_min + i*cell, g = (p - box_min) n / L, nearest node
// c = floor(g + 1/2), d = g - c; weights 0.5(0.5-d)^2, 0.75-d^2, 0.5(0.5+d)^2.
__device__ __forceinline__ bool tsc_axis(float p, float bmin, float fn, float L, int n, int wrap,
                                         int idx[3], float wt[3]) {
  float gc = __fdiv_rn(__fmul_rn(__fsub_rn(p, bmin), fn), L);
  int c = (int)floorf(__fadd_rn(gc, 0.5f));
  float d = __fsub_rn(gc, (float)c);
  float a = __fsub_rn(0.5f, d), b = __fadd_rn(0.5f, d);
  wt[0] = __fmul_rn(__fmul_rn(0.5f, a), a);
  wt[1] = __fsub_rn(0.75f, __fmul_rn(d, d));
  wt[2] = __fmul_rn(__fmul_rn(0.5f, b), b);
  bool ok = true;
  for (int k = 0; k < 3; ++k) {
    int i = c - 1 + k;
    if (wrap) { i %= n; if (i < 0) i += n; }
    else if (i < 0 || i >= n) ok = false;
    idx[k] = i;
  }
  return ok;
}

inline PaintGeom paint_geom(const baorec_ctx* c, int wrap) {
  PaintGeom g;
  g.n[0] = c->n1; g.n[1] = c->n2; g.n[2] = c->n3;
  for (int a = 0; a < 3; ++a) {
    g.fn[a] = (float)g.n[a];
    g.L[a] = c->cfg.box_size[a];
    g.bmin[a] = c->cfg.box_min[a];
  }
  g.wrap = wrap ? 1 : 0;
  return g;
}

}  // namespace
}  // namespace baorec
