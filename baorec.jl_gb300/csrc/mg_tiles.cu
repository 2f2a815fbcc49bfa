// Shared-memory tile kernels of the residual-driven multigrid solver.
//
// A block owns a 32 x TY x TZ tile of a periodic level mesh.  It stages the
// tile plus a halo (y/z: 2 cells for the red-black sweep, 1 for residuals;
// x: 4 cells, so that every window row is ten aligned 16-byte chunks) in
// shared memory.  Each chunk is either wholly inside the mesh or wholly
// wrapped, and the wrapped offsets of the window rows are tabulated once per
// block, so a chunk costs a handful of instructions.  Right-hand sides have
// no reuse and are read straight from global memory.  Every launch is
// specialised on the line-of-sight mode (local: per-cell coefficients from p
// tables; global: uniform coefficients) and on whether the level has cells
// next to the observer whose first-derivative coefficients need clamping.
#include <mutex>
#include <set>
#include <utility>

#include "mg_common.cuh"

namespace baorec {
namespace {

constexpr int TX = 32, XH = 4, WX = TX + 2 * XH;   // tile width, x-halo, window pitch
constexpr int NT = 512, NWARP = NT / 32;           // threads per block
constexpr int CH = WX / 4;                         // 16-byte chunks per window row

// The right-hand side of a warp's output rows (row = warp + i NWARP, interior
// cells, no wrap) is read through a ring of PF registers filled PF rows
// ahead, so those loads overlap the window loads and the stencil work
// instead of stalling the row that consumes them.
template <int TY, int TZ, int NW = NWARP>
struct RowPrefetch {
  static constexpr int RPW = (TY * TZ + NW - 1) / NW;   // rows per warp
  static constexpr int PF = RPW < 4 ? RPW : 4;
  float v[PF];
  __device__ __forceinline__ static int offset(int i, int warp, int lane, int x0, int y0, int z0, const int* n) {
    const int row = warp + i * NW;
    const int ly = row % TY, lz = row / TY;
    return ((z0 + lz) * n[1] + (y0 + ly)) * n[0] + x0 + lane;
  }
  __device__ __forceinline__ void issue(int i, const float* __restrict__ src, int warp, int lane, int x0, int y0,
                                        int z0, const int* n) {
    if (i < RPW && warp + i * NW < TY * TZ) v[i % PF] = __ldg(src + offset(i, warp, lane, x0, y0, z0, n));
  }
};

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Row offsets (ix = 0 of the row) of the periodic window rows
// y in [y0-HY, y0+TY+HY), z in [z0-HY, z0+TZ+HY).
template <int HY, int TY, int TZ, int NTB = NT>
__device__ __forceinline__ void row_table(int* __restrict__ ro, int y0, int z0, const int n[3]) {
  constexpr int SY = TY + 2 * HY, SZ = TZ + 2 * HY;
  for (int r = threadIdx.x; r < SY * SZ; r += NTB) {
    const int ly = r % SY, lz = r / SY;
    ro[r] = n[0] * (wrapi(y0 - HY + ly, n[1]) + n[1] * wrapi(z0 - HY + lz, n[2]));
  }
}

// Window chunks: s[row][4c .. 4c+3] = g[row offset + wrap(x0 - XH + 4c) ..].
template <int HY, int TY, int TZ, int NTB = NT>
__device__ __forceinline__ void load_rows(float* __restrict__ s, const int* __restrict__ ro, const float* __restrict__ g,
                                          int x0, int n0) {
  constexpr int ROWS = (TY + 2 * HY) * (TZ + 2 * HY);
  constexpr int K = (ROWS * CH + NTB - 1) / NTB;   // chunks per thread, all in flight together
  float4* s4 = reinterpret_cast<float4*>(s);
  float4 v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int t = threadIdx.x + k * NTB;
    if (t < ROWS * CH) {
      const int row = t / CH, c = t - CH * row;
      v[k] = __ldg(reinterpret_cast<const float4*>(g + ro[row] + wrapi(x0 - XH + 4 * c, n0)));
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int t = threadIdx.x + k * NTB;
    if (t < ROWS * CH) s4[t] = v[k];
  }
}

template <int HY, int TY, int TZ, int NTB = NT>
__device__ __forceinline__ void load_ptab(float* __restrict__ sp, const LG& G, int x0, int y0, int z0) {
  for (int q = threadIdx.x; q < WX; q += NTB) sp[q] = G.P[0][wrapi(x0 - XH + q, G.n[0])];
  for (int q = threadIdx.x; q < TY + 2 * HY; q += NTB) sp[WX + q] = G.P[1][wrapi(y0 - HY + q, G.n[1])];
  for (int q = threadIdx.x; q < TZ + 2 * HY; q += NTB) sp[2 * WX + q] = G.P[2][wrapi(z0 - HY + q, G.n[2])];
}

// Operator coefficients of one cell (approximate division: smoother and
// correction residual of a defect correction).
struct Cf {
  float gpx, gpy, gpz, hxy, hxz, hyz, dx, dy, dz, diag;
};

template <bool LOCAL, bool CLAMP>
__device__ __forceinline__ Cf coef_fast(float px, float py, float pz, const LG& G) {
  Cf c;
  const float px2 = px * px, py2 = py * py, pz2 = pz * pz;
  const float g = __fdividef(G.beta, G.cell2[0] * px2 + G.cell2[1] * py2 + G.cell2[2] * pz2);
  c.gpx = G.icell2[0] + g * px2;
  c.gpy = G.icell2[1] + g * py2;
  c.gpz = G.icell2[2] + g * pz2;
  const float hg = 0.5f * g;
  c.hxy = hg * (px * py); c.hxz = hg * (px * pz); c.hyz = hg * (py * pz);
  if (LOCAL) {
    c.dx = g * px; c.dy = g * py; c.dz = g * pz;
    if (CLAMP) {
      const float k = kClamp;
      c.dx = fminf(fmaxf(c.dx, -k * c.gpx), k * c.gpx);
      c.dy = fminf(fmaxf(c.dy, -k * c.gpy), k * c.gpy);
      c.dz = fminf(fmaxf(c.dz, -k * c.gpz), k * c.gpz);
    }
  } else {
    c.dx = c.dy = c.dz = 0.0f;
  }
  c.diag = 2.0f * (c.gpx + c.gpy + c.gpz);
  return c;
}

// Neighbour sum (the bracket of the operator) at shared index q.
template <bool LOCAL, int SXY>
__device__ __forceinline__ float nbr(const float* __restrict__ s, int q, const Cf& c) {
  constexpr int SX = WX;
  const float xp = s[q + 1], xm = s[q - 1], yp = s[q + SX], ym = s[q - SX], zp = s[q + SXY], zm = s[q - SXY];
  float o = c.gpx * (xp + xm) + c.gpy * (yp + ym) + c.gpz * (zp + zm) +
            c.hxy * ((s[q + 1 + SX] + s[q - 1 - SX]) - (s[q - 1 + SX] + s[q + 1 - SX])) +
            c.hxz * ((s[q + 1 + SXY] + s[q - 1 - SXY]) - (s[q - 1 + SXY] + s[q + 1 - SXY])) +
            c.hyz * ((s[q + SX + SXY] + s[q - SX - SXY]) - (s[q - SX + SXY] + s[q + SX - SXY]));
  if (LOCAL) o += c.dx * (xp - xm) + c.dy * (yp - ym) + c.dz * (zp - zm);
  return o;
}

// The same bracket over differences D = s_nb - s_q.  The operator's row sums
// vanish, so A s = -bracket(D); for smooth s the differences are exact to a
// rounding of their own size, where diag*s_q - bracket(s) cancels to a
// rounding of s_q's size (relative error growing like 1/(k h)^2).
template <bool LOCAL, int SXY>
__device__ __forceinline__ float nbr_diff(const float* __restrict__ s, int q, const Cf& c) {
  constexpr int SX = WX;
  const float s0 = s[q];
  auto D = [&](int o) { return s[q + o] - s0; };
  const float xp = s[q + 1], xm = s[q - 1], yp = s[q + SX], ym = s[q - SX], zp = s[q + SXY], zm = s[q - SXY];
  float o = c.gpx * ((xp - s0) + (xm - s0)) + c.gpy * ((yp - s0) + (ym - s0)) + c.gpz * ((zp - s0) + (zm - s0)) +
            c.hxy * ((D(1 + SX) + D(-1 - SX)) - (D(-1 + SX) + D(1 - SX))) +
            c.hxz * ((D(1 + SXY) + D(-1 - SXY)) - (D(-1 + SXY) + D(1 - SXY))) +
            c.hyz * ((D(SX + SXY) + D(-SX - SXY)) - (D(-SX + SXY) + D(SX - SXY)));
  if (LOCAL) o += c.dx * (xp - xm) + c.dy * (yp - ym) + c.dz * (zp - zm);
  return o;
}

// r = rhs - shift - Ã e (correction equation, clamped operator).
template <bool LOCAL, bool CLAMP, int TY, int TZ, bool DIFF = false>
__global__ void __launch_bounds__(NT) resid_kernel(const float* __restrict__ e, const float* __restrict__ rhs,
                                                   float* __restrict__ r, LG G, float shift,
                                                   float* __restrict__ acc) {
  constexpr int SY = TY + 2, SZ = TZ + 2, SXY = WX * SY;
  extern __shared__ __align__(16) float smem[];
  float* sv = smem;
  int* ro = reinterpret_cast<int*>(sv + WX * SY * SZ);
  float* sp = reinterpret_cast<float*>(ro + SY * SZ);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  using RP = RowPrefetch<TY, TZ>;
  RP pr, pa;
#pragma unroll
  for (int i = 0; i < RP::PF; ++i) {
    pr.issue(i, rhs, warp, lane, x0, y0, z0, G.n);
    if (acc) pa.issue(i, acc, warp, lane, x0, y0, z0, G.n);
  }
  row_table<1, TY, TZ>(ro, y0, z0, G.n);
  if (LOCAL) load_ptab<1, TY, TZ>(sp, G, x0, y0, z0);
  __syncthreads();
  load_rows<1, TY, TZ>(sv, ro, e, x0, G.n[0]);
  Cf cu;
  if (!LOCAL) cu = coef_fast<false, false>(G.pg[0], G.pg[1], G.pg[2], G);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < RP::RPW; ++i) {
    const int row = warp + i * NWARP;
    if (row >= TY * TZ) break;
    const float rv = pr.v[i % RP::PF];
    const float av = acc ? pa.v[i % RP::PF] : 0.0f;
    pr.issue(i + RP::PF, rhs, warp, lane, x0, y0, z0, G.n);
    if (acc) pa.issue(i + RP::PF, acc, warp, lane, x0, y0, z0, G.n);
    const int ly = 1 + row % TY, lz = 1 + row / TY, lx = XH + lane;
    const int q = lx + WX * ly + SXY * lz;
    const Cf cf = LOCAL ? coef_fast<true, CLAMP>(sp[lx], sp[WX + ly], sp[2 * WX + lz], G) : cu;
    const int o = ro[ly + SY * lz] + x0 + lane;
    if (DIFF)
      r[o] = (rv - shift) + nbr_diff<LOCAL, SXY>(sv, q, cf);
    else
      r[o] = (rv - shift) - (cf.diag * sv[q] - nbr<LOCAL, SXY>(sv, q, cf));
    if (acc) acc[o] = av + sv[q];   // optional: accumulate the operand into a running sum
  }
}

// The reference schedule's stencils on 32 x TY x TZ tiles of NTH threads, with
// the per-cell arithmetic of jacobi_kernel / residual_kernel (coef_at, the
// neighbours in gather's order, offdiag) and the neighbours read from the
// tile window instead of global memory:
//   JACOBI  one damped-Jacobi sweep (src/multigrid.jl:137-191, 207),
//           out = (1-ω) v + ω (f + bracket(v)) / diag;
//   else    the residual (src/multigrid.jl:328-376, 393),
//           out = (f - shift) - (diag v - bracket(v)), shift passed as omega.
template <int TY, int TZ, int NTH, bool JACOBI>
__global__ void __launch_bounds__(NTH, 1024 / NTH) jacobi_tile_kernel(const float* __restrict__ v,
                                                                     const float* __restrict__ f,
                                                                     float* __restrict__ out, LG G, float omega) {
  constexpr int SY = TY + 2, SZ = TZ + 2, SXY = WX * SY, NW = NTH / 32;
  extern __shared__ __align__(16) float smem[];
  float* sv = smem;
  int* ro = reinterpret_cast<int*>(sv + WX * SY * SZ);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  using RP = RowPrefetch<TY, TZ, NW>;
  RP pf;
#pragma unroll
  for (int i = 0; i < RP::PF; ++i) pf.issue(i, f, warp, lane, x0, y0, z0, G.n);
  row_table<1, TY, TZ, NTH>(ro, y0, z0, G.n);
  __syncthreads();
  load_rows<1, TY, TZ, NTH>(sv, ro, v, x0, G.n[0]);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < RP::RPW; ++i) {
    const int row = warp + i * NW;
    if (row >= TY * TZ) break;
    const float fv = pf.v[i % RP::PF];
    pf.issue(i + RP::PF, f, warp, lane, x0, y0, z0, G.n);
    const int ly = 1 + row % TY, lz = 1 + row / TY, lx = XH + lane;
    const int q = lx + WX * ly + SXY * lz;
    const Coef c = coef_at(G, x0 + lane, y0 + ly - 1, z0 + lz - 1);
    Nb b;
    b.xp = sv[q + 1]; b.xm = sv[q - 1];
    b.yp = sv[q + WX]; b.ym = sv[q - WX];
    b.zp = sv[q + SXY]; b.zm = sv[q - SXY];
    b.pp0 = sv[q + 1 + WX]; b.mm0 = sv[q - 1 - WX]; b.mp0 = sv[q - 1 + WX]; b.pm0 = sv[q + 1 - WX];
    b.p0p = sv[q + 1 + SXY]; b.m0m = sv[q - 1 - SXY]; b.m0p = sv[q - 1 + SXY]; b.p0m = sv[q + 1 - SXY];
    b._pp = sv[q + WX + SXY]; b._mm = sv[q - WX - SXY]; b._mp = sv[q - WX + SXY]; b._pm = sv[q + WX - SXY];
    if (JACOBI) {
      float jac = fv + offdiag(c, b, G.local);
      jac /= 2.0f * (c.gpx + c.gpy + c.gpz);
      out[ro[ly + SY * lz] + x0 + lane] = (1.0f - omega) * sv[q] + omega * jac;
    } else {
      const float av = 2.0f * (c.gpx + c.gpy + c.gpz) * sv[q] - offdiag(c, b, G.local);
      out[ro[ly + SY * lz] + x0 + lane] = (fv - omega) - av;
    }
  }
}

// Gauss-Seidel values of two cells (shared indices qa, qb) that share p_y:
// (rhs + neighbours) / diagonal, clamped operator, fast reciprocals.
template <bool LOCAL, bool CLAMP, int SXY>
__device__ __forceinline__ f2 gs_two(const float* __restrict__ s, int qa, int qb, f2 fr, f2 Px, float py, f2 Pz,
                                     const Cf& cu, const LG& G) {
  constexpr int SX = WX;
  auto L2 = [&](int off) { return P2(s[qa + off], s[qb + off]); };
  const f2 xp = L2(1), xm = L2(-1), yp = L2(SX), ym = L2(-SX), zp = L2(SXY), zm = L2(-SXY);
  const f2 Sx = add2(xp, xm), Sy = add2(yp, ym), Sz = add2(zp, zm);
  const f2 Xxy = sub2(add2(L2(1 + SX), L2(-1 - SX)), add2(L2(-1 + SX), L2(1 - SX)));
  const f2 Xxz = sub2(add2(L2(1 + SXY), L2(-1 - SXY)), add2(L2(-1 + SXY), L2(1 - SXY)));
  const f2 Xyz = sub2(add2(L2(SX + SXY), L2(-SX - SXY)), add2(L2(-SX + SXY), L2(SX - SXY)));
  f2 gpx, gpy, gpz, hxy, hxz, hyz;
  if (LOCAL) {
    const f2 px2 = mul2(Px, Px), pz2 = mul2(Pz, Pz);
    const float py2 = py * py;
    const f2 den = fma2(B2(G.cell2[0]), px2, fma2(B2(G.cell2[2]), pz2, B2(G.cell2[1] * py2)));
    const f2 g = mul2(B2(G.beta), rcp2(den));
    gpx = fma2(g, px2, B2(G.icell2[0]));
    gpy = fma2(g, B2(py2), B2(G.icell2[1]));
    gpz = fma2(g, pz2, B2(G.icell2[2]));
    f2 dx = mul2(g, Px), dy = mul2(g, B2(py)), dz = mul2(g, Pz);
    const f2 hPz = mul2(B2(0.5f), Pz);
    hxy = mul2(dx, B2(0.5f * py));
    hxz = mul2(dx, hPz);
    hyz = mul2(dy, hPz);
    if (CLAMP) {
      float a[3], b[3], la[3], lb[3];
      U2(dx, a[0], b[0]); U2(dy, a[1], b[1]); U2(dz, a[2], b[2]);
      U2(gpx, la[0], lb[0]); U2(gpy, la[1], lb[1]); U2(gpz, la[2], lb[2]);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        a[q] = fminf(fmaxf(a[q], -kClamp * la[q]), kClamp * la[q]);
        b[q] = fminf(fmaxf(b[q], -kClamp * lb[q]), kClamp * lb[q]);
      }
      dx = P2(a[0], b[0]); dy = P2(a[1], b[1]); dz = P2(a[2], b[2]);
    }
    f2 o = mul2(gpx, Sx);
    o = fma2(gpy, Sy, o);
    o = fma2(gpz, Sz, o);
    o = fma2(hxy, Xxy, o);
    o = fma2(hxz, Xxz, o);
    o = fma2(hyz, Xyz, o);
    o = fma2(dx, sub2(xp, xm), o);
    o = fma2(dy, sub2(yp, ym), o);
    o = fma2(dz, sub2(zp, zm), o);
    return mul2(add2(fr, o), mul2(B2(0.5f), rcp2(add2(add2(gpx, gpy), gpz))));
  }
  f2 o = mul2(B2(cu.gpx), Sx);
  o = fma2(B2(cu.gpy), Sy, o);
  o = fma2(B2(cu.gpz), Sz, o);
  o = fma2(B2(cu.hxy), Xxy, o);
  o = fma2(B2(cu.hxz), Xxz, o);
  o = fma2(B2(cu.hyz), Xyz, o);
  return mul2(add2(fr, o), B2(1.0f / cu.diag));
}

// One red-black Gauss-Seidel sweep, both colours in one pass, out of place.
// Red cells of the tile and of a one-cell ring around it are updated from the
// old window; then the black cells of the tile from the red-updated window.
// Window frame: x = x0 - 4 + lx, y = y0 - 2 + ly, z = z0 - 2 + lz; all three
// origins are even, so window parity is mesh parity.  Cell positions are fixed
// per thread, two cells per packed evaluation.  Red (ring rows ly, lz in [1, S-1), 17 cells per
// row): thread -> (row slot, cell t) once; rows of plane lz pair with plane
// lz + H (H = TZ/2 + 1 is odd, so the pair's parities differ and so do their
// x positions).  Black (tile rows, 16 cells per row): planes lz and lz + TZ/2
// pair (same parity, same x position).
template <bool LOCAL, bool CLAMP, int TY, int TZ>
__global__ void __launch_bounds__(NT, 2) rb_sweep2_kernel(const float* __restrict__ vin, float* __restrict__ vout,
                                                          const float* __restrict__ rhs, LG G, float shift) {
  constexpr int SY = TY + 4, SZ = TZ + 4, SXY = WX * SY;
  extern __shared__ __align__(16) float smem[];
  float* sv = smem;
  int* ro = reinterpret_cast<int*>(sv + WX * SY * SZ);
  float* sp = reinterpret_cast<float*>(ro + SY * SZ);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  row_table<2, TY, TZ>(ro, y0, z0, G.n);
  if (LOCAL) load_ptab<2, TY, TZ>(sp, G, x0, y0, z0);
  __syncthreads();
  load_rows<2, TY, TZ>(sv, ro, vin, x0, G.n[0]);
  Cf cu;
  if (!LOCAL) cu = coef_fast<false, false>(G.pg[0], G.pg[1], G.pg[2], G);
  __syncthreads();
  const f2 sh2 = B2(shift);
  // ---- red
  constexpr int RPR = 17, RSL = NT / RPR, RY = SY - 2, HP = TZ / 2 + 1, PR = RY * HP;
  constexpr int KR = (PR + RSL - 1) / RSL;
  static_assert(HP % 2 == 1, "red pairs need planes of opposite parity");
  const unsigned slot = threadIdx.x / RPR, t = threadIdx.x - RPR * slot;
  const int lxo = 3 + 2 * (int)t, lxe = lxo + 1;   // odd and even x positions of this thread's cells
  const float pxe = LOCAL ? sp[lxe] : 0.0f, pxo = LOCAL ? sp[lxo] : 0.0f;
  const int gxe = wrapi(x0 - XH + lxe, G.n[0]), gxo = wrapi(x0 - XH + lxo, G.n[0]);
  f2 nv[KR];
  int qa[KR], qb[KR];
#pragma unroll
  for (int k = 0; k < KR; ++k) {
    const unsigned pr = slot + RSL * k;
    qa[k] = -1;
    if (slot < RSL && pr < PR) {
      const int ly = 1 + pr % RY, lza = 1 + pr / RY, lzb = lza + HP;
      const bool ea = ((ly + lza) & 1) == 0;   // red: lx+ly+lz even, so cell a sits at an even lx
      const int lxa = ea ? lxe : lxo, lxb = ea ? lxo : lxe;
      qa[k] = lxa + WX * ly + SXY * lza;
      qb[k] = lxb + WX * ly + SXY * lzb;
      const f2 Px = P2(ea ? pxe : pxo, ea ? pxo : pxe);
      const f2 Pz = LOCAL ? P2(sp[2 * WX + lza], sp[2 * WX + lzb]) : B2(0.0f);
      const float py = LOCAL ? sp[WX + ly] : 0.0f;
      const f2 fr = sub2(P2(__ldg(rhs + ro[ly + SY * lza] + (ea ? gxe : gxo)),
                            __ldg(rhs + ro[ly + SY * lzb] + (ea ? gxo : gxe))), sh2);
      nv[k] = gs_two<LOCAL, CLAMP, SXY>(sv, qa[k], qb[k], fr, Px, py, Pz, cu, G);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < KR; ++k)
    if (qa[k] >= 0) {
      float a, b;
      U2(nv[k], a, b);
      sv[qa[k]] = a;
      sv[qb[k]] = b;
    }
  __syncthreads();
  // ---- black
  constexpr int BSL = NT / 16, HB = TZ / 2, PB = TY * HB, KB = (PB + BSL - 1) / BSL;
  const unsigned bslot = threadIdx.x >> 4, tb = threadIdx.x & 15;
  f2 nb[KB];
  int qc[KB];
#pragma unroll
  for (int k = 0; k < KB; ++k) {
    const unsigned pr = bslot + BSL * k;
    qc[k] = -1;
    if (pr < PB) {
      const int ly = 2 + pr % TY, lza = 2 + pr / TY, lzb = lza + HB;
      const int lx = 4 + ((ly + lza + 1) & 1) + 2 * (int)tb;
      qc[k] = lx + WX * ly + SXY * lza;
      const float px = LOCAL ? sp[lx] : 0.0f, py = LOCAL ? sp[WX + ly] : 0.0f;
      const f2 Pz = LOCAL ? P2(sp[2 * WX + lza], sp[2 * WX + lzb]) : B2(0.0f);
      const int gx = x0 - XH + lx;
      const f2 fr = sub2(P2(__ldg(rhs + ro[ly + SY * lza] + gx), __ldg(rhs + ro[ly + SY * lzb] + gx)), sh2);
      nb[k] = gs_two<LOCAL, CLAMP, SXY>(sv, qc[k], qc[k] + HB * SXY, fr, B2(px), py, Pz, cu, G);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < KB; ++k)
    if (qc[k] >= 0) {
      float a, b;
      U2(nb[k], a, b);
      sv[qc[k]] = a;
      sv[qc[k] + HB * SXY] = b;
    }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int row = warp; row < TY * TZ; row += NWARP) {
    const int ly = 2 + row % TY, lz = 2 + row / TY;
    vout[ro[ly + SY * lz] + x0 + lane] = sv[XH + lane + WX * ly + SXY * lz];
  }
}

// The FP32 running residual of the FFT corrections on 32 x TY x 16 tiles (TY =
// 16: two blocks of 512 threads per SM; TY = 8: four of 256), two
// z-adjacent cells per thread in packed FP32x2 arithmetic:
//   r = (rhs - shift) + bracket(e_nb - e_0),  acc += e  (optional).
// The window is stored as plane pairs: pair j interleaves window planes 2j
// and 2j+1 per cell, so one 8-byte shared load at an in-plane offset gives a
// cell column's values in two planes.  A thread computes window planes 2k+1
// (cell A) and 2k+2 (cell B); pairs k and k+1 at the nine in-plane offsets
// hold every value of both stencils: the z-1 and z+1 values of (A, B) are
// the pairs themselves, the in-plane values one register move from a pair.
// Warp w computes window row y = 1 + w, lane l column x = XH + l.
template <bool LOCAL, int TY, int TZ = 16>
__global__ void __launch_bounds__(32 * TY, 32 / TY) resid_pairs_kernel(const float* __restrict__ e,
                                                                     const float* __restrict__ rhs,
                                                                     float* __restrict__ r, LG G, float shift,
                                                                     float* __restrict__ acc) {
  constexpr int NTH = 32 * TY;       // one warp per output row
  constexpr int SY = TY + 2, SZ = TZ + 2;
  constexpr int NPR = SZ / 2;        // plane pairs in the window
  constexpr int PR = 2 * WX;         // floats per row of a plane pair
  constexpr int PP = SY * PR;        // floats per plane pair
  constexpr int NK = TZ / 2;         // output pairs per thread
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;
  int* ro = reinterpret_cast<int*>(sw + NPR * PP);
  float* sp = reinterpret_cast<float*>(ro + SY * SZ);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ly = 1 + warp, lx = XH + lane;
  const size_t plane = (size_t)G.n[0] * G.n[1];
  const size_t col = (size_t)(y0 + warp) * G.n[0] + x0 + lane;   // (x, y) of the thread's cells at z = 0
  // right-hand side (and acc) of the thread's cells: pair k in (r0, a0), pair
  // k + 1 in (r1, a1), loaded two pairs ahead of use
  float r0[2] = {0.0f, 0.0f}, r1[2] = {0.0f, 0.0f}, a0[2] = {0.0f, 0.0f}, a1[2] = {0.0f, 0.0f};
  auto issue = [&](int k, float* rr, float* aa) {
    if (k < NK) {
      const size_t o = col + (size_t)(z0 + 2 * k) * plane;
      rr[0] = __ldg(rhs + o);
      rr[1] = __ldg(rhs + o + plane);
      if (acc) { aa[0] = acc[o]; aa[1] = acc[o + plane]; }
    }
  };
  issue(0, r0, a0);
  issue(1, r1, a1);
  row_table<1, TY, TZ, NTH>(ro, y0, z0, G.n);
  if (LOCAL) load_ptab<1, TY, TZ, NTH>(sp, G, x0, y0, z0);
  __syncthreads();
  {
    constexpr int TOT = NPR * SY * CH;
    // every chunk of the thread in flight at once, or in rounds of four
    constexpr int K = (TOT + NTH - 1) / NTH, B = K <= 4 ? K : 4;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += B) {
      float4 a[B], b[B];
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const int t = threadIdx.x + (k0 + i) * NTH;
        if (k0 + i < K && t < TOT) {
          const int row = t / CH, c = t - CH * row;   // row = pair * SY + y
          const int j = row / SY, yy = row - SY * j;
          const int xo = wrapi(x0 - XH + 4 * c, G.n[0]);
          a[i] = __ldg(reinterpret_cast<const float4*>(e + ro[yy + SY * (2 * j)] + xo));
          b[i] = __ldg(reinterpret_cast<const float4*>(e + ro[yy + SY * (2 * j + 1)] + xo));
        }
      }
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const int t = threadIdx.x + (k0 + i) * NTH;
        if (k0 + i < K && t < TOT) {
          const int row = t / CH, c = t - CH * row;
          float4* d = reinterpret_cast<float4*>(sw + row * PR + 8 * c);
          d[0] = make_float4(a[i].x, b[i].x, a[i].y, b[i].y);
          d[1] = make_float4(a[i].z, b[i].z, a[i].w, b[i].w);
        }
      }
    }
  }
  __syncthreads();
  const float px = LOCAL ? sp[lx] : G.pg[0], py = LOCAL ? sp[WX + ly] : G.pg[1];
  const float px2 = px * px, py2 = py * py;
  const float dxy = coef_dxy(G, px2, py2);
  auto L = [&](int q) { return *reinterpret_cast<const f2*>(sw + q); };
  // (second plane of pair a, first plane of pair b): the in-plane values of (A, B)
  auto C = [](f2 a, f2 b) {
    float a0, a1, b0, b1;
    U2(a, a0, a1);
    U2(b, b0, b1);
    return P2(a1, b0);
  };
  constexpr int OX = 2, OY = PR;
#pragma unroll 1
  for (int k = 0; k < NK; ++k) {
    const float rA = r0[0], rB = r0[1], aA = a0[0], aB = a0[1];
    r0[0] = r1[0]; r0[1] = r1[1]; a0[0] = a1[0]; a0[1] = a1[1];
    issue(k + 2, r1, a1);
    const f2 Pz = LOCAL ? P2(sp[2 * WX + 2 * k + 1], sp[2 * WX + 2 * k + 2]) : B2(G.pg[2]);
    const f2 pz2 = mul2(Pz, Pz);
    float dA, dB;
    U2(fma2(B2(G.cell2[2]), pz2, B2(dxy)), dA, dB);
    const f2 g = P2(__fdividef(G.beta, dA), __fdividef(G.beta, dB));
    const f2 gpz = fma2(g, pz2, B2(G.icell2[2]));
    const f2 hg = mul2(B2(0.5f), g);
    const int q0 = (k * SY + ly) * PR + 2 * lx, q1 = q0 + PP;   // pairs k and k + 1 at (y, x)
    // (A, B) one plane down is pair k, one plane up pair k + 1
    const f2 zm = L(q0), zp = L(q1);
    const f2 s0 = C(zm, zp);
    f2 o = mul2(gpz, add2(sub2(zp, s0), sub2(zm, s0)));
    if (LOCAL) o = fma2(mul2(g, Pz), sub2(zp, zm), o);
    {   // x neighbours and the x-z diagonals
      const f2 kp = L(q0 + OX), km = L(q0 - OX), lp = L(q1 + OX), lm = L(q1 - OX);
      const f2 xp = C(kp, lp), xm = C(km, lm);
      o = fma2(fma2(g, B2(px2), B2(G.icell2[0])), add2(sub2(xp, s0), sub2(xm, s0)), o);
      o = fma2(mul2(hg, mul2(B2(px), Pz)), sub2(add2(sub2(lp, s0), sub2(km, s0)), add2(sub2(lm, s0), sub2(kp, s0))), o);
      if (LOCAL) o = fma2(mul2(g, B2(px)), sub2(xp, xm), o);
    }
    {   // y neighbours and the y-z diagonals
      const f2 kp = L(q0 + OY), km = L(q0 - OY), lp = L(q1 + OY), lm = L(q1 - OY);
      const f2 yp = C(kp, lp), ym = C(km, lm);
      o = fma2(fma2(g, B2(py2), B2(G.icell2[1])), add2(sub2(yp, s0), sub2(ym, s0)), o);
      o = fma2(mul2(hg, mul2(B2(py), Pz)), sub2(add2(sub2(lp, s0), sub2(km, s0)), add2(sub2(lm, s0), sub2(kp, s0))), o);
      if (LOCAL) o = fma2(mul2(g, B2(py)), sub2(yp, ym), o);
    }
    {   // x-y diagonals (in-plane)
      const f2 pp = C(L(q0 + OX + OY), L(q1 + OX + OY)), mm = C(L(q0 - OX - OY), L(q1 - OX - OY));
      const f2 mp = C(L(q0 - OX + OY), L(q1 - OX + OY)), pm = C(L(q0 + OX - OY), L(q1 + OX - OY));
      o = fma2(mul2(hg, B2(px * py)), sub2(add2(sub2(pp, s0), sub2(mm, s0)), add2(sub2(mp, s0), sub2(pm, s0))), o);
    }
    float oA, oB, sA, sB;
    U2(o, oA, oB);
    U2(s0, sA, sB);
    const size_t ga = col + (size_t)(z0 + 2 * k) * plane;
    r[ga] = (rA - shift) + oA;
    r[ga + plane] = (rB - shift) + oB;
    if (acc) {
      acc[ga] = aA + sA;
      acc[ga + plane] = aB + sB;
    }
  }
}

// The running residual of resid_pairs_kernel with the window streamed in z:
// a block owns a 32 x 16 x TZ tile and keeps only three plane pairs of its
// window in shared memory, a ring of slots.  Output pair k reads pairs k and
// k + 1; the loads of pair k + 2 are issued into registers before pair k is
// computed and stored into the slot pair k - 1 held after it, so they land
// while the stencil runs instead of in a separate load phase (one barrier per
// pair).  Per-cell arithmetic, thread mapping and window layout within a
// pair are those of resid_pairs_kernel, so the results are the same bits.
template <bool LOCAL, int TZ>
__global__ void __launch_bounds__(NT, 2) resid_pairz_kernel(const float* __restrict__ e, const float* __restrict__ rhs,
                                                          float* __restrict__ r, LG G, float shift,
                                                          float* __restrict__ acc) {
  constexpr int TY = 16, SY = TY + 2;
  constexpr int PR = 2 * WX;         // floats per row of a plane pair
  constexpr int PP = SY * PR;        // floats per plane pair (one ring slot)
  constexpr int NK = TZ / 2;         // output pairs per thread
  constexpr int NS = 3;              // ring slots
  constexpr int LT = SY * CH;        // 16-byte chunks of one plane of a pair: one per loading thread
  static_assert(NWARP == TY, "one warp per output row");
  static_assert(LT <= NT, "one chunk per thread and plane");
  extern __shared__ __align__(16) float smem[];
  float* sw = smem;                                   // NS slots
  int* roy = reinterpret_cast<int*>(sw + NS * PP);    // SY row offsets (y part)
  float* sp = reinterpret_cast<float*>(roy + SY);     // px (WX) | py (SY) | pz (TZ + 2)
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ly = 1 + warp, lx = XH + lane;
  const size_t plane = (size_t)G.n[0] * G.n[1];
  const size_t col = (size_t)(y0 + warp) * G.n[0] + x0 + lane;
  float r0[2] = {0.0f, 0.0f}, r1[2] = {0.0f, 0.0f}, a0[2] = {0.0f, 0.0f}, a1[2] = {0.0f, 0.0f};
  auto issue = [&](int k, float* rr, float* aa) {
    if (k < NK) {
      const size_t o = col + (size_t)(z0 + 2 * k) * plane;
      rr[0] = __ldg(rhs + o);
      rr[1] = __ldg(rhs + o + plane);
      if (acc) { aa[0] = acc[o]; aa[1] = acc[o + plane]; }
    }
  };
  issue(0, r0, a0);
  issue(1, r1, a1);
  // this thread's chunk of a plane pair: window row yy, x chunk c
  const int lrow = threadIdx.x / CH, lc = threadIdx.x - CH * lrow;
  const bool loader = threadIdx.x < LT;
  const int xo = wrapi(x0 - XH + 4 * lc, G.n[0]);
  const int yoff = loader ? G.n[0] * wrapi(y0 - 1 + lrow, G.n[1]) : 0;
  // window plane w (0 = z0 - 1) of the mesh: periodic plane offset
  auto zoff = [&](int w) { return (size_t)wrapi(z0 - 1 + w, G.n[2]) * plane; };
  float4 pa, pb;   // chunk of plane pair j in flight
  auto fetch = [&](int j) {
    if (loader) {
      pa = __ldg(reinterpret_cast<const float4*>(e + zoff(2 * j) + yoff + xo));
      pb = __ldg(reinterpret_cast<const float4*>(e + zoff(2 * j + 1) + yoff + xo));
    }
  };
  auto put = [&](int slot) {
    if (loader) {
      float4* d = reinterpret_cast<float4*>(sw + slot * PP + lrow * PR + 8 * lc);
      d[0] = make_float4(pa.x, pb.x, pa.y, pb.y);
      d[1] = make_float4(pa.z, pb.z, pa.w, pb.w);
    }
  };
  fetch(0);
  {
    const float4 qa = pa, qb = pb;
    fetch(1);
    if (loader) {
      float4* d = reinterpret_cast<float4*>(sw + lrow * PR + 8 * lc);
      d[0] = make_float4(qa.x, qb.x, qa.y, qb.y);
      d[1] = make_float4(qa.z, qb.z, qa.w, qb.w);
    }
  }
  put(1);
  if (LOCAL) {
    for (int q = threadIdx.x; q < WX; q += NT) sp[q] = G.P[0][wrapi(x0 - XH + q, G.n[0])];
    for (int q = threadIdx.x; q < SY; q += NT) sp[WX + q] = G.P[1][wrapi(y0 - 1 + q, G.n[1])];
    for (int q = threadIdx.x; q < TZ + 2; q += NT) sp[WX + SY + q] = G.P[2][wrapi(z0 - 1 + q, G.n[2])];
  }
  __syncthreads();
  const float px = LOCAL ? sp[lx] : G.pg[0], py = LOCAL ? sp[WX + ly] : G.pg[1];
  const float px2 = px * px, py2 = py * py;
  const float dxy = coef_dxy(G, px2, py2);
  auto L = [&](int q) { return *reinterpret_cast<const f2*>(sw + q); };
  auto C = [](f2 a, f2 b) {
    float a0, a1, b0, b1;
    U2(a, a0, a1);
    U2(b, b0, b1);
    return P2(a1, b0);
  };
  constexpr int OX = 2, OY = PR;
#pragma unroll 1
  for (int k = 0; k < NK; ++k) {
    const float rA = r0[0], rB = r0[1], aA = a0[0], aB = a0[1];
    r0[0] = r1[0]; r0[1] = r1[1]; a0[0] = a1[0]; a0[1] = a1[1];
    issue(k + 2, r1, a1);
    if (k + 2 <= NK) fetch(k + 2);   // pairs 0 .. NK of the window
    const f2 Pz = LOCAL ? P2(sp[WX + SY + 2 * k + 1], sp[WX + SY + 2 * k + 2]) : B2(G.pg[2]);
    const f2 pz2 = mul2(Pz, Pz);
    float dA, dB;
    U2(fma2(B2(G.cell2[2]), pz2, B2(dxy)), dA, dB);
    const f2 g = P2(__fdividef(G.beta, dA), __fdividef(G.beta, dB));
    const f2 gpz = fma2(g, pz2, B2(G.icell2[2]));
    const f2 hg = mul2(B2(0.5f), g);
    const int q0 = ((k % NS) * SY + ly) * PR + 2 * lx, q1 = (((k + 1) % NS) * SY + ly) * PR + 2 * lx;
    const f2 zm = L(q0), zp = L(q1);
    const f2 s0 = C(zm, zp);
    f2 o = mul2(gpz, add2(sub2(zp, s0), sub2(zm, s0)));
    if (LOCAL) o = fma2(mul2(g, Pz), sub2(zp, zm), o);
    {   // x neighbours and the x-z diagonals
      const f2 kp = L(q0 + OX), km = L(q0 - OX), lp = L(q1 + OX), lm = L(q1 - OX);
      const f2 xp = C(kp, lp), xm = C(km, lm);
      o = fma2(fma2(g, B2(px2), B2(G.icell2[0])), add2(sub2(xp, s0), sub2(xm, s0)), o);
      o = fma2(mul2(hg, mul2(B2(px), Pz)), sub2(add2(sub2(lp, s0), sub2(km, s0)), add2(sub2(lm, s0), sub2(kp, s0))), o);
      if (LOCAL) o = fma2(mul2(g, B2(px)), sub2(xp, xm), o);
    }
    {   // y neighbours and the y-z diagonals
      const f2 kp = L(q0 + OY), km = L(q0 - OY), lp = L(q1 + OY), lm = L(q1 - OY);
      const f2 yp = C(kp, lp), ym = C(km, lm);
      o = fma2(fma2(g, B2(py2), B2(G.icell2[1])), add2(sub2(yp, s0), sub2(ym, s0)), o);
      o = fma2(mul2(hg, mul2(B2(py), Pz)), sub2(add2(sub2(lp, s0), sub2(km, s0)), add2(sub2(lm, s0), sub2(kp, s0))), o);
      if (LOCAL) o = fma2(mul2(g, B2(py)), sub2(yp, ym), o);
    }
    {   // x-y diagonals (in-plane)
      const f2 pp = C(L(q0 + OX + OY), L(q1 + OX + OY)), mm = C(L(q0 - OX - OY), L(q1 - OX - OY));
      const f2 mp = C(L(q0 - OX + OY), L(q1 - OX + OY)), pm = C(L(q0 + OX - OY), L(q1 + OX - OY));
      o = fma2(mul2(hg, B2(px * py)), sub2(add2(sub2(pp, s0), sub2(mm, s0)), add2(sub2(mp, s0), sub2(pm, s0))), o);
    }
    float oA, oB, sA, sB;
    U2(o, oA, oB);
    U2(s0, sA, sB);
    const size_t ga = col + (size_t)(z0 + 2 * k) * plane;
    r[ga] = (rA - shift) + oA;
    r[ga + plane] = (rB - shift) + oB;
    if (acc) {
      acc[ga] = aA + sA;
      acc[ga + plane] = aB + sB;
    }
    // pair k + 2 goes where pair k - 1 was: every thread finished with that
    // slot before the barrier that ended iteration k - 1
    if (k + 2 <= NK) put((k + 2) % NS);
    __syncthreads();
  }
}

// Accurate residual with solution update: each window chunk of (hi, lo) + e
// becomes the updated double-float pair as it is loaded, held as interleaved
// (hi, lo) pairs (one 8-byte shared load per neighbour and one packed
// subtraction give both parts of a difference); then
// r = (f - α) + bracket over differences D = v_nb - v_0 with the exact
// operator, whose coefficients are evaluated with IEEE round-to-nearest
// operations in the reference's order.  Per-block (Σr, Σr²) to part.  The
// solution pair is (hi, lo) + ec first; with HASD the correction is ec + ed,
// added in FP32 as a separate e += d pass would.  NTH threads per block
// (512, or 256 for four blocks per SM on 32 x 8 x 8 / 32 x 8 x 16 tiles).
template <bool LOCAL, int TY, int TZ, bool HASD, int NTH = NT>
__global__ void __launch_bounds__(NTH, 1024 / NTH) resid_acc2_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                                                        const float* __restrict__ ec, const float* __restrict__ ed,
                                                        const float* __restrict__ f,
                                                        float* __restrict__ ohi, float* __restrict__ olo,
                                                        float* __restrict__ r, LG G, float alpha,
                                                        double* __restrict__ part) {
  constexpr int SY = TY + 2, SZ = TZ + 2, SXY = WX * SY, SN = WX * SY * SZ;
  extern __shared__ __align__(16) float smem[];
  f2* sw = reinterpret_cast<f2*>(smem);                      // SN (hi, lo) pairs
  int* ro = reinterpret_cast<int*>(smem + 2 * SN);
  float* sp = reinterpret_cast<float*>(ro + SY * SZ);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = NTH / 32;
  using RP = RowPrefetch<TY, TZ, NW>;
  RP pf;
#pragma unroll
  for (int i = 0; i < RP::PF; ++i) pf.issue(i, f, warp, lane, x0, y0, z0, G.n);
  row_table<1, TY, TZ, NTH>(ro, y0, z0, G.n);
  if (LOCAL) load_ptab<1, TY, TZ, NTH>(sp, G, x0, y0, z0);
  __syncthreads();
  {
    float4* sw4 = reinterpret_cast<float4*>(smem);
    constexpr int TOT = SY * SZ * CH, K = (TOT + NTH - 1) / NTH, B = HASD ? 3 : 4;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += B) {
      float4 h[B], l[B], e[B], d[B];
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int t = threadIdx.x + (k0 + b) * NTH;
        if (k0 + b < K && t < TOT) {
          const int row = t / CH, c = t - CH * row;
          const int o = ro[row] + wrapi(x0 - XH + 4 * c, G.n[0]);
          h[b] = __ldg(reinterpret_cast<const float4*>(hi + o));
          l[b] = __ldg(reinterpret_cast<const float4*>(lo + o));
          if (ec) e[b] = __ldg(reinterpret_cast<const float4*>(ec + o));
          if (HASD) d[b] = __ldg(reinterpret_cast<const float4*>(ed + o));
        }
      }
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int t = threadIdx.x + (k0 + b) * NTH;
        if (k0 + b < K && t < TOT) {
          if (HASD) {
            e[b].x = e[b].x + d[b].x;
            e[b].y = e[b].y + d[b].y;
            e[b].z = e[b].z + d[b].z;
            e[b].w = e[b].w + d[b].w;
          }
          if (ec) {
            df_add(h[b].x, l[b].x, e[b].x, h[b].x, l[b].x);
            df_add(h[b].y, l[b].y, e[b].y, h[b].y, l[b].y);
            df_add(h[b].z, l[b].z, e[b].z, h[b].z, l[b].z);
            df_add(h[b].w, l[b].w, e[b].w, h[b].w, l[b].w);
          }
          sw4[2 * t] = make_float4(h[b].x, l[b].x, h[b].y, l[b].y);
          sw4[2 * t + 1] = make_float4(h[b].z, l[b].z, h[b].w, l[b].w);
        }
      }
    }
  }
  __syncthreads();
  float s1 = 0.0f, s2 = 0.0f;
  constexpr int SX = WX;
#pragma unroll
  for (int i = 0; i < RP::RPW; ++i) {
    const int row = warp + i * NW;
    if (row >= TY * TZ) break;
    const float fv = pf.v[i % RP::PF];
    pf.issue(i + RP::PF, f, warp, lane, x0, y0, z0, G.n);
    const int ly = 1 + row % TY, lz = 1 + row / TY, lx = XH + lane;
    const int q = lx + SX * ly + SXY * lz;
    const float px = LOCAL ? sp[lx] : G.pg[0], py = LOCAL ? sp[WX + ly] : G.pg[1], pz = LOCAL ? sp[2 * WX + lz] : G.pg[2];
    const float px2 = __fmul_rn(px, px), py2 = __fmul_rn(py, py), pz2 = __fmul_rn(pz, pz);
    const float den = __fadd_rn(__fadd_rn(__fmul_rn(G.cell2[0], px2), __fmul_rn(G.cell2[1], py2)),
                                __fmul_rn(G.cell2[2], pz2));
    const float g = __fdiv_rn(G.beta, den);
    const float gpx = __fadd_rn(G.icell2[0], __fmul_rn(g, px2));
    const float gpy = __fadd_rn(G.icell2[1], __fmul_rn(g, py2));
    const float gpz = __fadd_rn(G.icell2[2], __fmul_rn(g, pz2));
    const f2 c0 = sw[q];
    auto D = [&](int u) {
      float a, b;
      U2(sub2(sw[u], c0), a, b);   // (h_u - h_0, l_u - l_0), each exact for neighbouring values
      return make_float2(a, b);
    };
    const float2 xp = D(q + 1), xm = D(q - 1), yp = D(q + SX), ym = D(q - SX), zp = D(q + SXY), zm = D(q - SXY);
    float br = gpx * dd_sum2(xp, xm) + gpy * dd_sum2(yp, ym) + gpz * dd_sum2(zp, zm) +
               g / 2.0f *
                   (__fmul_rn(px, py) * dd_cross(D(q + 1 + SX), D(q - 1 - SX), D(q - 1 + SX), D(q + 1 - SX)) +
                    __fmul_rn(px, pz) * dd_cross(D(q + 1 + SXY), D(q - 1 - SXY), D(q - 1 + SXY), D(q + 1 - SXY)) +
                    __fmul_rn(py, pz) * dd_cross(D(q + SX + SXY), D(q - SX - SXY), D(q - SX + SXY), D(q + SX - SXY)));
    if (LOCAL)
      br += __fmul_rn(g, px) * dd_diff2(xp, xm) + __fmul_rn(g, py) * dd_diff2(yp, ym) +
            __fmul_rn(g, pz) * dd_diff2(zp, zm);
    const int o = ro[ly + SY * lz] + x0 + lane;
    const float rv = (fv - alpha) + br;
    float h0, l0;
    U2(c0, h0, l0);
    ohi[o] = h0;
    olo[o] = l0;
    r[o] = rv;
    s1 += rv;
    s2 += rv * rv;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double red[2][NW];
  if (lane == 0) { red[0][warp] = s1; red[1][warp] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < NW; ++k) { a += red[0][k]; b += red[1][k]; }
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    part[2 * bid] = a;
    part[2 * bid + 1] = b;
  }
}

template <int HY, int TY, int TZ>
constexpr size_t win_bytes(int arrays) {
  return sizeof(float) * (size_t)arrays * WX * (TY + 2 * HY) * (TZ + 2 * HY) +
         sizeof(int) * (TY + 2 * HY) * (TZ + 2 * HY) + sizeof(float) * 3 * WX;
}

// Tile height/depth for a level: the autotuner's choice when it made one, else
// 16 x 16 when that still gives every SM a block, else 8 x 8.
bool big_tiles(const LG& G) {
  const int* n = G.n;
  if (n[1] % 16 || n[2] % 16) return false;
  if (G.tile16 >= 0) return G.tile16 == 1;
  return (n[0] / TX) * (n[1] / 16) * (n[2] / 16) >= kNumSMs;
}

template <int TY, int TZ>
dim3 grid_of(const int n[3]) { return dim3(n[0] / TX, n[1] / TY, n[2] / TZ); }

// Opt each kernel into its dynamic shared memory once per device.  Kernels
// of the same signature share a function-pointer type, so the cache is keyed
// by the kernel's address as well as the device.
template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const std::pair<const void*, int> key((const void*)kernel, dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(key)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.insert(key);
  return e;
}

template <bool LOCAL, bool CLAMP, int TY, int TZ>
cudaError_t sweep_t(cudaStream_t s, const float* vin, float* vout, const float* rhs, const LG& G, float shift) {
  auto k = rb_sweep2_kernel<LOCAL, CLAMP, TY, TZ>;
  constexpr size_t b = win_bytes<2, TY, TZ>(1);
  cudaError_t e = allow_smem(k, b);
  if (e != cudaSuccess) return e;
  (k<<<grid_of<TY, TZ>(G.n), NT, b, s>>>(vin, vout, rhs, G, shift), ::baorec::count_launch());
  return cudaGetLastError();
}

template <bool LOCAL, bool CLAMP, int TY, int TZ, bool DIFF = false>
cudaError_t resid_t(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float shift,
                    float* acc) {
  auto k = resid_kernel<LOCAL, CLAMP, TY, TZ, DIFF>;
  constexpr size_t b = win_bytes<1, TY, TZ>(1);
  cudaError_t e = allow_smem(k, b);
  if (e != cudaSuccess) return e;
  (k<<<grid_of<TY, TZ>(G.n), NT, b, s>>>(ec, rhs, r, G, shift, acc), ::baorec::count_launch());
  return cudaGetLastError();
}

template <bool LOCAL, int TZ>
cudaError_t pairz_t(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float* acc,
                    float shift) {
  auto k = resid_pairz_kernel<LOCAL, TZ>;
  constexpr size_t b = sizeof(float) * (3 * (16 + 2) * 2 * WX + WX + (16 + 2) + TZ + 2) + sizeof(int) * (16 + 2);
  cudaError_t e = allow_smem(k, b);
  if (e != cudaSuccess) return e;
  (k<<<dim3(G.n[0] / TX, G.n[1] / 16, G.n[2] / TZ), NT, b, s>>>(ec, rhs, r, G, shift, acc), ::baorec::count_launch());
  return cudaGetLastError();
}

template <bool LOCAL, int TY = 16, int TZ = 16>
cudaError_t pairs_t(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float* acc,
                    float shift) {
  auto k = resid_pairs_kernel<LOCAL, TY, TZ>;
  constexpr size_t b = win_bytes<1, TY, TZ>(1);
  cudaError_t e = allow_smem(k, b);
  if (e != cudaSuccess) return e;
  (k<<<grid_of<TY, TZ>(G.n), 32 * TY, b, s>>>(ec, rhs, r, G, shift, acc), ::baorec::count_launch());
  return cudaGetLastError();
}

template <bool LOCAL, int TY, int TZ, int NTH = NT>
cudaError_t acc_t(cudaStream_t s, const float* hi, const float* lo, const float* ec, const float* ed, const float* f,
                  float* ohi, float* olo, float* r, const LG& G, float alpha, double* part) {
  auto k = (ed && ec) ? resid_acc2_kernel<LOCAL, TY, TZ, true, NTH> : resid_acc2_kernel<LOCAL, TY, TZ, false, NTH>;
  constexpr size_t b = win_bytes<1, TY, TZ>(2);
  cudaError_t e = allow_smem(k, b);
  if (e != cudaSuccess) return e;
  (k<<<grid_of<TY, TZ>(G.n), NTH, b, s>>>(hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace

bool tile_ok(const int n[3]) { return n[0] % TX == 0 && n[1] % 8 == 0 && n[2] % 8 == 0; }

// accurate residual: 32 x 8 x 16 tiles of 256 threads (form 2), 32 x 8 x 8
// tiles of 256 threads (form 1), else the level's tiles with 512 threads
static int acc_form(const LG& G) {
  const int* n = G.n;
  if (G.accf == 2 && n[1] % 8 == 0 && n[2] % 16 == 0) return 2;
  if (G.accf == 1 && n[1] % 8 == 0 && n[2] % 8 == 0) return 1;
  return 0;
}

int tile_blocks(const LG& G) {
  const int* n = G.n;
  const int f = acc_form(G);
  if (f == 2) return (n[0] / TX) * (n[1] / 8) * (n[2] / 16);
  if (f == 1) return (n[0] / TX) * (n[1] / 8) * (n[2] / 8);
  return big_tiles(G) ? (n[0] / TX) * (n[1] / 16) * (n[2] / 16) : (n[0] / TX) * (n[1] / 8) * (n[2] / 8);
}

template <bool JACOBI>
cudaError_t ref_stencil_t(cudaStream_t s, const float* v, const float* f, float* out, const LG& G, float w) {
  auto run = [&](auto k, dim3 grid, size_t b) {
    cudaError_t e = allow_smem(k, b);
    if (e != cudaSuccess) return e;
    (k<<<grid, 256, b, s>>>(v, f, out, G, w), ::baorec::count_launch());
    return cudaGetLastError();
  };
  if (G.n[2] % 16 == 0)
    return run(jacobi_tile_kernel<8, 16, 256, JACOBI>, grid_of<8, 16>(G.n), win_bytes<1, 8, 16>(1));
  return run(jacobi_tile_kernel<8, 8, 256, JACOBI>, grid_of<8, 8>(G.n), win_bytes<1, 8, 8>(1));
}

cudaError_t launch_jacobi(cudaStream_t s, const float* v, const float* f, float* out, const LG& G, float omega) {
  return ref_stencil_t<true>(s, v, f, out, G, omega);
}

cudaError_t launch_ref_residual(cudaStream_t s, const float* v, const float* f, float* r, const LG& G, float shift) {
  return ref_stencil_t<false>(s, v, f, r, G, shift);
}

cudaError_t launch_rb_sweep(cudaStream_t s, const float* vin, float* vout, const float* rhs, const LG& G, float shift,
                            bool clamp) {
  const bool big = big_tiles(G);
  if (!G.local)
    return big ? sweep_t<false, false, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<false, false, 8, 8>(s, vin, vout, rhs, G, shift);
  if (clamp)
    return big ? sweep_t<true, true, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<true, true, 8, 8>(s, vin, vout, rhs, G, shift);
  return big ? sweep_t<true, false, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<true, false, 8, 8>(s, vin, vout, rhs, G, shift);
}

cudaError_t launch_resid(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float shift,
                         bool clamp, float* acc) {
  const bool big = big_tiles(G);
  if (!G.local)
    return big ? resid_t<false, false, 16, 16>(s, ec, rhs, r, G, shift, acc)
               : resid_t<false, false, 8, 8>(s, ec, rhs, r, G, shift, acc);
  if (clamp)
    return big ? resid_t<true, true, 16, 16>(s, ec, rhs, r, G, shift, acc)
               : resid_t<true, true, 8, 8>(s, ec, rhs, r, G, shift, acc);
  return big ? resid_t<true, false, 16, 16>(s, ec, rhs, r, G, shift, acc)
             : resid_t<true, false, 8, 8>(s, ec, rhs, r, G, shift, acc);
}

cudaError_t launch_resid_diff(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float* acc,
                              float shift) {
  if (G.pairs == 6 && G.n[1] % 8 == 0 && G.n[2] % 16 == 0)   // the pair kernel on 32 x 8 x 16 tiles
    return G.local ? pairs_t<true, 8>(s, ec, rhs, r, G, acc, shift) : pairs_t<false, 8>(s, ec, rhs, r, G, acc, shift);
  if (G.pairs == 4 || G.pairs == 5) {   // TMA-staged operands, 64 x 16 columns of 32 (form 4) or 16 (form 5) planes
    const int tz = G.pairs == 4 ? 32 : 16;
    if (resid_tma_ok(G, tz) && ((uintptr_t)ec | (uintptr_t)rhs | (uintptr_t)acc) % 16 == 0)
      return launch_resid_diff_tma(s, ec, rhs, r, G, acc, tz, shift);
  }
  const bool big = big_tiles(G);
  if (big && G.pairs == 3 && G.n[2] % 32 == 0)
    return G.local ? pairz_t<true, 32>(s, ec, rhs, r, G, acc, shift) : pairz_t<false, 32>(s, ec, rhs, r, G, acc, shift);
  if (big && (G.pairs == 2 || G.pairs == 3))
    return G.local ? pairz_t<true, 16>(s, ec, rhs, r, G, acc, shift) : pairz_t<false, 16>(s, ec, rhs, r, G, acc, shift);
  if (big && G.pairs) return G.local ? pairs_t<true>(s, ec, rhs, r, G, acc, shift) : pairs_t<false>(s, ec, rhs, r, G, acc, shift);
  if (!G.local)
    return big ? resid_t<false, false, 16, 16, true>(s, ec, rhs, r, G, shift, acc)
               : resid_t<false, false, 8, 8, true>(s, ec, rhs, r, G, shift, acc);
  return big ? resid_t<true, false, 16, 16, true>(s, ec, rhs, r, G, shift, acc)
             : resid_t<true, false, 8, 8, true>(s, ec, rhs, r, G, shift, acc);
}

cudaError_t launch_resid_acc(cudaStream_t s, const float* hi, const float* lo, const float* ec, const float* f,
                             float* ohi, float* olo, float* r, const LG& G, float alpha, double* part, int* nparts,
                             const float* ed) {
  *nparts = tile_blocks(G);
  const int form = acc_form(G);
  if (form == 2)
    return G.local ? acc_t<true, 8, 16, 256>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part)
                   : acc_t<false, 8, 16, 256>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part);
  if (form == 1)
    return G.local ? acc_t<true, 8, 8, 256>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part)
                   : acc_t<false, 8, 8, 256>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part);
  const bool big = big_tiles(G);
  if (G.local)
    return big ? acc_t<true, 16, 16>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part)
               : acc_t<true, 8, 8>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part);
  return big ? acc_t<false, 16, 16>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part)
             : acc_t<false, 8, 8>(s, hi, lo, ec, ed, f, ohi, olo, r, G, alpha, part);
}

}  // namespace baorec
