// Streaming (2.5-D) forms of the two finest-level residual kernels of the
// residual-driven solve: each block owns a 32 x 16 column of cells and walks
// a segment of z planes, holding four window planes (z-1, z, z+1 and the one
// in flight) in shared memory.  The next plane's window is copied with
// cp.async while the current plane is computed, so the loads of a block
// never stop for its arithmetic.
//
//   accurate residual: (hi, lo) += e (double-float), r = (f - α) + bracket(D)
//                      over differences D = v_nb - v_0 with the exact
//                      operator's IEEE-ordered coefficients; per-block (Σr, Σr²)
//   running residual:  r_out = r_in + bracket(d_nb - d_0) (FP32, fast
//                      coefficients), acc += d
//
// Window plane: rows y0-1 .. y0+16 (18), x from x0-4 (40 floats = ten 16-byte
// chunks, wrapped per chunk; x0 and n0 are multiples of 4).
#include <mutex>
#include <set>
#include <utility>

#include "mg_common.cuh"

namespace baorec {
namespace {

constexpr int SX = 32, SYT = 16;          // cells of a column: x, y
constexpr int WXS = 40, WYS = SYT + 2;    // window plane: floats per row, rows
constexpr int PLANE = WXS * WYS;          // floats per window plane
constexpr int CHP = WYS * (WXS / 4);      // 16-byte chunks per window plane (180)
constexpr int NTS = 256;                  // threads per block: 8 warps, 2 rows each
constexpr int NWS = NTS / 32;
constexpr int NSLOT = 8;                  // window planes held per block (ring)
constexpr int AHEAD = 6;                  // planes in flight ahead of the one computed (AHEAD + 2 <= NSLOT)
static_assert(AHEAD + 2 <= NSLOT, "ring too small for the prefetch distance");

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
// wait until at most AHEAD-1 of this thread's copy groups are pending
__device__ __forceinline__ void cp_wait_ahead() { asm volatile("cp.async.wait_group %0;\n" ::"n"(AHEAD - 1)); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ int wrapc(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Global offset of window chunk c of plane z (wrapped in every axis).
__device__ __forceinline__ size_t chunk_src(int c, int z, int x0, int y0, const int n[3]) {
  const int r = c / (WXS / 4), cx = c - r * (WXS / 4);
  const int x = wrapc(x0 - 4 + 4 * cx, n[0]);
  const int y = wrapc(y0 - 1 + r, n[1]);
  const int zz = wrapc(z, n[2]);
  return (size_t)x + (size_t)n[0] * ((size_t)y + (size_t)n[1] * (size_t)zz);
}
__device__ __forceinline__ int chunk_dst(int c) {
  const int r = c / (WXS / 4), cx = c - r * (WXS / 4);
  return r * WXS + 4 * cx;
}


// Accurate residual with the double-float update; see the file comment.
template <bool LOCAL>
__global__ void __launch_bounds__(NTS) resid_acc_stream_kernel(const float* __restrict__ hi,
                                                               const float* __restrict__ lo,
                                                               const float* __restrict__ ec,
                                                               const float* __restrict__ f, float* __restrict__ ohi,
                                                               float* __restrict__ olo, float* __restrict__ r, LG G,
                                                               float alpha, int zseg, double* __restrict__ part) {
  extern __shared__ __align__(16) float smem_stream[];
  float (*H)[PLANE] = reinterpret_cast<float (*)[PLANE]>(smem_stream);
  float (*Lo)[PLANE] = reinterpret_cast<float (*)[PLANE]>(smem_stream + NSLOT * PLANE);
  float (*E)[PLANE] = reinterpret_cast<float (*)[PLANE]>(smem_stream + 2 * NSLOT * PLANE);
  const int x0 = blockIdx.x * SX, y0 = blockIdx.y * SYT, z0 = blockIdx.z * zseg;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const bool loader = t < CHP;
  const bool has_e = ec != nullptr;
  const int dst = loader ? chunk_dst(t) : 0;
  auto issue = [&](int z) {   // plane z into slot z mod NSLOT (z >= -1)
    if (loader) {
      const size_t o = chunk_src(t, z, x0, y0, G.n);
      const int s = z & (NSLOT - 1);
      cp16(&H[s][dst], hi + o);
      cp16(&Lo[s][dst], lo + o);
      if (has_e) cp16(&E[s][dst], ec + o);
    }
    cp_commit();
  };
  auto fix = [&](int z) {     // (h, l) += e on this thread's own chunk, once its copies landed
    if (loader && has_e) {
      const int s = z & (NSLOT - 1);
#pragma unroll
      for (int k = 0; k < 4; ++k) df_add(H[s][dst + k], Lo[s][dst + k], E[s][dst + k], H[s][dst + k], Lo[s][dst + k]);
    }
  };
  // prologue: planes z0-1 .. z0+AHEAD-1 in flight, then z0-1 and z0 landed
  for (int k = -1; k < AHEAD; ++k) {
    if (k <= zseg) issue(z0 + k);
    else cp_commit();
  }
  cp_wait_ahead();
  fix(z0 - 1);
  fix(z0);
  float s1 = 0.0f, s2 = 0.0f;
  for (int i = 0; i < zseg; ++i) {
    const int z = z0 + i;
    if (i + AHEAD <= zseg) issue(z + AHEAD);
    else cp_commit();
    cp_wait_ahead();
    fix(z + 1);
    __syncthreads();
    const int sm = (z - 1) & (NSLOT - 1), s0 = z & (NSLOT - 1), sp = (z + 1) & (NSLOT - 1);
    const float pz = LOCAL ? __ldg(G.P[2] + z) : G.pg[2];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int ly = w + NWS * rr;
      const int x = x0 + lane, y = y0 + ly;
      const float px = LOCAL ? __ldg(G.P[0] + x) : G.pg[0];
      const float py = LOCAL ? __ldg(G.P[1] + y) : G.pg[1];
      const float px2 = __fmul_rn(px, px), py2 = __fmul_rn(py, py), pz2 = __fmul_rn(pz, pz);
      const float den = __fadd_rn(__fadd_rn(__fmul_rn(G.cell2[0], px2), __fmul_rn(G.cell2[1], py2)),
                                  __fmul_rn(G.cell2[2], pz2));
      const float g = __fdiv_rn(G.beta, den);
      const float gpx = __fadd_rn(G.icell2[0], __fmul_rn(g, px2));
      const float gpy = __fadd_rn(G.icell2[1], __fmul_rn(g, py2));
      const float gpz = __fadd_rn(G.icell2[2], __fmul_rn(g, pz2));
      const int q = (ly + 1) * WXS + lane + 4;
      const float h0 = H[s0][q], l0 = Lo[s0][q];
      auto D = [&](int s, int u) { return make_float2(__fsub_rn(H[s][u], h0), __fsub_rn(Lo[s][u], l0)); };
      const float2 xp = D(s0, q + 1), xm = D(s0, q - 1), yp = D(s0, q + WXS), ym = D(s0, q - WXS);
      const float2 zp = D(sp, q), zm = D(sm, q);
      float br = gpx * dd_sum2(xp, xm) + gpy * dd_sum2(yp, ym) + gpz * dd_sum2(zp, zm) +
                 g / 2.0f *
                     (__fmul_rn(px, py) * dd_cross(D(s0, q + 1 + WXS), D(s0, q - 1 - WXS), D(s0, q - 1 + WXS),
                                                   D(s0, q + 1 - WXS)) +
                      __fmul_rn(px, pz) * dd_cross(D(sp, q + 1), D(sm, q - 1), D(sp, q - 1), D(sm, q + 1)) +
                      __fmul_rn(py, pz) * dd_cross(D(sp, q + WXS), D(sm, q - WXS), D(sp, q - WXS), D(sm, q + WXS)));
      if (LOCAL)
        br += __fmul_rn(g, px) * dd_diff2(xp, xm) + __fmul_rn(g, py) * dd_diff2(yp, ym) +
              __fmul_rn(g, pz) * dd_diff2(zp, zm);
      const size_t o = (size_t)x + (size_t)G.n[0] * ((size_t)y + (size_t)G.n[1] * (size_t)z);
      const float rv = (__ldg(f + o) - alpha) + br;
      ohi[o] = h0;
      olo[o] = l0;
      r[o] = rv;
      s1 += rv;   // FP32 over this thread's cells; FP64 across warps and blocks
      s2 += rv * rv;
    }
    __syncthreads();
  }
  cp_wait0();
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double red[2][NWS];
  if (lane == 0) { red[0][w] = s1; red[1][w] = s2; }
  __syncthreads();
  if (t == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < NWS; ++k) { a += red[0][k]; b += red[1][k]; }
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    part[2 * bid] = a;
    part[2 * bid + 1] = b;
  }
}


// FP32 running residual of the FFT corrections; see the file comment.
template <bool LOCAL>
__global__ void __launch_bounds__(NTS) resid_diff_stream_kernel(const float* __restrict__ d,
                                                                const float* __restrict__ rin,
                                                                float* __restrict__ rout, LG G, int zseg,
                                                                float* __restrict__ acc, float shift) {
  __shared__ __align__(16) float W[NSLOT][PLANE];
  const int x0 = blockIdx.x * SX, y0 = blockIdx.y * SYT, z0 = blockIdx.z * zseg;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const bool loader = t < CHP;
  const int dst = loader ? chunk_dst(t) : 0;
  auto issue = [&](int z) {
    if (loader) cp16(&W[z & (NSLOT - 1)][dst], d + chunk_src(t, z, x0, y0, G.n));
    cp_commit();
  };
  for (int k = -1; k < AHEAD; ++k) {
    if (k <= zseg) issue(z0 + k);
    else cp_commit();
  }
  for (int i = 0; i < zseg; ++i) {
    const int z = z0 + i;
    if (i + AHEAD <= zseg) issue(z + AHEAD);
    else cp_commit();
    cp_wait_ahead();
    __syncthreads();
    const int sm = (z - 1) & (NSLOT - 1), s0 = z & (NSLOT - 1), sp = (z + 1) & (NSLOT - 1);
    const float pz = LOCAL ? __ldg(G.P[2] + z) : G.pg[2];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int ly = w + NWS * rr;
      const int x = x0 + lane, y = y0 + ly;
      const float px = LOCAL ? __ldg(G.P[0] + x) : G.pg[0];
      const float py = LOCAL ? __ldg(G.P[1] + y) : G.pg[1];
      const float px2 = px * px, py2 = py * py, pz2 = pz * pz;
      const float g = __fdividef(G.beta, G.cell2[0] * px2 + G.cell2[1] * py2 + G.cell2[2] * pz2);
      const float gpx = G.icell2[0] + g * px2, gpy = G.icell2[1] + g * py2, gpz = G.icell2[2] + g * pz2;
      const float hg = 0.5f * g;
      const int q = (ly + 1) * WXS + lane + 4;
      const float c0 = W[s0][q];
      auto D = [&](int s, int u) { return W[s][u] - c0; };
      const float xp = W[s0][q + 1], xm = W[s0][q - 1], yp = W[s0][q + WXS], ym = W[s0][q - WXS];
      const float zp = W[sp][q], zm = W[sm][q];
      float br = gpx * ((xp - c0) + (xm - c0)) + gpy * ((yp - c0) + (ym - c0)) + gpz * ((zp - c0) + (zm - c0)) +
                 hg * (px * py) * ((D(s0, q + 1 + WXS) + D(s0, q - 1 - WXS)) - (D(s0, q - 1 + WXS) + D(s0, q + 1 - WXS))) +
                 hg * (px * pz) * ((D(sp, q + 1) + D(sm, q - 1)) - (D(sp, q - 1) + D(sm, q + 1))) +
                 hg * (py * pz) * ((D(sp, q + WXS) + D(sm, q - WXS)) - (D(sp, q - WXS) + D(sm, q + WXS)));
      if (LOCAL) br += (g * px) * (xp - xm) + (g * py) * (yp - ym) + (g * pz) * (zp - zm);
      const size_t o = (size_t)x + (size_t)G.n[0] * ((size_t)y + (size_t)G.n[1] * (size_t)z);
      rout[o] = (__ldg(rin + o) - shift) + br;
      if (acc) acc[o] += c0;
    }
    __syncthreads();
  }
  cp_wait0();
}

// Dynamic shared memory above 48 KB, opted in once per kernel and device.
cudaError_t smem_optin(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({kernel, dev})) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.insert({kernel, dev});
  return e;
}

// z planes per block: halve the segment while the grid is below three
// blocks per SM (and the segment stays even and at least 8 planes).
int zseg_of(const int n[3]) {
  const int cols = (n[0] / SX) * (n[1] / SYT);
  int z = n[2];
  while (z % 2 == 0 && z > 8 && (long long)cols * (n[2] / z) < 3LL * kNumSMs) z /= 2;
  return z;
}

}  // namespace

bool stream_ok(const int n[3]) { return n[0] % SX == 0 && n[1] % SYT == 0 && n[2] >= 2; }

int stream_blocks(const int n[3]) { return (n[0] / SX) * (n[1] / SYT) * (n[2] / zseg_of(n)); }

cudaError_t launch_resid_acc_stream(cudaStream_t s, const float* hi, const float* lo, const float* ec, const float* f,
                                    float* ohi, float* olo, float* r, const LG& G, float alpha, double* part,
                                    int* nparts) {
  const int zs = zseg_of(G.n);
  const dim3 grid(G.n[0] / SX, G.n[1] / SYT, G.n[2] / zs);
  *nparts = (int)(grid.x * grid.y * grid.z);
  const size_t bytes = 3u * NSLOT * PLANE * sizeof(float);
  auto k = G.local ? resid_acc_stream_kernel<true> : resid_acc_stream_kernel<false>;
  cudaError_t e = smem_optin((const void*)k, bytes);
  if (e != cudaSuccess) return e;
  (k<<<grid, NTS, bytes, s>>>(hi, lo, ec, f, ohi, olo, r, G, alpha, zs, part), ::baorec::count_launch());
  return cudaGetLastError();
}

cudaError_t launch_resid_diff_stream(cudaStream_t s, const float* d, const float* rin, float* rout, const LG& G,
                                     float* acc, float shift) {
  const int zs = zseg_of(G.n);
  const dim3 grid(G.n[0] / SX, G.n[1] / SYT, G.n[2] / zs);
  if (G.local) (resid_diff_stream_kernel<true><<<grid, NTS, 0, s>>>(d, rin, rout, G, zs, acc, shift), ::baorec::count_launch());
  else (resid_diff_stream_kernel<false><<<grid, NTS, 0, s>>>(d, rin, rout, G, zs, acc, shift), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace baorec
