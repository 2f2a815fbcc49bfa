// Shared-memory tile kernels of the residual-driven multigrid solver.
//
// A block owns a TX x TY x TZ tile of a periodic level mesh.  It stages the
// tile plus a halo (2 cells for the red-black sweep, 1 for residuals) in
// shared memory with row-coalesced loads, computes from shared memory and
// writes the tile.  Every launch is specialised on the line-of-sight mode
// (local: per-cell coefficients from p tables; global: uniform coefficients)
// and on whether the level has cells next to the observer whose
// first-derivative coefficients need clamping.
#include <mutex>

#include "mg_common.cuh"

namespace baorec {
namespace {

constexpr int TX = 32, NT = 512;   // tile width and threads per block (tile height/depth: template)
constexpr int NWARP = NT / 32;

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Periodic window [x0-H, x0+TX+H) x [y0-H, ..) x [z0-H, ..) of g into s (pitch TX+2H).
template <int H, int TY, int TZ>
__device__ __forceinline__ void load_window(float* __restrict__ s, const float* __restrict__ g, int x0, int y0, int z0,
                                            const int n[3]) {
  constexpr int SX = TX + 2 * H, SY = TY + 2 * H, SZ = TZ + 2 * H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gxa = wrapi(x0 - H + lane, n[0]);
  const bool has_b = lane < SX - 32;
  const int gxb = has_b ? wrapi(x0 - H + 32 + lane, n[0]) : 0;
  const size_t plane = (size_t)n[0] * n[1];
  for (int row = warp; row < SY * SZ; row += NWARP) {
    const int ly = row % SY, lz = row / SY;
    const float* gr = g + (size_t)n[0] * wrapi(y0 - H + ly, n[1]) + plane * wrapi(z0 - H + lz, n[2]);
    float* sr = s + row * SX;
    sr[lane] = __ldg(gr + gxa);
    if (has_b) sr[32 + lane] = __ldg(gr + gxb);
  }
}

template <int H, int TY, int TZ>
__device__ __forceinline__ void load_ptab(float* __restrict__ sp, const LG& G, int x0, int y0, int z0) {
  constexpr int SX = TX + 2 * H;
  for (int q = threadIdx.x; q < TX + 2 * H; q += NT) sp[q] = G.P[0][wrapi(x0 - H + q, G.n[0])];
  for (int q = threadIdx.x; q < TY + 2 * H; q += NT) sp[SX + q] = G.P[1][wrapi(y0 - H + q, G.n[1])];
  for (int q = threadIdx.x; q < TZ + 2 * H; q += NT) sp[2 * SX + q] = G.P[2][wrapi(z0 - H + q, G.n[2])];
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
template <bool LOCAL, int SX, int SXY>
__device__ __forceinline__ float nbr(const float* __restrict__ s, int q, const Cf& c) {
  const float xp = s[q + 1], xm = s[q - 1], yp = s[q + SX], ym = s[q - SX], zp = s[q + SXY], zm = s[q - SXY];
  float o = c.gpx * (xp + xm) + c.gpy * (yp + ym) + c.gpz * (zp + zm) +
            c.hxy * ((s[q + 1 + SX] + s[q - 1 - SX]) - (s[q - 1 + SX] + s[q + 1 - SX])) +
            c.hxz * ((s[q + 1 + SXY] + s[q - 1 - SXY]) - (s[q - 1 + SXY] + s[q + 1 - SXY])) +
            c.hyz * ((s[q + SX + SXY] + s[q - SX - SXY]) - (s[q - SX + SXY] + s[q + SX - SXY]));
  if (LOCAL) o += c.dx * (xp - xm) + c.dy * (yp - ym) + c.dz * (zp - zm);
  return o;
}

// One red-black Gauss-Seidel sweep, both colours in one pass, out of place.
// Red cells of the tile and of a one-cell ring around it are updated from the
// old window; then the black cells of the tile from the red-updated window.
template <bool LOCAL, bool CLAMP, int TY, int TZ>
__global__ void __launch_bounds__(NT) rb_sweep_kernel(const float* __restrict__ vin, float* __restrict__ vout,
                                                      const float* __restrict__ rhs, LG G, float shift) {
  constexpr int SX = TX + 4, SY = TY + 4, SZ = TZ + 4, SXY = SX * SY;
  constexpr int FX = TX + 2, FY = TY + 2, FXY = FX * FY;
  extern __shared__ float smem[];
  float* sv = smem;                         // SX*SY*SZ
  float* sf = sv + SX * SY * SZ;            // FX*FY*(TZ+2)
  float* sp = sf + FX * FY * (TZ + 2);      // 3*SX
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  load_window<2, TY, TZ>(sv, vin, x0, y0, z0, G.n);
  load_window<1, TY, TZ>(sf, rhs, x0, y0, z0, G.n);
  if (LOCAL) load_ptab<2, TY, TZ>(sp, G, x0, y0, z0);
  Cf cu;
  if (!LOCAL) cu = coef_fast<false, false>(G.pg[0], G.pg[1], G.pg[2], G);
  __syncthreads();
  // red: 1 <= l < S-1, (lx+ly+lz) even (the tile origin and halo are even, so
  // window parity is mesh parity)
  constexpr int RPR = (SX - 2) / 2, RROWY = SY - 2, NRED = RPR * RROWY * (SZ - 2);
  constexpr int KR = (NRED + NT - 1) / NT;
  float nv[KR];
  int qr[KR];
#pragma unroll
  for (int k = 0; k < KR; ++k) {
    const int c = threadIdx.x + k * NT;
    qr[k] = -1;
    if (c < NRED) {
      const int t = c % RPR, row = c / RPR;
      const int ly = 1 + row % RROWY, lz = 1 + row / RROWY;
      const int lx = 1 + ((ly + lz + 1) & 1) + 2 * t;
      const int q = lx + SX * ly + SXY * lz;
      qr[k] = q;
      const Cf cf = LOCAL ? coef_fast<true, CLAMP>(sp[lx], sp[SX + ly], sp[2 * SX + lz], G) : cu;
      const float f = sf[(lx - 1) + FX * (ly - 1) + FXY * (lz - 1)] - shift;
      nv[k] = __fdividef(f + nbr<LOCAL, SX, SXY>(sv, q, cf), cf.diag);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < KR; ++k)
    if (qr[k] >= 0) sv[qr[k]] = nv[k];
  __syncthreads();
  // black: tile cells (2 <= l < S-2) with odd (lx+ly+lz)
  constexpr int BPR = TX / 2, NBLK = BPR * TY * TZ, KB = NBLK / NT;
  static_assert(NBLK % NT == 0, "black cells must divide evenly");
  float nb[KB];
  int qb[KB];
#pragma unroll
  for (int k = 0; k < KB; ++k) {
    const int c = threadIdx.x + k * NT;
    const int t = c % BPR, row = c / BPR;
    const int ly = 2 + row % TY, lz = 2 + row / TY;
    const int lx = 2 + ((ly + lz + 1) & 1) + 2 * t;
    const int q = lx + SX * ly + SXY * lz;
    qb[k] = q;
    const Cf cf = LOCAL ? coef_fast<true, CLAMP>(sp[lx], sp[SX + ly], sp[2 * SX + lz], G) : cu;
    const float f = sf[(lx - 1) + FX * (ly - 1) + FXY * (lz - 1)] - shift;
    nb[k] = __fdividef(f + nbr<LOCAL, SX, SXY>(sv, q, cf), cf.diag);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < KB; ++k) sv[qb[k]] = nb[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t plane = (size_t)G.n[0] * G.n[1];
  for (int row = warp; row < TY * TZ; row += NWARP) {
    const int ly = row % TY, lz = row / TY;
    vout[(size_t)(x0 + lane) + (size_t)G.n[0] * (y0 + ly) + plane * (z0 + lz)] = sv[2 + lane + SX * (ly + 2) + SXY * (lz + 2)];
  }
}

// r = rhs - shift - Ã e (correction equation, clamped operator).
template <bool LOCAL, bool CLAMP, int TY, int TZ>
__global__ void __launch_bounds__(NT) resid_kernel(const float* __restrict__ e, const float* __restrict__ rhs,
                                                   float* __restrict__ r, LG G, float shift) {
  constexpr int SX = TX + 2, SY = TY + 2, SZ = TZ + 2, SXY = SX * SY;
  extern __shared__ float smem[];
  float* sv = smem;
  float* sp = sv + SX * SY * SZ;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  load_window<1, TY, TZ>(sv, e, x0, y0, z0, G.n);
  if (LOCAL) load_ptab<1, TY, TZ>(sp, G, x0, y0, z0);
  Cf cu;
  if (!LOCAL) cu = coef_fast<false, false>(G.pg[0], G.pg[1], G.pg[2], G);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t plane = (size_t)G.n[0] * G.n[1];
  for (int row = warp; row < TY * TZ; row += NWARP) {
    const int ly = 1 + row % TY, lz = 1 + row / TY, lx = 1 + lane;
    const int q = lx + SX * ly + SXY * lz;
    const Cf cf = LOCAL ? coef_fast<true, CLAMP>(sp[lx], sp[SX + ly], sp[2 * SX + lz], G) : cu;
    const size_t o = (size_t)(x0 + lane) + (size_t)G.n[0] * (y0 + ly - 1) + plane * (z0 + lz - 1);
    r[o] = (rhs[o] - shift) - (cf.diag * sv[q] - nbr<LOCAL, SX, SXY>(sv, q, cf));
  }
}

// Accurate residual with solution update: the window of (hi, lo) + e is
// turned into the updated double-float pair as it is loaded; then
// r = (f - α) + bracket over differences D = v_nb - v_0 with the exact
// operator, whose coefficients are evaluated with IEEE round-to-nearest
// operations in the reference's order.  Per-block (Σr, Σr²) to part.
template <bool LOCAL, int TY, int TZ>
__global__ void __launch_bounds__(NT) resid_acc_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                                                       const float* __restrict__ ec, const float* __restrict__ f,
                                                       float* __restrict__ ohi, float* __restrict__ olo,
                                                       float* __restrict__ r, LG G, float alpha,
                                                       double* __restrict__ part) {
  constexpr int SX = TX + 2, SY = TY + 2, SZ = TZ + 2, SXY = SX * SY, SN = SX * SY * SZ;
  extern __shared__ float smem[];
  float* sh = smem;
  float* sl = sh + SN;
  float* sp = sl + SN;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gxa = wrapi(x0 - 1 + lane, G.n[0]);
    const bool has_b = lane < SX - 32;
    const int gxb = has_b ? wrapi(x0 - 1 + 32 + lane, G.n[0]) : 0;
    const size_t plane = (size_t)G.n[0] * G.n[1];
    for (int row = warp; row < SY * SZ; row += NWARP) {
      const int ly = row % SY, lz = row / SY;
      const size_t base = (size_t)G.n[0] * wrapi(y0 - 1 + ly, G.n[1]) + plane * wrapi(z0 - 1 + lz, G.n[2]);
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        if (half && !has_b) break;
        const size_t gidx = base + (half ? gxb : gxa);
        float h = __ldg(hi + gidx), l = __ldg(lo + gidx);
        if (ec) df_add(h, l, __ldg(ec + gidx), h, l);
        sh[row * SX + half * 32 + lane] = h;
        sl[row * SX + half * 32 + lane] = l;
      }
    }
  }
  if (LOCAL) load_ptab<1, TY, TZ>(sp, G, x0, y0, z0);
  __syncthreads();
  float s1 = 0.0f, s2 = 0.0f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t plane = (size_t)G.n[0] * G.n[1];
  for (int row = warp; row < TY * TZ; row += NWARP) {
    const int ly = 1 + row % TY, lz = 1 + row / TY, lx = 1 + lane;
    const int q = lx + SX * ly + SXY * lz;
    const float px = LOCAL ? sp[lx] : G.pg[0], py = LOCAL ? sp[SX + ly] : G.pg[1], pz = LOCAL ? sp[2 * SX + lz] : G.pg[2];
    const float px2 = __fmul_rn(px, px), py2 = __fmul_rn(py, py), pz2 = __fmul_rn(pz, pz);
    const float den = __fadd_rn(__fadd_rn(__fmul_rn(G.cell2[0], px2), __fmul_rn(G.cell2[1], py2)),
                                __fmul_rn(G.cell2[2], pz2));
    const float g = __fdiv_rn(G.beta, den);
    const float gpx = __fadd_rn(G.icell2[0], __fmul_rn(g, px2));
    const float gpy = __fadd_rn(G.icell2[1], __fmul_rn(g, py2));
    const float gpz = __fadd_rn(G.icell2[2], __fmul_rn(g, pz2));
    const float h0 = sh[q], l0 = sl[q];
    auto D = [&](int u) { return __fadd_rn(__fsub_rn(sh[u], h0), __fsub_rn(sl[u], l0)); };
    const float dxp = D(q + 1), dxm = D(q - 1), dyp = D(q + SX), dym = D(q - SX), dzp = D(q + SXY), dzm = D(q - SXY);
    float br = gpx * (dxp + dxm) + gpy * (dyp + dym) + gpz * (dzp + dzm) +
               g / 2.0f *
                   (__fmul_rn(px, py) * ((D(q + 1 + SX) + D(q - 1 - SX)) - (D(q - 1 + SX) + D(q + 1 - SX))) +
                    __fmul_rn(px, pz) * ((D(q + 1 + SXY) + D(q - 1 - SXY)) - (D(q - 1 + SXY) + D(q + 1 - SXY))) +
                    __fmul_rn(py, pz) * ((D(q + SX + SXY) + D(q - SX - SXY)) - (D(q - SX + SXY) + D(q + SX - SXY))));
    if (LOCAL) br += __fmul_rn(g, px) * (dxp - dxm) + __fmul_rn(g, py) * (dyp - dym) + __fmul_rn(g, pz) * (dzp - dzm);
    const size_t o = (size_t)(x0 + lane) + (size_t)G.n[0] * (y0 + ly - 1) + plane * (z0 + lz - 1);
    const float rv = (f[o] - alpha) + br;
    ohi[o] = h0;
    olo[o] = l0;
    r[o] = rv;
    s1 += rv;          // FP32 over this thread's 16 cells; FP64 across warps and blocks
    s2 += rv * rv;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double red[2][NWARP];
  if (lane == 0) { red[0][warp] = s1; red[1][warp] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < NWARP; ++k) { a += red[0][k]; b += red[1][k]; }
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    part[2 * bid] = a;
    part[2 * bid + 1] = b;
  }
}

template <int TY, int TZ>
constexpr size_t sweep_smem() {
  return sizeof(float) * ((TX + 4) * (TY + 4) * (TZ + 4) + (TX + 2) * (TY + 2) * (TZ + 2) + 3 * (TX + 4));
}
template <int TY, int TZ>
constexpr size_t resid_smem() { return sizeof(float) * ((TX + 2) * (TY + 2) * (TZ + 2) + 3 * (TX + 2)); }
template <int TY, int TZ>
constexpr size_t acc_smem() { return sizeof(float) * (2 * (TX + 2) * (TY + 2) * (TZ + 2) + 3 * (TX + 2)); }

// Tile height/depth for a level: 16 x 16 when that still gives >= 2 blocks per SM, else 8 x 8.
bool big_tiles(const int n[3]) {
  return n[1] % 16 == 0 && n[2] % 16 == 0 && (n[0] / TX) * (n[1] / 16) * (n[2] / 16) >= 2 * kNumSMs;
}

template <int TY, int TZ>
dim3 grid_of(const int n[3]) { return dim3(n[0] / TX, n[1] / TY, n[2] / TZ); }

// Opt each kernel into its dynamic shared memory once per device.
template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

template <bool LOCAL, bool CLAMP, int TY, int TZ>
cudaError_t sweep_t(cudaStream_t s, const float* vin, float* vout, const float* rhs, const LG& G, float shift) {
  auto k = rb_sweep_kernel<LOCAL, CLAMP, TY, TZ>;
  cudaError_t e = allow_smem(k, sweep_smem<TY, TZ>());
  if (e != cudaSuccess) return e;
  k<<<grid_of<TY, TZ>(G.n), NT, sweep_smem<TY, TZ>(), s>>>(vin, vout, rhs, G, shift);
  return cudaGetLastError();
}

template <bool LOCAL, bool CLAMP, int TY, int TZ>
cudaError_t resid_t(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float shift) {
  auto k = resid_kernel<LOCAL, CLAMP, TY, TZ>;
  cudaError_t e = allow_smem(k, resid_smem<TY, TZ>());
  if (e != cudaSuccess) return e;
  k<<<grid_of<TY, TZ>(G.n), NT, resid_smem<TY, TZ>(), s>>>(ec, rhs, r, G, shift);
  return cudaGetLastError();
}

template <bool LOCAL, int TY, int TZ>
cudaError_t acc_t(cudaStream_t s, const float* hi, const float* lo, const float* ec, const float* f, float* ohi,
                  float* olo, float* r, const LG& G, float alpha, double* part) {
  auto k = resid_acc_kernel<LOCAL, TY, TZ>;
  cudaError_t e = allow_smem(k, acc_smem<TY, TZ>());
  if (e != cudaSuccess) return e;
  k<<<grid_of<TY, TZ>(G.n), NT, acc_smem<TY, TZ>(), s>>>(hi, lo, ec, f, ohi, olo, r, G, alpha, part);
  return cudaGetLastError();
}

}  // namespace

bool tile_ok(const int n[3]) { return n[0] % TX == 0 && n[1] % 8 == 0 && n[2] % 8 == 0; }

int tile_blocks(const int n[3]) {
  return big_tiles(n) ? (n[0] / TX) * (n[1] / 16) * (n[2] / 16) : (n[0] / TX) * (n[1] / 8) * (n[2] / 8);
}

cudaError_t launch_rb_sweep(cudaStream_t s, const float* vin, float* vout, const float* rhs, const LG& G, float shift,
                            bool clamp) {
  const bool big = big_tiles(G.n);
  if (!G.local)
    return big ? sweep_t<false, false, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<false, false, 8, 8>(s, vin, vout, rhs, G, shift);
  if (clamp)
    return big ? sweep_t<true, true, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<true, true, 8, 8>(s, vin, vout, rhs, G, shift);
  return big ? sweep_t<true, false, 16, 16>(s, vin, vout, rhs, G, shift) : sweep_t<true, false, 8, 8>(s, vin, vout, rhs, G, shift);
}

cudaError_t launch_resid(cudaStream_t s, const float* ec, const float* rhs, float* r, const LG& G, float shift,
                         bool clamp) {
  const bool big = big_tiles(G.n);
  if (!G.local)
    return big ? resid_t<false, false, 16, 16>(s, ec, rhs, r, G, shift) : resid_t<false, false, 8, 8>(s, ec, rhs, r, G, shift);
  if (clamp)
    return big ? resid_t<true, true, 16, 16>(s, ec, rhs, r, G, shift) : resid_t<true, true, 8, 8>(s, ec, rhs, r, G, shift);
  return big ? resid_t<true, false, 16, 16>(s, ec, rhs, r, G, shift) : resid_t<true, false, 8, 8>(s, ec, rhs, r, G, shift);
}

cudaError_t launch_resid_acc(cudaStream_t s, const float* hi, const float* lo, const float* ec, const float* f,
                             float* ohi, float* olo, float* r, const LG& G, float alpha, double* part, int* nparts) {
  *nparts = tile_blocks(G.n);
  const bool big = big_tiles(G.n);
  if (G.local)
    return big ? acc_t<true, 16, 16>(s, hi, lo, ec, f, ohi, olo, r, G, alpha, part)
               : acc_t<true, 8, 8>(s, hi, lo, ec, f, ohi, olo, r, G, alpha, part);
  return big ? acc_t<false, 16, 16>(s, hi, lo, ec, f, ohi, olo, r, G, alpha, part)
             : acc_t<false, 8, 8>(s, hi, lo, ec, f, ohi, olo, r, G, alpha, part);
}

}  // namespace baorec
