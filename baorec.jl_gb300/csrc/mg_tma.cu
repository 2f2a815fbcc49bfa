// FP32 running residual of the FFT corrections with its operands staged in
// shared memory by the tensor-memory-access (TMA) engine:
//   r_out = (r_in - shift) + bracket(d_nb - d_0),   acc += d  (optional),
// with the per-cell arithmetic of resid_pairs_kernel (mg_tiles.cu) in the
// same order, so that every form of the running residual gives the same bits.
//
// Work: a block owns a 64 x 16 column of cells (x, y) and walks a segment of
// tz planes in z.  Warp w computes row y0 + w, lane l the two x-adjacent
// cells x0 + 2l, x0 + 2l + 1 in packed FP32x2 arithmetic.  The values of d
// travel in registers from plane to plane: of planes z-1, z, z+1 a thread
// keeps the four values x-1 .. x+2 of its row and of the rows y-1, y+1 (of
// plane z-1 only the pair x, x+1 of the side rows), so the 19-point stencil
// of two cells costs the nine shared loads of one new plane.
//
// Staging: a ring of NS plane slots in shared memory.  The slot of plane p
// holds
//   d     rows y0-1 .. y0+16 of the columns x0 .. x0+63 (18 x 256 B), and the
//         4-float x halos left and right of the same rows;
//   r_in  the tile's 16 rows of plane p, and acc the same (when accumulated).
// The mesh is periodic and TMA does not wrap, so the edge rows y0-1, y0+16
// and the x halos are boxes of their own, taken at wrapped coordinates:
// every box lies inside the mesh, every x coordinate is a multiple of four
// floats (16 bytes), every destination is 128-byte aligned.
//
// Thread 0 issues the boxes of a plane into the slot that the warps released
// the step before (NS - 2 planes ahead of the one computed); full (TMA
// transaction bytes) and empty (one arrival per warp) mbarriers hand slots
// between it and the warps.  Every wait is bounded in time: on expiry the
// warp sets kErrTimeout in the error word and the block stops; thread 0 waits
// for the copies it issued before the block exits.
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <utility>

#include "mg_common.cuh"
#include "tma_util.cuh"

namespace baorec {
namespace {

using namespace ::baorec::tma;

constexpr int kTX = 64, kTY = 16;                   // tile: cells along x (two per lane), rows (one per warp)
constexpr int kThreadsR = 32 * kTY;
constexpr int kRowB = kTX * 4;                      // bytes of one tile row
// slot layout (bytes)
constexpr int kOffD = 0;                            // d rows y0-1 .. y0+16
constexpr int kOffL = kOffD + (kTY + 2) * kRowB;    // left halo of rows y0 .. y0+15 (16 B each)
constexpr int kOffR = kOffL + kTY * 16;             // right halo of rows y0 .. y0+15
constexpr int kOffLT = kOffR + kTY * 16;            // left halo of row y0-1 (one 128-B cell each)
constexpr int kOffLB = kOffLT + 128;                // left halo of row y0+16
constexpr int kOffRT = kOffLB + 128;                // right halo of row y0-1
constexpr int kOffRB = kOffRT + 128;                // right halo of row y0+16
constexpr int kOffIn = kOffRB + 128;                // r_in rows y0 .. y0+15
constexpr int kOffAcc = kOffIn + kTY * kRowB;       // acc rows y0 .. y0+15
constexpr int kSlotB = kOffAcc + kTY * kRowB;
constexpr uint32_t kTxD = (kTY + 2) * kRowB + 2 * (kTY + 2) * 16;   // bytes of d per plane
constexpr uint32_t kTxPlane = kTY * kRowB;                          // bytes of r_in (or acc) per plane
static_assert(kOffL % 128 == 0 && kOffR % 128 == 0 && kOffLT % 128 == 0 && kOffIn % 128 == 0 &&
                  kOffAcc % 128 == 0 && kSlotB % 128 == 0,
              "128-byte aligned TMA destinations");

// 3-D tensor maps {x, y, z} of FP32 meshes: d with boxes {64, 16, 1} (rows),
// {64, 1, 1} (edge row), {4, 16, 1} (x halo), {4, 1, 1} (x halo of an edge
// row); r_in and acc with {64, 16, 1}.
struct ResidMaps {
  CUtensorMap d16, d1, h16, h1, rin, acc;
};

struct Row4 {
  float m, a, b, p;   // x-1, x, x+1, x+2
};

template <bool LOCAL, int NS>
__global__ void __launch_bounds__(kThreadsR, 1)
    resid_tma_kernel(const __grid_constant__ ResidMaps maps, float* __restrict__ rout, float* __restrict__ acc,
                     const LG G, const float shift, const int tz, unsigned* __restrict__ err,
                     const unsigned long long wait_ns) {
  static_assert(NS >= 3 && (NS & (NS - 1)) == 0, "a power of two, and a plane is issued while the two before it are read");
  extern __shared__ __align__(128) unsigned char smem_rt[];
  __shared__ __align__(8) uint64_t full[NS];
  __shared__ __align__(8) uint64_t empty[NS];
  __shared__ int abort_flag;
  const uint32_t raw = smem_u32(smem_rt);
  const uint32_t sbase = (raw + 127u) & ~127u;
  const float* S0 = reinterpret_cast<const float*>(smem_rt + (sbase - raw));
  const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z0 = blockIdx.z * tz;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool has_acc = acc != nullptr;
  const int nplanes = tz + 2;   // planes z0-1 .. z0+tz; plane index ip = z - z0 + 1
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < NS; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), kTY);
    }
    mbar_init_fence();
  }
  __syncthreads();

  // ---- thread 0: the boxes of plane ip into slot ip % NS ----
  const int yt = y0 == 0 ? n1 - 1 : y0 - 1, yb = y0 + kTY == n1 ? 0 : y0 + kTY;
  const int xl = x0 == 0 ? n0 - 4 : x0 - 4, xr = x0 + kTX == n0 ? 0 : x0 + kTX;
  int issued = 0;
  auto issue = [&](int ip) {
    const int s = ip & (NS - 1);
    const uint32_t d = sbase + (uint32_t)(s * kSlotB), bar = smem_u32(&full[s]);
    int z = z0 - 1 + ip;
    z = z < 0 ? z + n2 : (z >= n2 ? z - n2 : z);
    const bool own = ip >= 1 && ip <= tz;   // a plane of the tile's own cells: r_in and acc as well
    mbar_expect_tx(bar, kTxD + (own ? kTxPlane * (has_acc ? 2u : 1u) : 0u));
    tma_load_3d(d + kOffD + kRowB, &maps.d16, bar, x0, y0, z);
    tma_load_3d(d + kOffD, &maps.d1, bar, x0, yt, z);
    tma_load_3d(d + kOffD + (kTY + 1) * kRowB, &maps.d1, bar, x0, yb, z);
    tma_load_3d(d + kOffL, &maps.h16, bar, xl, y0, z);
    tma_load_3d(d + kOffR, &maps.h16, bar, xr, y0, z);
    tma_load_3d(d + kOffLT, &maps.h1, bar, xl, yt, z);
    tma_load_3d(d + kOffLB, &maps.h1, bar, xl, yb, z);
    tma_load_3d(d + kOffRT, &maps.h1, bar, xr, yt, z);
    tma_load_3d(d + kOffRB, &maps.h1, bar, xr, yb, z);
    if (own) {
      tma_load_3d(d + kOffIn, &maps.rin, bar, x0, y0, z);
      if (has_acc) tma_load_3d(d + kOffAcc, &maps.acc, bar, x0, y0, z);
    }
    issued = ip + 1;
  };
  // once every warp has released plane ip, its slot takes plane ip + NS
  auto refill = [&](int ip) -> bool {
    if (ip + NS >= nplanes) return true;
    if (!mbar_wait(smem_u32(&empty[ip & (NS - 1)]), (uint32_t)((ip / NS) & 1), &abort_flag, wait_ns)) return false;
    issue(ip + NS);
    return true;
  };

  // ---- every warp: shared-memory offsets (floats) of the thread's loads ----
  // slot rows R = warp (y-1), warp + 1 (y), warp + 2 (y+1)
  auto off_c = [&](int R) { return R * kTX + 2 * lane; };
  auto off_l = [&](int R) {
    if (lane > 0) return R * kTX + 2 * lane - 1;
    return (R == 0 ? kOffLT / 4 : R == kTY + 1 ? kOffLB / 4 : kOffL / 4 + 4 * (R - 1)) + 3;
  };
  auto off_r = [&](int R) {
    if (lane < 31) return R * kTX + 2 * lane + 2;
    return R == 0 ? kOffRT / 4 : R == kTY + 1 ? kOffRB / 4 : kOffR / 4 + 4 * (R - 1);
  };
  const int cm = off_c(warp), c0 = off_c(warp + 1), cp = off_c(warp + 2);
  const int lm = off_l(warp), l0 = off_l(warp + 1), lp = off_l(warp + 2);
  const int rm = off_r(warp), r0 = off_r(warp + 1), rp = off_r(warp + 2);
  const int o_in = kOffIn / 4 + warp * kTX + 2 * lane, o_acc = kOffAcc / 4 + warp * kTX + 2 * lane;
  auto slot = [&](int ip) { return S0 + (ip & (NS - 1)) * (kSlotB / 4); };
  auto row = [](const float* s, int c, int l, int r) {
    const float2 ab = *reinterpret_cast<const float2*>(s + c);
    Row4 v;
    v.m = s[l];
    v.a = ab.x;
    v.b = ab.y;
    v.p = s[r];
    return v;
  };
  auto pair = [](const float* s, int c) { return *reinterpret_cast<const float2*>(s + c); };
  auto wait_full = [&](int ip) -> bool {
    const bool w = mbar_wait(smem_u32(&full[ip & (NS - 1)]), (uint32_t)((ip / NS) & 1), &abort_flag, wait_ns);
    return __all_sync(0xffffffffu, w) != 0;
  };
  auto release = [&](int ip) {
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_u32(&empty[ip & (NS - 1)]));
  };
  auto producer_step = [&](int ip) -> bool {   // warp 0: thread 0 refills, the warp agrees on the outcome
    if (warp != 0) return true;
    const bool r = threadIdx.x == 0 ? refill(ip) : true;
    return __all_sync(0xffffffffu, r) != 0;
  };

  // ---- per-cell coefficients that do not change along z ----
  const int x = x0 + 2 * lane, y = y0 + warp;
  float pxa, pxb, py;
  if (LOCAL) {
    pxa = __ldg(G.P[0] + x);
    pxb = __ldg(G.P[0] + x + 1);
    py = __ldg(G.P[1] + y);
  } else {
    pxa = pxb = G.pg[0];
    py = G.pg[1];
  }
  const float pxa2 = pxa * pxa, pxb2 = pxb * pxb, py2 = py * py;
  const f2 Px = P2(pxa, pxb), Px2 = P2(pxa2, pxb2);
  const f2 Dxy = P2(coef_dxy(G, pxa2, py2), coef_dxy(G, pxb2, py2));
  const f2 PxPy = P2(pxa * py, pxb * py);
  const size_t plane = (size_t)n0 * n1;
  const size_t first = (size_t)z0 * plane + (size_t)y * n0 + x;
  float* out_r = rout + first;
  float* out_a = has_acc ? acc + first : nullptr;
  const float* pzs = LOCAL ? G.P[2] + z0 : nullptr;

  // Output plane z = z0 + j from planes z-1 (M), z (C) and z+1 (P, loaded
  // here from slot j + 2); r_in and acc of plane z come from slot j + 1,
  // released at the end.  The three plane roles rotate over consecutive
  // steps, so the loop below is unrolled by three and no value is copied.
  struct Plane {
    Row4 y, u, d;   // rows y, y+1, y-1
  };
  auto step = [&](int j, const Plane& M, const Plane& Cc, Plane& P) -> bool {
    if (j >= 1 && !producer_step(j)) return false;
    if (!wait_full(j + 2)) return false;
    const float* sn = slot(j + 2);
    const float* sc = slot(j + 1);
    P.y = row(sn, c0, l0, r0);
    P.u = row(sn, cp, lp, rp);
    P.d = row(sn, cm, lm, rm);
    const float2 rin = pair(sc, o_in);
    const float2 av = has_acc ? pair(sc, o_acc) : make_float2(0.0f, 0.0f);
    const float pz = LOCAL ? __ldg(pzs + j) : G.pg[2];
    const float pz2 = pz * pz;
    const f2 Pz = B2(pz);
    float dA, dB;
    U2(fma2(B2(G.cell2[2]), B2(pz2), Dxy), dA, dB);
    const f2 g = P2(__fdividef(G.beta, dA), __fdividef(G.beta, dB));
    const f2 gpz = fma2(g, B2(pz2), B2(G.icell2[2]));
    const f2 hg = mul2(B2(0.5f), g);
    const Row4 &mr = M.y, &cr = Cc.y, &cu = Cc.u, &cd = Cc.d, &pr = P.y, &pu = P.u, &pd = P.d;
    const f2 s0 = P2(cr.a, cr.b);
    const f2 zp = P2(pr.a, pr.b), zm = P2(mr.a, mr.b);
    f2 o = mul2(gpz, add2(sub2(zp, s0), sub2(zm, s0)));
    if (LOCAL) o = fma2(mul2(g, Pz), sub2(zp, zm), o);
    {   // x neighbours and the x-z diagonals
      const f2 xp = P2(cr.b, cr.p), xm = P2(cr.m, cr.a);
      const f2 upp = P2(pr.b, pr.p), dmm = P2(mr.m, mr.a), upm = P2(pr.m, pr.a), dmp = P2(mr.b, mr.p);
      o = fma2(fma2(g, Px2, B2(G.icell2[0])), add2(sub2(xp, s0), sub2(xm, s0)), o);
      o = fma2(mul2(hg, mul2(Px, Pz)), sub2(add2(sub2(upp, s0), sub2(dmm, s0)), add2(sub2(upm, s0), sub2(dmp, s0))),
               o);
      if (LOCAL) o = fma2(mul2(g, Px), sub2(xp, xm), o);
    }
    {   // y neighbours and the y-z diagonals
      const f2 yp = P2(cu.a, cu.b), ym = P2(cd.a, cd.b);
      const f2 upp = P2(pu.a, pu.b), dmm = P2(M.d.a, M.d.b), upm = P2(pd.a, pd.b), dmp = P2(M.u.a, M.u.b);
      o = fma2(fma2(g, B2(py2), B2(G.icell2[1])), add2(sub2(yp, s0), sub2(ym, s0)), o);
      o = fma2(mul2(hg, mul2(B2(py), Pz)), sub2(add2(sub2(upp, s0), sub2(dmm, s0)), add2(sub2(upm, s0), sub2(dmp, s0))),
               o);
      if (LOCAL) o = fma2(mul2(g, B2(py)), sub2(yp, ym), o);
    }
    {   // x-y diagonals (in-plane)
      const f2 pp = P2(cu.b, cu.p), mm = P2(cd.m, cd.a), mp = P2(cu.m, cu.a), pm = P2(cd.b, cd.p);
      o = fma2(mul2(hg, PxPy), sub2(add2(sub2(pp, s0), sub2(mm, s0)), add2(sub2(mp, s0), sub2(pm, s0))), o);
    }
    release(j + 1);
    float oA, oB;
    U2(o, oA, oB);
    *reinterpret_cast<float2*>(out_r) = make_float2((rin.x - shift) + oA, (rin.y - shift) + oB);
    out_r += plane;
    if (has_acc) {
      *reinterpret_cast<float2*>(out_a) = make_float2(av.x + cr.a, av.y + cr.b);
      out_a += plane;
    }
    return true;
  };

  if (threadIdx.x == 0)
    for (int ip = 0; ip < NS && ip < nplanes; ++ip) issue(ip);
  Plane A{}, B{}, C{};   // planes z0-1 and z0 first
  bool ok = wait_full(0);
  if (ok) {
    const float* s = slot(0);
    A.y = row(s, c0, l0, r0);
    A.u = row(s, cp, lp, rp);
    A.d = row(s, cm, lm, rm);
    release(0);
    ok = producer_step(0);
  }
  if (ok) ok = wait_full(1);
  if (ok) {
    const float* s = slot(1);
    B.y = row(s, c0, l0, r0);
    B.u = row(s, cp, lp, rp);
    B.d = row(s, cm, lm, rm);
  }
#pragma unroll 1
  for (int j = 0; ok && j < tz; j += 3) {
    if (!(ok = step(j, A, B, C)) || j + 1 >= tz) break;
    if (!(ok = step(j + 1, B, C, A)) || j + 2 >= tz) break;
    ok = step(j + 2, C, A, B);
  }
  if (!ok && lane == 0) {
    abort_flag = 1;
    atomicOr(err, kErrTimeout);
  }
  // the copies this block issued land before its shared memory is released
  if (threadIdx.x == 0)
    for (int ip = issued > NS ? issued - NS : 0; ip < issued; ++ip)
      mbar_drain(smem_u32(&full[ip & (NS - 1)]), (uint32_t)((ip / NS) & 1));
}

constexpr int kRing = 8;   // plane slots per block: planes are issued six steps ahead

cudaError_t encode_mesh_map(CUtensorMap* m, const float* p, const int n[3], uint32_t bx, uint32_t by) {
  // the maps depend only on (address, extents, box): cached, so that a
  // launch costs no driver call after the first with the same buffers
  using Key = std::tuple<const float*, int, int, int, uint32_t, uint32_t>;
  static std::mutex mu;
  static std::map<Key, CUtensorMap> cache;
  const Key k{p, n[0], n[1], n[2], bx, by};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(k);
    if (it != cache.end()) {
      *m = it->second;
      return cudaSuccess;
    }
  }
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[3] = {(cuuint64_t)n[0], (cuuint64_t)n[1], (cuuint64_t)n[2]};
  const cuuint64_t strides[2] = {(cuuint64_t)n[0] * 4, (cuuint64_t)n[0] * n[1] * 4};
  const cuuint32_t box[3] = {bx, by, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(p), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() >= 256) cache.clear();
  cache.emplace(k, *m);
  return cudaSuccess;
}

template <bool LOCAL>
cudaError_t tma_t(cudaStream_t s, const ResidMaps& maps, float* rout, float* acc, const LG& G, int tz, float shift) {
  auto k = resid_tma_kernel<LOCAL, kRing>;
  constexpr size_t bytes = (size_t)kRing * kSlotB + 128;
  static std::mutex mu;
  static std::set<int> opted;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!opted.count(dev)) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
      if (e != cudaSuccess) return e;
      opted.insert(dev);
    }
  }
  const dim3 grid(G.n[0] / kTX, G.n[1] / kTY, G.n[2] / tz);
  (k<<<grid, kThreadsR, bytes, s>>>(maps, rout, acc, G, shift, tz, G.err, kWaitNs), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace

bool resid_tma_ok(const LG& G, int tz) {
  const int* n = G.n;
  return G.err && n[0] % kTX == 0 && n[1] % kTY == 0 && tz > 0 && n[2] % tz == 0;
}

cudaError_t launch_resid_diff_tma(cudaStream_t s, const float* d, const float* rin, float* rout, const LG& G,
                                  float* acc, int tz, float shift) {
  if (!resid_tma_ok(G, tz)) return cudaErrorInvalidValue;
  for (const float* p : {d, rin, (const float*)acc})
    if ((uintptr_t)p % 16) return cudaErrorInvalidValue;
  ResidMaps m;
  cudaError_t e;
  if ((e = encode_mesh_map(&m.d16, d, G.n, kTX, kTY)) != cudaSuccess) return e;
  if ((e = encode_mesh_map(&m.d1, d, G.n, kTX, 1)) != cudaSuccess) return e;
  if ((e = encode_mesh_map(&m.h16, d, G.n, 4, kTY)) != cudaSuccess) return e;
  if ((e = encode_mesh_map(&m.h1, d, G.n, 4, 1)) != cudaSuccess) return e;
  if ((e = encode_mesh_map(&m.rin, rin, G.n, kTX, kTY)) != cudaSuccess) return e;
  if (acc) {
    if ((e = encode_mesh_map(&m.acc, acc, G.n, kTX, kTY)) != cudaSuccess) return e;
  } else {
    m.acc = m.rin;   // not read
  }
  return G.local ? tma_t<true>(s, m, rout, acc, G, tz, shift) : tma_t<false>(s, m, rout, acc, G, tz, shift);
}

}  // namespace baorec
