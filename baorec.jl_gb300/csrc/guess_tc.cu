// 3x3x3 convolution of the learned initial guess on the fifth-generation
// tensor cores: an implicit GEMM with M = 128 voxels of one output row,
// N = output channels, K = 27 taps x input channels, BF16 operands in shared
// memory, FP32 accumulators in tensor memory (TMEM).
//
// Shared-memory layout (no swizzle, K-major canonical form: a "core matrix"
// is 8 rows of 16 bytes, rows 16 bytes apart):
//   weights  [tap (dx, dy)][chunk of 8 input channels][dz][output channel][8]
//            BF16, one bulk TMA copy of a pre-arranged image per CTA.
//            B descriptor of (dx, dy, k step, first dz): LBO = 3*COUT*16
//            (chunk 2ks -> 2ks+1), SBO = 128 (8 output channels)
//   slabs    ring of S input "slabs"; a slab is one z plane of the input
//            restricted to the rows y-1..y+1 and voxels x0-1..x0+128 of the
//            tile: [chunk c][dy][x slot][8 channels], zero outside the grid
//            (the convolution's zero padding).
//            A descriptor of tap (dx, dy) and k step ks: start = slab +
//            2ks*kPlane + dy*2080 + dx*16, LBO = kPlane (chunk 2ks -> 2ks+1),
//            SBO = 128 (8 voxels).  Shifting the start by dx*16 bytes selects
//            the voxels x+dx-1: the halo is read in place, never copied.
//
// Slabs are filled by one of two loaders (identical slabs, checked bit for
// bit by the tests):
//   kLoadTma      (default) one thread issues a 4-D TMA box {8 channels,
//                 130 x, 3 y, 1 z} per chunk, zero-filled outside the grid;
//   kLoadCpAsync  two producer warps copy the 16-byte pieces with cp.async
//                 (consecutive threads read consecutive bytes of the
//                 channels-last activations), zero-filling the padding.
//
// Each CTA is persistent and walks "columns" (x segment, YR rows y0 ..
// y0+YR-1, zc consecutive z), marching in z.  Output row z needs input
// planes z-1, z, z+1 (taps dz = 0, 1, 2), so plane p feeds rows p+1, p, p-1;
// the MMA multiplies each slab ONCE by the three dz weight blocks side by
// side (N = 3*COUT, B image [dx,dy][k chunk][dz][n]) and the three N blocks
// land in the accumulators of those three rows.  Each output row y0+yy has
// a TMEM ring of kRing accumulators in descending-row order, so the three
// blocks are adjacent columns; the ring is followed by kShadow extra slots,
// where blocks past its end land, and the epilogue adds a shadow slot to
// ring slot 0 or 1 (one contiguous MMA per tap instead of two where the
// ring wraps: split MMAs cost several times a plain one on GB300).  Every
// MMA accumulates: the ring starts at zero and the epilogue zeroes what it
// reads.  A slab of YR+2 rows serves YR output rows (fewer TMA rows per
// output), and is freed right after its MMAs.
//
// Measured on GB300 (M=128, K=16, one issuing thread): an MMA costs
// max(~45, N/2) cycles whatever the smem layout or alignment, so N = 3*COUT
// (48-192) sits near the floor where N = COUT did not.
//
// Roles (352 threads): warps 0-1 load slabs (thread 0 also issues the bulk
// copy of the weight image); warp 2 owns the TMEM allocation and its lane 0
// issues the MMAs; warps 3-10 are two epilogue teams of four warps taking
// alternate output rows: tcgen05.ld of the row's accumulator (one voxel per
// thread), bias, addend, ReLU, BF16 channels-last stores, zeroing the
// accumulator behind them.  mbarriers hand slabs, weights and accumulators
// between the roles; every wait is bounded in time and on expiry sets
// kErrTimeout and stops its role, and the block drains its copies and MMAs
// before freeing TMEM (drain waits are not cut short by another role giving
// up; they are bounded by kWaitNs).  The pipeline waits' limit is a launch
// argument; a test hook holds the slab loader back so that they expire.
#include <algorithm>

#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "guess.cuh"
#include "tma_util.cuh"

namespace baorec {
namespace guess {
namespace {

using namespace ::baorec::tma;

typedef __nv_bfloat16 bf16;

constexpr int kTM = 128;                 // voxels per tile (MMA M)
constexpr int kSlots = kTM + 2;          // x slots of a slab row (halo of 1 each side)
constexpr int kRowBytes = kSlots * 16;   // 2080: one dy row of one chunk
constexpr int kProducers = 64;           // warps 0-1 load slabs
constexpr int kMmaWarp = 2;              // MMA issuer and TMEM owner
constexpr int kEpiWarp0 = 3;             // warps 3-10: two epilogue teams of 4 warps
constexpr int kThreads = 32 * (kEpiWarp0 + 8);
enum Loader { kLoadCpAsync = 0, kLoadTma = 1 };
constexpr int kSmemMax = 232448;         // opt-in dynamic shared memory per block
constexpr int kSmemBudget = kSmemMax - 1024 - 512;
constexpr int kRing = 6;                 // TMEM accumulators (output rows in flight) per output-row ring
constexpr int kShadow = 2;               // shadow slots past a ring's end: the MMA never wraps
constexpr int kCols = kRing + kShadow;   // slots of TMEM columns per ring

template <int CIN, int COUT>
struct Tc {
  // 8 input channels: one K=16 MMA covers the tap pair (dx, dx+1) of a
  // (dy, dz), the A operand's second K chunk being the next voxel (LBO 16 B);
  // pairs (0, 1) and (2, 3), tap 3 with zero weights
  static constexpr bool PAIRED = CIN == 8;
  static constexpr int KS = PAIRED ? 1 : CIN / 16;   // K steps of 16 channels per tap
  static constexpr int NMMA = PAIRED ? 6 : 9 * KS;   // MMAs per slab and dz group
  static constexpr int CH = CIN / 8;                 // 16-byte chunks per voxel
  static constexpr int WB = NMMA * 2 * 3 * COUT * 16; // weight image bytes
  // a unit covers YR output rows (y0 .. y0+YR-1) from a slab of YR+2 input
  // rows; one chunk plane = the TMA box plus a zeroed 32-byte pad (the
  // 8-channel MMAs read 16 bytes past the box), rounded to 128 bytes
  static constexpr int plane_of(int yr) { return ((yr + 2) * kRowBytes + 32 + 127) / 128 * 128; }
  static constexpr int s_of(int yr) {
    return (kSmemBudget - WB) / (CH * plane_of(yr)) > 6 ? 6 : (kSmemBudget - WB) / (CH * plane_of(yr));
  }
  // the most rows whose accumulator rings fit the 512 TMEM columns and whose
  // slabs still leave a ring of two in shared memory
  static constexpr int YR = (4 * kCols * COUT <= 512 && s_of(4) >= 2) ? 4
                            : (2 * kCols * COUT <= 512 && s_of(2) >= 2) ? 2 : 1;
  static constexpr int BOX = (YR + 2) * kRowBytes;   // bytes one TMA box delivers
  static constexpr int PLANE = plane_of(YR);
  static constexpr int SLAB = CH * PLANE;
  static constexpr int S = s_of(YR);                 // slab ring depth
  static constexpr int SMEM = WB + S * SLAB + 1024;  // + alignment slack
  static constexpr int TCOLS = YR * kCols * COUT;    // TMEM columns: one accumulator ring per output row
  // S >= 2: a slab is freed as soon as its own MMAs complete, so the loader
  // refills one slot while the MMAs read the other
  static_assert(S >= 2, "slab ring too shallow for this shape");
  static_assert(WB % 128 == 0 && SLAB % 128 == 0, "128-byte aligned regions");
  static_assert(TCOLS >= 32 && TCOLS <= 512 && (TCOLS & (TCOLS - 1)) == 0, "TMEM allocation: power of 2 in [32, 512]");
  static_assert(3 * COUT <= 256 && COUT % 16 == 0, "MMA N = 3 COUT in [16, 256], multiple of 16");
};

struct TcArgs {
  const bf16* in;     // input activations at their channel offset
  int in_cs;          // voxel pitch of the input (elements)
  const bf16* wimg;   // weight image in global memory (layout above)
  const float* bias;
  bf16* out;
  int out_cs;
  const bf16* add;
  int add_cs;
  int relu;
  int n;              // grid edge (input = output)
  int zc;             // output rows per column
  unsigned* err;
  unsigned long long wait_ns;   // limit of every pipeline wait
  int hold_back;      // test hook: the TMA slab loader issues no slab
};

// ---- PTX wrappers -----------------------------------------------------------

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
               : "memory");
}

// 16 bytes global -> shared; src_bytes 0 writes zeros (src is not read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// shared-memory matrix descriptor: no swizzle, fixed field 0b001 at bit 46
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// One accumulator row block (COUT FP32 columns of this warp's 32 TMEM
// lanes) into registers; a single wait in the same statement, so no
// register is read before the loads have landed.
template <int COUT>
__device__ __forceinline__ void tmem_ld_row(uint32_t addr, float* v);

template <>
__device__ __forceinline__ void tmem_ld_row<16>(uint32_t addr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

template <>
__device__ __forceinline__ void tmem_ld_row<32>(uint32_t addr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

template <>
__device__ __forceinline__ void tmem_ld_row<64>(uint32_t addr, float* v) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(addr), "r"(addr + 32u)
      : "memory");
#pragma unroll
  for (int j = 0; j < 64; ++j) v[j] = __uint_as_float(r[j]);
}

// zeros into 16 consecutive columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_zero16(uint32_t addr) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(addr),
      "r"(0u)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

struct Unit {
  int x0, y, z0;
};

// unit u = (x segment, group of yr rows, column of zc z planes), x fastest
__device__ __forceinline__ Unit unit_of(long long u, int n, int zc, int yr) {
  const int xsegs = (n + kTM - 1) / kTM, ny = n / yr;
  Unit t;
  t.x0 = (int)(u % xsegs) * kTM;
  const long long r = u / xsegs;
  t.y = (int)(r % ny) * yr;
  t.z0 = (int)(r / ny) * zc;
  return t;
}

__device__ __forceinline__ void give_up(volatile int* abort_flag, unsigned* err) {
  *abort_flag = 1;
  atomicOr(err, kErrTimeout);
}

// One slab (plane z_in of unit t, rows y0-1 .. y0+YR) into shared memory at
// dst: this producer thread's share of the 16-byte pieces, piece
// q = (row*130 + slot)*CH + chunk.
template <int CH, int YR, int PLANE>
__device__ __forceinline__ void load_slab(const TcArgs& a, const Unit& t, int z_in, uint32_t dst, int pt) {
  constexpr int PIECES = (YR + 2) * kSlots * CH;
  const int n = a.n;
  const bool zok = (unsigned)z_in < (unsigned)n;
#pragma unroll 4
  for (int q = pt; q < PIECES; q += kProducers) {
    const int c = q % CH, r = q / CH;
    const int sl = r % kSlots, dy = r / kSlots;
    const int xx = t.x0 - 1 + sl, yy = t.y + dy - 1;
    const bool ok = zok && (unsigned)xx < (unsigned)n && (unsigned)yy < (unsigned)n;
    const bf16* src = ok ? a.in + (((size_t)z_in * n + yy) * n + xx) * a.in_cs + 8 * c : a.in;
    cp_async16(dst + (uint32_t)(c * PLANE + dy * kRowBytes + sl * 16), src, ok ? 16u : 0u);
  }
}

// Descriptor offset (16-byte units) of the A window of MMA k of a slab: k =
// (dy*3 + dx)*KS + ks, or for 8 channels k = dy*2 + q (taps dx = 2q, 2q+1).
// The B image holds the matching weights at k * 2 * 3*COUT*16 bytes.
template <bool PAIRED, int KS, int PLANE>
__device__ __forceinline__ uint64_t a_off(int k) {
  if (PAIRED) return (uint64_t)(((k >> 1) * kRowBytes + (k & 1) * 32) >> 4);
  const int ks = k % KS, dx = (k / KS) % 3, dy = k / (3 * KS);
  return (uint64_t)((2 * ks * PLANE + dy * kRowBytes + dx * 16) >> 4);
}

// TMEM accumulator of output row i (rows counted across the CTA's columns):
// consecutive rows take descending slots, so rows z+1, z, z-1 sit in
// ascending, mostly adjacent column blocks.
__device__ __forceinline__ int acc_slot(long long i) { return (int)((kRing - (int)(i % kRing)) % kRing); }

template <int CIN, int COUT, int LOADER>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_kernel(const __grid_constant__ CUtensorMap tmap, TcArgs a) {
  using P = Tc<CIN, COUT>;
  constexpr int S = P::S;
  constexpr int AHEAD = S - 1;   // cp.async groups in flight per producer (deadlock-free bound: <= S)
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar_w, bar_fin, bar_full[S], bar_empty[S], bar_accf[kRing], bar_acce[kRing];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
  const uint32_t wsm = base, ssm = base + P::WB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = a.n, zc = a.zc;
  constexpr int YR = P::YR;
  // a 64-voxel row is one tile whose upper half reads the TMA fill (zeros) and is not stored
  const long long nunits = (long long)((n + kTM - 1) / kTM) * (n / YR) * (n / zc);

  if (threadIdx.x == 0) {
    abort_flag = 0;
    mbar_init(smem_u32(&bar_w), 1);
    mbar_init(smem_u32(&bar_fin), 1);
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&bar_full[s]), LOADER == kLoadTma ? 1 : kProducers);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int b = 0; b < kRing; ++b) {
      mbar_init(smem_u32(&bar_accf[b]), 1);
      mbar_init(smem_u32(&bar_acce[b]), 128);
    }
    mbar_init_fence();
  }
  // the 32-byte pad after each chunk of a slab is never loaded; an 8-channel
  // MMA reads it (times zero weights), so it must hold finite values
  for (int q = threadIdx.x; q < S * P::CH * 2; q += blockDim.x)
    asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(ssm + (uint32_t)(q >> 1) * P::PLANE + P::BOX + (q & 1) * 16),
                 "r"(0u)
                 : "memory");
  fence_proxy_async();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)P::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = tmem_slot;
  // every MMA accumulates: the ring starts at zero, and the epilogue zeroes
  // each accumulator after reading it
  if (warp >= kEpiWarp0 && warp < kEpiWarp0 + 4) {
    const uint32_t la = tm + ((uint32_t)(32 * (warp & 3)) << 16);
#pragma unroll 1
    for (int c = 0; c < P::TCOLS; c += 16) tmem_zero16(la + (uint32_t)c);
    tmem_wait_st();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  if (warp < kMmaWarp) {
    // ---- slab loaders (and the weight copy) ----
    const int pt = threadIdx.x;
    if (pt == 0) {
      mbar_expect_tx(smem_u32(&bar_w), (uint32_t)P::WB);
      bulk_load(wsm, a.wimg, (uint32_t)P::WB, smem_u32(&bar_w));
    }
    if (LOADER == kLoadTma) {
      if (pt == 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
        bool ok = true;
        long long j = 0;   // slab loads issued
        for (long long u = blockIdx.x; ok && !a.hold_back && u < nunits; u += gridDim.x) {
          const Unit t = unit_of(u, n, zc, YR);
          for (int p = 0; p < zc + 2; ++p, ++j) {
            const int slot = (int)(j % S);
            const long long use = j / S;
            if (use > 0 && !mbar_wait(smem_u32(&bar_empty[slot]), (uint32_t)((use - 1) & 1), &abort_flag, a.wait_ns)) {
              ok = false;
              break;
            }
            const uint32_t full = smem_u32(&bar_full[slot]);
            mbar_expect_tx(full, (uint32_t)(P::CH * P::BOX));
            const uint32_t dst = ssm + (uint32_t)slot * P::SLAB;
#pragma unroll
            for (int c = 0; c < P::CH; ++c)
              tma_load_4d(dst + c * P::PLANE, &tmap, full, 8 * c, t.x0 - 1, t.y - 1, t.z0 - 1 + p);
          }
        }
        if (!ok) give_up(&abort_flag, a.err);
        // drain: the last load of every slot has landed
        for (int s = 0; s < S; ++s) {
          if (j <= s) break;
          const long long last = j - 1 - ((j - 1 - s) % S);
          mbar_drain(smem_u32(&bar_full[s]), (uint32_t)((last / S) & 1));
        }
      }
    } else {
      // A producer holds at most AHEAD-1 slabs un-signalled while it waits
      // for a free slot; the slot's previous slab (S loads back) is then
      // signalled, and the MMA frees it without waiting for anything else
      // this producer owes.
      bool ok = true;
      long long j = 0, signalled = 0;
      for (long long u = blockIdx.x; ok && u < nunits; u += gridDim.x) {
        const Unit t = unit_of(u, n, zc, YR);
        for (int p = 0; p < zc + 2; ++p, ++j) {
          if (j - signalled >= AHEAD) {
            cp_async_wait<AHEAD - 1>();
            fence_proxy_async();
            mbar_arrive(smem_u32(&bar_full[(int)(signalled % S)]));
            ++signalled;
          }
          const int slot = (int)(j % S);
          const long long use = j / S;
          if (use > 0 && !mbar_wait(smem_u32(&bar_empty[slot]), (uint32_t)((use - 1) & 1), &abort_flag, a.wait_ns)) {
            ok = false;
            break;
          }
          load_slab<P::CH, YR, P::PLANE>(a, t, t.z0 - 1 + p, ssm + (uint32_t)slot * P::SLAB, pt);
          cp_async_commit();
        }
      }
      if (!ok) give_up(&abort_flag, a.err);
      cp_async_wait<0>();
      fence_proxy_async();
      for (; signalled < j; ++signalled) mbar_arrive(smem_u32(&bar_full[(int)(signalled % S)]));
    }
    if (pt == 0) mbar_drain(smem_u32(&bar_w), 0);   // the weight copy has landed
  } else if (warp == kMmaWarp) {
    // ---- MMA issuer: slab p of a column feeds output rows p, p-1, p-2
    //      (dz = 0, 1, 2) in one MMA per tap (dx, dy) and k step ----
    if (lane == 0) {
      constexpr uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTM >> 4) << 24);
      constexpr uint32_t kBlk = COUT * 16;          // bytes of one dz block of B
      constexpr uint32_t kLboB = 3 * COUT * 16;     // chunk stride of B
      bool ok = mbar_wait(smem_u32(&bar_w), 0, &abort_flag, a.wait_ns);
      long long j = 0, i0 = 0;   // slab loads and output rows before this column
      for (long long u = blockIdx.x; ok && u < nunits; u += gridDim.x) {
        for (int p = 0; p < zc + 2; ++p) {
          if (p < zc) {   // row p is first written now: its accumulator must be drained
            const long long i = i0 + p, use = i / kRing;
            if (use > 0 && !mbar_wait(smem_u32(&bar_acce[acc_slot(i)]), (uint32_t)((use - 1) & 1), &abort_flag,
                                      a.wait_ns)) {
              ok = false;
              break;
            }
          }
          const long long jj = j + p;
          const int slot = (int)(jj % S);
          if (!mbar_wait(smem_u32(&bar_full[slot]), (uint32_t)((jj / S) & 1), &abort_flag, a.wait_ns)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const int dz_lo = p - zc + 1 > 0 ? p - zc + 1 : 0;
          const int dz_hi = p < 2 ? p : 2;
          const int nd = dz_hi - dz_lo + 1;
          const int s_lo = acc_slot(i0 + p - dz_lo);
          // the nd blocks occupy slots s_lo .. s_lo+nd-1 <= kRing+1: past the
          // ring's end they land in its shadow slots, which the epilogue adds
          // to slots 0 and 1; every MMA is one contiguous N = nd*COUT
          const uint32_t id = idesc0 | ((uint32_t)(nd * COUT >> 3) << 17);
          // descriptors are linear in the start address (14-bit field, smem
          // below 256 KB): per MMA only compile-time offsets are added
          const uint64_t a_base = sdesc(ssm + (uint32_t)slot * P::SLAB, P::PAIRED ? 16u : (uint32_t)P::PLANE, 128);
          const uint64_t b_base = sdesc(wsm + (uint32_t)dz_lo * kBlk, kLboB, 128);
          // output row y0 + yy reads slab rows yy .. yy+2 and accumulates in
          // its own ring (TMEM columns yy*kCols*COUT ..)
#pragma unroll
          for (int yy = 0; yy < YR; ++yy) {
            const uint32_t d = tm + (uint32_t)((yy * kCols + s_lo) * COUT);
            const uint64_t a_row = a_base + (uint64_t)((yy * kRowBytes) >> 4);
#pragma unroll
            for (int k = 0; k < P::NMMA; ++k) {
              const uint64_t ad = a_row + a_off<P::PAIRED, P::KS, P::PLANE>(k);
              const uint64_t bo = (uint64_t)((k * 2 * kLboB) >> 4);
              mma_bf16(d, ad, b_base + bo, id, 1u);
            }
          }
          mma_commit(smem_u32(&bar_empty[slot]));
          if (p >= 2) mma_commit(smem_u32(&bar_accf[acc_slot(i0 + p - 2)]));   // row p-2 is complete
        }
        j += zc + 2;
        i0 += zc;
      }
      if (!ok) give_up(&abort_flag, a.err);
      // every MMA issued has completed before TMEM is freed
      mma_commit(smem_u32(&bar_fin));
      mbar_drain(smem_u32(&bar_fin), 0);
    }
  } else {
    // ---- epilogue: two teams of 4 warps take alternate output rows (a ring
    //      slot always belongs to the same team); one voxel per thread ----
    const int team = (warp - kEpiWarp0) >> 2;
    const int qd = warp & 3;   // TMEM lane quarter this warp may access
    const int m = 32 * qd + lane;
    const uint32_t lane_addr = tm + ((uint32_t)(32 * qd) << 16);
    bool ok = true;
    long long i = 0;
    for (long long u = blockIdx.x; ok && u < nunits; u += gridDim.x) {
      const Unit t = unit_of(u, n, zc, YR);
      for (int zl = 0; zl < zc; ++zl, ++i) {
        if ((int)(i & 1) != team) continue;
        const int s = acc_slot(i);
        const bool w = mbar_wait(smem_u32(&bar_accf[s]), (uint32_t)((i / kRing) & 1), &abort_flag, a.wait_ns);
        if (!__all_sync(0xffffffffu, w)) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll 1
        for (int yy = 0; yy < YR; ++yy) {
          const uint32_t acc = lane_addr + (uint32_t)((yy * kCols + s) * COUT);
          float v[COUT];
          tmem_ld_row<COUT>(acc, v);
          // zero the accumulator for its next row; the wait comes after the stores
#pragma unroll
          for (int c = 0; c < COUT; c += 16) tmem_zero16(acc + (uint32_t)c);
          if (s < kShadow) {   // the part that landed past the ring's end
            const uint32_t sh = lane_addr + (uint32_t)((yy * kCols + kRing + s) * COUT);
            float w[COUT];
            tmem_ld_row<COUT>(sh, w);
#pragma unroll
            for (int c = 0; c < COUT; ++c) v[c] += w[c];
#pragma unroll
            for (int c = 0; c < COUT; c += 16) tmem_zero16(sh + (uint32_t)c);
          }
          const bool inside = t.x0 + m < n;   // false only for the unused half of a 64-voxel row
          const size_t vo = ((size_t)(t.z0 + zl) * n + (t.y + yy)) * n + (inside ? t.x0 + m : 0);
          if (a.bias) {
#pragma unroll
            for (int c = 0; c < COUT; ++c) v[c] += __ldg(a.bias + c);
          }
          if (a.add && inside) {
            const uint4* ap = reinterpret_cast<const uint4*>(a.add + vo * a.add_cs);
#pragma unroll
            for (int g = 0; g < COUT / 8; ++g) {
              const uint4 q = ap[g];
              const uint32_t wd[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
              for (int h = 0; h < 4; ++h) {
                const __nv_bfloat162 p2 = *reinterpret_cast<const __nv_bfloat162*>(&wd[h]);
                v[8 * g + 2 * h] += __bfloat162float(p2.x);
                v[8 * g + 2 * h + 1] += __bfloat162float(p2.y);
              }
            }
          }
          if (a.relu) {
#pragma unroll
            for (int c = 0; c < COUT; ++c) v[c] = fmaxf(v[c], 0.0f);
          }
          uint4* op = reinterpret_cast<uint4*>(a.out + vo * a.out_cs);
#pragma unroll
          for (int g = 0; g < COUT / 8; ++g)
            if (inside)
              op[g] = make_uint4(pack_bf2(v[8 * g], v[8 * g + 1]), pack_bf2(v[8 * g + 2], v[8 * g + 3]),
                               pack_bf2(v[8 * g + 4], v[8 * g + 5]), pack_bf2(v[8 * g + 6], v[8 * g + 7]));
        }
        tmem_wait_st();
        tc_fence_before();
        mbar_arrive(smem_u32(&bar_acce[s]));
      }
    }
    if (!ok) give_up(&abort_flag, a.err);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"((uint32_t)P::TCOLS)
                 : "memory");
  }
}

// img[(((k*2 + c)*3 + dz)*CO + n)*8 + e] for MMA k of a slab and its K
// chunk c: for 16+ channels k = (dy*3 + dx)*KS + ks holds W(dx + 3dy + 9dz,
// 16ks + 8c + e, n); for 8 channels k = dy*2 + q holds W(tap of dx = 2q + c,
// e, n), zero for dx = 3.  The backward-data weights of a layer are
// W'(t, k, n) = W[26-t][n][k].
__global__ void image_kernel(int cin, int cout, const float* __restrict__ w, bf16* __restrict__ img, int backward) {
  const int ci2 = backward ? cout : cin, co2 = backward ? cin : cout;
  const bool paired = ci2 == 8;
  const int ks_n = paired ? 1 : ci2 / 16;
  const int nmma = paired ? 6 : 9 * ks_n;
  const size_t total = (size_t)nmma * 2 * 3 * co2 * 8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int e = (int)(i % 8);
    size_t r = i / 8;
    const int nn = (int)(r % co2);
    r /= co2;
    const int dz = (int)(r % 3);
    r /= 3;
    const int c = (int)(r % 2);
    const int k = (int)(r / 2);
    int dx, dy, ch;
    if (paired) {
      dy = k >> 1;
      dx = 2 * (k & 1) + c;
      ch = e;
    } else {
      const int ks = k % ks_n;
      dx = (k / ks_n) % 3;
      dy = k / (3 * ks_n);
      ch = 16 * ks + 8 * c + e;
    }
    float v = 0.0f;
    if (dx < 3) {
      const int t = dx + 3 * dy + 9 * dz;
      v = backward ? w[((size_t)(26 - t) * cin + nn) * cout + ch] : w[((size_t)t * cin + ch) * cout + nn];
    }
    img[i] = __float2bfloat16(v);
  }
}


// Input activations as a 4-D tensor {channels, x, y, z} (channels fastest,
// voxel pitch in_cs elements); box {8, 130, yr + 2, 1}.
cudaError_t input_map(CUtensorMap* map, const bf16* in, int in_cs, int cin, int n, int yr) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  if (((uintptr_t)in & 15) || (in_cs * 2) % 16) return cudaErrorInvalidValue;
  const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t pitch = (cuuint64_t)in_cs * 2;
  const cuuint64_t strides[3] = {pitch, pitch * n, pitch * n * n};
  const cuuint32_t box[4] = {8, (cuuint32_t)kSlots, (cuuint32_t)(yr + 2), 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(in), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int CIN, int COUT, int LOADER>
cudaError_t launch_tc(cudaStream_t s, const ConvArgs& c, int n) {
  using P = Tc<CIN, COUT>;
  static int blocks_per_sm[8] = {};   // per device ordinal (attribute set once)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 8) return cudaErrorInvalidDevice;
  if (!blocks_per_sm[dev]) {
    e = cudaFuncSetAttribute(conv_tc_kernel<CIN, COUT, LOADER>, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM);
    if (e != cudaSuccess) return e;
    int b = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, conv_tc_kernel<CIN, COUT, LOADER>, kThreads, P::SMEM);
    if (e != cudaSuccess) return e;
    // every resident CTA holds TCOLS of the SM's 512 TMEM columns for its
    // whole (persistent) life: a CTA that cannot allocate would wait for the
    // others to finish
    const int by_tmem = 512 / P::TCOLS;
    blocks_per_sm[dev] = std::max(1, std::min(b, by_tmem));
  }
  // 16-byte pieces of every voxel: aligned base and pitch
  if (((uintptr_t)c.in & 15) || (c.in_cs * 2) % 16 || ((uintptr_t)c.wimg & 15)) return cudaErrorInvalidValue;
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  if (LOADER == kLoadTma) {
    e = input_map(&map, c.in, c.in_cs, CIN, n, P::YR);
    if (e != cudaSuccess) return e;
  }
  TcArgs a;
  a.in = c.in;
  a.in_cs = c.in_cs;
  a.wimg = c.wimg;
  a.bias = c.bias;
  a.out = c.out;
  a.out_cs = c.out_cs;
  a.add = c.add;
  a.add_cs = c.add_cs;
  a.relu = c.relu;
  a.n = n;
  a.err = c.err;
  a.wait_ns = c.wait_ns;
  a.hold_back = LOADER == kLoadTma ? c.hold_back : 0;
  // rows per column: the choice that balances the persistent CTAs best
  const long long ctas = (long long)kNumSMs * blocks_per_sm[dev];
  int best = 0;
  long long best_rows = 0;
  for (int zc = 16; zc >= 4; zc /= 2) {
    if (n % zc) continue;
    const long long units = (long long)((n + kTM - 1) / kTM) * (n / P::YR) * (n / zc);
    const long long rows = ((units + ctas - 1) / ctas) * (zc + 2);   // slab loads of the busiest CTA
    if (!best || rows < best_rows) { best = zc; best_rows = rows; }
  }
  a.zc = best;
  const long long units = (long long)((n + kTM - 1) / kTM) * (n / P::YR) * (n / best);
  const unsigned grid = (unsigned)(units < ctas ? units : ctas);
  (conv_tc_kernel<CIN, COUT, LOADER><<<grid, kThreads, P::SMEM, s>>>(map, a), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace

bool tc_supported(int kind, int cin, int cout, int n) {
  // rows of 128k voxels, or a 64-voxel row as one half-used tile (the n/2
  // level of a 128^3 network)
  if (kind != C3 || !(n % kTM == 0 || n == kTM / 2)) return false;
#define X(I, O) if (cin == I && cout == O) return true;
  BAOREC_GUESS_TC_SHAPES(X)
#undef X
  return false;
}

cudaError_t conv_forward_tc(cudaStream_t s, int cin, int cout, const ConvArgs& c) {
  if (!c.wimg || !c.err || c.n_in != c.n_out) return cudaErrorInvalidValue;
#define X(I, O)                                                                          \
  if (cin == I && cout == O)                                                             \
    return c.tc_loader == 1 ? launch_tc<I, O, kLoadCpAsync>(s, c, c.n_out) : launch_tc<I, O, kLoadTma>(s, c, c.n_out);
  BAOREC_GUESS_TC_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t weight_image(cudaStream_t s, int cin, int cout, const float* w, __nv_bfloat16* img, bool backward) {
  (image_kernel<<<64, 256, 0, s>>>(cin, cout, w, img, backward ? 1 : 0), ::baorec::count_launch());
  return cudaGetLastError();
}

}  // namespace guess
}  // namespace baorec
