// The coarse end of a correction V-cycle in one cooperative kernel.
//
// Levels of at most kTailMaxCells cells are too small to fill the GPU one
// launch at a time (tens of blocks, microseconds of launch latency per step).
// This kernel runs all of them — pre-smoothing, residual, restriction, the
// dense FP64 solve on the coarsest level, prolongation and post-smoothing —
// with every block of a co-resident grid and a grid-wide barrier between
// steps.  Red-black half sweeps are out of place (v -> t -> v), so the result
// does not depend on thread scheduling.
#include <cooperative_groups.h>

#include "mg_common.cuh"

namespace cg = cooperative_groups;

namespace baorec {
namespace {

__device__ __forceinline__ void ijk_of(int e, const int n[3], int& i, int& j, int& k) {
  i = e % n[0];
  const int r = e / n[0];
  j = r % n[1];
  k = r / n[1];
}

__device__ __forceinline__ int id3(const int n[3], int i, int j, int k) { return i + n[0] * (j + n[1] * k); }

// coef_at with fast division (the tail is a preconditioner)
__device__ __forceinline__ Coef coef_tail(const LG& G, int i, int j, int k) {
  float px, py, pz;
  if (G.local) { px = G.P[0][i]; py = G.P[1][j]; pz = G.P[2][k]; }
  else { px = G.pg[0]; py = G.pg[1]; pz = G.pg[2]; }
  Coef c;
  const float px2 = px * px, py2 = py * py, pz2 = pz * pz;
  c.g = __fdividef(G.beta, G.cell2[0] * px2 + G.cell2[1] * py2 + G.cell2[2] * pz2);
  c.gpx = G.icell2[0] + c.g * px2;
  c.gpy = G.icell2[1] + c.g * py2;
  c.gpz = G.icell2[2] + c.g * pz2;
  c.pxy = px * py; c.pxz = px * pz; c.pyz = py * pz;
  if (G.local) {
    c.dx = fminf(fmaxf(c.g * px, -G.clamp * c.gpx), G.clamp * c.gpx);
    c.dy = fminf(fmaxf(c.g * py, -G.clamp * c.gpy), G.clamp * c.gpy);
    c.dz = fminf(fmaxf(c.g * pz, -G.clamp * c.gpz), G.clamp * c.gpz);
  } else {
    c.dx = c.dy = c.dz = 0.0f;
  }
  return c;
}

// (rhs - shift + neighbours(in)) / diag for cell e of level T; in == nullptr
// means a zero field (the first half sweep after zeroing the correction).
__device__ __forceinline__ float gs_cell(const TailLevel& T, const float* __restrict__ in, int e, float shift) {
  int i, j, k;
  ijk_of(e, T.G.n, i, j, k);
  const Coef c = coef_tail(T.G, i, j, k);
  float o = 0.0f;
  if (in) {
    const Nb b = gather([&](int a, int bb, int cc) { return in[id3(T.G.n, a, bb, cc)]; }, T.G.n, i, j, k);
    o = offdiag(c, b, T.G.local);
  }
  return __fdividef(T.f[e] - shift + o, 2.0f * (c.gpx + c.gpy + c.gpz));
}

__global__ void coarse_tail_kernel(TailArgs A) {
  cg::grid_group grid = cg::this_grid();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const int last = A.nl - 1;
  auto half_sweep = [&](const TailLevel& T, const float* in, float* out, int colour, float shift) {
    for (int e = tid; e < T.N; e += nth) {
      int i, j, k;
      ijk_of(e, T.G.n, i, j, k);
      out[e] = (((i + j + k) & 1) == colour) ? gs_cell(T, in, e, shift) : (in ? in[e] : 0.0f);
    }
    grid.sync();
  };
  // ---- down
  for (int l = 0; l < last; ++l) {
    const TailLevel& T = A.L[l];
    const float shift = l == 0 ? A.shift0 : 0.0f;
    // the correction starts at zero: the first half sweep reads no field
    for (int s = 0; s < A.nu1; ++s) {
      half_sweep(T, s == 0 ? nullptr : T.v, T.t, 0, shift);
      half_sweep(T, T.t, T.v, 1, shift);
    }
    if (A.nu1 == 0) {
      for (int e = tid; e < T.N; e += nth) T.v[e] = 0.0f;
      grid.sync();
    }
    // residual r = rhs - shift - A v
    for (int e = tid; e < T.N; e += nth) {
      int i, j, k;
      ijk_of(e, T.G.n, i, j, k);
      const Coef c = coef_at(T.G, i, j, k);
      const Nb b = gather([&](int a, int bb, int cc) { return T.v[id3(T.G.n, a, bb, cc)]; }, T.G.n, i, j, k);
      T.r[e] = (T.f[e] - shift) - (2.0f * (c.gpx + c.gpy + c.gpz) * T.v[e] - offdiag(c, b, T.G.local));
    }
    grid.sync();
    // full-weighting restriction into the next level's right-hand side
    const TailLevel& C = A.L[l + 1];
    for (int e = tid; e < C.N; e += nth) {
      int ci, cj, ck;
      ijk_of(e, C.G.n, ci, cj, ck);
      const int* nf = T.G.n;
      const int i = 2 * ci + 1, j = 2 * cj + 1, k = 2 * ck + 1;
      const int ip = i + 1 == nf[0] ? 0 : i + 1, im = i - 1, jp = j + 1 == nf[1] ? 0 : j + 1, jm = j - 1;
      const int kp = k + 1 == nf[2] ? 0 : k + 1, km = k - 1;
      auto F = [&](int a, int b, int cc) { return T.r[id3(nf, a, b, cc)]; };
      const float s = 8.0f * F(i, j, k) +
                      4.0f * (F(ip, j, k) + F(im, j, k) + F(i, jp, k) + F(i, jm, k) + F(i, j, kp) + F(i, j, km)) +
                      2.0f * (F(ip, jp, k) + F(im, jp, k) + F(ip, jm, k) + F(im, jm, k) + F(ip, j, kp) +
                              F(im, j, kp) + F(ip, j, km) + F(im, j, km) + F(i, jp, kp) + F(i, jm, kp) +
                              F(i, jp, km) + F(i, jm, km)) +
                      F(ip, jp, kp) + F(im, jp, kp) + F(ip, jm, kp) + F(im, jm, kp) + F(ip, jp, km) +
                      F(im, jp, km) + F(ip, jm, km) + F(im, jm, km);
      C.f[e] = s / 64.0f;
    }
    grid.sync();
  }
  // ---- coarsest: dense FP64 solve v = M f (one warp per row, coalesced columns)
  {
    const TailLevel& C = A.L[last];
    const int lane = threadIdx.x & 31;
    const int warp = tid >> 5, nwarp = nth >> 5;
    const float shift = last == 0 ? A.shift0 : 0.0f;   // M 1 = 0: the shift drops out
    (void)shift;
    for (int row = warp; row < C.N; row += nwarp) {
      double s = 0.0;
      const double* Mr = A.M + (size_t)row * C.N;
      for (int q = lane; q < C.N; q += 32) s += Mr[q] * (double)C.f[q];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) C.v[row] = (float)s;
    }
    grid.sync();
  }
  // ---- up
  for (int l = last - 1; l >= 0; --l) {
    const TailLevel& T = A.L[l];
    const TailLevel& C = A.L[l + 1];
    const float shift = l == 0 ? A.shift0 : 0.0f;
    // v += prolong(v_coarse): coarse c -> fine 2c+1, midpoints 2c+2 (periodic)
    for (int e = tid; e < C.N; e += nth) {
      int i, j, k;
      ijk_of(e, C.G.n, i, j, k);
      const int* nc = C.G.n;
      const int* nf = T.G.n;
      const int ip = i + 1 == nc[0] ? 0 : i + 1, jp = j + 1 == nc[1] ? 0 : j + 1, kp = k + 1 == nc[2] ? 0 : k + 1;
      auto Cv = [&](int a, int b, int cc) { return C.v[id3(nc, a, b, cc)]; };
      const float c000 = Cv(i, j, k), c100 = Cv(ip, j, k), c010 = Cv(i, jp, k), c001 = Cv(i, j, kp);
      const float c110 = Cv(ip, jp, k), c011 = Cv(i, jp, kp), c101 = Cv(ip, j, kp), c111 = Cv(ip, jp, kp);
      const int x0 = 2 * i + 1, y0 = 2 * j + 1, z0 = 2 * k + 1;
      const int x1 = x0 + 1 == nf[0] ? 0 : x0 + 1, y1 = y0 + 1 == nf[1] ? 0 : y0 + 1, z1 = z0 + 1 == nf[2] ? 0 : z0 + 1;
      T.v[id3(nf, x0, y0, z0)] += c000;
      T.v[id3(nf, x1, y0, z0)] += (c000 + c100) / 2.0f;
      T.v[id3(nf, x0, y1, z0)] += (c000 + c010) / 2.0f;
      T.v[id3(nf, x0, y0, z1)] += (c000 + c001) / 2.0f;
      T.v[id3(nf, x1, y1, z0)] += (c000 + c100 + c010 + c110) / 4.0f;
      T.v[id3(nf, x0, y1, z1)] += (c000 + c010 + c001 + c011) / 4.0f;
      T.v[id3(nf, x1, y0, z1)] += (c000 + c100 + c001 + c101) / 4.0f;
      T.v[id3(nf, x1, y1, z1)] += (c000 + c100 + c010 + c001 + c110 + c101 + c011 + c111) / 8.0f;
    }
    grid.sync();
    for (int s = 0; s < A.nu2; ++s) {
      half_sweep(T, T.v, T.t, 0, shift);
      half_sweep(T, T.t, T.v, 1, shift);
    }
  }
}

}  // namespace

// Largest grid that can be co-resident (the cooperative launch checks it).
cudaError_t launch_coarse_tail(cudaStream_t s, const TailArgs& args) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coarse_tail_kernel, 256, 0)) != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorLaunchOutOfResources;
  const int want = (args.L[0].N + 255) / 256;
  int blocks = sms * (per_sm < 2 ? per_sm : 2);
  if (blocks > want) blocks = want > 0 ? want : 1;
  TailArgs a = args;
  void* params[] = {&a};
  const cudaError_t le = cudaLaunchCooperativeKernel((void*)coarse_tail_kernel, dim3(blocks), dim3(256), params, 0, s);
  ::baorec::count_launch();
  return le;
}

}  // namespace baorec
