// Catalog coordinates on the device: sky <-> comoving Cartesian positions and
// FKP weights, the steps either side of the reconstruction in the reference's
// lightcone scripts (examples/lightcone.jl:30-82, test/benchmarks_cpu.jl:29-81).
// The cosmology stays on the host (src/cosmo.jl:83-98): the caller passes the
// comoving-distance table r(z) on a uniform z grid (FP64, Mpc, no h), and the
// kernels interpolate it linearly as Interpolations' Gridded(Linear()) does.
//
//   sky -> Cartesian:  ra, dec in degrees (FP32 ra * π / 180 as Julia rounds
//                      it), dist = r(z) in FP64, x = dist cos(dec) cos(ra) h,
//                      y = dist cos(dec) sin(ra) h, z = dist sin(dec) h
//   Cartesian -> sky:  r = |p| / h (FP32), z = r^-1(r) by binary search and
//                      linear interpolation on the (monotonic) table, ra =
//                      (atan2(y, x) 180/π - 360) rem 360 (the scripts' quirk:
//                      ra comes back in (-360, 0]), dec = atan2(z, |p_xy|) 180/π
//   FKP:               w = 1 / (1 + n(z) P0)
#include "common.cuh"

namespace baorec {
namespace {

struct Table {
  const double* r;
  int n;
  double z0, dz;
};

// Outside the table the reference's interpolation throws: flag kErrOOB.
__device__ __forceinline__ double r_of_z(const Table& t, double z, unsigned* err) {
  double u = (z - t.z0) / t.dz;
  if (!(u >= 0.0 && u <= (double)(t.n - 1))) atomicOr(err, kErrOOB);
  int i = (int)floor(u);
  i = i < 0 ? 0 : (i > t.n - 2 ? t.n - 2 : i);
  const double s = u - (double)i;
  return t.r[i] + s * (t.r[i + 1] - t.r[i]);
}

__device__ __forceinline__ double z_of_r(const Table& t, double r, unsigned* err) {
  if (!(r >= t.r[0] && r <= t.r[t.n - 1])) atomicOr(err, kErrOOB);
  int lo = 0, hi = t.n - 1;   // the largest lo with r[lo] <= r, within [0, n-2]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (t.r[mid] <= r) lo = mid;
    else hi = mid;
  }
  const double s = (r - t.r[lo]) / (t.r[lo + 1] - t.r[lo]);
  return t.z0 + t.dz * ((double)lo + s);
}

__global__ void sky_to_cart_kernel(const float* __restrict__ ra, const float* __restrict__ dec,
                                   const float* __restrict__ red, int64_t n, Table t, float h,
                                   float* __restrict__ x, float* __restrict__ y, float* __restrict__ z,
                                   unsigned* err) {
  const float pi = 3.14159265358979323846f;   // Float32(π)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double dist = r_of_z(t, (double)red[i], err);
    const float a = __fdiv_rn(__fmul_rn(ra[i], pi), 180.0f);
    const float d = __fdiv_rn(__fmul_rn(dec[i], pi), 180.0f);
    const double cd = (double)cosf(d), sd = (double)sinf(d), ca = (double)cosf(a), sa = (double)sinf(a);
    x[i] = (float)(dist * cd * ca * (double)h);
    y[i] = (float)(dist * cd * sa * (double)h);
    z[i] = (float)(dist * sd * (double)h);
  }
}

__global__ void cart_to_sky_kernel(const float* __restrict__ px, const float* __restrict__ py,
                                   const float* __restrict__ pz, int64_t n, Table t, float h,
                                   float* __restrict__ ra, float* __restrict__ dec, float* __restrict__ red,
                                   unsigned* err) {
  const float pi = 3.14159265358979323846f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = px[i], y = py[i], z = pz[i];
    const float r = __fdiv_rn(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z))), h);
    const float s = __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
    float lon = __fdiv_rn(__fmul_rn(atan2f(y, x), 180.0f), pi);
    const float lat = __fdiv_rn(__fmul_rn(atan2f(z, s), 180.0f), pi);
    lon = fmodf(__fsub_rn(lon, 360.0f), 360.0f);
    ra[i] = lon;
    dec[i] = lat;
    red[i] = (float)z_of_r(t, (double)r, err);
  }
}

__global__ void fkp_kernel(const float* __restrict__ nz, int64_t n, float P0, float* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = __fdiv_rn(1.0f, __fadd_rn(1.0f, __fmul_rn(nz[i], P0)));
}

int table_in(baorec_ctx* ctx, const double* r_table, int ntab, double z_min, double z_max, Table* t) {
  if (!r_table || ntab < 2 || !(z_max > z_min))
    return set_error(ctx, BAOREC_ERR_ARG, "distance table: need >= 2 entries on z_max > z_min");
  CKS(ensure(ctx, ctx->stage[7], (size_t)ntab * sizeof(double)));
  CK(cudaMemcpyAsync(ctx->stage[7].p, r_table, (size_t)ntab * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  t->r = (const double*)ctx->stage[7].p;
  t->n = ntab;
  t->z0 = z_min;
  t->dz = (z_max - z_min) / (double)(ntab - 1);
  return BAOREC_OK;
}

unsigned grid_of_n(int64_t n) {
  unsigned g = grid_for((size_t)n, 256);
  return g > 64u * kNumSMs ? 64u * kNumSMs : (g ? g : 1u);
}

}  // namespace
}  // namespace baorec

using namespace baorec;

extern "C" int baorec_sky_to_cartesian(baorec_ctx* ctx, const float* ra, const float* dec, const float* z, int64_t n,
                                       const double* r_table, int32_t ntab, double z_min, double z_max, float h,
                                       float* x, float* y, float* zc, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || (n > 0 && (!ra || !dec || !z || !x || !y || !zc)))
    return set_error(ctx, BAOREC_ERR_ARG, "sky_to_cartesian: bad arrays");
  Table t;
  CKS(table_in(ctx, r_table, ntab, z_min, z_max, &t));
  const float *dra, *ddec, *dz;
  CKS(stage_in(ctx, 0, ra, n, flags, &dra));
  CKS(stage_in(ctx, 1, dec, n, flags, &ddec));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float *ox, *oy, *oz;
  CKS(stage_out_alloc(ctx, 4, n, flags, x, &ox));
  CKS(stage_out_alloc(ctx, 5, n, flags, y, &oy));
  CKS(stage_out_alloc(ctx, 6, n, flags, zc, &oz));
  if (n > 0) {
    (sky_to_cart_kernel<<<grid_of_n(n), 256, 0, ctx->stream>>>(dra, ddec, dz, n, t, h, ox, oy, oz, ctx->derr), ::baorec::count_launch());
    CKLAUNCH();
  }
  CKS(stage_out_copy(ctx, x, ox, n, flags));
  CKS(stage_out_copy(ctx, y, oy, n, flags));
  CKS(stage_out_copy(ctx, zc, oz, n, flags));
  // the table sits in a staging buffer: wait before returning unless the caller owns the ordering
  return finish(ctx, flags & ~BAOREC_ASYNC);
}

extern "C" int baorec_cartesian_to_sky(baorec_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                                       const double* r_table, int32_t ntab, double z_min, double z_max, float h,
                                       float* ra, float* dec, float* red, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || (n > 0 && (!x || !y || !z || !ra || !dec || !red)))
    return set_error(ctx, BAOREC_ERR_ARG, "cartesian_to_sky: bad arrays");
  Table t;
  CKS(table_in(ctx, r_table, ntab, z_min, z_max, &t));
  const float *dx, *dy, *dz;
  CKS(stage_in(ctx, 0, x, n, flags, &dx));
  CKS(stage_in(ctx, 1, y, n, flags, &dy));
  CKS(stage_in(ctx, 2, z, n, flags, &dz));
  float *o0, *o1, *o2;
  CKS(stage_out_alloc(ctx, 4, n, flags, ra, &o0));
  CKS(stage_out_alloc(ctx, 5, n, flags, dec, &o1));
  CKS(stage_out_alloc(ctx, 6, n, flags, red, &o2));
  if (n > 0) {
    (cart_to_sky_kernel<<<grid_of_n(n), 256, 0, ctx->stream>>>(dx, dy, dz, n, t, h, o0, o1, o2, ctx->derr), ::baorec::count_launch());
    CKLAUNCH();
  }
  CKS(stage_out_copy(ctx, ra, o0, n, flags));
  CKS(stage_out_copy(ctx, dec, o1, n, flags));
  CKS(stage_out_copy(ctx, red, o2, n, flags));
  return finish(ctx, flags & ~BAOREC_ASYNC);
}

extern "C" int baorec_fkp_weights(baorec_ctx* ctx, const float* nz, int64_t n, float P0, float* w, uint32_t flags) {
  if (!ctx) return BAOREC_ERR_ARG;
  if (n < 0 || (n > 0 && (!nz || !w))) return set_error(ctx, BAOREC_ERR_ARG, "fkp_weights: bad arrays");
  const float* dnz;
  CKS(stage_in(ctx, 0, nz, n, flags, &dnz));
  float* dw;
  CKS(stage_out_alloc(ctx, 4, n, flags, w, &dw));
  if (n > 0) {
    (fkp_kernel<<<grid_of_n(n), 256, 0, ctx->stream>>>(dnz, n, P0, dw), ::baorec::count_launch());
    CKLAUNCH();
  }
  CKS(stage_out_copy(ctx, w, dw, n, flags));
  return finish(ctx, (flags & BAOREC_HOST) ? (flags & ~BAOREC_ASYNC) : flags);
}
