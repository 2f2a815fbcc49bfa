// Bounding box of a particle catalog without any device allocation.
//
// Some callers cannot let this library allocate device memory: a Julia or
// Python host whose pool allocator (CUDA.jl, PyTorch's caching allocator)
// already owns the device memory budget, and latency-sensitive pipelines
// where the implicit device-wide synchronisation of cudaMalloc / cudaFree
// would stall their other streams.  For them baorec_setup_box_noalloc
// computes what baorec_setup_box computes (setup_box, src/utils.jl:100-109)
// with no context and no allocation: the per-block partial minima/maxima live
// in a fixed file-scope device array instead of a context buffer.
//
// The array is sized for kMaxBlocks blocks of kThreads x kItemsPerThread
// particles, so a call accepts at most kMaxParticles = 16,777,216 particles
// and rejects larger catalogs with BAOREC_ERR_TOO_LARGE.  Every GPU that
// loads the library holds the 24.6 KB array until the process exits.
//
// The call is synchronous: it waits for its stream and copies six values into
// host stack memory, neither of which is allowed while the stream is being
// captured, so a call on a capturing stream is refused (BAOREC_ERR_ARG)
// before anything is enqueued.  The array's device address is looked up once
// per device and cached; cudaDeviceReset unloads the module that holds the
// array, so a process that resets a device must not call this entry point on
// that device again.
#include <mutex>

#include "common.cuh"

namespace baorec {
namespace {

constexpr int kThreads = 256;
constexpr int kItemsPerThread = 64;
constexpr int kMaxBlocks = 1024;
constexpr int64_t kMaxParticles = (int64_t)kMaxBlocks * kThreads * kItemsPerThread;
constexpr int kFinal = kMaxBlocks * 6;   // offset of the final 6 values
constexpr int kMaxDevices = 64;

// Shared by every call on a device; each call overwrites the partials of the
// blocks it launches and the final 6 values, so nothing needs clearing.
static __device__ __align__(256) float g_box_scratch[kMaxBlocks * 6 + 8];

std::mutex g_setup_mu;
float* g_scratch_ptr[kMaxDevices] = {};

// One block reduces kThreads * kItemsPerThread particles into 6 partials.
__global__ void box_partial_noalloc_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                           const float* __restrict__ z, int64_t n, float* __restrict__ part) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  const int64_t base = (int64_t)blockIdx.x * kThreads * kItemsPerThread + threadIdx.x;
#pragma unroll 4
  for (int k = 0; k < kItemsPerThread; ++k) {
    int64_t i = base + (int64_t)k * kThreads;
    if (i >= n) break;
    float v[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int a = 0; a < 3; ++a) { mn[a] = fminf(mn[a], v[a]); mx[a] = fmaxf(mx[a], v[a]); }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  __shared__ float s[6][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int a = 0; a < 3; ++a) { s[a][wid] = mn[a]; s[3 + a][wid] = mx[a]; }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int a = threadIdx.x;
    float r = s[a][0];
    for (int q = 1; q < kThreads / 32; ++q) r = a < 3 ? fminf(r, s[a][q]) : fmaxf(r, s[a][q]);
    part[blockIdx.x * 6 + a] = r;
  }
}

// One block folds the nblocks partials into part[kFinal .. kFinal+5].
__global__ void box_final_noalloc_kernel(float* __restrict__ part, int nblocks) {
  __shared__ float s[6][kThreads];
  float r[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int b = threadIdx.x; b < nblocks; b += kThreads)
    for (int a = 0; a < 6; ++a) r[a] = a < 3 ? fminf(r[a], part[b * 6 + a]) : fmaxf(r[a], part[b * 6 + a]);
  for (int a = 0; a < 6; ++a) s[a][threadIdx.x] = r[a];
  __syncthreads();
  if (threadIdx.x < 6) {
    const int a = threadIdx.x;
    float v = s[a][0];
    for (int q = 1; q < kThreads; ++q) v = a < 3 ? fminf(v, s[a][q]) : fmaxf(v, s[a][q]);
    part[kFinal + a] = v;
  }
}

// Device address of g_box_scratch on the current device, looked up once per
// device (the host-side symbol is only a stand-in, not a device address).
cudaError_t scratch_for_current_device(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_box_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = (float*)p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// The particle arrays must be device (or managed) memory of the current
// device: the kernels run there, next to the scratch array of that device.
bool on_current_device(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) return false;
  return at.type == cudaMemoryTypeManaged || at.device == dev;
}

}  // namespace
}  // namespace baorec

extern "C" int baorec_setup_box_noalloc(const float* x, const float* y, const float* z, int64_t n, float pad,
                                        void* stream, float box_size_out[3], float box_min_out[3]) {
  using namespace baorec;
  if (!x || !y || !z || !box_size_out || !box_min_out || n < 1) return BAOREC_ERR_ARG;
  if (n > kMaxParticles) return BAOREC_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BAOREC_ERR_CUDA;
  if (!on_current_device(x, dev) || !on_current_device(y, dev) || !on_current_device(z, dev)) return BAOREC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    return BAOREC_ERR_ARG;
  }
  if (cap != cudaStreamCaptureStatusNone) return BAOREC_ERR_ARG;
  float* part = nullptr;
  if (scratch_for_current_device(&part) != cudaSuccess) return BAOREC_ERR_CUDA;
  const int nblocks = (int)((n + (int64_t)kThreads * kItemsPerThread - 1) / ((int64_t)kThreads * kItemsPerThread));
  (box_partial_noalloc_kernel<<<nblocks, kThreads, 0, s>>>(x, y, z, n, part), ::baorec::count_launch());
  if (cudaGetLastError() != cudaSuccess) return BAOREC_ERR_CUDA;
  (box_final_noalloc_kernel<<<1, kThreads, 0, s>>>(part, nblocks), ::baorec::count_launch());
  if (cudaGetLastError() != cudaSuccess) return BAOREC_ERR_CUDA;
  float h[6];
  if (cudaMemcpyAsync(h, part + kFinal, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return BAOREC_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return BAOREC_ERR_CUDA;
  // src/utils.jl:103-105 in FP32, as baorec_setup_box does
  const float half = pad / 2.0f;
  float side = -INFINITY;
  for (int a = 0; a < 3; ++a) {
    box_min_out[a] = h[a] - half;
    side = fmaxf(side, (h[3 + a] + half) - box_min_out[a]);
  }
  for (int a = 0; a < 3; ++a) box_size_out[a] = side;
  return BAOREC_OK;
}
