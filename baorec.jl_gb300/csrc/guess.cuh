// Learned initial guess: a 3-level 3-D U-Net over BF16 channels-last
// activations with FP32 accumulation on the tensor cores.
//
// Kernels (guess_kernels.cu) are implicit GEMMs over a "gather" convolution:
// every output voxel v of a layer is  y[v][o] = b[o] + Σ_t Σ_i W[t][i][o] x[src(v,t)][i]
// with three tap geometries:
//   C3  3x3x3, stride 1, zero padding 1      (taps t = (dx,dy,dz) in {0,1,2}^3, src = v + d - 1)
//   DN  2x2x2, stride 2 (down-sampling)      (taps d in {0,1}^3, src = 2v + d)
//   UP  2x2x2 transposed, stride 2           (one tap per output voxel: d = v & 1, src = v >> 1)
// M = voxels (16 consecutive x per MMA tile), N = output channels, K = taps x
// input channels.  The backward data pass of C3 is C3 with flipped,
// transposed weights; that of DN is UP-shaped and vice versa, so one forward
// kernel serves both directions.  The weight gradient is a second implicit
// GEMM with the voxels as the reduction dimension.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace baorec {
namespace guess {

enum Kind { C3 = 0, DN = 1, UP = 2 };

inline int taps_of(int kind) { return kind == C3 ? 27 : 8; }

struct ConvArgs {
  const __nv_bfloat16* in;   // input at its channel offset
  int in_cs;                 // input channel stride (voxel pitch in elements)
  __nv_bfloat16* out;        // output at its channel offset
  int out_cs;
  const __nv_bfloat16* add;  // optional addend, same voxel layout as out (may alias out)
  int add_cs;
  const uint2* w;            // weights in MMA fragment order (see weight_frag_index)
  const float* bias;         // per output channel, or null
  int relu;
  int n_in, n_out;           // cube edge of the input and output grids
  // tensor-core (tcgen05) path, taken for the shapes tc_supported() accepts:
  const __nv_bfloat16* wimg = nullptr;   // weight image (weight_image), null = mma.sync path
  unsigned* err = nullptr;               // device error word (kErrTimeout)
  int tc_loader = 0;                     // slab loader: 0 TMA boxes, 1 cp.async warps
  // limit of every pipeline wait of the tcgen05 kernel (ns); the drains at
  // the end of a block always allow 2 s
  unsigned long long wait_ns = 2000000000ull;
  int hold_back = 0;                     // test hook: the TMA slab loader issues no slab (waits expire)
};

struct WgradArgs {
  const __nv_bfloat16* in;   // forward input
  int in_cs;
  const __nv_bfloat16* dy;   // gradient of the forward output (ReLU already applied)
  int dy_cs;
  float* dw;                 // [t][ci][co] FP32, accumulated
  int n_in, n_out;
};

// Fragment-ordered weights of one layer: for tap t, K step ks (16 input
// channels; 8 when the layer has 8), N block nb (8 output channels) and lane:
//   {pack(W[t][k0+2q][n], W[t][k0+2q+1][n]), pack(W[t][k0+8+2q][n], W[t][k0+9+2q][n])}
// with k0 = 16 ks, q = lane & 3, n = 8 nb + (lane >> 2).
inline size_t frag_count(int kind, int cin, int cout) {
  const int ks = cin >= 16 ? cin / 16 : 1;
  return (size_t)taps_of(kind) * ks * (cout / 8) * 32;
}

// layer shapes with an mma.sync kernel (guess_kernels.cu)
#define BAOREC_GUESS_SHAPES(X)                                                                     \
  X(C3, 8, 16) X(C3, 16, 16) X(C3, 32, 32) X(C3, 64, 64) X(C3, 64, 32) X(C3, 32, 16) X(C3, 16, 32) \
  X(C3, 32, 64) X(DN, 16, 32) X(DN, 32, 64) X(UP, 64, 32) X(UP, 32, 16)

// C3 shapes with a tcgen05 kernel (guess_tc.cu); grids with n % 128 == 0 or n == 64
#define BAOREC_GUESS_TC_SHAPES(X) X(8, 16) X(16, 16) X(32, 32) X(32, 16) X(16, 32) X(32, 64) X(64, 32)

// BF16 entries of a tcgen05 weight image: one 16-wide K step per MMA of a
// slab (9 taps x cin/16 steps, or 6 tap pairs for 8 channels), 3 dz blocks
inline size_t image_count(int cin, int cout) { return (size_t)(cin == 8 ? 6 : 9 * (cin / 16)) * 16 * 3 * cout; }

// Dispatches to the tcgen05 kernel when a.wimg is set and the shape is
// covered, to the mma.sync kernel otherwise.
cudaError_t conv_forward(cudaStream_t s, int kind, int cin, int cout, const ConvArgs& a);
bool tc_supported(int kind, int cin, int cout, int n);
cudaError_t conv_forward_tc(cudaStream_t s, int cin, int cout, const ConvArgs& a);
// fp32 master W[t][ci][co] -> the tcgen05 weight image of the forward (or,
// with backward, the backward-data) convolution of a C3 layer
cudaError_t weight_image(cudaStream_t s, int cin, int cout, const float* w, __nv_bfloat16* img, bool backward);
cudaError_t conv_wgrad(cudaStream_t s, int kind, int cin, int cout, const WgradArgs& a);
// fp32 master W[t][ci][co] -> fragments; transpose_flip selects the backward
// data weights (W'[t'][co][ci] = W[flip(t)][ci][co], flip only for C3).
cudaError_t weight_frags(cudaStream_t s, int kind, int cin, int cout, const float* w, uint2* frag, bool backward);

}  // namespace guess
}  // namespace baorec
