// cuFFT load callback of the FFT preconditioner (compiled to LTO IR and
// linked into the inverse-transform plan at plan creation): the C2R reads
// each half-complex mode already multiplied by 1 / (N S(k)), so the k-space
// multiply costs no pass over the spectrum of its own.  S(k) and the table
// layout are those of spectral_inverse_kernel in fft.cu.
#include <cufftXt.h>

struct SpecCallbackInfo {
  const float* tab;   // hx2[n1h] | sx[n1h] | hy2[n2] | sy[n2] | hz2[n3] | sz[n3]
  unsigned long long nk;   // modes of the spectrum
  int n1h, n2, n3;
  float diag[3], cross[3];
  float invN;
};

extern "C" __device__ cufftComplex baorec_spectral_load(void* dataIn, unsigned long long offset, void* callerInfo,
                                                        void* sharedPointer) {
  const SpecCallbackInfo* p = static_cast<const SpecCallbackInfo*>(callerInfo);
  if (offset >= p->nk) return make_cuComplex(0.0f, 0.0f);   // never read outside the spectrum
  cufftComplex v = static_cast<const cufftComplex*>(dataIn)[offset];
  const unsigned int o = (unsigned int)offset;   // one spectrum, fewer than 2^32 modes
  const unsigned int row = o / (unsigned int)p->n1h;
  const int i = (int)(o - row * (unsigned int)p->n1h);
  const int k = (int)(row / (unsigned int)p->n2), j = (int)row - k * p->n2;
  const float* hx2 = p->tab;
  const float* sx = hx2 + p->n1h;
  const float* hy2 = sx + p->n1h;
  const float* sy = hy2 + p->n2;
  const float* hz2 = sy + p->n2;
  const float* sz = hz2 + p->n3;
  const float syj = sy[j], szk = sz[k];
  const float A = p->diag[0] * hx2[i] + p->diag[1] * hy2[j] + p->diag[2] * hz2[k] + p->cross[2] * syj * szk +
                  (p->cross[0] * syj + p->cross[1] * szk) * sx[i];
  const float s = o == 0u ? 0.0f : p->invN * __frcp_rn(A);
  v.x *= s;
  v.y *= s;
  return v;
}

// The same callback with C++ linkage, for cuFFT builds that look the symbol
// up by its mangled name.
__device__ cufftComplex baorec_spectral_load2(void* dataIn, unsigned long long offset, void* callerInfo,
                                              void* sharedPointer) {
  return baorec_spectral_load(dataIn, offset, callerInfo, sharedPointer);
}
