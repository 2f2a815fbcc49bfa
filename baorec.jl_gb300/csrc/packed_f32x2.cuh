// Packed FP32x2 arithmetic (add / sub / mul / fma .rn.f32x2): two
// independent IEEE round-to-nearest FP32 operations per instruction, each
// lane rounded exactly as the scalar operation.
#pragma once

namespace baorec {

typedef unsigned long long f2;
__device__ __forceinline__ f2 P2(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void U2(f2 r, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ f2 B2(float a) { return P2(a, a); }
#define BAOREC_F2OP(name, op)                                                 \
  __device__ __forceinline__ f2 name(f2 a, f2 b) {                            \
    f2 d;                                                                     \
    asm(op ".rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));               \
    return d;                                                                 \
  }
BAOREC_F2OP(add2, "add")
BAOREC_F2OP(sub2, "sub")
BAOREC_F2OP(mul2, "mul")
#undef BAOREC_F2OP
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

}  // namespace baorec
