// pn_f32x2.cuh -- two FP32 lanes per instruction (sm_100 and later: add/sub/mul/fma .f32x2).
//
// The FP32 tile kernels update two x-neighbouring points per thread.  Every operation below is
// the IEEE round-to-nearest FP32 operation applied to each lane separately, so a lane's result is
// bit for bit the one the scalar code gives; only the instruction count halves.
#pragma once

#include <cuda_runtime.h>

namespace pn {

// the two-lane fma below must not hide the scalar ones inside this namespace
using ::fma;

struct __align__(8) f2 {
  float x, y;
};

__device__ __forceinline__ f2 splat(float v) { return f2{v, v}; }

__device__ __forceinline__ unsigned long long pk(f2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}

__device__ __forceinline__ f2 upk(unsigned long long r) {
  f2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}

__device__ __forceinline__ f2 fma(f2 a, f2 b, f2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)), "l"(pk(c)));
  return upk(d);
}

__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
  return upk(d);
}

__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
  return upk(d);
}

__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
  return upk(d);
}

// exact negation (the sign of zero included): a product with -1
__device__ __forceinline__ f2 neg(f2 a) { return a * splat(-1.0f); }

__device__ __forceinline__ f2 ld2(const float* p) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  return f2{v.x, v.y};
}

__device__ __forceinline__ void st2(float* p, f2 v) { *reinterpret_cast<float2*>(p) = make_float2(v.x, v.y); }

}  // namespace pn
