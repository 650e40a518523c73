// pn_f32x2.cuh -- two FP32 lanes per instruction (sm_100 and later: add/sub/mul/fma .f32x2).
//
// The FP32 tile kernels can update two x-neighbouring points per thread (PN_TMA_PPT = 2).  Every
// operation below is the IEEE round-to-nearest FP32 operation applied to each lane separately, so
// a lane's result is bit for bit the one the scalar code gives; only the instruction count halves.
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

// The lanes of one thread of a tile kernel: one point (float) or two x-neighbouring points (f2).
// Code written against Lanes<P> is the same arithmetic for either, lane by lane.
template <int P>
struct Lanes;

template <>
struct Lanes<1> {
  using V = float;
  static __device__ __forceinline__ V splat(float v) { return v; }
  static __device__ __forceinline__ V ld(const float* p) { return *p; }
  // global memory another CTA of the same launch may have written: cached at L2 only
  static __device__ __forceinline__ V ldcg(const float* p) { return __ldcg(p); }
  static __device__ __forceinline__ void st(float* p, V v) { *p = v; }
  static __device__ __forceinline__ float get(V v, int) { return v; }
  static __device__ __forceinline__ void set(V& v, int, float x) { v = x; }
  static __device__ __forceinline__ V neg(V v) { return -v; }
  static __device__ __forceinline__ V rcp(V v) { return 1.0f / v; }
  // right (a) and left (b) x neighbours of the thread's point: a at r, b at l = r - 1
  static __device__ __forceinline__ void xpair(const float* p, int r, int l, bool, V& a, V& b) {
    a = p[r];
    b = p[l];
  }
};

template <>
struct Lanes<2> {
  using V = f2;
  static __device__ __forceinline__ V splat(float v) { return pn::splat(v); }
  static __device__ __forceinline__ V ld(const float* p) { return ld2(p); }
  static __device__ __forceinline__ V ldcg(const float* p) {
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return f2{v.x, v.y};
  }
  static __device__ __forceinline__ void st(float* p, V v) { st2(p, v); }
  static __device__ __forceinline__ float get(V v, int k) { return k ? v.y : v.x; }
  static __device__ __forceinline__ void set(V& v, int k, float x) {
    if (k) v.y = x;
    else v.x = x;
  }
  static __device__ __forceinline__ V neg(V v) { return pn::neg(v); }
  static __device__ __forceinline__ V rcp(V v) { return f2{1.0f / v.x, 1.0f / v.y}; }
  // the pair reads three consecutive values: the right value of the first point is the left value
  // of the second.  `r_even`: r is even (then the pair (r, r + 1) is aligned), else l is.
  static __device__ __forceinline__ void xpair(const float* p, int r, int l, bool r_even, V& a, V& b) {
    if (r_even) {
      a = ld2(p + r);
      b = f2{p[l], a.x};
    } else {
      b = ld2(p + l);
      a = f2{b.y, p[r + 1]};
    }
  }
};

}  // namespace pn
