// tlr_complex.cuh -- complex arithmetic on double2 / float2.
#pragma once

#include <cuda_runtime.h>

namespace tlr {

template <class C> struct Real;
template <> struct Real<double2> { using T = double; };
template <> struct Real<float2> { using T = float; };

__host__ __device__ __forceinline__ double2 mkc(double a, double b, double2 *) {
  return make_double2(a, b);
}
__host__ __device__ __forceinline__ float2 mkc(float a, float b, float2 *) {
  return make_float2(a, b);
}
template <class C>
__host__ __device__ __forceinline__ C cmake(typename Real<C>::T a,
                                            typename Real<C>::T b) {
  return mkc(a, b, (C *)nullptr);
}
template <class C>
__host__ __device__ __forceinline__ C czero() {
  return cmake<C>(0, 0);
}
template <class C>
__device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <class C>
__device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc - a*b
template <class C>
__device__ __forceinline__ C cfms(C acc, C a, C b) {
  acc.x = fma(-a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
// acc + a*b
template <class C>
__device__ __forceinline__ C cfma(C acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
template <class C>
__device__ __forceinline__ typename Real<C>::T cabs1(C a) {
  return fabs(a.x) + fabs(a.y);
}
// 1 / a with scaling (Smith's method) to avoid overflow.
template <class C>
__device__ __forceinline__ C cinv(C a) {
  using T = typename Real<C>::T;
  if (fabs(a.x) >= fabs(a.y)) {
    const T r = a.y / a.x, d = a.x + a.y * r;
    return cmake<C>(T(1) / d, -r / d);
  }
  const T r = a.x / a.y, d = a.y + a.x * r;
  return cmake<C>(r / d, T(-1) / d);
}
__device__ __forceinline__ double2 to_c(double2 v, double2 *) { return v; }
__device__ __forceinline__ float2 to_c(double2 v, float2 *) {
  return make_float2((float)v.x, (float)v.y);
}
template <class C>
__device__ __forceinline__ C from64(double2 v) { return to_c(v, (C *)nullptr); }
__device__ __forceinline__ double2 to64(double2 v) { return v; }
__device__ __forceinline__ double2 to64(float2 v) { return make_double2(v.x, v.y); }

}  // namespace tlr
