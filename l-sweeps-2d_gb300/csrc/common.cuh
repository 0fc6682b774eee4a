// Shared device/host helpers for the GB300 L-sweeps library: complex arithmetic
// on float2/double2, precision traits and error plumbing.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace lsw {

template <typename T> struct Cx;
template <> struct Cx<float>  { using type = float2; };
template <> struct Cx<double> { using type = double2; };
template <typename T> using cx_t = typename Cx<T>::type;

template <typename C> __host__ __device__ __forceinline__ C cmake(double re, double im) {
  C r; r.x = (decltype(r.x))re; r.y = (decltype(r.y))im; return r;
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc += a*b
__host__ __device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x); acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y); acc.y = fmaf(a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc -= a*b
__host__ __device__ __forceinline__ void cfms(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(-a.x, b.x, acc.x); acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(-a.x, b.y, acc.y); acc.y = fmaf(-a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ void cfms(double2& acc, double2 a, double2 b) {
  acc.x = fma(-a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ float abs2(float2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// 1/a computed as conj(a)/|a|^2
__host__ __device__ __forceinline__ float2 crcp(float2 a) {
  float d = 1.0f / abs2(a); return make_float2(a.x * d, -a.y * d);
}
__host__ __device__ __forceinline__ double2 crcp(double2 a) {
  double d = 1.0 / abs2(a); return make_double2(a.x * d, -a.y * d);
}
__host__ __device__ __forceinline__ float2 to_c(float2 a, float2) { return a; }
__host__ __device__ __forceinline__ double2 to_c(double2 a, double2) { return a; }
__host__ __device__ __forceinline__ float2 to_c(double2 a, float2) { return make_float2((float)a.x, (float)a.y); }
__host__ __device__ __forceinline__ double2 to_c(float2 a, double2) { return make_double2(a.x, a.y); }

template <typename C> __host__ __device__ __forceinline__ C czero() { C r; r.x = 0; r.y = 0; return r; }

}  // namespace lsw
