// Shared device/host helpers of the GB300 boost-factor library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

namespace bf {

// ---- complex arithmetic on float2 / double2 -------------------------------
template <typename R> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename R> using cplx_t = typename cplx_of<R>::type;

__host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename C>
__host__ __device__ __forceinline__ C cadd(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
template <typename C>
__host__ __device__ __forceinline__ C csub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
template <typename C>
__host__ __device__ __forceinline__ C cmul(C a, C b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C>
__host__ __device__ __forceinline__ C cmulc(C a, C b) {
  return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C, typename R>
__host__ __device__ __forceinline__ C cscale(C a, R s) { return mk(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C>
__host__ __device__ __forceinline__ C cmul_mi(C a) {
  return INV ? mk(-a.y, a.x) : mk(a.y, -a.x);
}
template <typename C>
__host__ __device__ __forceinline__ C cconj(C a) { return mk(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 czero_of(float2) { return make_float2(0.0f, 0.0f); }
__host__ __device__ __forceinline__ double2 czero_of(double2) { return make_double2(0.0, 0.0); }

__device__ __forceinline__ float2 to_c(double2 v, float2) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ double2 to_c(double2 v, double2) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

// ---- host error plumbing ---------------------------------------------------
struct Status {
  int code = 0;
  std::string msg;
};

}  // namespace bf
