// Shared device helpers for the oqupy_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace otb {

// aligned to its size so that an element is one vector load / store
template <typename T>
struct __align__(2 * sizeof(T)) cx {
  T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}

template <typename T>
__device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) {
  return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) {
  return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <typename T>
__device__ __forceinline__ cx<T> cjmul(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
// acc += a * b
template <typename T>
__device__ __forceinline__ void cfma(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename T>
__device__ __forceinline__ void cjfma(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
template <typename T>
__device__ __forceinline__ cx<T> cscale(cx<T> a, T s) {
  return mk<T>(a.x * s, a.y * s);
}
template <typename T>
__device__ __forceinline__ cx<T> cconj(cx<T> a) {
  return mk<T>(a.x, -a.y);
}
template <typename To, typename From>
__device__ __forceinline__ cx<To> ccast(cx<From> a) {
  return mk<To>((To)a.x, (To)a.y);
}

template <typename T>
struct num;
template <>
struct num<double> {
  static __device__ __forceinline__ double eps() { return 1.1102230246251565e-16; }
  static __device__ __forceinline__ double big_zeta() { return 1.0e150; }
};
template <>
struct num<float> {
  static __device__ __forceinline__ float eps() { return 5.9604645e-08f; }
  static __device__ __forceinline__ float big_zeta() { return 1.0e18f; }
};

// Status codes shared with the host (mirrored in include/oqupy_gb300.h).
enum : int {
  ST_OK = 0,
  ST_NO_CONVERGENCE = -4,
  ST_CHI_OVERFLOW = -7,
  ST_NONFINITE = -6,
};

}  // namespace otb
