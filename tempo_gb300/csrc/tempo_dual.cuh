// tempo_dual.cuh -- forward-mode dual numbers for the tangent-linear and adjoint
// kernels of the column step.
//
// Dual<T, N> carries a value v and N directional derivatives d[0..N-1].  The physics
// templates of tempo_level.cuh / tempo_rates.cuh instantiated with R = Dual<T, N>
// compute, for a point, its outputs and their derivatives along N input directions in
// one pass.  Every branch, clip and table index is decided on the value v alone, so the
// derivatives are those of the forward trajectory with its branches and table bins held
// fixed; where the value arithmetic is T, the value part reproduces the forward kernel
// bit for bit (the FP64 path is compiled without FMA contraction).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#if defined(__CUDACC__)
#define TG_UNROLL _Pragma("unroll")
#else
#define TG_UNROLL
#endif

namespace tg {

template <class T, int N>
struct Dual {
  T v;
  T d[N];
  Dual() = default;
  __host__ __device__ Dual(T x) : v(x) {
TG_UNROLL
    for (int i = 0; i < N; i++) d[i] = T(0);
  }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value &&
                                                     !std::is_same<U, T>::value>::type>
  __host__ __device__ Dual(U x) : Dual(T(x)) {}
  __host__ __device__ explicit operator T() const { return v; }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value &&
                                                     !std::is_same<U, T>::value>::type>
  __host__ __device__ explicit operator U() const { return U(v); }
};

template <class X> struct IsDual : std::false_type {};
template <class T, int N> struct IsDual<Dual<T, N>> : std::true_type {};

#define TG_DUAL_T template <class T, int N>
#define TG_D Dual<T, N>

// arithmetic (value in T exactly as the plain kernel computes it)
TG_DUAL_T __host__ __device__ __forceinline__ TG_D operator-(const TG_D& a) {
  TG_D r;
  r.v = -a.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
  return r;
}
TG_DUAL_T __host__ __device__ __forceinline__ TG_D operator+(const TG_D& a, const TG_D& b) {
  TG_D r;
  r.v = a.v + b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
  return r;
}
TG_DUAL_T __host__ __device__ __forceinline__ TG_D operator-(const TG_D& a, const TG_D& b) {
  TG_D r;
  r.v = a.v - b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i];
  return r;
}
TG_DUAL_T __host__ __device__ __forceinline__ TG_D operator*(const TG_D& a, const TG_D& b) {
  TG_D r;
  r.v = a.v * b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
TG_DUAL_T __host__ __device__ __forceinline__ TG_D operator/(const TG_D& a, const TG_D& b) {
  TG_D r;
  r.v = a.v / b.v;
  const T ib = T(1) / b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
// mixed operands: the plain operand is a constant of the forward trajectory
#define TG_DUAL_ARITH template <class T, int N, class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator+(const TG_D& a, U b) {
  TG_D r = a;
  r.v = a.v + T(b);
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator+(U a, const TG_D& b) {
  TG_D r = b;
  r.v = T(a) + b.v;
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator-(const TG_D& a, U b) {
  TG_D r = a;
  r.v = a.v - T(b);
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator-(U a, const TG_D& b) {
  TG_D r = -b;
  r.v = T(a) - b.v;
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator*(const TG_D& a, U b) {
  TG_D r;
  r.v = a.v * T(b);
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * T(b);
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator*(U a, const TG_D& b) {
  TG_D r;
  r.v = T(a) * b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = T(a) * b.d[i];
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator/(const TG_D& a, U b) {
  TG_D r;
  r.v = a.v / T(b);
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] / T(b);
  return r;
}
TG_DUAL_ARITH __host__ __device__ __forceinline__ TG_D operator/(U a, const TG_D& b) {
  TG_D r;
  r.v = T(a) / b.v;
  const T g = -r.v / b.v;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = g * b.d[i];
  return r;
}

TG_DUAL_T __host__ __device__ __forceinline__ TG_D& operator+=(TG_D& a, const TG_D& b) { return a = a + b; }
TG_DUAL_T __host__ __device__ __forceinline__ TG_D& operator-=(TG_D& a, const TG_D& b) { return a = a - b; }
TG_DUAL_T __host__ __device__ __forceinline__ TG_D& operator*=(TG_D& a, const TG_D& b) { return a = a * b; }

// comparisons on values
#define TG_DUAL_CMP(op)                                                                       \
  TG_DUAL_T __host__ __device__ __forceinline__ bool operator op(const TG_D& a, const TG_D& b) { \
    return a.v op b.v;                                                                        \
  }                                                                                           \
  template <class T, int N, class U,                                                          \
            class = typename std::enable_if<std::is_arithmetic<U>::value>::type>              \
  __host__ __device__ __forceinline__ bool operator op(const TG_D& a, U b) {                  \
    return a.v op T(b);                                                                       \
  }                                                                                           \
  template <class T, int N, class U,                                                          \
            class = typename std::enable_if<std::is_arithmetic<U>::value>::type>              \
  __host__ __device__ __forceinline__ bool operator op(U a, const TG_D& b) {                  \
    return T(a) op b.v;                                                                       \
  }
TG_DUAL_CMP(<)
TG_DUAL_CMP(>)
TG_DUAL_CMP(<=)
TG_DUAL_CMP(>=)
TG_DUAL_CMP(==)
TG_DUAL_CMP(!=)
#undef TG_DUAL_CMP

// y = f(a) with f'(a) given: chain rule on every direction
TG_DUAL_T __host__ __device__ __forceinline__ TG_D dual_chain(const TG_D& a, T fv, T dfda) {
  TG_D r;
  r.v = fv;
TG_UNROLL
  for (int i = 0; i < N; i++) r.d[i] = dfda * a.d[i];
  return r;
}

}  // namespace tg
