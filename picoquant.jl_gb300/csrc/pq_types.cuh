// Element types and arithmetic helpers shared by the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include "pq_internal.h"

namespace pq {

template <int DT>
struct ElemOf;
template <>
struct ElemOf<PQ_C64> {
  using T = float2;
};
template <>
struct ElemOf<PQ_C128> {
  using T = double2;
};

template <typename A>
struct Acc;
template <>
struct Acc<float> {
  using C = float2;
};
template <>
struct Acc<double> {
  using C = double2;
};

__device__ __forceinline__ float2 czero(float) { return make_float2(0.f, 0.f); }
__device__ __forceinline__ double2 czero(double) { return make_double2(0.0, 0.0); }

template <typename R>
__device__ __forceinline__ typename Acc<R>::C cvt(float2 v);
template <>
__device__ __forceinline__ float2 cvt<float>(float2 v) {
  return v;
}
template <>
__device__ __forceinline__ double2 cvt<double>(float2 v) {
  return make_double2(v.x, v.y);
}
template <typename R>
__device__ __forceinline__ typename Acc<R>::C cvt(double2 v);
template <>
__device__ __forceinline__ float2 cvt<float>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}
template <>
__device__ __forceinline__ double2 cvt<double>(double2 v) {
  return v;
}

template <typename T>
__device__ __forceinline__ T store_as(float2 v);
template <>
__device__ __forceinline__ float2 store_as<float2>(float2 v) {
  return v;
}
template <>
__device__ __forceinline__ double2 store_as<double2>(float2 v) {
  return make_double2(v.x, v.y);
}
template <typename T>
__device__ __forceinline__ T store_as(double2 v);
template <>
__device__ __forceinline__ float2 store_as<float2>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}
template <>
__device__ __forceinline__ double2 store_as<double2>(double2 v) {
  return v;
}

__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

// Kahan-compensated complex accumulator: partial sums of short K chunks are
// accumulated in FP32 and folded into (s, c) here, so the accumulation error
// grows with the chunk length rather than with K.
struct KahanC {
  float2 s, c;
};
__device__ __forceinline__ void kahan_init(KahanC& k) {
  k.s = make_float2(0.f, 0.f);
  k.c = make_float2(0.f, 0.f);
}
__device__ __forceinline__ void kahan_add1(float& s, float& c, float x) {
  float y = x - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}
__device__ __forceinline__ void kahan_add(KahanC& k, float2 x) {
  kahan_add1(k.s.x, k.c.x, x.x);
  kahan_add1(k.s.y, k.c.y, x.y);
}
__device__ __forceinline__ float2 kahan_value(const KahanC& k) { return make_float2(k.s.x - k.c.x, k.s.y - k.c.y); }

// Number of K terms accumulated in plain FP32 before a compensated fold.
constexpr int kChunk = 16;

inline int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = 152 * 8;  // 8 resident 256-thread blocks per SM
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace pq
