// Device helpers shared by the pass and decode kernels.
#pragma once

#include "puck_internal.h"

#include <math_constants.h>

namespace puck {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ long long tri(int n) { return (long long)n * (n + 1) / 2; }

// ChartHalf.chartIndex (src/main/scala/puck/parser/ParseChart.scala:58-65):
// span-major triangular index of the cell (min(b,e), max(b,e)).
__device__ __forceinline__ int chart_index(int b, int e, int n) {
  int sp = abs(e - b) - 1;
  return min(b, e) + sp * n - sp * (sp - 1) / 2;
}

// Entry k of a work list holding unit i (pref[k] <= i < pref[k+1]).
__device__ __forceinline__ int entry_of(const DevWork& W, int i) {
  int lo = 0, hi = W.nent;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (W.pref[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int span_of(const DevWork& W, int k) { return W.span ? W.span[k] : W.span_all; }
__device__ __forceinline__ int ways_of(const DevWork& W, int k) { return W.ways ? W.ways[k] : W.ways_all; }

// Semirings (src/main/scala/puck/parser/RuleSemiring.scala:22-98).
template <int S> struct Sr;
template <> struct Sr<SEMI_VITERBI> {
  static __device__ __forceinline__ float zero() { return -CUDART_INF_F; }
  static __device__ __forceinline__ float one() { return 0.f; }
  static __device__ __forceinline__ float add(float x, float y) { return fmaxf(x, y); }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return fmaxf(acc, child + w); }
  static __device__ __forceinline__ bool live(float v) { return v != -CUDART_INF_F; }
};
template <> struct Sr<SEMI_REAL> {
  static __device__ __forceinline__ float zero() { return 0.f; }
  static __device__ __forceinline__ float one() { return 1.f; }
  static __device__ __forceinline__ float add(float x, float y) { return x + y; }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return fmaf(child, w, acc); }
  static __device__ __forceinline__ bool live(float v) { return v != 0.f; }
};
template <> struct Sr<SEMI_LOGSUM> {
  static __device__ __forceinline__ float zero() { return -1000000.0f; }
  static __device__ __forceinline__ float one() { return 0.f; }
  static __device__ __forceinline__ float add(float x, float y) {
    float lo = fminf(x, y), hi = fmaxf(x, y);
    return hi + log1pf(expf(lo - hi));
  }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return add(acc, child + w); }
  static __device__ __forceinline__ bool live(float) { return true; }  // no exact zero: never skipped
};

template <int S> __device__ __forceinline__ float warp_reduce(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = Sr<S>::add(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ bool mask_any(const DevMask& M, long long c) {
  if (!M.bits) return true;
  const int* m = M.bits + c * M.mask_size;
  for (int i = 0; i < M.mask_size; ++i)
    if (m[i]) return true;
  return false;
}

__device__ __forceinline__ float scale_of(const float* sc, long long c) { return sc ? sc[c] : 0.f; }

}  // namespace dev
}  // namespace puck
