// Shared device helpers and host-side bookkeeping for libgbsv.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbsv.h"

namespace gbsv {

// ---------------------------------------------------------------- types --
template <typename R> struct CxT;
template <> struct CxT<float> { using T = float2; };
template <> struct CxT<double> { using T = double2; };
template <typename R> using Cx = typename CxT<R>::T;

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// acc + a * b
template <typename C>
__device__ __forceinline__ C cmad(C a, C b, C acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}

template <typename C>
__device__ __forceinline__ C czero() {
  C r;
  r.x = 0;
  r.y = 0;
  return r;
}

// Streaming (evict-first) loads and stores.  Coherent, so in-place updates
// (each thread reads then writes its own amplitudes) are safe.
__device__ __forceinline__ float2 ld_cs(const float2* p) { return __ldcs(p); }
__device__ __forceinline__ double2 ld_cs(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ void st_cs(float2* p, float2 v) { __stcs(p, v); }
__device__ __forceinline__ void st_cs(double2* p, double2 v) { __stcs(p, v); }

// Load / store a chunk of V consecutive amplitudes with 16-byte vectors.
template <int V>
__device__ __forceinline__ void load_chunk(const float2* p, float2* r) {
  if constexpr (V == 1) {
    r[0] = __ldcs(p);
  } else {
#pragma unroll
    for (int j = 0; j < V / 2; ++j) {
      float4 v = __ldcs(reinterpret_cast<const float4*>(p) + j);
      r[2 * j] = make_float2(v.x, v.y);
      r[2 * j + 1] = make_float2(v.z, v.w);
    }
  }
}
template <int V>
__device__ __forceinline__ void store_chunk(float2* p, const float2* r) {
  if constexpr (V == 1) {
    __stcs(p, r[0]);
  } else {
#pragma unroll
    for (int j = 0; j < V / 2; ++j) {
      __stcs(reinterpret_cast<float4*>(p) + j,
             make_float4(r[2 * j].x, r[2 * j].y, r[2 * j + 1].x,
                         r[2 * j + 1].y));
    }
  }
}
template <int V>
__device__ __forceinline__ void load_chunk(const double2* p, double2* r) {
#pragma unroll
  for (int j = 0; j < V; ++j) r[j] = __ldcs(p + j);
}
template <int V>
__device__ __forceinline__ void store_chunk(double2* p, const double2* r) {
#pragma unroll
  for (int j = 0; j < V; ++j) __stcs(p + j, r[j]);
}

// Per-thread accumulator for reductions.  GB300 issues FP64 at a small
// fraction of its FP32 rate, so complex64 data is accumulated per thread as
// an unevaluated float pair (hi, lo): each product a*b enters exactly
// (p = a*b, its rounding error e = fma(a, b, -p)) and each addition keeps
// its rounding error (TwoSum, Knuth), so the per-thread result carries
// about twice float precision (near FP64) using only FP32 operations.  Only
// the per-thread results meet in FP64.  complex128 data uses FP64.
template <typename R> struct Acc;
template <> struct Acc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
  }
  // += a * b exactly
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    lo += fmaf(a, b, -p);
    add(p);
  }
  __device__ __forceinline__ double value() const {
    return (double)hi + (double)lo;
  }
};
template <> struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void add_prod(double a, double b) {
    s = fma(a, b, s);
  }
  __device__ __forceinline__ double value() const { return s; }
};

// Insert a zero bit at position pos of x (bits >= pos move up by one).
__device__ __forceinline__ uint64_t insert_zero(uint64_t x, int pos) {
  uint64_t lo = x & ((uint64_t(1) << pos) - 1);
  return ((x >> pos) << (pos + 1)) | lo;
}

// Gate record of the fused stages (layout identical to gbsv_fused_gate_t).
struct FusedGate {
  int32_t kind;
  int32_t nq;          // diagonal: number of qubits (1 or 2)
  int32_t b0, b1;      // tile / register bit, or -1 - position outside
  uint64_t cmask;      // apply only where (tile base & cmask) == cval
  uint64_t cval;
  int64_t mat;         // complex-element offset into the matrix pool
  int64_t mat_bstride; // per-state stride in the pool (0 = shared)
};

// 16-byte asynchronous global -> shared copy (cp.async, L2 only).
template <typename R>
__device__ __forceinline__ void cp_async16(Cx<R>* smem, const Cx<R>* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s),
               "l"(gmem)
               : "memory");
}

// 8-byte asynchronous global -> shared copy (cp.async.ca, through L1).
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s),
               "l"(gmem)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// --------------------------------------------------------------- host ----
// Records a launch and converts a pending CUDA error into a status.
int after_launch(const char* what);
int set_error(int status, const char* fmt, ...);
// GBSV_C128_PAIRS or GBSV_C128_FP64 (gbsv_set_c128_arith)
int c128_arith();
inline int dtype_bytes(int dtype) {
  switch (dtype) {
    case GBSV_C64: return 8;
    case GBSV_C128: return 16;
    case GBSV_F32: return 4;
    case GBSV_F64: return 8;
    default: return 0;
  }
}
inline int sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached = v > 0 ? v : 148;
  }
  return cached;
}

}  // namespace gbsv
