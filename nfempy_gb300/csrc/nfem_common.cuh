// Shared definitions for the nfempy GB300 kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nfem_gb300.h"

#define NFEM_TRY_CUDA(expr)                         \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return NFEM_ERR_CUDA;    \
  } while (0)

#define NFEM_CHECK_LAUNCH()                                   \
  do {                                                        \
    cudaError_t _e = cudaGetLastError();                      \
    if (_e != cudaSuccess) return NFEM_ERR_CUDA;              \
  } while (0)

namespace nfem {

constexpr int kWarp = 32;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Grid size for a grid-stride loop: a multiple of the SM count (152 on GB300)
// times the resident blocks per SM, capped by the work.
int grid_for(int64_t n_items, int block, int blocks_per_sm = 8);

// Device-side status word: the first nonzero code written wins.
__device__ __forceinline__ void set_status(int32_t* status, int32_t code) {
  if (status) atomicCAS(status, 0, code);
}

// Align a byte offset up to 256 bytes (workspace carving).
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Carver {
  char* base;
  size_t off;
  size_t cap;
  template <typename T>
  T* take(size_t count) {
    size_t o = align256(off);
    off = o + count * sizeof(T);
    return reinterpret_cast<T*>(base + o);
  }
  bool ok() const { return off <= cap; }
};

// Packed FP32 point records written by nfem_points_split: record 0 holds
// (lo_scale, cx, cy, cz); record v + 1 holds (hx, hy, hz, q) for point v,
// where hi + lo = point - c (c = the bounding-box centre rounded to float),
// h = float(point - c) and q packs three signed 10-bit integers
// (bits 0-9, 10-19, 20-29) with lo_d ~= q_d * lo_scale.  An edge component
// is then (h1 - h0) + float(q1 - q0) * lo_scale: one 16-byte load per point,
// no FP64 arithmetic, and an absolute error of lo_scale (about 2^-33 times
// the half-extent of the mesh).
__device__ __forceinline__ float4 packed_point(const float* split, int32_t v) {
  return __ldg(reinterpret_cast<const float4*>(split) + 1 + v);
}
__device__ __forceinline__ float packed_lo_scale(const float* split) { return __ldg(split); }
__device__ __forceinline__ int packed_q(float w, int d) {
  return int(__float_as_uint(w) << (22 - 10 * d)) >> 22;
}
// edge component d of x1 - x0 from two packed records
__device__ __forceinline__ float packed_diff(const float4& r1, const float4& r0, int d, float lo_scale) {
  const float h1 = d == 0 ? r1.x : (d == 1 ? r1.y : r1.z);
  const float h0 = d == 0 ? r0.x : (d == 1 ? r0.y : r0.z);
  return (h1 - h0) + float(packed_q(r1.w, d) - packed_q(r0.w, d)) * lo_scale;
}

// 4-wide slot of a node column in a row image of the node-row kernels:
// (component j = 0, 1, 2, pad), read and written as 16-byte vectors
template <typename T>
struct Slot4;
template <>
struct Slot4<float> {
  float4 v;
  __device__ __forceinline__ void load(const float* a) { v = *reinterpret_cast<const float4*>(a); }
  __device__ __forceinline__ void store(float* a) const { *reinterpret_cast<float4*>(a) = v; }
  __device__ __forceinline__ float& operator[](int j) { return j == 0 ? v.x : (j == 1 ? v.y : v.z); }
  __device__ __forceinline__ void zero() { v = make_float4(0.f, 0.f, 0.f, 0.f); }
};
template <>
struct Slot4<double> {
  double2 lo, hi;
  __device__ __forceinline__ void load(const double* a) {
    lo = reinterpret_cast<const double2*>(a)[0];
    hi = reinterpret_cast<const double2*>(a)[1];
  }
  __device__ __forceinline__ void store(double* a) const {
    reinterpret_cast<double2*>(a)[0] = lo;
    reinterpret_cast<double2*>(a)[1] = hi;
  }
  __device__ __forceinline__ double& operator[](int j) { return j == 0 ? lo.x : (j == 1 ? lo.y : hi.x); }
  __device__ __forceinline__ void zero() {
    lo = make_double2(0.0, 0.0);
    hi = lo;
  }
};

// exclusive scan of int32 counts into int64 offsets (n + 1 entries)
size_t scan_workspace_bytes(int64_t n);
int exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* ws,
                       size_t ws_bytes, cudaStream_t stream);

}  // namespace nfem
