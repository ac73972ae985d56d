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

// Current value of a launch knob (nfem_knob_set; 0 = built-in choice).
int knob(int key);

// Device-side status word: the first nonzero code written wins.
__device__ __forceinline__ void set_status(int32_t* status, int32_t code) {
  if (status) atomicCAS(status, 0, code);
}

// A coefficient that must be finite: NaN or +-Inf sets NFEM_ERR_NONFINITE.
template <typename T>
__device__ __forceinline__ void check_finite(int32_t* status, T v) {
  if (!isfinite(v)) set_status(status, NFEM_ERR_NONFINITE);
}
// A coefficient that must be finite and positive (a permeability, a shear
// modulus): NaN / Inf -> NFEM_ERR_NONFINITE, v <= 0 -> NFEM_ERR_DOMAIN.
template <typename T>
__device__ __forceinline__ void check_positive(int32_t* status, T v) {
  if (!(v > T(0)) || !isfinite(v)) set_status(status, isfinite(v) ? NFEM_ERR_DOMAIN : NFEM_ERR_NONFINITE);
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

// Packed point records written by nfem_points_split: record 0 holds
// (scale, cx, cy, cz) as floats; record v + 1 holds point v as three 32-bit
// fixed-point integers q = round((x - c) / scale) (and a zero), with c the
// bounding-box centre rounded to float and scale = 2^(e - 30) for a
// half-extent below 2^e, so |q| < 2^30 and differences of two q fit in 32
// bits.  An edge component is float(q1 - q0) * scale: one 16-byte load per
// point, an exact integer difference, no FP64 arithmetic; absolute error at
// most scale, i.e. a relative edge error below 1e-9 x (cells across the mesh).
__device__ __forceinline__ float4 packed_point(const float* split, int32_t v) {
  return __ldg(reinterpret_cast<const float4*>(split) + 1 + v);
}
__device__ __forceinline__ float packed_lo_scale(const float* split) { return __ldg(split); }
// edge component d of x1 - x0 from two packed records
__device__ __forceinline__ float packed_diff(const float4& r1, const float4& r0, int d, float scale) {
  const float a = d == 0 ? r1.x : (d == 1 ? r1.y : r1.z);
  const float b = d == 0 ? r0.x : (d == 1 ? r0.y : r0.z);
  return float(__float_as_int(a) - __float_as_int(b)) * scale;
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
