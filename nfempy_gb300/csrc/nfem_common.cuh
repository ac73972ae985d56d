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

// exclusive scan of int32 counts into int64 offsets (n + 1 entries)
size_t scan_workspace_bytes(int64_t n);
int exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* ws,
                       size_t ws_bytes, cudaStream_t stream);

}  // namespace nfem
