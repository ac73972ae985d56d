// K5 + K7: device-resident Krylov solve with FP64 iterative refinement.
//
// Reference: the drivers hand the assembled PETSc matrix to a KSP
// (examples/md_elliptic_scalar/md_elliptic_scalar.py:343-363 MUMPS LU;
// examples/cauchy_elasticity/cg_elasticity_example_1.py:159-170 ICC-CG;
// examples/cosserat_elasticity/mfe_cosserat_elasticity_example_3.py:256-297
// MINRES + fieldsplit) and solve A x = b with b = -r(0).
//
// GPU design:
//  * CSR SpMV in FP32 (inner) and FP64 (outer residual r = b - A x), warp
//    chunks of 32 rows whose contiguous CSR segment is streamed with
//    coalesced loads into shared memory, then reduced per row.
//  * Deterministic reductions: a fixed grid of blocks writes partial sums
//    and the last block to finish adds them in a fixed order (bitwise
//    reproducible dots and norms, no separate reduction launch).
//  * Preconditioners: point Jacobi; cell-patch block Jacobi (weighted
//    additive Schwarz over the element cliques: z = sum_c R_c^T D_c A_c^-1 R_c v
//    with D_c = 1 / multiplicity), applied row-owner or, stored in A's CSR
//    pattern, as one SpMV; and a two-level Galerkin cycle (damped smoother
//    before and after a coarse correction with a dense or block-diagonal
//    stored inverse, A P kept to update residuals without an SpMV).
//  * Flexible GMRES(m) with classical Gram-Schmidt and one
//    re-orthogonalisation, the second pass and the norm fused with the
//    updates; the Hessenberg matrix, Givens rotations and residual
//    estimates live on the device, so a restart cycle synchronises with the
//    host once, and cycles after the first are replayed as a CUDA graph.
//  * Mixed precision: inner FGMRES in FP32 on the FP32 matrix, outer
//    refinement with the FP64 residual of the FP64 matrix until
//    ||b - A x|| / ||b|| <= rtol (the stopping test is always FP64).
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include <type_traits>

#include "nfem_common.cuh"
#include "tc_common.cuh"

#define NFEM_RC(...)                \
  do {                              \
    int _rc = (__VA_ARGS__);        \
    if (_rc != NFEM_OK) return _rc; \
  } while (0)

extern "C" int nfem_mlp_forward(const int32_t* dims, int weight_type, const void* params, const float* params_f32,
                                int64_t batch, const float* x, float* h1, float* h2, float* y, void* stream);

namespace nfem {

constexpr int kRedBlocks = 1216;  // 8 x 152 SMs; the widest reduction grid (partial buffers)
constexpr int kRedThreads = 256;
constexpr int kSpmvWarps = 8;
constexpr int kSpmvCap = 32 * 16;
#ifndef NFEM_SPMV_UNROLL
#define NFEM_SPMV_UNROLL 4
#endif
constexpr int kSpmvUnroll = NFEM_SPMV_UNROLL;
constexpr int kMaxRestart = 128;

// type of the coarse inverse's trailing updates (FP64 diagonal blocks)
#ifndef NFEM_COARSE_T
#define NFEM_COARSE_T float
#endif

// Gate of a restart cycle (a device word written by an earlier kernel of the
// same stream): a kernel given the gate returns at once while it is nonzero.
// givens_update sets it when the cycle reaches its inner tolerance, so the
// cycle's remaining steps cost only their launches.
#define NFEM_GATE(g) \
  if ((g) != nullptr && *static_cast<const volatile int32_t*>(g) != 0) return

// ------------------------------------------------------------------ SpMV
template <typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(32 * kSpmvWarps)
    spmv_kernel(int64_t n_rows, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                const VT* __restrict__ val, const XT* __restrict__ x, XT* __restrict__ y,
                const XT* __restrict__ b, int residual, const float* __restrict__ yscale,
                const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ AT stage[kSpmvWarps][kSpmvCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  AT* st = stage[warp];
  for (int64_t r0 = (int64_t(blockIdx.x) * kSpmvWarps + warp) * 32; r0 < n_rows;
       r0 += int64_t(gridDim.x) * kSpmvWarps * 32) {
    const int64_t r = r0 + lane;
    const bool valid = r < n_rows;
    const int32_t rb = valid ? __ldg(row_ptr + r) : 0;
    const int32_t re = valid ? __ldg(row_ptr + r + 1) : 0;
    const int last = int(min(int64_t(31), n_rows - 1 - r0));
    const int32_t base = __shfl_sync(0xffffffffu, rb, 0);
    const int32_t end = __shfl_sync(0xffffffffu, re, last);
    const int span = end - base;
    AT acc = AT(0);
    // the warp's contiguous segment in pieces of kSpmvCap products, each
    // loaded coalesced; every lane then sums its own row's part in column
    // order (long rows, e.g. vector P2 elasticity, take several pieces)
    for (int c0 = 0; c0 < span; c0 += kSpmvCap) {
      const int cl = min(kSpmvCap, span - c0);
      // kSpmvUnroll products per lane in flight: the columns and values
      // first, then the gathers of x they name
      for (int i0 = lane; i0 < cl; i0 += 32 * kSpmvUnroll) {
        int32_t cc[kSpmvUnroll];
        VT vv[kSpmvUnroll];
#pragma unroll
        for (int u = 0; u < kSpmvUnroll; ++u) {
          const int i = i0 + 32 * u;
          const int64_t k = int64_t(base) + c0 + i;
          cc[u] = i < cl ? __ldg(col + k) : 0;
          vv[u] = i < cl ? __ldg(val + k) : VT(0);
        }
#pragma unroll
        for (int u = 0; u < kSpmvUnroll; ++u) {
          const int i = i0 + 32 * u;
          if (i < cl) st[i] = AT(vv[u]) * AT(__ldg(x + cc[u]));
        }
      }
      __syncwarp();
      if (valid) {
        const int k0 = max(rb - base, c0), k1 = min(re - base, c0 + cl);
        for (int k = k0; k < k1; ++k) acc += st[k - c0];
      }
      __syncwarp();
    }
    if (valid) {
      AT out = residual == 1 ? AT(b[r]) - acc : (residual == 2 ? AT(b[r]) + acc : acc);
      if (yscale) out *= AT(yscale[r]);
      y[r] = XT(out);
    }
  }
}

template <typename VT, typename XT, typename AT>
static int spmv(int64_t n, const int32_t* rp, const int32_t* ci, const VT* v, const XT* x, XT* y, const XT* b,
                int residual, cudaStream_t s, const float* yscale = nullptr, const int32_t* gate = nullptr) {
  if (n == 0) return NFEM_OK;
  const int grid = grid_for(ceil_div(n, 32 * kSpmvWarps), 1, 8);
  spmv_kernel<VT, XT, AT><<<grid, 32 * kSpmvWarps, 0, s>>>(n, rp, ci, v, x, y, b, residual, yscale, gate);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < (blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

// partial[j * gridDim.x + block] = sum_i X_j[i] * y[i] for j < k (X_j = X + j * ldx).
// Eight basis vectors per pass share one read of y; each thread keeps two
// elements in flight per vector (memory-level parallelism for HBM).
constexpr int kDotGroup = 8;

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    multidot_partial(int64_t n, int k, const T* __restrict__ X, int64_t ldx, const T* __restrict__ y,
                     double* __restrict__ partial, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ double sh[kDotGroup][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int j0 = 0; j0 < k; j0 += kDotGroup) {
    const int g = min(kDotGroup, k - j0);
    double acc[kDotGroup];
    float accf[kDotGroup];
#pragma unroll
    for (int q = 0; q < kDotGroup; ++q) { acc[q] = 0.0; accf[q] = 0.f; }
    int cnt = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += 2 * stride) {
      const int64_t i2 = i + stride;
      const bool has2 = i2 < n;
      const float y0 = float(__ldg(y + i));
      const float y1 = has2 ? float(__ldg(y + i2)) : 0.f;
#pragma unroll
      for (int q = 0; q < kDotGroup; ++q) {
        if (q < g) {
          const T* xj = X + int64_t(j0 + q) * ldx;
          const float x0 = float(__ldg(xj + i));
          const float x1 = has2 ? float(__ldg(xj + i2)) : 0.f;
          if constexpr (sizeof(T) == 4) {
            accf[q] = fmaf(x0, y0, fmaf(x1, y1, accf[q]));
          } else {
            acc[q] += double(__ldg(xj + i)) * double(__ldg(y + i)) +
                      (has2 ? double(__ldg(xj + i2)) * double(__ldg(y + i2)) : 0.0);
          }
        }
      }
      if constexpr (sizeof(T) == 4) {
        if (++cnt == 32) {
#pragma unroll
          for (int q = 0; q < kDotGroup; ++q) { acc[q] += double(accf[q]); accf[q] = 0.f; }
          cnt = 0;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kDotGroup; ++q) {
      double v = acc[q] + double(accf[q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) sh[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < g) {
      double t = 0.0;
      for (int w = 0; w < (kRedThreads / 32); ++w) t += sh[threadIdx.x][w];
      partial[int64_t(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
    }
    __syncthreads();
  }
}

// out[j] = sum_b partial[j][b] (fixed order, one block per j); mode 1: sqrt
__global__ void reduce_partials(const double* __restrict__ partial, int nb, int k, double* __restrict__ out,
                                int mode, double sign) {
  __shared__ double sh[32];
  const int j = blockIdx.x;
  if (j >= k) return;
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v += partial[int64_t(j) * nb + b];
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) out[j] = mode == 1 ? sqrt(t) : sign * t;
}

// ---- FP32 reductions over 16-byte rows
// Partial sums: FP32 per thread, folded into FP64 in shared memory every 16
// elements (the registers stay with the loads), a fixed-order block
// reduction, one partial per (vector, block).  With a counter, the last
// block to finish adds the partials of each vector in block order and
// writes the result (sqrt for mode 1) -- no separate reduction launch; the
// counter returns to 0.  The grids are the resident grids of the kernels
// (blocks per SM x SMs), so every block streams its share in one wave.

// Called by all threads of every block after the partials of vectors
// q < k were written (partial[q * gridDim.x + blockIdx.x]).
__device__ __forceinline__ void finish_partials(const double* partial, int k, double* __restrict__ out, int mode,
                                                unsigned int* counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int q = warp; q < k; q += nw) {
    double v = 0.0;
    for (int b = lane; b < int(gridDim.x); b += 32) v += __ldcg(partial + int64_t(q) * gridDim.x + b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[q] = mode == 1 ? sqrt(v) : v;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

template <int KM>
__device__ __forceinline__ void block_partials(int k, const float (&accf)[KM], double (*sacc)[kRedThreads],
                                               double (*sh)[kRedThreads / 32], double* __restrict__ partial) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < KM; ++q) {
    if (q < k) {
      double v = sacc[q][threadIdx.x] + double(accf[q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) sh[q][warp] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double t = 0.0;
    for (int w = 0; w < (kRedThreads / 32); ++w) t += sh[threadIdx.x][w];
    partial[int64_t(threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
}

// partial[q][block] = sum_i X_q[i] . y[i], q < k, eight vectors per pass
// sharing one read of y
__global__ void __launch_bounds__(kRedThreads)
    multidot_partial_v4(int64_t n4, int k, const float4* __restrict__ X, int64_t ldx4,
                        const float4* __restrict__ y, double* __restrict__ partial, double* __restrict__ out,
                        int mode, unsigned int* counter, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ double sacc[kDotGroup][kRedThreads];
  __shared__ double sh[kDotGroup][kRedThreads / 32];
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int j0 = 0; j0 < k; j0 += kDotGroup) {
    const int g = min(kDotGroup, k - j0);
#pragma unroll
    for (int q = 0; q < kDotGroup; ++q) sacc[q][threadIdx.x] = 0.0;
    float accf[kDotGroup];
#pragma unroll
    for (int q = 0; q < kDotGroup; ++q) accf[q] = 0.f;
    int cnt = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += stride) {
      const float4 yv = __ldg(y + i);
      const float4* xq = X + int64_t(j0) * ldx4 + i;
#pragma unroll
      for (int q = 0; q < kDotGroup; ++q) {
        if (q < g) {
          const float4 xv = __ldg(xq);
          accf[q] = fmaf(xv.x, yv.x, fmaf(xv.y, yv.y, fmaf(xv.z, yv.z, fmaf(xv.w, yv.w, accf[q]))));
        }
        xq += ldx4;
      }
      if (++cnt == 16) {
#pragma unroll
        for (int q = 0; q < kDotGroup; ++q) {
          sacc[q][threadIdx.x] += double(accf[q]);
          accf[q] = 0.f;
        }
        cnt = 0;
      }
    }
    block_partials<kDotGroup>(g, accf, sacc, sh, partial + int64_t(j0) * gridDim.x);
    __syncthreads();
  }
  if (counter) finish_partials(partial, k, out, mode, counter);
}

static bool rows16(int64_t n, int64_t ldx, const void* a, const void* b) {
  return n % 4 == 0 && ldx % 4 == 0 && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
}

// Blocks of `kernel` resident on the whole device at kRedThreads threads
// (at most kRedBlocks, the partial buffers' width); cached per kernel.
template <typename K>
static int resident_grid(K kernel, int* cache) {
  if (*cache > 0) return *cache;
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kRedThreads, 0) != cudaSuccess || per < 1)
    return kRedBlocks;
  *cache = std::min(per * sms, kRedBlocks);
  return *cache;
}

// out[q] = X_q . y (q < k), sqrt of it for mode 1.  counter: the FP32
// 16-byte-row form finishes the sum in the kernel (see finish_partials).
template <typename T>
static int multidot(int64_t n, int k, const T* X, int64_t ldx, const T* y, double* partial, double* out, int mode,
                    cudaStream_t s, const int32_t* gate = nullptr, unsigned int* counter = nullptr) {
  if constexpr (sizeof(T) == 4) {
    if (rows16(n, ldx, X, y)) {
      static int cache = 0;
      const int nb = resident_grid(multidot_partial_v4, &cache);
      multidot_partial_v4<<<nb, kRedThreads, 0, s>>>(n / 4, k, reinterpret_cast<const float4*>(X), ldx / 4,
                                                     reinterpret_cast<const float4*>(y), partial, out, mode, counter,
                                                     gate);
      if (!counter) reduce_partials<<<k, 256, 0, s>>>(partial, nb, k, out, mode, 1.0);
      NFEM_CHECK_LAUNCH();
      return NFEM_OK;
    }
  }
  multidot_partial<T><<<kRedBlocks, kRedThreads, 0, s>>>(n, k, X, ldx, y, partial, gate);
  reduce_partials<<<k, 256, 0, s>>>(partial, kRedBlocks, k, out, mode, 1.0);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// w -= sum_{j<k} h[j] X_j   (h on the device; FP64 coefficients)
template <typename T>
__global__ void multi_axpy(int64_t n, int k, const T* __restrict__ X, int64_t ldx, const double* __restrict__ h,
                           T* __restrict__ w, double hsign, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ double hs[kMaxRestart + 1];
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = hsign * h[j];
  __syncthreads();
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += 2 * stride) {
    const int64_t i2 = i + stride;
    const bool has2 = i2 < n;
    float a0 = 0.f, a1 = 0.f;
#pragma unroll 4
    for (int j = 0; j < k; ++j) {
      const float hj = float(hs[j]);
      const T* xj = X + int64_t(j) * ldx;
      a0 = fmaf(hj, float(__ldg(xj + i)), a0);
      if (has2) a1 = fmaf(hj, float(__ldg(xj + i2)), a1);
    }
    w[i] = T(float(w[i]) - a0);
    if (has2) w[i2] = T(float(w[i2]) - a1);
  }
}

// float4 form of multi_axpy for 16-byte rows
__global__ void multi_axpy_v4(int64_t n4, int k, const float4* __restrict__ X, int64_t ldx4,
                              const double* __restrict__ h, float4* __restrict__ w, double hsign,
                              const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ float hs[kMaxRestart + 1];
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = float(hsign * h[j]);
  __syncthreads();
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += int64_t(gridDim.x) * blockDim.x) {
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int j = 0; j < k; ++j) {
      const float hj = hs[j];
      const float4 xv = __ldg(X + int64_t(j) * ldx4 + i);
      a.x = fmaf(hj, xv.x, a.x);
      a.y = fmaf(hj, xv.y, a.y);
      a.z = fmaf(hj, xv.z, a.z);
      a.w = fmaf(hj, xv.w, a.w);
    }
    float4 v = w[i];
    v.x -= a.x;
    v.y -= a.y;
    v.z -= a.z;
    v.w -= a.w;
    w[i] = v;
  }
}

// ---- fused Gram-Schmidt passes (16-byte rows, k <= KM basis vectors)
// The second classical Gram-Schmidt pass needs w' = w - X h before its dot
// products X^T w'; each thread holds its k basis entries in registers, so
// the update and the products share one read of X.  The last update and
// the norm of its result share the next read.  Partial sums follow
// multidot_partial_v4: FP32 per thread, folded into FP64 every 16
// elements (here into shared memory, to keep the registers for X), a
// fixed-order block reduction, one partial per (vector, block).
// w <- w - X h;  partial = per-block sums of X^T w (the updated w)
#ifndef NFEM_CGS_MIN_BLOCKS
#define NFEM_CGS_MIN_BLOCKS 2
#endif
template <int KM>
__global__ void __launch_bounds__(kRedThreads, NFEM_CGS_MIN_BLOCKS)
    axpy_dot_v4(int64_t n4, int k, const float4* __restrict__ X, int64_t ldx4, const double* __restrict__ h,
                float4* __restrict__ w, double* __restrict__ partial, double* __restrict__ out,
                unsigned int* counter, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ float hs[KM];
  __shared__ double sacc[KM][kRedThreads];
  __shared__ double sh[KM][kRedThreads / 32];
  for (int q = threadIdx.x; q < k; q += blockDim.x) hs[q] = float(h[q]);
#pragma unroll
  for (int q = 0; q < KM; ++q) sacc[q][threadIdx.x] = 0.0;
  __syncthreads();
  float accf[KM];
#pragma unroll
  for (int q = 0; q < KM; ++q) accf[q] = 0.f;
  int cnt = 0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += stride) {
    float4 xv[KM];
    const float4* xq = X + i;
#pragma unroll
    for (int q = 0; q < KM; ++q) {
      if (q < k) xv[q] = __ldg(xq);
      xq += ldx4;
    }
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < KM; ++q) {
      if (q < k) {
        const float hq = hs[q];
        a.x = fmaf(hq, xv[q].x, a.x);
        a.y = fmaf(hq, xv[q].y, a.y);
        a.z = fmaf(hq, xv[q].z, a.z);
        a.w = fmaf(hq, xv[q].w, a.w);
      }
    }
    float4 v = w[i];
    v.x -= a.x;
    v.y -= a.y;
    v.z -= a.z;
    v.w -= a.w;
    w[i] = v;
#pragma unroll
    for (int q = 0; q < KM; ++q)
      if (q < k) accf[q] = fmaf(xv[q].x, v.x, fmaf(xv[q].y, v.y, fmaf(xv[q].z, v.z, fmaf(xv[q].w, v.w, accf[q]))));
    if (++cnt == 16) {
#pragma unroll
      for (int q = 0; q < KM; ++q) {
        sacc[q][threadIdx.x] += double(accf[q]);
        accf[q] = 0.f;
      }
      cnt = 0;
    }
  }
  block_partials<KM>(k, accf, sacc, sh, partial);
  finish_partials(partial, k, out, 0, counter);
}

// w <- w - X h;  partial = per-block sums of w . w (the updated w)
template <int KM>
__global__ void __launch_bounds__(kRedThreads)
    axpy_norm_v4(int64_t n4, int k, const float4* __restrict__ X, int64_t ldx4, const double* __restrict__ h,
                 float4* __restrict__ w, double* __restrict__ partial, double* __restrict__ out,
                 unsigned int* counter, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ float hs[KM];
  __shared__ double sacc[1][kRedThreads];
  __shared__ double sh[1][kRedThreads / 32];
  for (int q = threadIdx.x; q < k; q += blockDim.x) hs[q] = float(h[q]);
  sacc[0][threadIdx.x] = 0.0;
  __syncthreads();
  float accf[1] = {0.f};
  int cnt = 0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += stride) {
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < KM; ++q) {
      if (q < k) {
        const float hq = hs[q];
        const float4 xv = __ldg(X + int64_t(q) * ldx4 + i);
        a.x = fmaf(hq, xv.x, a.x);
        a.y = fmaf(hq, xv.y, a.y);
        a.z = fmaf(hq, xv.z, a.z);
        a.w = fmaf(hq, xv.w, a.w);
      }
    }
    float4 v = w[i];
    v.x -= a.x;
    v.y -= a.y;
    v.z -= a.z;
    v.w -= a.w;
    w[i] = v;
    accf[0] = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, accf[0]))));
    if (++cnt == 16) {
      sacc[0][threadIdx.x] += double(accf[0]);
      accf[0] = 0.f;
      cnt = 0;
    }
  }
  block_partials<1>(1, accf, sacc, sh, partial);
  finish_partials(partial, 1, out, 1, counter);
}

// The second Gram-Schmidt pass and the norm, given the first pass's
// coefficients h (k <= 16 basis vectors, 16-byte rows): w <- w - X h,
// y = X^T w, w <- w - X y, nrm = ||w||.  Returns false (nothing launched)
// when the fused form does not apply.
static bool cgs2_fused(int64_t n, int k, const float* X, int64_t ldx, const double* h, float* w, double* y,
                       double* nrm, double* partial, unsigned int* counter, cudaStream_t s,
                       const int32_t* gate) {
  if (k > 16 || !rows16(n, ldx, X, w)) return false;
  const auto* X4 = reinterpret_cast<const float4*>(X);
  auto* w4 = reinterpret_cast<float4*>(w);
  if (k <= 8) {
    static int c1 = 0, c2 = 0;
    axpy_dot_v4<8><<<resident_grid(axpy_dot_v4<8>, &c1), kRedThreads, 0, s>>>(n / 4, k, X4, ldx / 4, h, w4, partial,
                                                                              y, counter, gate);
    axpy_norm_v4<8><<<resident_grid(axpy_norm_v4<8>, &c2), kRedThreads, 0, s>>>(n / 4, k, X4, ldx / 4, y, w4,
                                                                                partial, nrm, counter, gate);
  } else {
    static int c1 = 0, c2 = 0;
    axpy_dot_v4<16><<<resident_grid(axpy_dot_v4<16>, &c1), kRedThreads, 0, s>>>(n / 4, k, X4, ldx / 4, h, w4,
                                                                                partial, y, counter, gate);
    axpy_norm_v4<16><<<resident_grid(axpy_norm_v4<16>, &c2), kRedThreads, 0, s>>>(n / 4, k, X4, ldx / 4, y, w4,
                                                                                  partial, nrm, counter, gate);
  }
  return true;
}

// w -= sign * X h over k vectors, choosing the float4 form when it applies
static void multi_axpy_f32(int64_t n, int k, const float* X, int64_t ldx, const double* h, float* w, double hsign,
                           cudaStream_t s, const int32_t* gate = nullptr) {
  if (rows16(n, ldx, X, w)) {
    multi_axpy_v4<<<grid_for(n / 4, 256), 256, 0, s>>>(n / 4, k, reinterpret_cast<const float4*>(X), ldx / 4, h,
                                                        reinterpret_cast<float4*>(w), hsign, gate);
  } else {
    multi_axpy<float><<<grid_for(n, 256), 256, 0, s>>>(n, k, X, ldx, h, w, hsign, gate);
  }
}

// v = w / nrm and, with a, t = a (.) v (the next preconditioner input of
// the weighted inner product)
// (w and v may be the same vector)
__global__ void scale_by_inv_w(int64_t n, const float* w, const double* __restrict__ nrm, float* v,
                               const float* __restrict__ a, float* __restrict__ t, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  const double d = *nrm;
  const float inv = d > 0.0 ? float(1.0 / d) : 0.f;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float x = w[i] * inv;
    v[i] = x;
    if (a) t[i] = a[i] * x;
  }
}

// y = a (.) x  (elementwise)
__global__ void scale_vec(int64_t n, const float* __restrict__ a, const float* __restrict__ x, float* __restrict__ y,
                          const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = a[i] * x[i];
}

// Weights of the inner product the flexible GMRES minimises in.  s_i^2 is
// |a_ii|^-1 for rows with a diagonal and (sum_j a_ij^2 / |a_jj|)^-1 for rows
// without one (the pressure rows of a saddle point, a Schur-complement
// diagonal); c_i^2 is the squared column norm of the preconditioner (1 when
// there is none).  W_i = sqrt(s_i^2 c_i^2), stored as W^1/2 and W^-1/2.
__global__ void weights_rows(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ v, double* __restrict__ s2) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n; r += int64_t(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] == r) d = fabs(v[k]);
    if (d > 0.0) {
      s2[r] = 1.0 / d;
    } else {
      double acc = 0.0;
      for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
        const int32_t j = ci[k];
        double dj = 0.0;
        for (int32_t q = rp[j]; q < rp[j + 1]; ++q)
          if (ci[q] == j) dj = fabs(v[q]);
        if (dj > 0.0) acc += v[k] * v[k] / dj;
      }
      s2[r] = acc > 0.0 ? 1.0 / acc : 1.0;
    }
  }
}

// c_i^2 = sum over the incidences (c, a) of column i of sum_b (inv[c][b][a] / m_b)^2
template <int NT>
__global__ void weights_blockcols(int64_t n_rows, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const int32_t* __restrict__ cd, const float* __restrict__ inv, double* __restrict__ c2,
                                  int n_run = 0) {
  const int N = NT > 0 ? NT : n_run;
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int32_t k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k) {
      const int32_t occ = inc[k];
      const int32_t c = occ / N;
      const int a = occ - c * N;
      for (int b = 0; b < N; ++b) {
        const int32_t db = cd[int64_t(c) * N + b];
        const double mb = double(inc_ptr[db + 1] - inc_ptr[db]);
        const double x = double(inv[(int64_t(c) * N + b) * N + a]) / mb;
        acc += x * x;
      }
    }
    c2[r] = acc > 0.0 ? acc : 1.0;
  }
}

__global__ void weights_final(int64_t n, const double* __restrict__ s2, const double* __restrict__ c2,
                              float* __restrict__ wsqrt, float* __restrict__ winvsqrt) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const double w = sqrt(s2[i] * (c2 ? c2[i] : 1.0));
    wsqrt[i] = float(sqrt(w));
    winvsqrt[i] = float(1.0 / sqrt(w));
  }
}

// ---- two-level (Galerkin) coarse correction
// p_val[2i + s]: pressure rows -> 1 for their aggregate; flux rows -> -w_i *
// (sum of row i's entries in the pressure columns of aggregate p_agg[2i + s]).
__global__ void twolevel_fill_p(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const double* __restrict__ v, int64_t p_base, int64_t n_cells,
                                const int32_t* __restrict__ cell_agg, const float* __restrict__ w,
                                const int32_t* __restrict__ p_agg, float* __restrict__ p_val) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x) {
    const bool prow = i >= p_base && i < p_base + n_cells;
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      const int32_t a = p_agg[2 * i + sl];
      float val = 0.f;
      if (a >= 0) {
        if (prow) {
          val = 1.f;
        } else {
          double acc = 0.0;
          for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int64_t j = ci[k];
            if (j >= p_base && j < p_base + n_cells && cell_agg[j - p_base] == a) acc += v[k];
          }
          val = float(-double(w[i]) * acc);
        }
      }
      p_val[2 * i + sl] = val;
    }
  }
}

// Position of coarse entry (alpha, beta): dense row-major, or inside the
// diagonal block of alpha (block layout); -1 when beta lies in another block.
struct CoarseIndex {
  int n_agg;
  const int32_t* blk_ptr;
  const int64_t* blk_off;
  const int32_t* agg_blk;  // nullptr: dense
  __device__ int64_t operator()(int32_t a, int32_t b) const {
    if (!agg_blk) return int64_t(a) * n_agg + b;
    const int32_t blk = agg_blk[a];
    if (agg_blk[b] != blk) return -1;
    const int32_t b0 = blk_ptr[blk];
    return blk_off[blk] + int64_t(a - b0) * (blk_ptr[blk + 1] - b0) + (b - b0);
  }
};

// ac[alpha, beta] += P[i, alpha] A[i, j] P[j, beta] over the nonzeros of A
__global__ void twolevel_galerkin(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                  const double* __restrict__ v, const int32_t* __restrict__ p_agg,
                                  const float* __restrict__ p_val, CoarseIndex at, double* __restrict__ ac,
                                  int32_t* status) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x) {
    const int32_t ai0 = p_agg[2 * i], ai1 = p_agg[2 * i + 1];
    const double pi0 = p_val[2 * i], pi1 = p_val[2 * i + 1];
    if ((ai0 < 0 || pi0 == 0.0) && (ai1 < 0 || pi1 == 0.0)) continue;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
      const int64_t j = ci[k];
      const double aij = v[k];
#pragma unroll
      for (int sj = 0; sj < 2; ++sj) {
        const int32_t bj = p_agg[2 * j + sj];
        const double pj = p_val[2 * j + sj];
        if (bj < 0 || pj == 0.0) continue;
#pragma unroll
        for (int si = 0; si < 2; ++si) {
          const int32_t ai = si ? ai1 : ai0;
          const double pi = si ? pi1 : pi0;
          if (ai < 0 || pi == 0.0) continue;
          const int64_t e = at(ai, bj);
          if (e < 0) {
            set_status(status, NFEM_ERR_INVALID_ARG);
            continue;
          }
          atomicAdd(ac + e, pi * aij * pj);
        }
      }
    }
  }
}

// Gauss-Jordan inversion of the dense [n, 2n] array [Ac | I] (FP64, row-major)
__global__ void gj_pivot(double* __restrict__ m, int n, int k, int32_t* __restrict__ piv, int32_t* status) {
  __shared__ double best[1024];
  __shared__ int besti[1024];
  double b = -1.0;
  int bi = k;
  for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
    const double x = fabs(m[int64_t(i) * 2 * n + k]);
    if (x > b) { b = x; bi = i; }
  }
  best[threadIdx.x] = b;
  besti[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double y = best[threadIdx.x + o];
      const int yi = besti[threadIdx.x + o];
      if (y > best[threadIdx.x] || (y == best[threadIdx.x] && yi < besti[threadIdx.x])) {
        best[threadIdx.x] = y;
        besti[threadIdx.x] = yi;
      }
    }
    __syncthreads();
  }
  const int p = besti[0];
  if (threadIdx.x == 0) {
    *piv = p;
    if (!(best[0] > 0.0)) set_status(status, NFEM_ERR_BREAKDOWN);
  }
  // swap rows k and p, then scale row k
  if (p != k)
    for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) {
      const double t = m[int64_t(k) * 2 * n + j];
      m[int64_t(k) * 2 * n + j] = m[int64_t(p) * 2 * n + j];
      m[int64_t(p) * 2 * n + j] = t;
    }
  __syncthreads();
  const double d = m[int64_t(k) * 2 * n + k];
  const double inv = d != 0.0 ? 1.0 / d : 0.0;
  __syncthreads();
  for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) m[int64_t(k) * 2 * n + j] *= inv;
}

// rows i != k: m[i, j] -= m[i, k] m[k, j] for j > k (columns < k of the left
// half are already unit vectors); column k is cleared afterwards
__global__ void gj_eliminate(double* __restrict__ m, int n, int k) {
  const int w = 2 * n - k - 1;
  const int64_t total = int64_t(n) * w;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(e / w);
    const int j = k + 1 + int(e - int64_t(i) * w);
    if (i == k) continue;
    const double f = m[int64_t(i) * 2 * n + k];
    if (f != 0.0) m[int64_t(i) * 2 * n + j] -= f * m[int64_t(k) * 2 * n + j];
  }
}

__global__ void gj_clear_col(double* __restrict__ m, int n, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (i != k) m[int64_t(i) * 2 * n + k] = 0.0;
}

__global__ void gj_extract(const double* __restrict__ m, int n, float* __restrict__ inv) {
  const int64_t total = int64_t(n) * n;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(e / n), j = int(e - int64_t(i) * n);
    inv[e] = float(m[int64_t(i) * 2 * n + n + j]);
  }
}

__global__ void gj_init(const double* __restrict__ ac, int n, double* __restrict__ m) {
  const int64_t total = int64_t(n) * 2 * n;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(e / (2 * n)), j = int(e - int64_t(i) * 2 * n);
    m[e] = j < n ? ac[int64_t(i) * n + j] : (j - n == i ? 1.0 : 0.0);
  }
}

// ------------------------------------------------------------------ blocked coarse inverse
// In-place block Gauss-Jordan inversion of the coarse matrix, 64 x 64
// blocks, no pivoting, FP32 (the inverse is stored and applied in FP32).  A_c = P^T A P is symmetric positive definite here
// (the flux extension cancels the saddle point's sign structure:
// A_c = (D B^T P_p)^T M (D B^T P_p) with M the flux mass matrix), so the
// unpivoted elimination is stable.  Per block column K:
//   D = A_KK^-1 (one block in shared memory);  A_KJ <- D A_KJ;
//   A_IJ <- A_IJ - A_IK A_KJ;  A_IK <- -A_IK D;  A_KK <- D   (I, J != K).
// The matrix is padded to a multiple of 64 with an identity block, whose
// inverse is the identity again.  T is the type of the trailing updates.
constexpr int kGjB = 64;

template <typename T>
__global__ void __launch_bounds__(256) bgj_pad(const double* __restrict__ ac, int n, int N, T* __restrict__ m) {
  const int64_t total = int64_t(N) * N;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(e / N), j = int(e - int64_t(i) * N);
    m[e] = (i < n && j < n) ? T(ac[int64_t(i) * n + j]) : T(i == j ? 1.0 : 0.0);
  }
}

#ifndef NFEM_COARSE_DIAG_T
#define NFEM_COARSE_DIAG_T float
#endif
// One 64 x 64 diagonal block inverted by 1,024 threads, four entries of a
// row in each thread's registers; per step the pivot row and column go
// through double-buffered shared memory (one barrier a step).  Measured at
// 4,096 aggregates: 1,024 threads 40 us per block, 256 threads (sixteen
// entries each) 47 us: the per-thread work of a step outweighs the cheaper
// barrier.
constexpr int kDiagThreads = 1024, kDiagE = kGjB * kGjB / kDiagThreads;  // 4 entries per thread
template <typename T>
__global__ void __launch_bounds__(kDiagThreads) bgj_inv_diag(T* __restrict__ m, int N, int k0, T* __restrict__ dblk,
                                                             int32_t* status) {
  using D = NFEM_COARSE_DIAG_T;
  static_assert(kGjB == 64 && kDiagE * kDiagThreads == kGjB * kGjB && kGjB % kDiagE == 0,
                "whole rows of kDiagE entries per thread");
  __shared__ D rowb[2][kGjB], colb[2][kGjB], ipb[2];
  const int r = threadIdx.x / (kGjB / kDiagE), c0 = (threadIdx.x % (kGjB / kDiagE)) * kDiagE;
  D a[kDiagE];
#pragma unroll
  for (int q = 0; q < kDiagE; ++q) a[q] = D(m[int64_t(k0 + r) * N + k0 + c0 + q]);
  for (int k = 0; k < kGjB; ++k) {
    const int b = k & 1;
    if (r == k) {
#pragma unroll
      for (int q = 0; q < kDiagE; ++q) rowb[b][c0 + q] = a[q];
    }
    if (k >= c0 && k < c0 + kDiagE) {
      D v = a[0];
#pragma unroll
      for (int q = 1; q < kDiagE; ++q) v = (k - c0 == q) ? a[q] : v;
      colb[b][r] = v;
      // the pivot's reciprocal, once per step (the one division of the step)
      if (r == k) ipb[b] = v != D(0) ? D(1) / v : D(0);
    }
    __syncthreads();
    const D p = rowb[b][k];
    const D ip = ipb[b];
    if (threadIdx.x == 0 && !(fabs(p) > 0.0)) set_status(status, NFEM_ERR_BREAKDOWN);
    const D cr = colb[b][r];
#pragma unroll
    for (int q = 0; q < kDiagE; ++q) {
      const int c = c0 + q;
      const D rc = rowb[b][c] * ip;
      if (r == k && c == k) a[q] = ip;
      else if (r == k) a[q] = rc;
      else if (c == k) a[q] = -cr * ip;
      else a[q] -= cr * rc;
    }
  }
#pragma unroll
  for (int q = 0; q < kDiagE; ++q) dblk[r * kGjB + c0 + q] = T(a[q]);
}

// 64 x 64 product of two shared-memory tiles, 4 x 4 outputs per thread
template <typename T>
__device__ __forceinline__ void tile_mma(const T (*x)[kGjB + 1], const T (*y)[kGjB + 1], T (&acc)[4][4]) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
#pragma unroll 8
  for (int k = 0; k < kGjB; ++k) {
    T xa[4], yb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) xa[a] = x[ty * 4 + a][k];
#pragma unroll
    for (int b = 0; b < 4; ++b) yb[b] = y[k][tx * 4 + b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] += xa[a] * yb[b];
  }
}

template <typename T>
__device__ __forceinline__ void load_tile(T (*t)[kGjB + 1], const T* __restrict__ src, int N, int r0, int c0) {
  for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) {
    const int r = e / kGjB, c = e - r * kGjB;
    t[r][c] = src[int64_t(r0 + r) * N + c0 + c];
  }
}

// mode 0: row block    A_KJ <- D A_KJ        (blockIdx.x = J tile)
// mode 1: column block A_IK <- -A_IK D       (blockIdx.x = I tile)
template <typename T>
__global__ void __launch_bounds__(256) bgj_panel(T* __restrict__ m, int N, int k0, const T* __restrict__ dblk,
                                                 int mode) {
  extern __shared__ __align__(16) unsigned char bgj_smem[];
  T(*d)[kGjB + 1] = reinterpret_cast<T(*)[kGjB + 1]>(bgj_smem);
  T(*x)[kGjB + 1] = d + kGjB;
  const int t0 = blockIdx.x * kGjB;
  if (t0 == k0) return;
  for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) d[e / kGjB][e % kGjB] = dblk[e];
  if (mode == 0) load_tile(x, m, N, k0, t0);
  else load_tile(x, m, N, t0, k0);
  __syncthreads();
  T acc[4][4] = {};
  if (mode == 0) tile_mma(d, x, acc);
  else tile_mma(x, d, acc);
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int r = ty * 4 + a, c = tx * 4 + b;
      if (mode == 0) m[int64_t(k0 + r) * N + t0 + c] = acc[a][b];
      else m[int64_t(t0 + r) * N + k0 + c] = -acc[a][b];
    }
}

// A_IJ -= A_IK A_KJ for tiles I, J != K (A_KJ already updated, A_IK not yet)
template <typename T>
__global__ void __launch_bounds__(256) bgj_trailing(T* __restrict__ m, int N, int k0) {
  extern __shared__ __align__(16) unsigned char bgj_smem[];
  T(*x)[kGjB + 1] = reinterpret_cast<T(*)[kGjB + 1]>(bgj_smem);
  T(*y)[kGjB + 1] = x + kGjB;
  const int i0 = blockIdx.y * kGjB, j0 = blockIdx.x * kGjB;
  if (i0 == k0 || j0 == k0) return;
  load_tile(x, m, N, i0, k0);
  load_tile(y, m, N, k0, j0);
  __syncthreads();
  T acc[4][4] = {};
  tile_mma(x, y, acc);
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      T* e = m + int64_t(i0 + ty * 4 + a) * N + j0 + tx * 4 + b;
      *e -= acc[a][b];
    }
}

// The trailing update on the tensor cores (FP32 trailing matrix): a tile of
// 128 rows x 256 columns of A_IJ -= A_IK A_KJ per CTA, as one 128 x 256 x 64
// product in tensor memory.  The operands are split into TF32 high and low
// parts (x = hi + lo, both TF32) and the product taken as hi.hi + hi.lo +
// lo.hi (24 tcgen05.mma kind::tf32, M 128, N 256, K 8), which keeps FP32
// accuracy (the dropped lo.lo term is below 2^-22 relative).  A_IK is staged
// K-major as it lies in memory; A_KJ is staged transposed (column n of the
// tile as row n of the B operand).  Rows and columns of the pivot block K
// and beyond N are left alone.
constexpr int kTcTM = 128, kTcTN = 256;
constexpr uint32_t kTcSbo = (kGjB / 4) * 128;  // 2048: row-group stride of the K = 64 operands
constexpr size_t kTcA = size_t(kTcTM) * kGjB * 4;   // 32 KB per part
constexpr size_t kTcB = size_t(kTcTN) * kGjB * 4;   // 64 KB per part
constexpr size_t kTcSmem = 2 * kTcA + 2 * kTcB + 64 + 1024;

__device__ __forceinline__ uint32_t tc_off(int row, int k) {
  return uint32_t((row & 7) * 16 + (row >> 3) * kTcSbo + (k & 3) * 4 + (k >> 2) * 128);
}

__global__ void __launch_bounds__(256, 1) bgj_trailing_tc(float* __restrict__ m, int N, int k0, int32_t* status) {
  extern __shared__ uint8_t tc_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sAh = sm;
  uint8_t* sAl = sAh + kTcA;
  uint8_t* sBh = sAl + kTcA;
  uint8_t* sBl = sBh + kTcB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sBl + kTcB);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  volatile int32_t* flag = reinterpret_cast<volatile int32_t*>(slot + 1);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int i0 = blockIdx.y * kTcTM, j0 = blockIdx.x * kTcTN;
  // A = A_IK: 128 rows x 64, 16-byte chunks; eight consecutive lanes take
  // eight rows of one chunk (one 128-byte core-matrix line).  Every load of
  // the thread is issued before the first is used (eight in flight)
  {
    constexpr int kIt = kTcTM * (kGjB / 4) / 256;  // 8
    float4 v[kIt];
#pragma unroll
    for (int it = 0; it < kIt; ++it) {
      const int q = t + 256 * it;
      const int r = (q & 7) + 8 * (q >> 7), c = (q >> 3) & 15;
      v[it] = i0 + r < N ? __ldg(reinterpret_cast<const float4*>(m + int64_t(i0 + r) * N + k0 + 4 * c))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int it = 0; it < kIt; ++it) {
      const int q = t + 256 * it;
      const int r = (q & 7) + 8 * (q >> 7), c = (q >> 3) & 15;
      const float e[4] = {v[it].x, v[it].y, v[it].z, v[it].w};
      float h[4], l[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        h[u] = tc::to_tf32(e[u]);
        l[u] = tc::to_tf32(e[u] - h[u]);
      }
      *reinterpret_cast<float4*>(sAh + tc_off(r, 4 * c)) = make_float4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<float4*>(sAl + tc_off(r, 4 * c)) = make_float4(l[0], l[1], l[2], l[3]);
    }
  }
  // B = A_KJ transposed: row n of B = column j0 + n of the 64 pivot rows.
  // Lane n takes the 16-byte chunk of four pivot rows of its column: the
  // global loads of a warp are 32 consecutive columns, its shared stores
  // whole 128-byte core-matrix lines
  // (sixteen chunks per thread, in two batches of eight: 32 loads in flight)
  const int n = t & (kTcTN - 1);
  const bool n_ok = j0 + n < N;
#pragma unroll
  for (int batch = 0; batch < 2; ++batch) {
    float e[8][4];
#pragma unroll
    for (int it = 0; it < 8; ++it) {
      const int c = batch * 8 + it;
#pragma unroll
      for (int u = 0; u < 4; ++u) e[it][u] = n_ok ? __ldg(m + int64_t(k0 + 4 * c + u) * N + j0 + n) : 0.f;
    }
#pragma unroll
    for (int it = 0; it < 8; ++it) {
      const int c = batch * 8 + it;
      float h[4], l[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        h[u] = tc::to_tf32(e[it][u]);
        l[u] = tc::to_tf32(e[it][u] - h[u]);
      }
      *reinterpret_cast<float4*>(sBh + tc_off(n, 4 * c)) = make_float4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<float4*>(sBl + tc_off(n, 4 * c)) = make_float4(l[0], l[1], l[2], l[3]);
    }
  }
  if (t == 0) {
    tc::bar_init(tc::smem_u32(bar));
    *flag = 0;
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(slot), kTcTN);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  if (t == 0) {
    constexpr uint32_t id = tc::idesc(tc::kTypeTF32, kTcTM, kTcTN);
    const uint32_t ah = tc::smem_u32(sAh), al = tc::smem_u32(sAl), bh = tc::smem_u32(sBh), bl = tc::smem_u32(sBl);
#pragma unroll 1
    for (int ks = 0; ks < kGjB / 8; ++ks) {  // K = 8 per MMA: two 16-byte chunks
      const uint32_t o = uint32_t(ks) * 256;
      tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, kTcSbo), tc::smem_desc(bh + o, 128, kTcSbo), id, ks > 0);
      tc::mma_tf32(tmem, tc::smem_desc(ah + o, 128, kTcSbo), tc::smem_desc(bl + o, 128, kTcSbo), id, 1u);
      tc::mma_tf32(tmem, tc::smem_desc(al + o, 128, kTcSbo), tc::smem_desc(bh + o, 128, kTcSbo), id, 1u);
    }
    tc::commit(tc::smem_u32(bar));
    if (!tc::wait_commit(tc::smem_u32(bar), 0, status)) *flag = 1;
  }
  __syncthreads();
  tc::fence_after_sync();
  if (!*flag) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. and columns 128 (w / 4) ..
    const int row = i0 + 32 * (warp & 3) + lane;
    const bool row_ok = row < N && (row < k0 || row >= k0 + kGjB);
#pragma unroll 1
    for (int c0 = 0; c0 < kTcTN / 2; c0 += 32) {
      uint32_t v[32];
      const int cb = (warp >> 2) * (kTcTN / 2) + c0;
      tc::tmem_ld32(tmem + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(cb), v);
      const int col0 = j0 + cb;
      if (row_ok && col0 < N && (col0 + 32 <= k0 || col0 >= k0 + kGjB)) {
        float4* dst = reinterpret_cast<float4*>(m + int64_t(row) * N + col0);
        float4 x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = dst[u];  // eight loads in flight
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          x[u].x -= __uint_as_float(v[4 * u]);
          x[u].y -= __uint_as_float(v[4 * u + 1]);
          x[u].z -= __uint_as_float(v[4 * u + 2]);
          x[u].w -= __uint_as_float(v[4 * u + 3]);
          dst[u] = x[u];
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcTN);
  }
}

template <typename T>
__global__ void bgj_put_diag(T* __restrict__ m, int N, int k0, const T* __restrict__ dblk) {
  for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x)
    m[int64_t(k0 + e / kGjB) * N + k0 + e % kGjB] = dblk[e];
}

template <typename T>
__global__ void bgj_extract(const T* __restrict__ m, int n, int N, float* __restrict__ inv) {
  const int64_t total = int64_t(n) * n;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(e / n), j = int(e - int64_t(i) * n);
    inv[e] = float(m[int64_t(i) * N + j]);
  }
}

// Inverts the n x n FP64 matrix ac into inv (FP32) using m (N x N of T,
// N = n rounded up to 64) and dblk (64 x 64 of T) as scratch.
template <typename T>
static int blocked_inverse(const double* ac, int n, T* m, T* dblk, float* inv, int32_t* status, cudaStream_t s) {
  const int N = int(ceil_div(n, kGjB) * kGjB);
  const int nt = N / kGjB;
  const size_t smem = 2 * kGjB * (kGjB + 1) * sizeof(T);
  static const bool attr = [smem] {
    return cudaFuncSetAttribute(bgj_trailing<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) ==
               cudaSuccess &&
           cudaFuncSetAttribute(bgj_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) == cudaSuccess;
  }();
  if (!attr) return NFEM_ERR_CUDA;
  // trailing updates on the tensor cores (FP32 trailing matrix) from N = 512
  // on, or from 128 with the knob at 2; 1 keeps the CUDA-core tiles
  const int tck = knob(NFEM_KNOB_COARSE_TC);
  bool tc = false;
  if constexpr (std::is_same<T, float>::value) tc = tck != 1 && N >= (tck == 2 ? 128 : 512);
  if (tc) {
    static const bool tc_attr = cudaFuncSetAttribute(bgj_trailing_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     int(kTcSmem)) == cudaSuccess;
    if (!tc_attr) return NFEM_ERR_CUDA;
  }
  bgj_pad<T><<<grid_for(int64_t(N) * N, 256), 256, 0, s>>>(ac, n, N, m);
  for (int kb = 0; kb < nt; ++kb) {
    const int k0 = kb * kGjB;
    bgj_inv_diag<T><<<1, kDiagThreads, 0, s>>>(m, N, k0, dblk, status);
    bgj_panel<T><<<nt, 256, smem, s>>>(m, N, k0, dblk, 0);
    if constexpr (std::is_same<T, float>::value) {
      if (tc)
        bgj_trailing_tc<<<dim3(unsigned(ceil_div(N, kTcTN)), unsigned(ceil_div(N, kTcTM))), 256, kTcSmem, s>>>(
            m, N, k0, status);
      else
        bgj_trailing<T><<<dim3(nt, nt), 256, smem, s>>>(m, N, k0);
    } else {
      bgj_trailing<T><<<dim3(nt, nt), 256, smem, s>>>(m, N, k0);
    }
    bgj_panel<T><<<nt, 256, smem, s>>>(m, N, k0, dblk, 1);
    bgj_put_diag<T><<<1, 256, 0, s>>>(m, N, k0, dblk);
  }
  bgj_extract<T><<<grid_for(int64_t(n) * n, 256), 256, 0, s>>>(m, n, N, inv);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ------------------------------------------------------------------ block-diagonal coarse inverse
// The blocked Gauss-Jordan above, batched over the diagonal blocks of a
// block-diagonal coarse matrix and run in place in ac_inv (FP32, the copy of
// ac): 64 x 64 tiles, edge tiles clipped to the block (loads zero-filled,
// stores masked), every block in the same launches (grid z or y = block).
// Per tile column K of each block with s_b > K:
//   A_KK <- A_KK^-1;  A_KJ <- A_KK^-1 A_KJ;  A_IJ -= A_IK A_KJ;
//   A_IK <- -A_IK A_KK^-1   (I, J != K).
// A_KK is read only by the panel products after its inversion, so the
// inverse is written to its place at once.
__device__ __forceinline__ void load_tile_clip(float (*t)[kGjB + 1], const float* __restrict__ src, int ld, int r0,
                                               int c0) {
  for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) {
    const int r = e / kGjB, c = e - r * kGjB;
    t[r][c] = (r0 + r < ld && c0 + c < ld) ? src[int64_t(r0 + r) * ld + c0 + c] : 0.f;
  }
}

__global__ void __launch_bounds__(256) bbgj_diag(int n_blocks, const int32_t* __restrict__ blk_ptr,
                                                 const int64_t* __restrict__ blk_off, float* __restrict__ inv,
                                                 int k0, int max_size, int32_t* status) {
  __shared__ float a[kGjB][kGjB + 1];
  __shared__ float row[kGjB], col[kGjB];
  for (int blk = blockIdx.x; blk < n_blocks; blk += gridDim.x) {
    const int s = blk_ptr[blk + 1] - blk_ptr[blk];
    if (k0 == 0 && s > max_size && threadIdx.x == 0) set_status(status, NFEM_ERR_INVALID_ARG);
    if (k0 >= s) continue;
    const int rem = min(kGjB, s - k0);
    float* m = inv + blk_off[blk] + int64_t(k0) * s + k0;
    for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) {
      const int r = e / kGjB, c = e - r * kGjB;
      a[r][c] = (r < rem && c < rem) ? m[int64_t(r) * s + c] : (r == c ? 1.f : 0.f);
    }
    __syncthreads();
    for (int k = 0; k < rem; ++k) {
      const float p = a[k][k];
      const float ip = p > 0.f ? 1.f / p : 0.f;
      if (threadIdx.x == 0 && !(p > 0.f)) set_status(status, NFEM_ERR_BREAKDOWN);
      if (threadIdx.x < kGjB) {
        row[threadIdx.x] = a[k][threadIdx.x] * ip;
        col[threadIdx.x] = a[threadIdx.x][k];
      }
      __syncthreads();
      for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) {
        const int r = e / kGjB, c = e - r * kGjB;
        if (r == k && c == k) a[r][c] = ip;
        else if (r == k) a[r][c] = row[c];
        else if (c == k) a[r][c] = -col[r] * ip;
        else a[r][c] = fmaf(-col[r], row[c], a[r][c]);
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < kGjB * kGjB; e += blockDim.x) {
      const int r = e / kGjB, c = e - r * kGjB;
      if (r < rem && c < rem) m[int64_t(r) * s + c] = a[r][c];
    }
    __syncthreads();
  }
}

// mode 0: A_KJ <- D A_KJ (blockIdx.x = J);  mode 1: A_IK <- -A_IK D (blockIdx.x = I)
__global__ void __launch_bounds__(256) bbgj_panel(int n_blocks, const int32_t* __restrict__ blk_ptr,
                                                  const int64_t* __restrict__ blk_off, float* __restrict__ inv,
                                                  int k0, int mode) {
  __shared__ float d[kGjB][kGjB + 1];
  __shared__ float x[kGjB][kGjB + 1];
  const int t0 = blockIdx.x * kGjB;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  for (int blk = blockIdx.y; blk < n_blocks; blk += gridDim.y) {
    const int s = blk_ptr[blk + 1] - blk_ptr[blk];
    if (k0 >= s || t0 >= s || t0 == k0) continue;
    float* m = inv + blk_off[blk];
    load_tile_clip(d, m, s, k0, k0);
    if (mode == 0) load_tile_clip(x, m, s, k0, t0);
    else load_tile_clip(x, m, s, t0, k0);
    __syncthreads();
    float acc[4][4] = {};
    if (mode == 0) tile_mma<float>(d, x, acc);
    else tile_mma<float>(x, d, acc);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int r = ty * 4 + a, c = tx * 4 + b;
        if (mode == 0) {
          if (k0 + r < s && t0 + c < s) m[int64_t(k0 + r) * s + t0 + c] = acc[a][b];
        } else {
          if (t0 + r < s && k0 + c < s) m[int64_t(t0 + r) * s + k0 + c] = -acc[a][b];
        }
      }
    __syncthreads();
  }
}

// A_IJ -= A_IK A_KJ for I, J != K (A_KJ updated, A_IK not yet)
__global__ void __launch_bounds__(256) bbgj_trailing(int n_blocks, const int32_t* __restrict__ blk_ptr,
                                                     const int64_t* __restrict__ blk_off, float* __restrict__ inv,
                                                     int k0) {
  __shared__ float x[kGjB][kGjB + 1];
  __shared__ float y[kGjB][kGjB + 1];
  const int i0 = blockIdx.y * kGjB, j0 = blockIdx.x * kGjB;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  for (int blk = blockIdx.z; blk < n_blocks; blk += gridDim.z) {
    const int s = blk_ptr[blk + 1] - blk_ptr[blk];
    if (k0 >= s || i0 >= s || j0 >= s || i0 == k0 || j0 == k0) continue;
    float* m = inv + blk_off[blk];
    load_tile_clip(x, m, s, i0, k0);
    load_tile_clip(y, m, s, k0, j0);
    __syncthreads();
    float acc[4][4] = {};
    tile_mma<float>(x, y, acc);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int r = i0 + ty * 4 + a, c = j0 + tx * 4 + b;
        if (r < s && c < s) m[int64_t(r) * s + c] -= acc[a][b];
      }
    __syncthreads();
  }
}

__global__ void cast_f64_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b);

static int block_diag_inverse(const nfem_two_level* L, int32_t* status, cudaStream_t s) {
  const int nt = int(ceil_div(L->blk_max, kGjB));
  const unsigned nb = unsigned(std::min(L->n_blocks, 65535));
  cast_f64_f32<<<grid_for(L->ac_entries, 256), 256, 0, s>>>(L->ac_entries, L->ac, L->ac_inv);
  for (int kb = 0; kb < nt; ++kb) {
    const int k0 = kb * kGjB;
    bbgj_diag<<<nb, 256, 0, s>>>(L->n_blocks, L->blk_ptr, L->blk_off, L->ac_inv, k0, nt * kGjB, status);
    if (nt > 1) {
      bbgj_panel<<<dim3(nt, nb), 256, 0, s>>>(L->n_blocks, L->blk_ptr, L->blk_off, L->ac_inv, k0, 0);
      bbgj_trailing<<<dim3(nt, nt, std::min(nb, 65535u)), 256, 0, s>>>(L->n_blocks, L->blk_ptr, L->blk_off,
                                                                        L->ac_inv, k0);
      bbgj_panel<<<dim3(nt, nb), 256, 0, s>>>(L->n_blocks, L->blk_ptr, L->blk_off, L->ac_inv, k0, 1);
    }
  }
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ec[alpha] = sum over alpha's block of Ainv[alpha, beta] rc[beta]  (one warp
// per aggregate)
__global__ void block_gemv(int n_agg, const int32_t* __restrict__ blk_ptr, const int64_t* __restrict__ blk_off,
                           const int32_t* __restrict__ agg_blk, const float* __restrict__ Ainv,
                           const float* __restrict__ x, float* __restrict__ y, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n_agg) return;
  const int32_t blk = __ldg(agg_blk + warp);
  const int32_t b0 = __ldg(blk_ptr + blk), s = __ldg(blk_ptr + blk + 1) - b0;
  const float* row = Ainv + __ldg(blk_off + blk) + int64_t(warp - b0) * s;
  const float* xb = x + b0;
  float acc = 0.f;
  for (int j = lane; j < s; j += 32) acc = fmaf(__ldg(row + j), __ldg(xb + j), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = acc;
}

// rc[alpha] = sum over P^T's list of alpha (rows in ascending order) of
// p_val * r: one block per aggregate (its list has thousands of entries),
// each thread a fixed stride of the list, partial sums added in a fixed order.
__global__ void twolevel_restrict(int n_agg, const int32_t* __restrict__ pt_ptr, const int32_t* __restrict__ pt_row,
                                  const float* __restrict__ pt_val, const float* __restrict__ r,
                                  float* __restrict__ rc, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  __shared__ double sh[32];
  const int agg = blockIdx.x;
  if (agg >= n_agg) return;
  float acc = 0.f;
  for (int32_t k = pt_ptr[agg] + threadIdx.x; k < pt_ptr[agg + 1]; k += blockDim.x)
    acc = fmaf(__ldg(pt_val + k), __ldg(r + __ldg(pt_row + k)), acc);
  const double t = block_sum(double(acc), sh);
  if (threadIdx.x == 0) rc[agg] = float(t);
}

// The same sum with one warp per aggregate, for short lists (many small
// aggregates): lanes take a fixed stride of the list, then a fixed-order
// shuffle reduction.
__global__ void twolevel_restrict_warp(int n_agg, const int32_t* __restrict__ pt_ptr,
                                       const int32_t* __restrict__ pt_row, const float* __restrict__ pt_val,
                                       const float* __restrict__ r, float* __restrict__ rc,
                                       const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  const int agg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (agg >= n_agg) return;
  float acc = 0.f;
  for (int32_t k = __ldg(pt_ptr + agg) + lane; k < __ldg(pt_ptr + agg + 1); k += 32)
    acc = fmaf(__ldg(pt_val + k), __ldg(r + __ldg(pt_row + k)), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) rc[agg] = acc;
}

// ec = Ainv rc  (one warp per row; 16-byte loads when n % 4 == 0 and both
// arrays are 16-byte aligned)
__global__ void dense_gemv(int n, const float* __restrict__ Ainv, const float* __restrict__ x, float* __restrict__ y,
                           const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const float* row = Ainv + int64_t(warp) * n;
  float acc = 0.f;
  if ((n & 3) == 0 && ((reinterpret_cast<uintptr_t>(Ainv) | reinterpret_cast<uintptr_t>(x)) & 15) == 0) {
    const float4* row4 = reinterpret_cast<const float4*>(row);
    const float4* x4 = reinterpret_cast<const float4*>(x);
#pragma unroll 4
    for (int j = lane; j < n / 4; j += 32) {
      const float4 a = __ldg(row4 + j), b = __ldg(x4 + j);
      acc = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc))));
    }
  } else {
    for (int j = lane; j < n; j += 32) acc = fmaf(row[j], x[j], acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = acc;
}

__global__ void twolevel_prolong(int64_t n_rows, const int32_t* __restrict__ p_agg, const float* __restrict__ p_val,
                                 const float* __restrict__ ec, float* __restrict__ z, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      const int32_t a = p_agg[2 * i + sl];
      if (a >= 0) acc = fmaf(p_val[2 * i + sl], ec[a], acc);
    }
    z[i] += acc;
  }
}

// ---- A P (FP32 matrix times prolongation), for the fused apply
constexpr int kApCap = 64;  // distinct aggregates of one row

// Sorted distinct aggregates of the P rows named by the columns of row i.
__device__ __forceinline__ int ap_row_aggs(int64_t i, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                           const int32_t* __restrict__ p_agg, int32_t (&list)[kApCap],
                                           int32_t* status) {
  int m = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
    const int64_t j = ci[k];
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      int32_t a = p_agg[2 * j + sl];
      if (a < 0) continue;
      int pos = 0;
      while (pos < m && list[pos] < a) ++pos;
      if (pos < m && list[pos] == a) continue;
      if (m == kApCap) {
        set_status(status, NFEM_ERR_CAPACITY);
        return m;
      }
      for (int t = m; t > pos; --t) list[t] = list[t - 1];
      list[pos] = a;
      ++m;
    }
  }
  return m;
}

__global__ void ap_count(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                         const int32_t* __restrict__ p_agg, int32_t* __restrict__ counts, int32_t* status) {
  int32_t list[kApCap];
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x)
    counts[i] = ap_row_aggs(i, rp, ci, p_agg, list, status);
}

__global__ void ap_fill_cols(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const int32_t* __restrict__ p_agg, const int32_t* __restrict__ ap_ptr,
                             int32_t* __restrict__ ap_col, int32_t* status) {
  int32_t list[kApCap];
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int m = ap_row_aggs(i, rp, ci, p_agg, list, status);
    if (m != ap_ptr[i + 1] - ap_ptr[i]) {
      set_status(status, NFEM_ERR_PATTERN);
      continue;
    }
    for (int t = 0; t < m; ++t) ap_col[ap_ptr[i] + t] = list[t];
  }
}

// ap_val = sum over the row's nonzeros j and P slots s of a_ij p_val[j, s],
// in column order (FP64 sums of the FP32 products' operands, rounded once)
__global__ void ap_fill_values(int64_t n_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                               const float* __restrict__ a32, const int32_t* __restrict__ p_agg,
                               const float* __restrict__ p_val, const int32_t* __restrict__ ap_ptr,
                               const int32_t* __restrict__ ap_col, float* __restrict__ ap_val, int32_t* status) {
  double acc[kApCap];
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int32_t e0 = ap_ptr[i];
    const int m = ap_ptr[i + 1] - e0;
    if (m > kApCap) {
      set_status(status, NFEM_ERR_CAPACITY);
      continue;
    }
    for (int t = 0; t < m; ++t) acc[t] = 0.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
      const int64_t j = ci[k];
#pragma unroll
      for (int sl = 0; sl < 2; ++sl) {
        const int32_t a = p_agg[2 * j + sl];
        if (a < 0) continue;
        int t = 0;
        while (t < m && ap_col[e0 + t] != a) ++t;
        if (t == m) {
          set_status(status, NFEM_ERR_PATTERN);
          continue;
        }
        acc[t] += double(a32[k]) * double(p_val[2 * j + sl]);
      }
    }
    for (int t = 0; t < m; ++t) ap_val[e0 + t] = float(acc[t]);
  }
}

__global__ void offsets_i32(const int64_t* __restrict__ in, int64_t n, int32_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = int32_t(in[i]);
}

// z += P ec and r -= (A P) ec: r stays the residual v - A z of the new z
__global__ void twolevel_prolong_res(int64_t n_rows, const int32_t* __restrict__ p_agg,
                                     const float* __restrict__ p_val, const float* __restrict__ ec,
                                     float* __restrict__ z, const int32_t* __restrict__ ap_ptr,
                                     const int32_t* __restrict__ ap_col, const float* __restrict__ ap_val,
                                     float* __restrict__ r, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      const int32_t a = p_agg[2 * i + sl];
      if (a >= 0) acc = fmaf(p_val[2 * i + sl], ec[a], acc);
    }
    z[i] += acc;
    float ap = 0.f;
    for (int32_t e = ap_ptr[i]; e < ap_ptr[i + 1]; ++e) ap = fmaf(__ldg(ap_val + e), __ldg(ec + __ldg(ap_col + e)), ap);
    r[i] -= ap;
  }
}

// z += P ec and, with A P, w = yscale (.) ((v - r) + (A P) ec) = yscale (.) A z
__global__ void twolevel_prolong_ap(int64_t n_rows, const int32_t* __restrict__ p_agg,
                                    const float* __restrict__ p_val, const float* __restrict__ ec,
                                    float* __restrict__ z, const int32_t* __restrict__ ap_ptr,
                                    const int32_t* __restrict__ ap_col, const float* __restrict__ ap_val,
                                    const float* __restrict__ v, const float* __restrict__ r,
                                    const float* __restrict__ yscale, float* __restrict__ w,
                                    const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_rows; i += int64_t(gridDim.x) * blockDim.x) {
    float acc = 0.f;
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      const int32_t a = p_agg[2 * i + sl];
      if (a >= 0) acc = fmaf(p_val[2 * i + sl], ec[a], acc);
    }
    z[i] += acc;
    float ap = 0.f;
    for (int32_t e = ap_ptr[i]; e < ap_ptr[i + 1]; ++e) ap = fmaf(__ldg(ap_val + e), __ldg(ec + __ldg(ap_col + e)), ap);
    const float az = (v[i] - r[i]) + ap;
    w[i] = yscale ? yscale[i] * az : az;
  }
}

// pt_val[k] = p_val of the (row, slot) that P^T entry k refers to
__global__ void twolevel_fill_pt(int64_t nnz, const int32_t* __restrict__ pt_slot, const float* __restrict__ p_val,
                                 float* __restrict__ pt_val) {
  for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < nnz; k += int64_t(gridDim.x) * blockDim.x)
    pt_val[k] = p_val[pt_slot[k]];
}

__global__ void snapshot_kernel(int64_t n, const double* __restrict__ x, const float* __restrict__ d,
                                float* __restrict__ out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = float(x[i] + double(d[i]));
}

__global__ void cast_f64_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    b[i] = float(a[i]);
}

// x64 += d32
__global__ void add_f32_to_f64(int64_t n, const float* __restrict__ d, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] += double(d[i]);
}

__global__ void fill_f32(int64_t n, float* __restrict__ x, float v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] = v;
}

// ------------------------------------------------------------------ preconditioners
__global__ void jacobi_setup(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ v, float* __restrict__ dinv, int32_t* status) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n; r += int64_t(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] == r) d = v[k];
    if (d == 0.0) set_status(status, NFEM_ERR_BREAKDOWN);
    dinv[r] = d != 0.0 ? float(1.0 / d) : 0.f;
  }
}

__global__ void jacobi_apply(int64_t n, const float* __restrict__ dinv, const float* __restrict__ v,
                             float* __restrict__ z, const int32_t* __restrict__ gate) {
  NFEM_GATE(gate);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    z[i] = dinv[i] * v[i];
}

// Extracts the principal submatrix A[dofs_c, dofs_c] of every cell and
// inverts it (Gauss-Jordan with partial pivoting, FP64); stores FP32.
template <int N>
__global__ void block_extract_invert(int64_t n_cells, const int32_t* __restrict__ cd, const int32_t* __restrict__ rp,
                                     const int32_t* __restrict__ ci, const double* __restrict__ v,
                                     float* __restrict__ inv, int32_t* status) {
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < n_cells;
       c += int64_t(gridDim.x) * blockDim.x) {
    double a[N][2 * N];
    int32_t d[N];
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = cd[c * N + i];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const int32_t b0 = rp[d[i]], b1 = rp[d[i] + 1];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        int32_t lo = b0, hi = b1;
        while (lo < hi) {
          int32_t mid = (lo + hi) >> 1;
          if (ci[mid] < d[j]) lo = mid + 1; else hi = mid;
        }
        a[i][j] = (lo < b1 && ci[lo] == d[j]) ? v[lo] : 0.0;
        a[i][N + j] = i == j ? 1.0 : 0.0;
      }
    }
    bool singular = false;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int p = k;
      double best = fabs(a[k][k]);
#pragma unroll
      for (int i = k + 1; i < N; ++i)
        if (fabs(a[i][k]) > best) { best = fabs(a[i][k]); p = i; }
      if (best == 0.0) { singular = true; break; }
      if (p != k) {
#pragma unroll
        for (int j = 0; j < 2 * N; ++j) { double t = a[k][j]; a[k][j] = a[p][j]; a[p][j] = t; }
      }
      const double ip = 1.0 / a[k][k];
#pragma unroll
      for (int j = 0; j < 2 * N; ++j) a[k][j] *= ip;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (i == k) continue;
        const double f = a[i][k];
#pragma unroll
        for (int j = 0; j < 2 * N; ++j) a[i][j] -= f * a[k][j];
      }
    }
    if (singular) set_status(status, NFEM_ERR_BREAKDOWN);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) inv[(c * N + i) * N + j] = singular ? 0.f : float(a[i][N + j]);
  }
}

// Cells with more local DoFs (6 .. 32, e.g. 30 for the four-field Cosserat
// layout): one warp per cell, the block and the identity side by side in
// shared memory, lane j owning columns j and N + j, Gauss-Jordan with partial
// pivoting in FP32 (the inverse is stored in FP32 and only preconditions).
constexpr int kBlkWarps = 4;
constexpr int kBlkMaxN = 32;
__global__ void __launch_bounds__(32 * kBlkWarps) block_extract_invert_warp(
    int64_t n_cells, int N, const int32_t* __restrict__ cd, const int32_t* __restrict__ rp,
    const int32_t* __restrict__ ci, const double* __restrict__ v, float* __restrict__ inv, int32_t* status) {
  __shared__ float sm[kBlkWarps][kBlkMaxN][2 * kBlkMaxN + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float(*m)[2 * kBlkMaxN + 1] = sm[warp];
  for (int64_t c = int64_t(blockIdx.x) * kBlkWarps + warp; c < n_cells; c += int64_t(gridDim.x) * kBlkWarps) {
    const int32_t dj = lane < N ? __ldg(cd + c * N + lane) : 0;
    for (int i = 0; i < N; ++i) {
      const int32_t di = __ldg(cd + c * N + i);
      const int32_t b0 = __ldg(rp + di), b1 = __ldg(rp + di + 1);
      if (lane < N) {
        int32_t lo = b0, hi = b1;
        while (lo < hi) {  // at most log2(row length) steps
          const int32_t mid = (lo + hi) >> 1;
          if (__ldg(ci + mid) < dj) lo = mid + 1; else hi = mid;
        }
        m[i][lane] = (lo < b1 && __ldg(ci + lo) == dj) ? float(__ldg(v + lo)) : 0.f;
        m[i][N + lane] = i == lane ? 1.f : 0.f;
      }
    }
    __syncwarp();
    bool singular = false;
    for (int k = 0; k < N; ++k) {
      float best = (lane >= k && lane < N) ? fabsf(m[lane][k]) : -1.f;
      int p = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {  // warp arg-max, lowest row on ties
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int op = __shfl_xor_sync(0xffffffffu, p, o);
        if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
      }
      if (!(best > 0.f)) {  // the same value in every lane: a uniform exit
        singular = true;
        break;
      }
      if (p != k && lane < N) {
        float t = m[k][lane]; m[k][lane] = m[p][lane]; m[p][lane] = t;
        t = m[k][N + lane]; m[k][N + lane] = m[p][N + lane]; m[p][N + lane] = t;
      }
      __syncwarp();
      const float ip = 1.f / m[k][k];
      __syncwarp();
      if (lane < N) {
        m[k][lane] *= ip;
        m[k][N + lane] *= ip;
      }
      __syncwarp();
      for (int i = 0; i < N; ++i) {
        if (i == k) continue;
        const float f = m[i][k];
        __syncwarp();
        if (lane < N) {
          m[i][lane] -= f * m[k][lane];
          m[i][N + lane] -= f * m[k][N + lane];
        }
        __syncwarp();
      }
    }
    if (singular && lane == 0) set_status(status, NFEM_ERR_BREAKDOWN);
    for (int i = 0; i < N; ++i)
      if (lane < N) inv[(c * N + i) * N + lane] = singular ? 0.f : m[i][N + lane];
    __syncwarp();
  }
}

// z_r = (1 / m_r) sum over the incidences (c, a) of row r of (A_c^-1 v[dofs_c])_a
// The cell-block smoother as a matrix in A's pattern: row r of
// omega / m_r sum over the incidences (c, a) of r of row a of A_c^-1, at the
// columns dofs_c (the pattern of A is the union of the cells' cliques).
// damping of the cell-block smoother (the two-level cycle's omega, else 1)
static float pre_omega(const nfem_precond* pc) {
  if (pc->kind != NFEM_PC_TWO_LEVEL || !pc->two_level) return 1.f;
  const float w = pc->two_level->omega;
  return w > 0.f ? w : 1.f;
}

// NT > 0: N = NT known at compile time; NT == 0: N = n_run (cells of 6..32 DoFs)
template <int NT>
__global__ void smoother_fill(int64_t n_rows, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                              const int32_t* __restrict__ cd, const float* __restrict__ inv,
                              const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, float omega,
                              float* __restrict__ sv, int32_t* status, int n_run = 0) {
  const int N = NT > 0 ? NT : n_run;
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t b0 = rp[r], b1 = rp[r + 1];
    for (int32_t e = b0; e < b1; ++e) sv[e] = 0.f;
    const int32_t kb = inc_ptr[r], ke = inc_ptr[r + 1];
    if (ke == kb) {  // a row of no cell: the smoother leaves it as it is
      int32_t e = b0;
      while (e < b1 && ci[e] != r) ++e;
      if (e < b1) sv[e] = omega;
      else set_status(status, NFEM_ERR_PATTERN);
      continue;
    }
    const float scale = omega / float(ke - kb);
    for (int32_t k = kb; k < ke; ++k) {
      const int32_t occ = inc[k];
      const int32_t c = occ / N;
      const int a = occ - c * N;
      const float* row = inv + (int64_t(c) * N + a) * N;
#pragma unroll
      for (int b = 0; b < N; ++b) {
        const int32_t j = cd[int64_t(c) * N + b];
        int32_t lo = b0, hi = b1;
        while (lo < hi) {
          const int32_t mid = (lo + hi) >> 1;
          if (ci[mid] < j) lo = mid + 1; else hi = mid;
        }
        if (lo < b1 && ci[lo] == j) sv[lo] += scale * row[b];
        else set_status(status, NFEM_ERR_PATTERN);
      }
    }
  }
}

// omega scales the result; accumulate adds it into z (a post-smoothing step)
template <int NT>
__global__ void block_apply(int64_t n_rows, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                            const int32_t* __restrict__ cd, const float* __restrict__ inv, const float* __restrict__ v,
                            float* __restrict__ z, const int32_t* __restrict__ gate, float omega = 1.f,
                            int accumulate = 0, int n_run = 0) {
  NFEM_GATE(gate);
  const int N = NT > 0 ? NT : n_run;
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t kb = inc_ptr[r], ke = inc_ptr[r + 1];
    float acc = 0.f;
    for (int32_t k = kb; k < ke; ++k) {
      const int32_t occ = inc[k];
      const int32_t c = occ / N;
      const int a = occ - c * N;
      const float* row = inv + (int64_t(c) * N + a) * N;
#pragma unroll
      for (int b = 0; b < N; ++b) acc = fmaf(__ldg(row + b), __ldg(v + __ldg(cd + int64_t(c) * N + b)), acc);
    }
    const float zr = ke > kb ? acc / float(ke - kb) : v[r];
    if (accumulate) z[r] += omega * zr;
    else z[r] = omega == 1.f ? zr : omega * zr;
  }
}

// ------------------------------------------------------------------ Hessenberg / Givens
// Column j of H holds h[0..j+1]; rotations cs/sn; g the rotated rhs.
__global__ void givens_update(double* __restrict__ H, int ldh, const double* __restrict__ h2,
                              double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g, int j,
                              double* __restrict__ hist, int32_t* status, int32_t* __restrict__ gate,
                              const double* __restrict__ target_ptr) {
  const double target = *target_ptr;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (gate && gate[0]) return;
  double* h = H + int64_t(j) * ldh;
  for (int i = 0; i <= j; ++i) h[i] += h2[i];  // second Gram-Schmidt pass
  for (int i = 0; i < j; ++i) {
    const double t = cs[i] * h[i] + sn[i] * h[i + 1];
    h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
    h[i] = t;
  }
  const double a = h[j], b = h[j + 1];
  const double rr = hypot(a, b);
  if (!(rr > 0.0) || !isfinite(rr)) {
    set_status(status, NFEM_ERR_BREAKDOWN);
    cs[j] = 1.0;
    sn[j] = 0.0;
    hist[j] = fabs(g[j]);
    return;
  }
  cs[j] = a / rr;
  sn[j] = b / rr;
  h[j] = rr;
  h[j + 1] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  hist[j] = fabs(g[j + 1]);
  if (gate && hist[j] <= target) gate[0] = 1;  // the rest of the cycle is skipped
}

// y = R^-1 g for the leading k x k triangle of H (stored by columns)
__global__ void upper_solve(const double* __restrict__ H, int ldh, const double* __restrict__ g, int k,
                            double* __restrict__ y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = k - 1; i >= 0; --i) {
    double s = g[i];
    for (int j = i + 1; j < k; ++j) s -= H[int64_t(j) * ldh + i] * y[j];
    y[i] = s / H[int64_t(i) * ldh + i];
  }
}

__global__ void set_scalar(double* __restrict__ p, double v) { *p = v; }

__global__ void init_cycle(double* __restrict__ g, int m, const double* __restrict__ beta, int32_t* __restrict__ gate) {
  for (int i = threadIdx.x; i <= m; i += blockDim.x) g[i] = i == 0 ? *beta : 0.0;
  if (threadIdx.x == 0 && gate) gate[0] = 0;
}


}  // namespace nfem

using namespace nfem;

// ===================================================================== C ABI
extern "C" int nfem_spmv(int value_type, int64_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
                         const void* values, const void* x, void* y, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!row_ptr || !col_idx || !values || !x || !y))) return NFEM_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (value_type == NFEM_F64)
    return spmv<double, double, double>(n_rows, row_ptr, col_idx, (const double*)values, (const double*)x,
                                        (double*)y, nullptr, 0, s);
  if (value_type == NFEM_F32)
    return spmv<float, float, float>(n_rows, row_ptr, col_idx, (const float*)values, (const float*)x, (float*)y,
                                     nullptr, 0, s);
  return NFEM_ERR_INVALID_ARG;
}

extern "C" int nfem_residual_f64(int64_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
                                 const double* values, const double* x, const double* b, double* r, void* stream) {
  if (n_rows < 0 || (n_rows > 0 && (!row_ptr || !col_idx || !values || !x || !b || !r))) return NFEM_ERR_INVALID_ARG;
  return spmv<double, double, double>(n_rows, row_ptr, col_idx, values, x, r, b, 1, (cudaStream_t)stream);
}

extern "C" int nfem_precond_setup(const nfem_precond* pc, const nfem_csr* A64, int32_t* dev_status, void* stream) {
  if (!pc || !A64 || A64->value_type != NFEM_F64) return NFEM_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (pc->kind == NFEM_PC_JACOBI) {
    if (!pc->diag_inv) return NFEM_ERR_INVALID_ARG;
    jacobi_setup<<<grid_for(A64->n_rows, 256), 256, 0, s>>>(A64->n_rows, A64->row_ptr, A64->col_idx,
                                                             (const double*)A64->values, pc->diag_inv, dev_status);
  } else if (pc->kind == NFEM_PC_CELL_BLOCK || pc->kind == NFEM_PC_TWO_LEVEL) {
    if (!pc->cell_dofs || !pc->block_inv) return NFEM_ERR_INVALID_ARG;
    if (pc->kind == NFEM_PC_TWO_LEVEL) {
      const nfem_two_level* L = pc->two_level;
      if (!L || L->n_agg < 1 || !L->cell_agg || !L->w || !L->p_agg || !L->p_val || !L->pt_ptr || !L->pt_row ||
          !L->pt_slot || !L->pt_val || !L->ac || !L->ac_inv || (!L->gj && L->n_blocks == 0) || !L->work)
        return NFEM_ERR_INVALID_ARG;
      if (L->n_blocks < 0 || (L->n_blocks > 0 && (!L->blk_ptr || !L->blk_off || !L->agg_blk || L->blk_max < 1 ||
                                                  L->blk_max > NFEM_COARSE_BLOCK_MAX || L->ac_entries < 1)))
        return NFEM_ERR_INVALID_ARG;
      if (L->ap_ptr && (!L->ap_col || !L->ap_val || !pc->a32 || pc->a32->value_type != NFEM_F32 ||
                        pc->a32->n_rows != A64->n_rows))
        return NFEM_ERR_INVALID_ARG;
    }
    // every argument is checked before the first launch
    if (pc->n_loc < 4 || pc->n_loc > kBlkMaxN) return NFEM_ERR_UNSUPPORTED;
    if (pc->smoother) {
      const nfem_csr* S = pc->smoother;
      if (S->value_type != NFEM_F32 || S->n_rows != A64->n_rows || !S->values || S->row_ptr != A64->row_ptr ||
          S->col_idx != A64->col_idx)
        return NFEM_ERR_INVALID_ARG;
    }
    const int g = grid_for(pc->n_cells, 128);
    switch (pc->n_loc) {
      case 4: block_extract_invert<4><<<g, 128, 0, s>>>(pc->n_cells, pc->cell_dofs, A64->row_ptr, A64->col_idx,
                                                        (const double*)A64->values, pc->block_inv, dev_status); break;
      case 5: block_extract_invert<5><<<g, 128, 0, s>>>(pc->n_cells, pc->cell_dofs, A64->row_ptr, A64->col_idx,
                                                        (const double*)A64->values, pc->block_inv, dev_status); break;
      default:
        block_extract_invert_warp<<<grid_for(ceil_div(pc->n_cells, kBlkWarps), 1, 8), 32 * kBlkWarps, 0, s>>>(
            pc->n_cells, pc->n_loc, pc->cell_dofs, A64->row_ptr, A64->col_idx, (const double*)A64->values,
            pc->block_inv, dev_status);
    }
    if (pc->smoother) {
      const nfem_csr* S = pc->smoother;
      const int gr = grid_for(A64->n_rows, 256);
      if (pc->n_loc == 5)
        smoother_fill<5><<<gr, 256, 0, s>>>(A64->n_rows, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv,
                                            A64->row_ptr, A64->col_idx, pre_omega(pc), (float*)S->values,
                                            dev_status);
      else if (pc->n_loc == 4)
        smoother_fill<4><<<gr, 256, 0, s>>>(A64->n_rows, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv,
                                            A64->row_ptr, A64->col_idx, pre_omega(pc), (float*)S->values,
                                            dev_status);
      else
        smoother_fill<0><<<gr, 256, 0, s>>>(A64->n_rows, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv,
                                            A64->row_ptr, A64->col_idx, pre_omega(pc), (float*)S->values,
                                            dev_status, pc->n_loc);
    }
  } else if (pc->kind != NFEM_PC_NONE) {
    return NFEM_ERR_UNSUPPORTED;
  }
  NFEM_CHECK_LAUNCH();
  if (pc->wsqrt) {
    if (!pc->winvsqrt || !pc->setup_scratch) return NFEM_ERR_INVALID_ARG;
    const int64_t n = A64->n_rows;
    double* s2 = pc->setup_scratch;
    double* c2 = pc->setup_scratch + n;
    const int g = grid_for(n, 256);
    weights_rows<<<g, 256, 0, s>>>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, s2);
    bool have_c = false;
    if (pc->kind == NFEM_PC_CELL_BLOCK || pc->kind == NFEM_PC_TWO_LEVEL) {
      have_c = true;
      if (pc->n_loc == 5)
        weights_blockcols<5><<<g, 256, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, c2);
      else if (pc->n_loc == 4)
        weights_blockcols<4><<<g, 256, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, c2);
      else
        weights_blockcols<0><<<g, 256, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, c2,
                                               pc->n_loc);
    }
    weights_final<<<g, 256, 0, s>>>(n, s2, have_c ? c2 : nullptr, pc->wsqrt, pc->winvsqrt);
    NFEM_CHECK_LAUNCH();
  }
  if (pc->kind == NFEM_PC_TWO_LEVEL) {
    const nfem_two_level* L = pc->two_level;
    const int64_t n = A64->n_rows;
    const int na = L->n_agg;
    const int g = grid_for(n, 256);
    twolevel_fill_p<<<g, 256, 0, s>>>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, L->p_base,
                                      pc->n_cells, L->cell_agg, L->w, L->p_agg, L->p_val);
    twolevel_fill_pt<<<grid_for(L->pt_nnz, 256), 256, 0, s>>>(L->pt_nnz, L->pt_slot, L->p_val, L->pt_val);
    if (L->ap_ptr) {  // (arguments checked above)
      ap_fill_values<<<g, 256, 0, s>>>(n, pc->a32->row_ptr, pc->a32->col_idx, (const float*)pc->a32->values,
                                       L->p_agg, L->p_val, L->ap_ptr, L->ap_col, L->ap_val, dev_status);
      NFEM_CHECK_LAUNCH();
    }
    const bool blocks = L->n_blocks > 0;
    const CoarseIndex at{na, L->blk_ptr, L->blk_off, blocks ? L->agg_blk : nullptr};
    NFEM_TRY_CUDA(cudaMemsetAsync(L->ac, 0, size_t(blocks ? L->ac_entries : int64_t(na) * na) * sizeof(double), s));
    twolevel_galerkin<<<g, 256, 0, s>>>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, L->p_agg,
                                        L->p_val, at, L->ac, dev_status);
    if (blocks) {
      return block_diag_inverse(L, dev_status, s);
    }
    // blocked inversion when the scratch holds the padded matrix (n >= 64:
    // (n + 63)^2 + 64^2 entries of T fit in the 2 n^2 doubles of gj)
    const int N = int(ceil_div(na, kGjB) * kGjB);
    if (na >= kGjB && size_t(N) * N + kGjB * kGjB <= size_t(2) * na * na * (sizeof(double) / sizeof(NFEM_COARSE_T))) {
      auto* m = reinterpret_cast<NFEM_COARSE_T*>(L->gj);
      NFEM_RC(blocked_inverse<NFEM_COARSE_T>(L->ac, na, m, m + size_t(N) * N, L->ac_inv, dev_status, s));
    } else {
      gj_init<<<grid_for(int64_t(na) * 2 * na, 256), 256, 0, s>>>(L->ac, na, L->gj);
      int32_t* piv = reinterpret_cast<int32_t*>(L->work);
      for (int k = 0; k < na; ++k) {
        gj_pivot<<<1, 1024, 0, s>>>(L->gj, na, k, piv, dev_status);
        gj_eliminate<<<grid_for(int64_t(na) * (2 * na - k - 1), 256), 256, 0, s>>>(L->gj, na, k);
        gj_clear_col<<<grid_for(na, 256), 256, 0, s>>>(L->gj, na, k);
      }
      gj_extract<<<grid_for(int64_t(na) * na, 256), 256, 0, s>>>(L->gj, na, L->ac_inv);
    }
    NFEM_CHECK_LAUNCH();
  }
  return NFEM_OK;
}

// cell-block smoother: z = omega B v, or z += omega B v
static int smoother(const nfem_precond* pc, int64_t n, const float* v, float* z, float omega, int accumulate,
                    cudaStream_t s, const int32_t* gate) {
  const int B = 256;
  if (pc->smoother) {  // omega B is stored in A's pattern: one SpMV
    const nfem_csr* S = pc->smoother;
    return spmv<float, float, float>(n, S->row_ptr, S->col_idx, (const float*)S->values, v, z, accumulate ? z : nullptr,
                                     accumulate ? 2 : 0, s, nullptr, gate);
  }
  if (pc->n_loc == 5)
    block_apply<5><<<grid_for(n, B), B, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, v, z, gate,
                                                omega, accumulate);
  else if (pc->n_loc == 4)
    block_apply<4><<<grid_for(n, B), B, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, v, z, gate,
                                                omega, accumulate);
  else
    block_apply<0><<<grid_for(n, B), B, 0, s>>>(n, pc->inc_ptr, pc->inc, pc->cell_dofs, pc->block_inv, v, z, gate,
                                                omega, accumulate, pc->n_loc);
  return NFEM_OK;
}


// z = M v.  With w_out and the two-level A P, also w_out = yscale (.) A z
// (*w_done = true); the caller's SpMV is then not needed.
static int precond_apply(const nfem_precond* pc, int64_t n, const float* v, float* z, cudaStream_t s,
                         const int32_t* gate = nullptr, float* w_out = nullptr, const float* yscale = nullptr,
                         bool* w_done = nullptr) {
  if (w_done) *w_done = false;
  const int B = 256;
  switch (pc->kind) {
    case NFEM_PC_NONE:
      NFEM_TRY_CUDA(cudaMemcpyAsync(z, v, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
      return NFEM_OK;
    case NFEM_PC_JACOBI:
      jacobi_apply<<<grid_for(n, B), B, 0, s>>>(n, pc->diag_inv, v, z, gate);
      break;
    case NFEM_PC_TWO_LEVEL:
    case NFEM_PC_CELL_BLOCK:
      NFEM_RC(smoother(pc, n, v, z, pre_omega(pc), 0, s, gate));
      break;
    default:
      return NFEM_ERR_UNSUPPORTED;
  }
  NFEM_CHECK_LAUNCH();
  if (pc->kind == NFEM_PC_TWO_LEVEL) {
    // z += P Ac^-1 P^T (v - A z)
    const nfem_two_level* L = pc->two_level;
    if (!L || !pc->a32) return NFEM_ERR_INVALID_ARG;
    const int na = L->n_agg;
    float* r2 = L->work + 64;
    float* rc = r2 + n;
    float* ec = rc + na;
    // multiplicative: the coarse problem sees the smoother's residual (the
    // additive form, restricting v itself, saves this SpMV but measured 249
    // against 205 iterations and a longer solve at 64^3 x 6)
    NFEM_RC(spmv<float, float, float>(n, pc->a32->row_ptr, pc->a32->col_idx, (const float*)pc->a32->values, z, r2, v,
                                      1, s, nullptr, gate));
    // a warp per aggregate for short P^T lists (under 64 entries on
    // average), else a block per aggregate with about four entries a thread
    const int64_t avg = L->pt_nnz / na;
    if (avg < 64) {
      twolevel_restrict_warp<<<unsigned(ceil_div(int64_t(na) * 32, 256)), 256, 0, s>>>(na, L->pt_ptr, L->pt_row,
                                                                                       L->pt_val, r2, rc, gate);
    } else {
      const int threads = int(std::min<int64_t>(256, ceil_div(avg, 4 * 32) * 32));
      twolevel_restrict<<<unsigned(na), threads, 0, s>>>(na, L->pt_ptr, L->pt_row, L->pt_val, r2, rc, gate);
    }
    if (L->n_blocks > 0)
      block_gemv<<<unsigned(ceil_div(int64_t(na) * 32, 256)), 256, 0, s>>>(na, L->blk_ptr, L->blk_off, L->agg_blk,
                                                                           L->ac_inv, rc, ec, gate);
    else
      dense_gemv<<<unsigned(ceil_div(int64_t(na) * 32, 256)), 256, 0, s>>>(na, L->ac_inv, rc, ec, gate);
    if (L->post_smooth) {
      // z += omega B (v - A z) after the coarse correction (symmetric cycle)
      if (L->ap_ptr) {
        twolevel_prolong_res<<<grid_for(n, 256), 256, 0, s>>>(n, L->p_agg, L->p_val, ec, z, L->ap_ptr, L->ap_col,
                                                              L->ap_val, r2, gate);
      } else {
        twolevel_prolong<<<grid_for(n, 256), 256, 0, s>>>(n, L->p_agg, L->p_val, ec, z, gate);
        NFEM_RC(spmv<float, float, float>(n, pc->a32->row_ptr, pc->a32->col_idx, (const float*)pc->a32->values, z,
                                          r2, v, 1, s, nullptr, gate));
      }
      NFEM_RC(smoother(pc, n, r2, z, pre_omega(pc), 1, s, gate));
    } else if (w_out && L->ap_ptr) {
      twolevel_prolong_ap<<<grid_for(n, 256), 256, 0, s>>>(n, L->p_agg, L->p_val, ec, z, L->ap_ptr, L->ap_col,
                                                           L->ap_val, v, r2, yscale, w_out, gate);
      if (w_done) *w_done = true;
    } else {
      twolevel_prolong<<<grid_for(n, 256), 256, 0, s>>>(n, L->p_agg, L->p_val, ec, z, gate);
    }
    NFEM_CHECK_LAUNCH();
  }
  return NFEM_OK;
}

extern "C" int nfem_precond_apply(const nfem_precond* pc, int64_t n, const float* v, float* z, void* stream) {
  if (!pc || n < 0 || (n > 0 && (!v || !z))) return NFEM_ERR_INVALID_ARG;
  if (n == 0) return NFEM_OK;
  return precond_apply(pc, n, v, z, (cudaStream_t)stream);
}

extern "C" int nfem_two_level_ap_workspace_bytes(int64_t n_rows, size_t* bytes) {
  if (!bytes || n_rows < 0) return NFEM_ERR_INVALID_ARG;
  *bytes = align256(size_t(n_rows) * 4) + align256(size_t(n_rows + 1) * 8) + scan_workspace_bytes(n_rows) + 1024;
  return NFEM_OK;
}

extern "C" int nfem_two_level_ap_pattern(const nfem_csr* A, const nfem_two_level* L, void* workspace,
                                         size_t workspace_bytes, int32_t* ap_ptr, int32_t* ap_col,
                                         int64_t* nnz_host, int32_t* dev_status, void* stream) {
  if (!A || !L || !ap_ptr || !nnz_host || !L->p_agg || A->n_rows < 0 || !A->row_ptr || !A->col_idx)
    return NFEM_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = A->n_rows;
  const int g = grid_for(n, 128);
  if (ap_col) {
    if (n > 0) ap_fill_cols<<<g, 128, 0, s>>>(n, A->row_ptr, A->col_idx, L->p_agg, ap_ptr, ap_col, dev_status);
    NFEM_CHECK_LAUNCH();
    return NFEM_OK;
  }
  size_t need = 0;
  nfem_two_level_ap_workspace_bytes(n, &need);
  if (!workspace || workspace_bytes < need) return NFEM_ERR_WORKSPACE;
  Carver cw{reinterpret_cast<char*>(workspace), 0, workspace_bytes};
  int32_t* counts = cw.take<int32_t>(n);
  int64_t* off = cw.take<int64_t>(n + 1);
  const size_t sws_b = scan_workspace_bytes(n);
  void* sws = cw.take<char>(sws_b);
  if (!cw.ok()) return NFEM_ERR_WORKSPACE;
  if (n > 0) ap_count<<<g, 128, 0, s>>>(n, A->row_ptr, A->col_idx, L->p_agg, counts, dev_status);
  NFEM_CHECK_LAUNCH();
  NFEM_RC(exclusive_scan_i32(counts, n, off, sws, sws_b, s));
  int64_t total = 0;
  NFEM_TRY_CUDA(cudaMemcpyAsync(&total, off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  NFEM_TRY_CUDA(cudaStreamSynchronize(s));
  if (total >= INT32_MAX) return NFEM_ERR_OVERFLOW;
  offsets_i32<<<grid_for(n + 1, 256), 256, 0, s>>>(off, n + 1, ap_ptr);
  NFEM_CHECK_LAUNCH();
  *nnz_host = total;
  return NFEM_OK;
}

// workspace layout of the solver
// entries n .. ld - 1 of count vectors of stride ld set to zero
__global__ void zero_tails(float* __restrict__ base, int count, int64_t ld, int64_t n) {
  const int w = int(ld - n);
  for (int e = threadIdx.x; e < count * w; e += blockDim.x) base[int64_t(e / w) * ld + n + e % w] = 0.f;
}

struct SolveWs {
  float *V, *Z, *w, *t32, *r32, *d32;
  double *r64, *partial, *H, *cs, *sn, *g, *hist, *y, *scal;
  int32_t *status, *gate;
  unsigned int* counter;  // finish_partials (returns to 0 after every use)
};

// FP32 Krylov vectors are padded to a multiple of four entries (zero tails)
// so that the Gram-Schmidt kernels always take 16-byte rows.
static int64_t padded4(int64_t n) { return (n + 3) & ~int64_t(3); }

static size_t solve_ws_bytes(int64_t n, int m, SolveWs* out, void* base) {
  Carver c{reinterpret_cast<char*>(base), 0, ~size_t(0)};
  SolveWs w;
  const int64_t ld = padded4(n);
  w.V = c.take<float>(size_t(m + 1) * ld);
  w.Z = c.take<float>(size_t(m) * ld);
  w.w = c.take<float>(ld);
  w.t32 = c.take<float>(ld);
  w.r32 = c.take<float>(ld);
  w.d32 = c.take<float>(ld);
  w.r64 = c.take<double>(n);
  w.partial = c.take<double>(size_t(kRedBlocks) * (m + 2));
  w.H = c.take<double>(size_t(m) * (m + 1));
  w.cs = c.take<double>(m + 1);
  w.sn = c.take<double>(m + 1);
  w.g = c.take<double>(m + 2);
  w.hist = c.take<double>(m + 1);
  w.y = c.take<double>(m + 1);
  w.scal = c.take<double>(8);
  w.status = c.take<int32_t>(4);
  w.gate = c.take<int32_t>(4);
  w.counter = c.take<unsigned int>(4);
  if (out) *out = w;
  return c.off + 256;
}

// The m Arnoldi steps of one FGMRES cycle (no host synchronisation, a fixed
// launch sequence: the Givens kernel's gate ends a converged cycle's work).
static int arnoldi_steps(const nfem_precond* pc, const nfem_csr* A32, int64_t n, int64_t ld, int m, int ldh,
                         const SolveWs& w, bool weighted, int gv, cudaStream_t s) {
  const int B = 256;
  for (int j = 0; j < m; ++j) {
    float* vj = w.V + int64_t(j) * ld;
    float* zj = w.Z + int64_t(j) * ld;
    const int32_t* done = w.gate;
    // w = W^1/2 A z_j: from the two-level apply when it carries A P
    bool w_done = false;
    if (weighted) {  // w.t32 = W^-1/2 v_j, written with v_j
      NFEM_RC(precond_apply(pc, n, w.t32, zj, s, done, w.w, pc->wsqrt, &w_done));
    } else {
      NFEM_RC(precond_apply(pc, n, vj, zj, s, done, w.w, nullptr, &w_done));
    }
    if (!w_done)
      NFEM_RC(spmv<float, float, float>(n, A32->row_ptr, A32->col_idx, (const float*)A32->values, zj, w.w,
                                        nullptr, 0, s, weighted ? pc->wsqrt : nullptr, done));
    double* hcol = w.H + int64_t(j) * ldh;
    // classical Gram-Schmidt, twice (the cancellation test of a selective
    // second pass fires on nearly every Arnoldi step, so it saves nothing)
    NFEM_RC(multidot<float>(ld, j + 1, w.V, ld, w.w, w.partial, hcol, 0, s, done, w.counter));
    if (!cgs2_fused(ld, j + 1, w.V, ld, hcol, w.w, w.y, hcol + j + 1, w.partial, w.counter, s, done)) {
      multi_axpy_f32(ld, j + 1, w.V, ld, hcol, w.w, 1.0, s, done);
      NFEM_RC(multidot<float>(ld, j + 1, w.V, ld, w.w, w.partial, w.y, 0, s, done, w.counter));
      multi_axpy_f32(ld, j + 1, w.V, ld, w.y, w.w, 1.0, s, done);
      NFEM_RC(multidot<float>(ld, 1, w.w, ld, w.w, w.partial, hcol + j + 1, 1, s, done, w.counter));
    }
    scale_by_inv_w<<<gv, B, 0, s>>>(n, w.w, hcol + j + 1, w.V + int64_t(j + 1) * ld,
                                    weighted ? pc->winvsqrt : nullptr, w.t32, done);
    // h += the second pass's coefficients w.y, then the rotations
    givens_update<<<1, 32, 0, s>>>(w.H, ldh, w.y, w.cs, w.sn, w.g, j, w.hist, w.status, w.gate, w.scal + 4);
    NFEM_CHECK_LAUNCH();
  }
  return NFEM_OK;
}

// A CUDA graph of one cycle's steps, captured on a private stream.
struct CycleGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  template <typename F>
  int capture(F&& launch) {
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return NFEM_ERR_CUDA;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return NFEM_ERR_CUDA;
    const int rc = launch(cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cap, &graph);
    if (rc != NFEM_OK || e != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return rc != NFEM_OK ? rc : NFEM_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      exec = nullptr;
      return NFEM_ERR_CUDA;
    }
    return NFEM_OK;
  }
  ~CycleGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (cap) cudaStreamDestroy(cap);
  }
};

extern "C" int nfem_solve_workspace_bytes(int64_t n, int restart, size_t* bytes) {
  if (!bytes || n < 0 || restart < 1 || restart > kMaxRestart) return NFEM_ERR_INVALID_ARG;
  *bytes = solve_ws_bytes(n, restart, nullptr, nullptr);
  return NFEM_OK;
}


// device scalars of the replayed schedule (no host round trip)
__global__ void set_inner_target(double* __restrict__ target, const double* __restrict__ wr0, double rtol) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *target = rtol * *wr0;
}
__global__ void final_relres(double* __restrict__ out, const double* __restrict__ scal) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = scal[1] / (scal[0] > 0.0 ? scal[0] : 1.0);
}

// The solve's launches in a recorded schedule, with no host synchronisation
// (capturable); see nfem_solve_params.schedule_mode.
static int solve_replay(const nfem_csr* A64, const nfem_csr* A32, const nfem_precond* pc, const double* b,
                        double* x, const nfem_solve_params* prm, SolveWs& w, bool weighted, int64_t n, int64_t ld,
                        int m, int ldh, int gv, cudaStream_t s, nfem_solve_info* info) {
  const int B = 256;
  const int32_t* sch = prm->schedule;
  const int cap = prm->schedule_capacity;
  if (!sch || cap < 1 || sch[0] < 0 || !prm->relres_out) return NFEM_ERR_INVALID_ARG;
  NFEM_RC(multidot<double>(n, 1, b, n, b, w.partial, w.scal + 0, 1, s));
  NFEM_RC(spmv<double, double, double>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, x, w.r64, b, 1, s));
  NFEM_RC(multidot<double>(n, 1, w.r64, n, w.r64, w.partial, w.scal + 1, 1, s));
  int pos = 1;
  const int n_outer = sch[0];
  for (int o = 0; o < n_outer; ++o) {
    if (pos >= cap) return NFEM_ERR_INVALID_ARG;
    const int n_cycles = sch[pos++];
    info->outer_iterations++;
    cast_f64_f32<<<gv, B, 0, s>>>(n, w.r64, w.r32);
    fill_f32<<<gv, B, 0, s>>>(n, w.d32, 0.f);
    if (weighted)
      scale_vec<<<gv, B, 0, s>>>(n, pc->wsqrt, w.r32, w.V, nullptr);
    else
      NFEM_TRY_CUDA(cudaMemcpyAsync(w.V, w.r32, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    NFEM_RC(multidot<float>(ld, 1, w.V, ld, w.V, w.partial, w.scal + 3, 1, s, nullptr, w.counter));
    set_inner_target<<<1, 1, 0, s>>>(w.scal + 4, w.scal + 3, prm->inner_rtol);
    for (int c = 0; c < n_cycles; ++c) {
      if (pos >= cap) return NFEM_ERR_INVALID_ARG;
      const int k = sch[pos++];
      if (k < 1 || k > m) return NFEM_ERR_INVALID_ARG;
      if (c > 0)
        NFEM_RC(spmv<float, float, float>(n, A32->row_ptr, A32->col_idx, (const float*)A32->values, w.d32, w.V,
                                          w.r32, 1, s, weighted ? pc->wsqrt : nullptr));
      NFEM_RC(multidot<float>(ld, 1, w.V, ld, w.V, w.partial, w.scal + 2, 1, s, nullptr, w.counter));
      scale_by_inv_w<<<gv, B, 0, s>>>(n, w.V, w.scal + 2, w.V, weighted ? pc->winvsqrt : nullptr, w.t32, nullptr);
      init_cycle<<<1, 128, 0, s>>>(w.g, m, w.scal + 2, w.gate);
      NFEM_CHECK_LAUNCH();
      NFEM_RC(arnoldi_steps(pc, A32, n, ld, m, ldh, w, weighted, gv, s));
      info->inner_iterations += k;
      upper_solve<<<1, 32, 0, s>>>(w.H, ldh, w.g, k, w.y);
      multi_axpy_f32(ld, k, w.Z, ld, w.y, w.d32, -1.0, s);
      NFEM_CHECK_LAUNCH();
    }
    add_f32_to_f64<<<gv, B, 0, s>>>(n, w.d32, x);
    NFEM_RC(spmv<double, double, double>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, x, w.r64, b, 1,
                                         s));
    NFEM_RC(multidot<double>(n, 1, w.r64, n, w.r64, w.partial, w.scal + 1, 1, s));
  }
  final_relres<<<1, 1, 0, s>>>(prm->relres_out, w.scal);
  NFEM_CHECK_LAUNCH();
  info->final_relres = -1.0;  // on the device (relres_out)
  return NFEM_OK;
}

extern "C" int nfem_solve_ir_fgmres(const nfem_csr* A64, const nfem_csr* A32, const nfem_precond* pc,
                                    const double* b, double* x, const nfem_solve_params* prm, void* workspace,
                                    size_t workspace_bytes, nfem_solve_info* info, void* stream) {
  if (!A64 || !A32 || !pc || !b || !x || !prm || !info) return NFEM_ERR_INVALID_ARG;
  if (A64->value_type != NFEM_F64 || A32->value_type != NFEM_F32 || A64->n_rows != A32->n_rows)
    return NFEM_ERR_INVALID_ARG;
  const int64_t n = A64->n_rows;
  const int m = prm->restart;
  if (m < 1 || m > kMaxRestart) return NFEM_ERR_INVALID_ARG;
  if (!workspace || workspace_bytes < solve_ws_bytes(n, m, nullptr, nullptr)) return NFEM_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  SolveWs w;
  solve_ws_bytes(n, m, &w, workspace);
  const bool weighted = pc->wsqrt != nullptr && pc->winvsqrt != nullptr;
  const int B = 256;
  const int gv = grid_for(n, B);
  const int ldh = m + 1;
  NFEM_TRY_CUDA(cudaMemsetAsync(w.status, 0, 4 * sizeof(int32_t), s));
  NFEM_TRY_CUDA(cudaMemsetAsync(w.counter, 0, 4 * sizeof(unsigned int), s));
  // ld: stride of the basis vectors; entries n .. ld - 1 of every FP32 vector
  // are zero and stay zero (kernels of length n never write them, the
  // Gram-Schmidt updates of length ld add zero to them)
  const int64_t ld = padded4(n);
  if (ld > n) {
    zero_tails<<<1, 256, 0, s>>>(w.V, m + 1, ld, n);
    zero_tails<<<1, 256, 0, s>>>(w.Z, m, ld, n);
    zero_tails<<<1, 64, 0, s>>>(w.w, 1, ld, n);
    zero_tails<<<1, 64, 0, s>>>(w.t32, 1, ld, n);
    zero_tails<<<1, 64, 0, s>>>(w.r32, 1, ld, n);
    zero_tails<<<1, 64, 0, s>>>(w.d32, 1, ld, n);
  }
  info->inner_iterations = 0;
  info->outer_iterations = 0;
  info->n_snapshots = 0;
  info->status = NFEM_OK;
  if (prm->schedule_mode == 2) return solve_replay(A64, A32, pc, b, x, prm, w, weighted, n, ld, m, ldh, gv, s, info);
  // schedule recording: {n_outer, then per step n_cycles and the cycles' steps}
  const bool record = prm->schedule_mode == 1 && prm->schedule && prm->schedule_capacity > 0;
  int rec_pos = 1, rec_cycles_at = -1;
  bool rec_ok = record;
  auto rec_push = [&](int v) {
    if (!rec_ok) return;
    if (rec_pos >= prm->schedule_capacity) { rec_ok = false; return; }
    prm->schedule[rec_pos++] = v;
  };
  double hb[2];
  // ||b||
  NFEM_RC(multidot<double>(n, 1, b, n, b, w.partial, w.scal + 0, 1, s));
  NFEM_RC(spmv<double, double, double>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, x, w.r64, b, 1, s));
  NFEM_RC(multidot<double>(n, 1, w.r64, n, w.r64, w.partial, w.scal + 1, 1, s));
  NFEM_TRY_CUDA(cudaMemcpyAsync(hb, w.scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  NFEM_TRY_CUDA(cudaStreamSynchronize(s));
  const double nb = hb[0] > 0.0 ? hb[0] : 1.0;
  double rel = hb[1] / nb;
  info->initial_relres = rel;
  std::vector<double> hist(m + 1);
  const bool graphs = prm->no_graphs == 0;
  CycleGraph cycle_graph;
  bool first_solve_cycle = true;
  while (rel > prm->rtol && info->outer_iterations < prm->max_outer &&
         info->inner_iterations < prm->max_inner) {
    info->outer_iterations++;
    rec_cycles_at = rec_pos;
    rec_push(0);
    // inner problem A32 d = r32, d0 = 0
    cast_f64_f32<<<gv, B, 0, s>>>(n, w.r64, w.r32);
    fill_f32<<<gv, B, 0, s>>>(n, w.d32, 0.f);
    if (weighted)
      scale_vec<<<gv, B, 0, s>>>(n, pc->wsqrt, w.r32, w.V, nullptr);
    else
      NFEM_TRY_CUDA(cudaMemcpyAsync(w.V, w.r32, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    // the inner solve reduces the W-weighted residual norm by inner_rtol;
    // the outer loop measures the true FP64 residual
    NFEM_RC(multidot<float>(ld, 1, w.V, ld, w.V, w.partial, w.scal + 3, 1, s, nullptr, w.counter));
    double wr0 = 0.0;
    NFEM_TRY_CUDA(cudaMemcpyAsync(&wr0, w.scal + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    NFEM_TRY_CUDA(cudaStreamSynchronize(s));
    const double inner_target = prm->inner_rtol * wr0;
    set_scalar<<<1, 1, 0, s>>>(w.scal + 4, inner_target);  // read by the Givens kernel
    double inner_res = wr0;
    bool inner_done = wr0 == 0.0;
    bool first_cycle = true;
    while (!inner_done && info->inner_iterations < prm->max_inner) {
      // V0 = W^1/2 (r32 - A32 d32) after the first cycle
      if (!first_cycle) {
        NFEM_RC(spmv<float, float, float>(n, A32->row_ptr, A32->col_idx, (const float*)A32->values, w.d32, w.V,
                                          w.r32, 1, s, weighted ? pc->wsqrt : nullptr));
      }
      first_cycle = false;
      NFEM_RC(multidot<float>(ld, 1, w.V, ld, w.V, w.partial, w.scal + 2, 1, s, nullptr, w.counter));
      // V0 = V0 / ||V0||, and the first preconditioner input W^-1/2 V0
      scale_by_inv_w<<<gv, B, 0, s>>>(n, w.V, w.scal + 2, w.V, weighted ? pc->winvsqrt : nullptr, w.t32, nullptr);
      init_cycle<<<1, 128, 0, s>>>(w.g, m, w.scal + 2, w.gate);
      NFEM_CHECK_LAUNCH();
      // Second cycle onwards: the m steps as one CUDA graph, captured once on
      // a private stream (the caller's may be the legacy stream) and
      // replayed on `s` every cycle; the launch sequence is fixed (the gate
      // ends a converged cycle's work on the device).  Large systems capture
      // it right after launching the first cycle, so the host's capture and
      // instantiation overlap that cycle on the GPU; small ones at the second
      // cycle, so a solve of one cycle captures nothing.
      auto capture = [&]() {
        return cycle_graph.capture([&](cudaStream_t cs_) {
          return arnoldi_steps(pc, A32, n, ld, m, ldh, w, weighted, gv, cs_);
        });
      };
      const bool early_capture = n >= (int64_t(1) << 20);
      if (graphs && cycle_graph.exec == nullptr && !first_solve_cycle && !early_capture) NFEM_RC(capture());
      if (cycle_graph.exec) {
        NFEM_TRY_CUDA(cudaGraphLaunch(cycle_graph.exec, s));
      } else {
        NFEM_RC(arnoldi_steps(pc, A32, n, ld, m, ldh, w, weighted, gv, s));
        if (graphs && early_capture && cycle_graph.exec == nullptr) NFEM_RC(capture());
      }
      first_solve_cycle = false;
      // one synchronisation per cycle: residual estimates of every step
      NFEM_TRY_CUDA(cudaMemcpyAsync(hist.data(), w.hist, m * sizeof(double), cudaMemcpyDeviceToHost, s));
      NFEM_TRY_CUDA(cudaStreamSynchronize(s));
      int k = m;
      for (int i = 0; i < m; ++i) {
        if (hist[i] <= inner_target || !std::isfinite(hist[i])) { k = i + 1; break; }
      }
      info->inner_iterations += k;
      inner_res = hist[k - 1];
      rec_push(k);
      if (rec_ok) prm->schedule[rec_cycles_at]++;
      upper_solve<<<1, 32, 0, s>>>(w.H, ldh, w.g, k, w.y);
      // d += Z y   (multi_axpy subtracts: pass -1 via hsign)
      multi_axpy_f32(ld, k, w.Z, ld, w.y, w.d32, -1.0, s);
      NFEM_CHECK_LAUNCH();
      if (prm->snapshots && info->n_snapshots < prm->max_snapshots) {
        snapshot_kernel<<<gv, B, 0, s>>>(n, x, w.d32, prm->snapshots + int64_t(info->n_snapshots) * n);
        info->n_snapshots++;
      }
      if (!std::isfinite(inner_res)) {
        info->status = NFEM_ERR_NONFINITE;
        return NFEM_ERR_NONFINITE;
      }
      if (inner_res <= inner_target) inner_done = true;
    }
    add_f32_to_f64<<<gv, B, 0, s>>>(n, w.d32, x);
    NFEM_RC(spmv<double, double, double>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, x, w.r64, b, 1,
                                         s));
    NFEM_RC(multidot<double>(n, 1, w.r64, n, w.r64, w.partial, w.scal + 1, 1, s));
    NFEM_TRY_CUDA(cudaMemcpyAsync(hb + 1, w.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    NFEM_TRY_CUDA(cudaStreamSynchronize(s));
    rel = hb[1] / nb;
    if (!std::isfinite(rel)) {
      info->status = NFEM_ERR_NONFINITE;
      info->final_relres = rel;
      return NFEM_ERR_NONFINITE;
    }
  }
  info->final_relres = rel;
  if (record) prm->schedule[0] = rec_ok ? info->outer_iterations : -1;
  int32_t st = 0;
  NFEM_TRY_CUDA(cudaMemcpyAsync(&st, w.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  NFEM_TRY_CUDA(cudaStreamSynchronize(s));
  if (rel > prm->rtol) info->status = st ? st : NFEM_ERR_NOT_CONVERGED;
  return info->status;
}
