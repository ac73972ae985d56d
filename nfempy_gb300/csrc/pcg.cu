// Preconditioned conjugate gradients for symmetric positive definite
// systems, FP32 inner iterations inside FP64 iterative refinement.
//
// Reference: the P2 elasticity driver solves with PETSc CG and an
// incomplete-Cholesky preconditioner
// (examples/cauchy_elasticity/cg_elasticity_example_1.py:159-170).  The
// triangular solves of ICC are sequential; the GPU form keeps CG and uses a
// block-diagonal preconditioner: point Jacobi, or the inverse of the 3 x 3
// diagonal block of every node (the three components of a vector P2 node,
// DoF = 3 node + component) for vector fields.
//
// Outer step (FP64): r = b - A x on the FP64 matrix; stop when
// ||r|| / ||b|| <= rtol; else solve A e = r / ||r|| with CG on the FP32 copy
// of A to the inner tolerance and add ||r|| e to x.
// Inner CG: one SpMV, one dot, one fused update (x, r, z = M r, r.z, r.r)
// and one fused direction update per iteration.  Reductions: per-block
// partial sums of a fixed grid, summed in a fixed order by every block that
// needs them (bitwise deterministic, no atomics, no host round trip).
// Convergence is read on the host every kCheck iterations.
#include "nfem_common.cuh"

namespace nfem {
namespace {

constexpr int kCgThreads = 256;
constexpr int kCgBlocks = 608;  // 4 x 152 SMs: the fixed grid of every reduction
constexpr int kCheck = 16;      // iterations between host convergence checks

__device__ __forceinline__ double cg_block_sum(double v, double* sh) {
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
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  t = sh[32];
  __syncthreads();
  return t;
}

// sum of the kCgBlocks partials, in the same order in every block
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < kCgBlocks; i += blockDim.x) v += part[i];
  return cg_block_sum(v, sh);
}

template <typename A, typename B>
__global__ void __launch_bounds__(kCgThreads) dot_kernel(int64_t n, const A* __restrict__ a, const B* __restrict__ b,
                                                         double* __restrict__ partial) {
  __shared__ double sh[33];
  double v = 0.0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    v += double(a[i]) * double(b[i]);
  v = cg_block_sum(v, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

// scal[slot] = sum of the partials (one block)
__global__ void finalize_kernel(const double* __restrict__ part, double* __restrict__ scal, int slot) {
  __shared__ double sh[33];
  const double v = sum_partials(part, sh);
  if (threadIdx.x == 0) scal[slot] = v;
}

// z = M r for the units [u0, u1) of this thread's grid stride; PC 0: point
// Jacobi (inv[i] = 1 / a_ii); PC 1: node blocks (inv[9 v ..] = the inverse of
// the 3 x 3 diagonal block of node v, rows 3 v .. 3 v + 2).  Also r.z, r.r.
template <int PC>
__device__ __forceinline__ void precond_unit(int64_t u, const float* __restrict__ r, float* __restrict__ z,
                                             const float* __restrict__ inv, double& rz, double& rr) {
  if constexpr (PC == 0) {
    const float ri = r[u];
    const float zi = inv[u] * ri;
    z[u] = zi;
    rz += double(ri) * zi;
    rr += double(ri) * ri;
  } else {
    const float r0 = r[3 * u], r1 = r[3 * u + 1], r2 = r[3 * u + 2];
    const float* m = inv + 9 * u;
    const float z0 = m[0] * r0 + m[1] * r1 + m[2] * r2;
    const float z1 = m[3] * r0 + m[4] * r1 + m[5] * r2;
    const float z2 = m[6] * r0 + m[7] * r1 + m[8] * r2;
    z[3 * u] = z0;
    z[3 * u + 1] = z1;
    z[3 * u + 2] = z2;
    rz += double(r0) * z0 + double(r1) * z1 + double(r2) * z2;
    rr += double(r0) * r0 + double(r1) * r1 + double(r2) * r2;
  }
}

// start: z = M r, partials of r.z and r.r (x = 0, r = the scaled residual)
template <int PC>
__global__ void __launch_bounds__(kCgThreads) cg_start_kernel(int64_t units, const float* __restrict__ r,
                                                              float* __restrict__ z, float* __restrict__ p,
                                                              const float* __restrict__ inv, double* rz_part,
                                                              double* rr_part) {
  __shared__ double sh[33];
  double rz = 0.0, rr = 0.0;
  for (int64_t u = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; u < units; u += int64_t(gridDim.x) * blockDim.x) {
    precond_unit<PC>(u, r, z, inv, rz, rr);
    const int w = PC == 0 ? 1 : 3;
#pragma unroll
    for (int k = 0; k < w; ++k) p[w * u + k] = z[w * u + k];  // p = z, the rows this thread just wrote
  }
  rz = cg_block_sum(rz, sh);
  rr = cg_block_sum(rr, sh);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = rz;
    rr_part[blockIdx.x] = rr;
  }
}

// alpha = rz / (p . q); x += alpha p; r -= alpha q; z = M r; partials of r.z, r.r
template <int PC>
__global__ void __launch_bounds__(kCgThreads)
    cg_update_kernel(int64_t units, const double* __restrict__ scal_cur, const double* __restrict__ pq_part,
                     float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
                     const float* __restrict__ q, float* __restrict__ z, const float* __restrict__ inv,
                     double* rz_part, double* rr_part, int32_t* status) {
  __shared__ double sh[33];
  const double pq = sum_partials(pq_part, sh);
  const double rz_old = scal_cur[0];
  if (rz_old == 0.0) {  // r = 0: converged exactly, nothing to update
    if (threadIdx.x == 0) rz_part[blockIdx.x] = rr_part[blockIdx.x] = 0.0;
    return;
  }
  if (!(pq > 0.0) || !isfinite(pq)) {  // A not positive definite on p, or a non-finite value
    if (blockIdx.x == 0 && threadIdx.x == 0) set_status(status, NFEM_ERR_BREAKDOWN);
    return;
  }
  const float alpha = float(rz_old / pq);
  double rz = 0.0, rr = 0.0;
  for (int64_t u = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; u < units; u += int64_t(gridDim.x) * blockDim.x) {
    const int w = PC == 0 ? 1 : 3;
#pragma unroll
    for (int k = 0; k < w; ++k) {
      const int64_t i = w * u + k;
      x[i] = fmaf(alpha, p[i], x[i]);
      r[i] = fmaf(-alpha, q[i], r[i]);
    }
    precond_unit<PC>(u, r, z, inv, rz, rr);
  }
  rz = cg_block_sum(rz, sh);
  rr = cg_block_sum(rr, sh);
  if (threadIdx.x == 0) {
    rz_part[blockIdx.x] = rz;
    rr_part[blockIdx.x] = rr;
  }
}

// beta = rz_new / rz_old; p = z + beta p; block 0 stores rz_new, rr_new
__global__ void __launch_bounds__(kCgThreads)
    cg_direction_kernel(int64_t n, const double* __restrict__ scal_cur, double* __restrict__ scal_next,
                        const double* __restrict__ rz_part, const double* __restrict__ rr_part,
                        const float* __restrict__ z, float* __restrict__ p, const int32_t* __restrict__ status) {
  __shared__ double sh[33];
  if (*status) return;
  const double rz_new = sum_partials(rz_part, sh);
  const double rr_new = sum_partials(rr_part, sh);
  const float beta = scal_cur[0] != 0.0 ? float(rz_new / scal_cur[0]) : 0.f;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    p[i] = fmaf(beta, p[i], z[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal_next[0] = rz_new;
    scal_next[1] = rr_new;
  }
}

__global__ void scale_to_f32_kernel(int64_t n, const double* __restrict__ r, const double* __restrict__ scal,
                                    float* __restrict__ r32, float* __restrict__ x32) {
  const double inv = 1.0 / sqrt(scal[0]);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    r32[i] = float(r[i] * inv);
    x32[i] = 0.f;
  }
}

__global__ void correct_kernel(int64_t n, const double* __restrict__ scal, const float* __restrict__ e,
                               double* __restrict__ x) {
  const double s = sqrt(scal[0]);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] += s * double(e[i]);
}

// point Jacobi: inv[i] = 1 / a_ii (FP64 matrix); zero or missing diagonal: degenerate
__global__ void jacobi_inv_kernel(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                  const double* __restrict__ v, float* __restrict__ inv, int32_t* status) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
      if (ci[k] == i) d = v[k];
    if (!(d != 0.0) || !isfinite(d)) set_status(status, NFEM_ERR_DEGENERATE);
    inv[i] = float(1.0 / d);
  }
}

// node blocks: the 3 x 3 diagonal block of node u (rows and columns 3 u ..
// 3 u + 2), inverted in FP64 by cofactors, stored FP32 row-major
__global__ void node_block_inv_kernel(int64_t n_nodes, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                      const double* __restrict__ v, float* __restrict__ inv, int32_t* status) {
  for (int64_t u = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; u < n_nodes; u += int64_t(gridDim.x) * blockDim.x) {
    double B[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < 3; ++i) {
      const int64_t row = 3 * u + i;
      int32_t lo = rp[row], hi = rp[row + 1];
      const int32_t end = hi;
      const int32_t c0 = int32_t(3 * u);
      while (lo < hi) {  // first column >= 3 u
        const int32_t mid = (lo + hi) >> 1;
        if (ci[mid] < c0) lo = mid + 1; else hi = mid;
      }
      for (int32_t k = lo; k < end && ci[k] < c0 + 3; ++k) B[i][ci[k] - c0] = v[k];
    }
    const double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
    const double c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
    const double c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
    const double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
    if (!(det != 0.0) || !isfinite(det)) set_status(status, NFEM_ERR_DEGENERATE);
    const double id = 1.0 / det;
    float* m = inv + 9 * u;
    m[0] = float(c00 * id);
    m[1] = float((B[0][2] * B[2][1] - B[0][1] * B[2][2]) * id);
    m[2] = float((B[0][1] * B[1][2] - B[0][2] * B[1][1]) * id);
    m[3] = float(c01 * id);
    m[4] = float((B[0][0] * B[2][2] - B[0][2] * B[2][0]) * id);
    m[5] = float((B[0][2] * B[1][0] - B[0][0] * B[1][2]) * id);
    m[6] = float(c02 * id);
    m[7] = float((B[0][1] * B[2][0] - B[0][0] * B[2][1]) * id);
    m[8] = float((B[0][0] * B[1][1] - B[0][1] * B[1][0]) * id);
  }
}

struct CgWork {
  double* r64;
  float *x32, *r32, *z32, *p32, *q32;
  double *pq_part, *rz_part, *rr_part;
  double* scal;  // [0..1] current (rz, rr), [2..3] next, [4] ||r64||^2, [5] ||b||^2
};

size_t cg_bytes(int64_t n) {
  return align256(size_t(n) * 8) + 5 * align256(size_t(n) * 4) + 3 * align256(size_t(kCgBlocks) * 8) + 256 + 1024;
}

CgWork carve(void* ws, int64_t n) {
  Carver c{static_cast<char*>(ws), 0, cg_bytes(n)};
  CgWork w;
  w.r64 = c.take<double>(size_t(n));
  w.x32 = c.take<float>(size_t(n));
  w.r32 = c.take<float>(size_t(n));
  w.z32 = c.take<float>(size_t(n));
  w.p32 = c.take<float>(size_t(n));
  w.q32 = c.take<float>(size_t(n));
  w.pq_part = c.take<double>(kCgBlocks);
  w.rz_part = c.take<double>(kCgBlocks);
  w.rr_part = c.take<double>(kCgBlocks);
  w.scal = c.take<double>(8);
  return w;
}

}  // namespace
}  // namespace nfem

using namespace nfem;

extern "C" int nfem_pcg_setup(int pc_kind, const nfem_csr* A64, float* inv, int32_t* dev_status, void* stream) {
  if (!A64 || A64->value_type != NFEM_F64 || !inv || A64->n_rows < 0) return NFEM_ERR_INVALID_ARG;
  const int64_t n = A64->n_rows;
  if (n == 0) return NFEM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (pc_kind == NFEM_PC_JACOBI) {
    jacobi_inv_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, A64->row_ptr, A64->col_idx, (const double*)A64->values,
                                                        inv, dev_status);
  } else if (pc_kind == NFEM_PC_NODE_BLOCK) {
    if (n % 3) return NFEM_ERR_UNSUPPORTED;
    node_block_inv_kernel<<<grid_for(n / 3, 256), 256, 0, s>>>(n / 3, A64->row_ptr, A64->col_idx,
                                                                (const double*)A64->values, inv, dev_status);
  } else {
    return NFEM_ERR_UNSUPPORTED;
  }
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_pcg_workspace_bytes(int64_t n_rows, size_t* bytes) {
  if (!bytes || n_rows < 0) return NFEM_ERR_INVALID_ARG;
  *bytes = cg_bytes(n_rows);
  return NFEM_OK;
}

extern "C" int nfem_solve_ir_pcg(const nfem_csr* A64, const nfem_csr* A32, int pc_kind, const float* inv,
                                 const double* b, double* x, double rtol, double inner_rtol, int max_inner,
                                 int max_outer, void* workspace, size_t workspace_bytes, nfem_solve_info* info,
                                 int32_t* dev_status, void* stream) {
  if (!A64 || !A32 || !b || !x || !info || !inv || !dev_status || A64->value_type != NFEM_F64 ||
      A32->value_type != NFEM_F32 || A64->n_rows != A32->n_rows || !(rtol > 0) || !(inner_rtol > 0) ||
      max_inner < 1 || max_outer < 1)
    return NFEM_ERR_INVALID_ARG;
  if (pc_kind != NFEM_PC_JACOBI && pc_kind != NFEM_PC_NODE_BLOCK) return NFEM_ERR_UNSUPPORTED;
  const int64_t n = A64->n_rows;
  if (pc_kind == NFEM_PC_NODE_BLOCK && n % 3) return NFEM_ERR_UNSUPPORTED;
  *info = nfem_solve_info{0, 0, 0.0, 0.0, NFEM_OK, 0};
  if (n == 0) return NFEM_OK;
  if (!workspace || workspace_bytes < cg_bytes(n) || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return NFEM_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  CgWork w = carve(workspace, n);
  const int64_t units = pc_kind == NFEM_PC_JACOBI ? n : n / 3;
  const int g = kCgBlocks;
  auto host_scalar = [&](const double* dptr, double& out) -> int {
    NFEM_TRY_CUDA(cudaMemcpyAsync(&out, dptr, sizeof(double), cudaMemcpyDeviceToHost, s));
    NFEM_TRY_CUDA(cudaStreamSynchronize(s));
    return NFEM_OK;
  };
  int rc;
  // ||b||^2
  dot_kernel<double, double><<<g, kCgThreads, 0, s>>>(n, b, b, w.pq_part);
  finalize_kernel<<<1, kCgThreads, 0, s>>>(w.pq_part, w.scal, 5);
  NFEM_CHECK_LAUNCH();
  double bb = 0.0;
  if ((rc = host_scalar(w.scal + 5, bb))) return rc;
  if (!isfinite(bb)) return NFEM_ERR_NONFINITE;
  if (bb == 0.0) {
    NFEM_TRY_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), s));
    return NFEM_OK;
  }
  const double nb = sqrt(bb);
  int inner_total = 0;
  for (int outer = 0;; ++outer) {
    // r64 = b - A64 x, its norm
    if ((rc = nfem_residual_f64(n, A64->row_ptr, A64->col_idx, (const double*)A64->values, x, b, w.r64, stream)))
      return rc;
    dot_kernel<double, double><<<g, kCgThreads, 0, s>>>(n, w.r64, w.r64, w.pq_part);
    finalize_kernel<<<1, kCgThreads, 0, s>>>(w.pq_part, w.scal, 4);
    NFEM_CHECK_LAUNCH();
    double rr64 = 0.0;
    if ((rc = host_scalar(w.scal + 4, rr64))) return rc;
    if (!isfinite(rr64)) {
      info->status = NFEM_ERR_NONFINITE;
      return NFEM_ERR_NONFINITE;
    }
    const double rel = sqrt(rr64) / nb;
    if (outer == 0) info->initial_relres = rel;
    info->final_relres = rel;
    info->outer_iterations = outer;
    info->inner_iterations = inner_total;
    if (rel <= rtol) return NFEM_OK;
    if (outer >= max_outer || inner_total >= max_inner) {
      info->status = NFEM_ERR_NOT_CONVERGED;
      return NFEM_ERR_NOT_CONVERGED;
    }
    // inner CG on A32 e = r64 / ||r64||, e0 = 0
    scale_to_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, w.r64, w.scal + 4, w.r32, w.x32);
    if (pc_kind == NFEM_PC_JACOBI)
      cg_start_kernel<0><<<g, kCgThreads, 0, s>>>(units, w.r32, w.z32, w.p32, inv, w.rz_part, w.rr_part);
    else
      cg_start_kernel<1><<<g, kCgThreads, 0, s>>>(units, w.r32, w.z32, w.p32, inv, w.rz_part, w.rr_part);
    finalize_kernel<<<1, kCgThreads, 0, s>>>(w.rz_part, w.scal, 0);
    finalize_kernel<<<1, kCgThreads, 0, s>>>(w.rr_part, w.scal, 1);
    NFEM_CHECK_LAUNCH();
    double rr0 = 0.0;
    if ((rc = host_scalar(w.scal + 1, rr0))) return rc;
    double* cur = w.scal;
    double* nxt = w.scal + 2;
    const double target = inner_rtol * inner_rtol * rr0;
    for (int it = 0; inner_total < max_inner; ++it) {
      if ((rc = nfem_spmv(NFEM_F32, n, A32->row_ptr, A32->col_idx, A32->values, w.p32, w.q32, stream))) return rc;
      dot_kernel<float, float><<<g, kCgThreads, 0, s>>>(n, w.p32, w.q32, w.pq_part);
      if (pc_kind == NFEM_PC_JACOBI)
        cg_update_kernel<0><<<g, kCgThreads, 0, s>>>(units, cur, w.pq_part, w.x32, w.r32, w.p32, w.q32, w.z32, inv,
                                                      w.rz_part, w.rr_part, dev_status);
      else
        cg_update_kernel<1><<<g, kCgThreads, 0, s>>>(units, cur, w.pq_part, w.x32, w.r32, w.p32, w.q32, w.z32, inv,
                                                      w.rz_part, w.rr_part, dev_status);
      cg_direction_kernel<<<g, kCgThreads, 0, s>>>(n, cur, nxt, w.rz_part, w.rr_part, w.z32, w.p32, dev_status);
      NFEM_CHECK_LAUNCH();
      double* t = cur;
      cur = nxt;
      nxt = t;
      ++inner_total;
      if ((it + 1) % kCheck == 0 || inner_total >= max_inner) {
        double rr = 0.0;
        int32_t st = 0;
        NFEM_TRY_CUDA(cudaMemcpyAsync(&st, dev_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        if ((rc = host_scalar(cur + 1, rr))) return rc;
        if (st) {
          info->status = st;
          info->inner_iterations = inner_total;
          return st;
        }
        if (!isfinite(rr)) {
          info->status = NFEM_ERR_NONFINITE;
          return NFEM_ERR_NONFINITE;
        }
        if (rr <= target) break;
      }
    }
    // x += ||r64|| e
    correct_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, w.scal + 4, w.x32, x);
    NFEM_CHECK_LAUNCH();
  }
}
