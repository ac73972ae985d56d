// Vector P2 linear elasticity: element integrals + CSR scatter (row owner),
// and the boundary penalty form.
//
// Reference: LEPrimalWeakForm.evaluate_form
// (src/weak_forms/le_primal_weak_form.py:10-129): for basis a, component i
// and basis b, component j,
//   j[(a,i),(b,j)] = int mu (grad phi_a . grad phi_b) delta_ij
//                  + mu d_j phi_a d_i phi_b + lambda d_i phi_a d_j phi_b
//   r[(a,i)]       = + int f_i phi_a        (alpha = 0)
// LEPrimalWeakFormBCDirichlet (le_primal_weak_form.py:131-177): on boundary
// facets j[(a,i),(b,i)] += beta int phi_a phi_b, beta = 1e12 (u_D = 0 here).
//
// Closed form on affine cells with cell-wise constant lambda, mu:
//   A_ab[p][q] = int d_p phi_a d_q phi_b = |det J| (J^-T S_ab J^-1)_pq,
//   S_ab[k][l] = int_ref dhat_k phihat_a dhat_l phihat_b  (exact reference table),
//   K_ab[i][j] = mu delta_ij tr(A_ab) + mu A_ab[j][i] + lambda A_ab[i][j].
//
// GPU design: one warp per node owns the node's three component rows (they
// are consecutive in the CSR and share one column structure of 3 x deg
// entries).  Three groups of ten lanes each take one (cell, local node a)
// incidence per step; lane b of a group evaluates the 3 x 3 block K_ab and
// adds it into its group's shared-memory image of the three rows at the node
// position given by the 8-bit node codes.  The three images are summed in a
// fixed order and stored coalesced: each value written once, no atomics,
// bitwise deterministic.
#include <string.h>

#include <mutex>

#include "nfem_common.cuh"

namespace nfem {

constexpr int kElasDegMax = 96;  // node columns per node row
#ifndef NFEM_ELAS_WARPS
#define NFEM_ELAS_WARPS 4
#endif
constexpr int kElasWarps32 = NFEM_ELAS_WARPS;
constexpr int kElasWarps64 = 2;

__constant__ double c_S[10 * 10 * 9];
__constant__ double c_m[10];
__constant__ double c_Mf[6 * 6];

static double h_S[10 * 10 * 9], h_m[10], h_Mf[36];
static bool h_tables_set = false;
static std::mutex h_tables_mutex;

static int upload_tables(const double* S, const double* m, const double* Mf, cudaStream_t s) {
  std::lock_guard<std::mutex> lock(h_tables_mutex);
  if (h_tables_set && !memcmp(S, h_S, sizeof(h_S)) && !memcmp(m, h_m, sizeof(h_m)) &&
      (!Mf || !memcmp(Mf, h_Mf, sizeof(h_Mf))))
    return NFEM_OK;
  memcpy(h_S, S, sizeof(h_S));
  memcpy(h_m, m, sizeof(h_m));
  if (Mf) memcpy(h_Mf, Mf, sizeof(h_Mf));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_S, h_S, sizeof(h_S), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_m, h_m, sizeof(h_m), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_Mf, h_Mf, sizeof(h_Mf), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaStreamSynchronize(s));
  h_tables_set = true;
  return NFEM_OK;
}

struct ElasParams {
  int64_t n_nodes;
  int deg_max;  // largest node degree (columns / 3) of any node row
  // rows a kernel takes by node degree: 0 every row, 1 degree <= 32 only,
  // 2 degree > 32 only (the split form: register rows for the short edge
  // rows, shared-memory images for the long vertex rows)
  int deg_filter;
  int64_t n_cells;
  void* geom;  // [n_cells][12]: J^-1 (row-major, 9), lambda |det J|, mu |det J|, |det J|
  int64_t row0;  // first row of the space (dof_shift)
  const double* points;
  const float* split;
  const int32_t* cv;
  const void* lam;
  const void* mu;
  const void* force;
  const int32_t* inc_ptr;
  const int32_t* inc;
  const uint8_t* codes;
  const int32_t* row_ptr;
  void* values;
  void* rhs;
  int accumulate;
  int32_t* status;
};

template <typename T>
__device__ __forceinline__ void tet_edges(const ElasParams& p, int32_t c, T (&J)[3][3]);

template <>
__device__ __forceinline__ void tet_edges<double>(const ElasParams& p, int32_t c, double (&J)[3][3]) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const int vs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      J[d][k] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - __ldg(p.points + int64_t(vs[0]) * 3 + d);
}

template <>
__device__ __forceinline__ void tet_edges<float>(const ElasParams& p, int32_t c, float (&J)[3][3]) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const float s = packed_lo_scale(p.split);
  const float4 r0 = packed_point(p.split, v.x), r1 = packed_point(p.split, v.y), r2 = packed_point(p.split, v.z),
               r3 = packed_point(p.split, v.w);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    J[d][0] = packed_diff(r1, r0, d, s);
    J[d][1] = packed_diff(r2, r0, d, s);
    J[d][2] = packed_diff(r3, r0, d, s);
  }
}

// J^-1 (row-major, g[0..8]) and det J of the edge matrix J (columns = edges)
template <typename T>
__device__ __forceinline__ T inverse_det(const T (&J)[3][3], T (&g)[12]) {
  const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const T det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const T id = T(1) / det;
  g[0] = c00 * id;
  g[3] = c01 * id;
  g[6] = c02 * id;
  g[1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  g[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  g[7] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  g[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  g[5] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  g[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

// Badly shaped cells in FP32: det J and J^-1 from FP32 edges carry a
// relative error of a few ulps over the shape quality q = |det J| /
// (|e_0| |e_1| |e_2|), and an edge shorter than 2^20 units of the
// fixed-point records a relative error above 2^-21 from their rounding;
// cells with q < 0.1 or such an edge take both in FP64, from the FP64
// points when the caller passed them, else from the fixed-point records'
// exact integer differences, rounded to FP32 once at the end.
constexpr float kElasSliverQ = 0.1f;

__device__ __noinline__ float refine_inverse(const ElasParams& p, int32_t c, float (&gf)[12]) {
  double J[3][3];
  if (p.points) {
    tet_edges<double>(p, c, J);
  } else {
    const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
    const double s = double(packed_lo_scale(p.split));
    const float4 r0 = packed_point(p.split, v.x);
    const float4 r[3] = {packed_point(p.split, v.y), packed_point(p.split, v.z), packed_point(p.split, v.w)};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      J[0][k] = double(int64_t(__float_as_int(r[k].x)) - __float_as_int(r0.x)) * s;
      J[1][k] = double(int64_t(__float_as_int(r[k].y)) - __float_as_int(r0.y)) * s;
      J[2][k] = double(int64_t(__float_as_int(r[k].z)) - __float_as_int(r0.z)) * s;
    }
  }
  double g[12];
  const double det = inverse_det<double>(J, g);
#pragma unroll
  for (int k = 0; k < 9; ++k) gf[k] = float(g[k]);
  return float(det);
}

// Per-cell geometry, once per cell (every cell is read by the rows of its
// ten nodes): J^-1, lambda |det J|, mu |det J|, |det J|.
template <typename T>
__global__ void elas_geom_kernel(const ElasParams p) {
  const T* lam = static_cast<const T*>(p.lam);
  const T* mu = static_cast<const T*>(p.mu);
  T* out = static_cast<T*>(p.geom);
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < p.n_cells;
       c += int64_t(gridDim.x) * blockDim.x) {
    T J[3][3];
    tet_edges<T>(p, int32_t(c), J);
    T g[12];
    T det = inverse_det<T>(J, g);
    if constexpr (sizeof(T) == 4) {
      const T n0 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
      const T n1 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
      const T n2 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
      const T q = (det < T(0) ? -det : det) * rsqrtf(n0) * rsqrtf(n1) * rsqrtf(n2);
      const float s = packed_lo_scale(p.split) * 1048576.0f;  // 2^20 units
      const T n_min = fminf(n0, fminf(n1, n2));
      if (q < T(kElasSliverQ) || n_min < s * s) det = refine_inverse(p, int32_t(c), g);
    }
    if (!(det != T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
    const T adet = det < T(0) ? -det : det;
    const T lam_c = __ldg(lam + c), mu_c = __ldg(mu + c);
    check_finite(p.status, lam_c);
    check_positive(p.status, mu_c);
    g[9] = lam_c * adet;
    g[10] = mu_c * adet;
    g[11] = adet;
#pragma unroll
    for (int k = 0; k < 12; ++k) out[c * 12 + k] = g[k];
  }
}

template <typename T>
__device__ __forceinline__ void load_geom(const ElasParams& p, int32_t c, T (&g)[12]);
template <>
__device__ __forceinline__ void load_geom<float>(const ElasParams& p, int32_t c, float (&g)[12]) {
  const float4* q = static_cast<const float4*>(p.geom) + int64_t(c) * 3;
  const float4 a = __ldg(q), b = __ldg(q + 1), d = __ldg(q + 2);
  g[0] = a.x; g[1] = a.y; g[2] = a.z; g[3] = a.w;
  g[4] = b.x; g[5] = b.y; g[6] = b.z; g[7] = b.w;
  g[8] = d.x; g[9] = d.y; g[10] = d.z; g[11] = d.w;
}
template <>
__device__ __forceinline__ void load_geom<double>(const ElasParams& p, int32_t c, double (&g)[12]) {
  const double2* q = static_cast<const double2*>(p.geom) + int64_t(c) * 6;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double2 v = __ldg(q + k);
    g[2 * k] = v.x;
    g[2 * k + 1] = v.y;
  }
}

// Row images: per warp, per group, rows i = 0..2 of the node, one 4-wide slot
// per node column (the column's components j = 0..2 and a pad), so a 3 x 3
// block is added with three 16-byte read-modify-writes.
// NFEM_ELAS_IMAGES: 3 = one image per group (the groups add at once, and
// the images are summed at the end); 1 = one image per warp, the groups'
// read-modify-writes in turn (a third of the shared memory per warp, so
// twice the resident warps).  Measured at 40^3 x 6 FP32: 3 images 0.690 ms,
// 1 image 0.612 ms.
#ifndef NFEM_ELAS_IMAGES
#define NFEM_ELAS_IMAGES 1
#endif
constexpr int kElasImages = NFEM_ELAS_IMAGES;
static_assert(kElasImages == 1 || kElasImages == 3, "one image per group or one per warp");

template <typename T>
__host__ __device__ constexpr size_t elas_image_words(int deg) {
  return size_t(kElasImages) * 3 * size_t(deg) * 4;
}

template <typename T, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) elasticity_rows_kernel(const ElasParams p) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int deg_max = p.deg_max;
  T* images = reinterpret_cast<T*>(dsm);  // [WARPS][3 groups][3 rows][deg_max][4]
  // reference tables read with per-lane indices (a, b): shared memory serves
  // those in one pass, the constant cache would serialise them
  T* sS = images + WARPS * elas_image_words<T>(deg_max);
  T* sm_m = sS + 900;
  for (int i = threadIdx.x; i < 900; i += blockDim.x) sS[i] = T(c_S[i]);
  if (threadIdx.x < 10) sm_m[threadIdx.x] = T(c_m[threadIdx.x]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / 10, b = lane - 10 * (lane / 10);
  const T* force = static_cast<const T*>(p.force);
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  T* wimg = images + warp * elas_image_words<T>(deg_max);
  for (int64_t v = int64_t(blockIdx.x) * WARPS + warp; v < p.n_nodes; v += int64_t(gridDim.x) * WARPS) {
    const int64_t r0 = p.row0 + 3 * v;
    const int32_t base = __ldg(p.row_ptr + r0);
    const int len = __ldg(p.row_ptr + r0 + 1) - base;  // 3 x deg
    const int deg = len / 3;
    if (deg > deg_max || len % 3 != 0 || deg < 1) {
      if (lane == 0) set_status(p.status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    if ((p.deg_filter == 1 && deg > 32) || (p.deg_filter == 2 && deg <= 32)) continue;  // the other kernel's row
    // the group images of this node: [images][3 rows][deg][4]
    const int gstride = kElasImages == 3 ? 3 * deg * 4 : 0;
    for (int q = lane; q < kElasImages * 3 * deg; q += 32) {
      Slot4<T> z;
      z.zero();
      z.store(wimg + q * 4);
    }
    __syncwarp();
    const int32_t kb = __ldg(p.inc_ptr + r0), ke = __ldg(p.inc_ptr + r0 + 1);
    T rhs_acc[3] = {T(0), T(0), T(0)};
    for (int32_t k0 = kb; k0 < ke; k0 += 3) {
      const int32_t k = k0 + g;
      const bool act = lane < 30 && k < ke;
      T K[3][3];
      int pos = 0;
      if (act) {
        const int32_t occ = __ldg(p.inc + k);
        const int32_t c = occ / 30;
        const int a = (occ - c * 30) / 3;
        // node position inside the row; the clamp keeps a corrupted code in
        // this node's image (a valid one is < deg)
        pos = min(int(__ldg(p.codes + int64_t(k) * 16 + b)), deg - 1);
        T gm[12];
        load_geom<T>(p, c, gm);
        const T(&Ji)[12] = gm;  // Ji[k * 3 + q] = (J^-1)_{kq}
        const T* S = sS + (a * 10 + b) * 9;
        // A / |det| = Ji^T S Ji; lambda |det| and mu |det| carry the |det|
        T SJ[3][3];
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            SJ[kk][q] = S[kk * 3 + 0] * Ji[0 * 3 + q] + S[kk * 3 + 1] * Ji[1 * 3 + q] + S[kk * 3 + 2] * Ji[2 * 3 + q];
        T A[3][3];
#pragma unroll
        for (int pp = 0; pp < 3; ++pp)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            A[pp][q] = Ji[0 * 3 + pp] * SJ[0][q] + Ji[1 * 3 + pp] * SJ[1][q] + Ji[2 * 3 + pp] * SJ[2][q];
        const T lc = gm[9], mc = gm[10], adet = gm[11];
        const T tr = A[0][0] + A[1][1] + A[2][2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) K[i][j] = (i == j ? mc * tr : T(0)) + mc * A[j][i] + lc * A[i][j];
        if (force && b == 0) {
#pragma unroll
          for (int i = 0; i < 3; ++i) rhs_acc[i] += adet * sm_m[a] * __ldg(force + int64_t(c) * 3 + i);
        }
      }
      // add the 3 x 3 block at the node column: three images take every
      // group at once; one image takes the groups in turn (two cells of the
      // node may share a column), the whole warp stepping together
#pragma unroll
      for (int gg = 0; gg < (kElasImages == 1 ? 3 : 1); ++gg) {
        if (act && (kElasImages == 3 || g == gg)) {
          T* im = wimg + g * gstride;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            T* slot = im + (i * deg + pos) * 4;
            Slot4<T> s4;
            s4.load(slot);
#pragma unroll
            for (int j = 0; j < 3; ++j) s4[j] += K[i][j];
            s4.store(slot);
          }
        }
        __syncwarp();
      }
    }
    // combine the group images in a fixed order: one (row i, column) slot per lane
    for (int q = lane; q < 3 * deg; q += 32) {
      Slot4<T> s0, s1, s2;
      s0.load(wimg + q * 4);
      if (kElasImages == 3) {
        s1.load(wimg + gstride + q * 4);
        s2.load(wimg + 2 * gstride + q * 4);
      }
      const int i = q / deg, pos = q - i * deg;
      T* out = values + int64_t(base) + i * len + 3 * pos;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T sum = kElasImages == 3 ? s0[j] + s1[j] + s2[j] : s0[j];
        if (p.accumulate) out[j] += sum; else out[j] = sum;
      }
    }
    T r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T a0 = __shfl_sync(0xffffffffu, rhs_acc[i], 0);
      const T a1 = __shfl_sync(0xffffffffu, rhs_acc[i], 10);
      const T a2 = __shfl_sync(0xffffffffu, rhs_acc[i], 20);
      r[i] = a0 + a1 + a2;
    }
    if (lane < 3) {
      const T rv = lane == 0 ? r[0] : (lane == 1 ? r[1] : r[2]);
      if (p.accumulate) rhs[r0 + lane] += rv; else rhs[r0 + lane] = rv;
    }
    __syncwarp();
  }
}

// Register form of the node rows: no shared-memory image.  Lane L owns the
// node columns L, L + 32 and L + 64 of the row (deg <= 96) and keeps their
// 3 x 3 blocks in registers.  The three groups of ten lanes evaluate the
// blocks K_ab of three incidences at once, as above; the blocks then reach
// their owners by warp shuffles: per incidence, each owner finds from the
// node codes which local node b falls on its column and pulls the nine
// values from lane 10 g + b (one round per column a lane owns that the
// incidence touches; usually one).  Every block is added by its owner in
// incidence order, so the sums are bitwise deterministic, and the row is
// stored once, coalesced, by the owners.
template <typename T>
__device__ __forceinline__ int code_match(uint4 cw, int col) {
  // position (0..9) of byte value `col` among the first ten code bytes, or -1
  const uint32_t rep = 0x01010101u * uint32_t(col);
  const uint32_t m0 = __vcmpeq4(cw.x, rep), m1 = __vcmpeq4(cw.y, rep), m2 = __vcmpeq4(cw.z, rep) & 0x0000ffffu;
  if (m0) return (__ffs(m0) - 1) >> 3;
  if (m1) return 4 + ((__ffs(m1) - 1) >> 3);
  if (m2) return 8 + ((__ffs(m2) - 1) >> 3);
  return -1;
}

template <typename T, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) elasticity_rows_reg_kernel(const ElasParams p) {
  __shared__ T sS[900];
  __shared__ T sm_m[10];
  for (int i = threadIdx.x; i < 900; i += blockDim.x) sS[i] = T(c_S[i]);
  if (threadIdx.x < 10) sm_m[threadIdx.x] = T(c_m[threadIdx.x]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / 10, b = lane - 10 * (lane / 10);
  const T* force = static_cast<const T*>(p.force);
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  const uint4* codes4 = reinterpret_cast<const uint4*>(p.codes);
  for (int64_t v = int64_t(blockIdx.x) * WARPS + warp; v < p.n_nodes; v += int64_t(gridDim.x) * WARPS) {
    const int64_t r0 = p.row0 + 3 * v;
    const int32_t base = __ldg(p.row_ptr + r0);
    const int len = __ldg(p.row_ptr + r0 + 1) - base;  // 3 x deg
    const int deg = len / 3;
    if (deg > 96 || len % 3 != 0 || deg < 1) {
      if (lane == 0) set_status(p.status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    if ((p.deg_filter == 1 && deg > 32) || (p.deg_filter == 2 && deg <= 32)) continue;  // the other kernel's row
    const int np = (deg + 31) >> 5;  // columns per lane
    T acc[3][9];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int e = 0; e < 9; ++e) acc[q][e] = T(0);
    const int32_t kb = __ldg(p.inc_ptr + r0), ke = __ldg(p.inc_ptr + r0 + 1);
    T rhs_acc[3] = {T(0), T(0), T(0)};
    for (int32_t k0 = kb; k0 < ke; k0 += 3) {
      const int32_t k = k0 + g;
      const bool act = lane < 30 && k < ke;
      T K[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) K[e] = T(0);
      if (act) {
        const int32_t occ = __ldg(p.inc + k);
        const int32_t c = occ / 30;
        const int a = (occ - c * 30) / 3;
        T gm[12];
        load_geom<T>(p, c, gm);
        const T(&Ji)[12] = gm;
        const T* S = sS + (a * 10 + b) * 9;
        T SJ[3][3];
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            SJ[kk][q] = S[kk * 3 + 0] * Ji[0 * 3 + q] + S[kk * 3 + 1] * Ji[1 * 3 + q] + S[kk * 3 + 2] * Ji[2 * 3 + q];
        T A[3][3];
#pragma unroll
        for (int pp = 0; pp < 3; ++pp)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            A[pp][q] = Ji[0 * 3 + pp] * SJ[0][q] + Ji[1 * 3 + pp] * SJ[1][q] + Ji[2 * 3 + pp] * SJ[2][q];
        const T lc = gm[9], mc = gm[10], adet = gm[11];
        const T tr = A[0][0] + A[1][1] + A[2][2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) K[i * 3 + j] = (i == j ? mc * tr : T(0)) + mc * A[j][i] + lc * A[i][j];
        if (force && b == 0) {
#pragma unroll
          for (int i = 0; i < 3; ++i) rhs_acc[i] += adet * sm_m[a] * __ldg(force + int64_t(c) * 3 + i);
        }
      }
      // route the blocks of the (up to) three incidences to their owners
#pragma unroll
      for (int gg = 0; gg < 3; ++gg) {
        if (k0 + gg >= ke) break;  // warp-uniform
        const uint4 cw = __ldg(codes4 + (k0 + gg));
        int src[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const int col = lane + 32 * q;
          const int m = (q < np && col < deg) ? code_match<T>(cw, col) : -1;
          src[q] = m;
        }
        // one round per owned column: lanes without a hit in a column pull
        // from themselves and discard
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          if (q >= np) break;  // warp-uniform
          if (!__any_sync(0xffffffffu, src[q] >= 0)) continue;
          const int from = src[q] >= 0 ? 10 * gg + src[q] : lane;
#pragma unroll
          for (int e = 0; e < 9; ++e) {
            const T val = __shfl_sync(0xffffffffu, K[e], from);
            if (src[q] >= 0) acc[q][e] += val;
          }
        }
      }
    }
    // store the owned columns: row i of the node, column 3 col + j
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int col = lane + 32 * q;
      if (q < np && col < deg) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          T* out = values + int64_t(base) + i * len + 3 * col;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            if (p.accumulate) out[j] += acc[q][i * 3 + j]; else out[j] = acc[q][i * 3 + j];
          }
        }
      }
    }
    T r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T a0 = __shfl_sync(0xffffffffu, rhs_acc[i], 0);
      const T a1 = __shfl_sync(0xffffffffu, rhs_acc[i], 10);
      const T a2 = __shfl_sync(0xffffffffu, rhs_acc[i], 20);
      r[i] = a0 + a1 + a2;
    }
    if (lane < 3) {
      const T rv = lane == 0 ? r[0] : (lane == 1 ? r[1] : r[2]);
      if (p.accumulate) rhs[r0 + lane] += rv; else rhs[r0 + lane] = rv;
    }
  }
}

// Boundary penalty: for each facet (6 P2 nodes), values at (dof_a,i),(dof_b,i)
// += beta |det_F| Mf_ab for every component i (atomics: a facet row sums
// contributions of the facets sharing its node).
template <typename T>
__global__ void penalty_kernel(int64_t n_facets, const int32_t* __restrict__ fdofs, const int32_t* __restrict__ fv,
                               const double* __restrict__ points, const int32_t* __restrict__ row_ptr,
                               const int32_t* __restrict__ col_idx, double beta, T* __restrict__ values,
                               int32_t* status) {
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_facets * 36;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t f = t / 36;
    const int ab = int(t - f * 36);
    const int a = ab / 6, b = ab - 6 * (ab / 6);
    double e1[3], e2[3];
    const int32_t v0 = fv[f * 3], v1 = fv[f * 3 + 1], v2 = fv[f * 3 + 2];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      e1[d] = points[int64_t(v1) * 3 + d] - points[int64_t(v0) * 3 + d];
      e2[d] = points[int64_t(v2) * 3 + d] - points[int64_t(v0) * 3 + d];
    }
    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                 cz = e1[0] * e2[1] - e1[1] * e2[0];
    const double detf = sqrt(cx * cx + cy * cy + cz * cz);
    const double val = beta * detf * c_Mf[a * 6 + b];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int32_t row = fdofs[f * 18 + a * 3 + i], col = fdofs[f * 18 + b * 3 + i];
      int32_t lo = row_ptr[row], hi = row_ptr[row + 1];
      const int32_t end = hi;
      while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (col_idx[mid] < col) lo = mid + 1; else hi = mid;
      }
      if (lo < end && col_idx[lo] == col) atomicAdd(values + lo, T(val));
      else set_status(status, NFEM_ERR_PATTERN);
    }
  }
}

// node codes: per incidence of a component-0 row, the node position (column
// position / n_comp) of each local node's first column in that row
__global__ void node_codes_kernel(const int32_t* __restrict__ cd, int n_loc, int n_comp, int64_t n_rows, int64_t row0,
                                  const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                                  uint8_t* __restrict__ codes, int32_t* status) {
  const int n_nodes_loc = n_loc / n_comp;
  for (int64_t r = row0 + (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) * n_comp; r < n_rows;
       r += int64_t(gridDim.x) * blockDim.x * n_comp) {
    const int32_t b0 = row_ptr[r], b1 = row_ptr[r + 1];
    for (int32_t k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k) {
      const int32_t c = inc[k] / n_loc;
      for (int b = 0; b < 16; ++b) {
        int code = 255;
        if (b < n_nodes_loc) {
          const int32_t col = cd[int64_t(c) * n_loc + b * n_comp];
          int32_t lo = b0, hi = b1;
          while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (col_idx[mid] < col) lo = mid + 1; else hi = mid;
          }
          if (lo >= b1 || col_idx[lo] != col) set_status(status, NFEM_ERR_PATTERN);
          const int np = (lo - b0) / n_comp;
          if (np > 254) set_status(status, NFEM_ERR_UNSUPPORTED);
          code = min(np, 254);
        }
        codes[int64_t(k) * 16 + b] = uint8_t(code);
      }
    }
  }
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_pattern_node_codes(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int n_comp,
                                       int64_t row0, int64_t n_rows, const int32_t* inc_ptr, const int32_t* inc,
                                       const int32_t* row_ptr, const int32_t* col_idx, uint8_t* codes,
                                       int32_t* dev_status, void* stream) {
  if (n_cells < 0 || n_loc < 1 || n_comp < 1 || n_loc % n_comp || n_loc / n_comp > 16 || row0 < 0 ||
      n_rows < row0 || (n_rows > row0 && (!cell_dofs || !inc_ptr || !inc || !row_ptr || !col_idx || !codes)))
    return NFEM_ERR_INVALID_ARG;
  if (n_rows == row0) return NFEM_OK;
  node_codes_kernel<<<grid_for(ceil_div(n_rows - row0, n_comp), 256), 256, 0, (cudaStream_t)stream>>>(
      cell_dofs, n_loc, n_comp, n_rows, row0, inc_ptr, inc, row_ptr, col_idx, codes, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

template <typename T, int WARPS>
static int launch_elasticity_reg(const ElasParams& p, cudaStream_t stream) {
  if (p.deg_max > 96) return NFEM_ERR_UNSUPPORTED;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, elasticity_rows_reg_kernel<T, WARPS>, 32 * WARPS, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  elasticity_rows_reg_kernel<T, WARPS><<<grid_for(ceil_div(p.n_nodes, WARPS), 1, per_sm), 32 * WARPS, 0, stream>>>(p);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

template <typename T, int WARPS>
static int launch_elasticity(const ElasParams& p, cudaStream_t stream) {
  const size_t smem = (WARPS * elas_image_words<T>(p.deg_max) + 910) * sizeof(T);
  if (smem > 227 * 1024) return NFEM_ERR_UNSUPPORTED;
  if (smem > 48 * 1024)
    NFEM_TRY_CUDA(cudaFuncSetAttribute(elasticity_rows_kernel<T, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(smem)));
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, elasticity_rows_kernel<T, WARPS>, 32 * WARPS, smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  elasticity_rows_kernel<T, WARPS>
      <<<grid_for(ceil_div(p.n_nodes, WARPS), 1, per_sm), 32 * WARPS, smem, stream>>>(p);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_elasticity_p2_workspace_bytes(int value_type, int64_t n_cells, size_t* bytes) {
  if (!bytes || n_cells < 0 || (value_type != NFEM_F64 && value_type != NFEM_F32)) return NFEM_ERR_INVALID_ARG;
  *bytes = size_t(n_cells) * 12 * (value_type == NFEM_F64 ? sizeof(double) : sizeof(float));
  return NFEM_OK;
}

extern "C" int nfem_elasticity_p2_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                           const double* points, const float* points_split,
                                           const int32_t* cell_vertices, const void* lambda_, const void* mu,
                                           const void* force, const double* ref_S, const double* ref_m,
                                           const int32_t* inc_ptr, const int32_t* inc, const uint8_t* node_codes,
                                           const int32_t* row_ptr, int max_node_degree, void* values, void* rhs,
                                           int accumulate, void* workspace, size_t workspace_bytes,
                                           int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0) return NFEM_ERR_INVALID_ARG;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n_nodes < 0 || row0 < 0) return NFEM_ERR_INVALID_ARG;
  if (n_nodes == 0) return NFEM_OK;
  if (!cell_vertices || !lambda_ || !mu || !ref_S || !ref_m || !inc_ptr || !inc || !node_codes || !row_ptr ||
      !values || !rhs)
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F64 && !points) return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F32 && (!points_split || (reinterpret_cast<uintptr_t>(points_split) & 15)))
    return NFEM_ERR_INVALID_ARG;
  if (reinterpret_cast<uintptr_t>(cell_vertices) & 15) return NFEM_ERR_INVALID_ARG;
  int rc = upload_tables(ref_S, ref_m, nullptr, stream);
  if (rc) return rc;
  ElasParams p;
  p.n_nodes = n_nodes;
  p.row0 = row0;
  p.points = points;
  p.split = points_split;
  p.cv = cell_vertices;
  p.lam = lambda_;
  p.mu = mu;
  p.force = force;
  p.inc_ptr = inc_ptr;
  p.inc = inc;
  p.codes = node_codes;
  p.row_ptr = row_ptr;
  p.values = values;
  p.rhs = rhs;
  p.accumulate = accumulate != 0;
  p.status = dev_status;
  const size_t vb = value_type == NFEM_F64 ? sizeof(double) : sizeof(float);
  if (!workspace || workspace_bytes < size_t(n_cells) * 12 * vb || (reinterpret_cast<uintptr_t>(workspace) & 15))
    return NFEM_ERR_WORKSPACE;
  p.n_cells = n_cells;
  p.geom = workspace;
  if (value_type == NFEM_F64)
    elas_geom_kernel<double><<<grid_for(n_cells, 256), 256, 0, stream>>>(p);
  else
    elas_geom_kernel<float><<<grid_for(n_cells, 256), 256, 0, stream>>>(p);
  p.deg_max = max_node_degree > 0 ? max_node_degree : kElasDegMax;
  if (p.deg_max > 255) return NFEM_ERR_UNSUPPORTED;  // node codes are bytes
  p.deg_filter = 0;
  if (knob(NFEM_KNOB_ELAS_ROWS) == 3 && p.deg_max <= 96) {
    // split: rows of at most 32 node columns in registers, longer rows in images
    p.deg_filter = 2;
    if (value_type == NFEM_F64)
      rc = launch_elasticity<double, kElasWarps64>(p, stream);
    else
      rc = launch_elasticity<float, kElasWarps32>(p, stream);
    if (rc) return rc;
    p.deg_filter = 1;
    if (value_type == NFEM_F64)
      rc = launch_elasticity_reg<double, 4>(p, stream);
    else
      rc = launch_elasticity_reg<float, 8>(p, stream);
  } else if (knob(NFEM_KNOB_ELAS_ROWS) == 2 && p.deg_max <= 96) {
    // register accumulation (opt-in: measured at 40^3 x 6 FP32 1.08 ms
    // against 0.61 ms for the shared-memory images)
    if (value_type == NFEM_F64)
      rc = launch_elasticity_reg<double, 4>(p, stream);
    else
      rc = launch_elasticity_reg<float, 8>(p, stream);
  } else if (value_type == NFEM_F64) {
    rc = launch_elasticity<double, kElasWarps64>(p, stream);
  } else {
    const int w = knob(NFEM_KNOB_ELAS_WARPS);
    if (w == 2)
      rc = launch_elasticity<float, 2>(p, stream);
    else if (w == 8)
      rc = launch_elasticity<float, 8>(p, stream);
    else if (w == 4)
      rc = launch_elasticity<float, 4>(p, stream);
    else
      rc = launch_elasticity<float, kElasWarps32>(p, stream);
  }
  if (rc) return rc;
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_elasticity_p2_penalty(int value_type, int64_t n_facets, const int32_t* facet_dofs,
                                          const int32_t* facet_vertices, const double* points, double beta,
                                          const double* ref_S, const double* ref_m, const double* ref_Mf,
                                          const int32_t* row_ptr, const int32_t* col_idx, void* values,
                                          int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n_facets < 0) return NFEM_ERR_INVALID_ARG;
  if (n_facets == 0) return NFEM_OK;
  if (!facet_dofs || !facet_vertices || !points || !ref_S || !ref_m || !ref_Mf || !row_ptr || !col_idx || !values)
    return NFEM_ERR_INVALID_ARG;
  int rc = upload_tables(ref_S, ref_m, ref_Mf, stream);
  if (rc) return rc;
  const int g = grid_for(n_facets * 36, 256);
  if (value_type == NFEM_F64)
    penalty_kernel<double><<<g, 256, 0, stream>>>(n_facets, facet_dofs, facet_vertices, points, row_ptr, col_idx,
                                                  beta, (double*)values, dev_status);
  else
    penalty_kernel<float><<<g, 256, 0, stream>>>(n_facets, facet_dofs, facet_vertices, points, row_ptr, col_idx,
                                                 beta, (float*)values, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
