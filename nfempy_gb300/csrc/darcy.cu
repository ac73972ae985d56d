// K1-K4 fused: mixed Darcy RT1 x P0 element integrals + CSR scatter.
//
// Reference: LaplaceDualWeakForm.evaluate_form
// (src/weak_forms/laplace_dual_weak_form.py:10-86) evaluated for every cell
// and scattered entry by entry (src/assembly/ScatterFormData.py:5-25).  Per
// cell, with psi_i the oriented, Piola-mapped RT1 functions and w = 1 the P0
// function:
//   j[i, j] =  int K^-1 psi_i . psi_j      j[i, p] = -int w div psi_i
//   j[p, j] =  int w div psi_j             j[p, p] = 0
//   r[p]    = -int f w                     r[i]    = 0      (alpha = 0)
//
// Closed forms used here (exact for affine cells and cell-wise constant K,
// so equal to the reference's order-3 quadrature up to round-off):
//   psi_i = (1/|det J|) J psihat_i,  psihat_i = sgn_i * kappa * (xhat - vhat_i)
//   with sgn_i = sigma_i * s_i (sigma: reference normal vs outward, s: the
//   orientation sign), kappa = 2 (tet) or 1 (triangle);
//   int psi_i . psi_j = sgn_i sgn_j kappa^2 / |det J| * T_ij,
//   T_ij = tr(G S) - m.G vhat_i - m.G vhat_j + |That| vhat_i^T G vhat_j,
//   G = J^T J, m = int xhat, S = int xhat xhat^T on the reference simplex;
//   int w div psi_i = sgn_i (the flux normalisation).
//
// GPU design (row owner): one thread per global row, 32 consecutive rows per
// warp.  A thread walks the (cell, local row) incidences of its row (two for
// an interior face, one for a boundary face or a pressure row), evaluates
// that row of the element matrix from the cell's vertices and adds it into a
// warp-private shared-memory image of the warp's contiguous CSR segment at
// the positions given by the precomputed 4-bit slot codes.  The segment is
// then stored with coalesced writes.  Every CSR value and residual entry is
// written exactly once: no atomics, no zero-fill pass, deterministic sums.
#include "nfem_common.cuh"

namespace nfem {

constexpr int kDarcyWarps = 8;
constexpr int kDarcyMaxRow = 16;

struct DarcyParams {
  int64_t n_rows;
  const double* points;
  const float* split;
  const int32_t* cv;
  const uint8_t* sign;
  const void* kappa;
  const void* source;
  const int32_t* pairs;
  const uint32_t* pair_codes;
  const int32_t* row_ptr;
  void* values;
  void* rhs;
  int32_t* status;
  int accumulate;
  int n_qp;
  double qw[32];
};

template <typename T, int DIM>
struct DarcyConst;
template <typename T>
struct DarcyConst<T, 3> {
  static __device__ __forceinline__ T sigma(int i) { return (i & 1) ? T(-1) : T(1); }
  static constexpr double kappa2 = 4.0, area = 1.0 / 6.0, f1 = 1.0 / 24.0, f2 = 1.0 / 120.0;
};
template <typename T>
struct DarcyConst<T, 2> {
  static __device__ __forceinline__ T sigma(int i) { return (i == 1) ? T(1) : T(-1); }
  static constexpr double kappa2 = 1.0, area = 0.5, f1 = 1.0 / 6.0, f2 = 1.0 / 24.0;
};

// Edge vectors J[k] = x_{k+1} - x_0 of cell c.
template <typename T, int DIM>
__device__ __forceinline__ void cell_edges(const DarcyParams& p, int32_t c, T (&J)[DIM][3]);

template <>
__device__ __forceinline__ void cell_edges<double, 3>(const DarcyParams& p, int32_t c, double (&J)[3][3]) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const int vs[4] = {v.x, v.y, v.z, v.w};
  double x0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) x0[d] = __ldg(p.points + int64_t(vs[0]) * 3 + d);
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) J[k][d] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - x0[d];
}

template <>
__device__ __forceinline__ void cell_edges<double, 2>(const DarcyParams& p, int32_t c, double (&J)[2][3]) {
  const int32_t* vp = p.cv + int64_t(c) * 3;
  const int vs[3] = {__ldg(vp), __ldg(vp + 1), __ldg(vp + 2)};
  double x0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) x0[d] = __ldg(p.points + int64_t(vs[0]) * 3 + d);
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) J[k][d] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - x0[d];
}

// FP32: coordinates as float (hi, lo) pairs; differences of hi parts of
// nearby points are exact, the lo parts restore what the split dropped.
__device__ __forceinline__ void load_split(const float* s, int v, float (&hi)[3], float (&lo)[3]) {
  const float2* q = reinterpret_cast<const float2*>(s + int64_t(v) * 6);
  const float2 a = __ldg(q), b = __ldg(q + 1), d = __ldg(q + 2);
  hi[0] = a.x; hi[1] = a.y; hi[2] = b.x;
  lo[0] = b.y; lo[1] = d.x; lo[2] = d.y;
}

template <>
__device__ __forceinline__ void cell_edges<float, 3>(const DarcyParams& p, int32_t c, float (&J)[3][3]) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const int vs[4] = {v.x, v.y, v.z, v.w};
  float h0[3], l0[3];
  load_split(p.split, vs[0], h0, l0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float h[3], l[3];
    load_split(p.split, vs[k + 1], h, l);
#pragma unroll
    for (int d = 0; d < 3; ++d) J[k][d] = (h[d] - h0[d]) + (l[d] - l0[d]);
  }
}

template <>
__device__ __forceinline__ void cell_edges<float, 2>(const DarcyParams& p, int32_t c, float (&J)[2][3]) {
  const int32_t* vp = p.cv + int64_t(c) * 3;
  const int vs[3] = {__ldg(vp), __ldg(vp + 1), __ldg(vp + 2)};
  float h0[3], l0[3];
  load_split(p.split, vs[0], h0, l0);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    float h[3], l[3];
    load_split(p.split, vs[k + 1], h, l);
#pragma unroll
    for (int d = 0; d < 3; ++d) J[k][d] = (h[d] - h0[d]) + (l[d] - l0[d]);
  }
}

template <typename T, int DIM>
__device__ __forceinline__ T abs_det(const T (&J)[DIM][3], const T (&G)[DIM][DIM]) {
  if constexpr (DIM == 3) {
    T d = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    return d < T(0) ? -d : d;
  } else {
    return sqrt(G[0][0] * G[1][1] - G[0][1] * G[0][1]);
  }
}

// One incidence (cell c, local row a) of a row: everything loaded up front so
// that the two incidences of a face row overlap their memory latency.
template <typename T, int DIM>
struct Incidence {
  T J[DIM][3];
  T kap;
  T src;
  uint32_t m;
};

template <typename T, int DIM, int SRC>
__device__ __forceinline__ void load_incidence(const DarcyParams& p, int32_t c, bool need_geo,
                                               Incidence<T, DIM>& x) {
  const T* kappa = static_cast<const T*>(p.kappa);
  const T* src = static_cast<const T*>(p.source);
  x.m = __ldg(p.sign + c);
  x.kap = __ldg(kappa + c);
  x.src = T(0);
  if constexpr (SRC == NFEM_COEF_CELL) x.src = __ldg(src + c);
  if constexpr (SRC == NFEM_COEF_QPOINT) {
    T acc = T(0);
#pragma unroll 4
    for (int q = 0; q < 32; ++q)
      if (q < p.n_qp) acc += T(p.qw[q]) * __ldg(src + int64_t(c) * p.n_qp + q);
    x.src = acc;
  }
  if (need_geo) {
    cell_edges<T, DIM>(p, c, x.J);
  } else {
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int d = 0; d < 3; ++d) x.J[i][d] = T(0);
  }
}

// Row a of the element matrix of the incidence (vals[0..NF) flux columns,
// vals[NF] pressure column) and, for the pressure row, the residual entry.
template <typename T, int DIM, int SRC>
__device__ __forceinline__ void element_row(const DarcyParams& p, const Incidence<T, DIM>& x, int a, bool need_geo,
                                            T (&vals)[DIM + 2], T& rhs_val) {
  constexpr int NF = DIM + 1;
  using C = DarcyConst<T, DIM>;
  T sg[NF];
#pragma unroll
  for (int i = 0; i < NF; ++i) sg[i] = ((x.m >> i) & 1u) ? -C::sigma(i) : C::sigma(i);
  T G[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) G[i][j] = x.J[i][0] * x.J[j][0] + x.J[i][1] * x.J[j][1] + x.J[i][2] * x.J[j][2];
  T det = T(1);
  if (need_geo) {
    det = abs_det<T, DIM>(x.J, G);
    if (!(det > T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
  }
  if (a < NF) {
    T R[DIM];
    T trG = T(0), sumG = T(0);
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      R[i] = T(0);
#pragma unroll
      for (int j = 0; j < DIM; ++j) R[i] += G[i][j];
      trG += G[i][i];
      sumG += R[i];
    }
    const T tgs = (trG + sumG) * T(C::f2);
    const T scale = T(C::kappa2) / (x.kap * det);
    // row a-1 of G and R[a-1] through selects (no local-memory indexing)
    T Ga[DIM];
    T Ra = T(0);
#pragma unroll
    for (int j = 0; j < DIM; ++j) Ga[j] = T(0);
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      const bool hit = (a == i + 1);
      Ra = hit ? R[i] : Ra;
#pragma unroll
      for (int j = 0; j < DIM; ++j) Ga[j] = hit ? G[i][j] : Ga[j];
    }
    T sga = sg[0];
#pragma unroll
    for (int i = 1; i < NF; ++i) sga = (a == i) ? sg[i] : sga;
    const T gma = Ra * T(C::f1);
#pragma unroll
    for (int b = 0; b < NF; ++b) {
      const T gmb = b > 0 ? R[b - 1] * T(C::f1) : T(0);
      const T gv = b > 0 ? Ga[b - 1] * T(C::area) : T(0);
      vals[b] = scale * sga * sg[b] * (tgs - gma - gmb + gv);
    }
    vals[NF] = -sga;
  } else {
#pragma unroll
    for (int b = 0; b < NF; ++b) vals[b] = sg[b];
    vals[NF] = T(0);
    if constexpr (SRC == NFEM_COEF_CELL) rhs_val += -det * T(C::area) * x.src;
    if constexpr (SRC == NFEM_COEF_QPOINT) rhs_val += -det * x.src;
  }
}

struct RowHead {
  int2 pr;
  uint2 cd;
};

__device__ __forceinline__ RowHead load_head(const DarcyParams& p, int64_t r) {
  RowHead h;
  if (r < p.n_rows) {
    h.pr = __ldg(reinterpret_cast<const int2*>(p.pairs) + r);
    h.cd = __ldg(reinterpret_cast<const uint2*>(p.pair_codes) + r);
  } else {
    h.pr = make_int2(-1, -1);
    h.cd = make_uint2(0u, 0u);
  }
  return h;
}

// Row length from the slot codes: 1 + the largest position any incidence
// writes (the positions of a row's columns are 0..len-1 and every column is
// written by some incidence).
template <int NLOC>
__device__ __forceinline__ int row_len_from_codes(const RowHead& h) {
  int len = 0;
  const int occ[2] = {h.pr.x, h.pr.y};
  const uint32_t code[2] = {h.cd.x, h.cd.y};
#pragma unroll
  for (int t = 0; t < 2; ++t)
    if (occ[t] >= 0)
#pragma unroll
      for (int b = 0; b < NLOC; ++b) len = max(len, int((code[t] >> (4 * b)) & 15u) + 1);
  return len;
}

template <typename T, int DIM, int SRC>
__global__ void __launch_bounds__(32 * kDarcyWarps) darcy_rows_kernel(const DarcyParams p) {
  constexpr int NLOC = DIM + 2;
  __shared__ T stage[kDarcyWarps][32 * kDarcyMaxRow];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* st = stage[warp];
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  const int64_t stride = int64_t(gridDim.x) * kDarcyWarps * 32;

  int64_t r0 = (int64_t(blockIdx.x) * kDarcyWarps + warp) * 32;
  RowHead head = load_head(p, r0 + lane);
  int32_t base_next = r0 < p.n_rows ? __ldg(p.row_ptr + r0) : 0;
  for (; r0 < p.n_rows; r0 += stride) {
    const int64_t r = r0 + lane;
    const bool valid = r < p.n_rows;
    const RowHead h = head;
    const int32_t base = base_next;
    // prefetch the next chunk of this warp (overlaps its latency with this one)
    head = load_head(p, r0 + stride + lane);
    base_next = (r0 + stride < p.n_rows) ? __ldg(p.row_ptr + r0 + stride) : 0;

    const int occ[2] = {h.pr.x, h.pr.y};
    const uint32_t code[2] = {h.cd.x, h.cd.y};
    int32_t c[2];
    int a[2];
    bool on[2], geo[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      on[t] = occ[t] >= 0;
      c[t] = on[t] ? occ[t] / NLOC : 0;
      a[t] = on[t] ? occ[t] - c[t] * NLOC : 0;
      geo[t] = on[t] && ((a[t] < DIM + 1) || (SRC != 0));
    }
    Incidence<T, DIM> inc[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) load_incidence<T, DIM, SRC>(p, c[t], geo[t], inc[t]);

    // row offsets inside the chunk: exclusive warp scan of the row lengths
    const int len = valid ? row_len_from_codes<NLOC>(h) : 0;
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int off = incl - len;
    const int span = __shfl_sync(0xffffffffu, incl, 31);
    if (span > 32 * kDarcyMaxRow) {  // cannot happen for codes built with rows <= 16
      if (lane == 0) set_status(p.status, NFEM_ERR_PATTERN);
      continue;
    }
    for (int i = lane; i < span; i += 32) st[i] = T(0);
    __syncwarp();
    T rhs_val = T(0);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (on[t]) {
        T vals[NLOC];
        element_row<T, DIM, SRC>(p, inc[t], a[t], geo[t], vals, rhs_val);
#pragma unroll
        for (int b = 0; b < NLOC; ++b) {
          // codes index inside the row (< 16 entries); the clamp keeps a
          // corrupted code inside this warp's staging buffer
          const int idx = min(off + int((code[t] >> (4 * b)) & 15u), 32 * kDarcyMaxRow - 1);
          st[idx] += vals[b];
        }
      }
    }
    __syncwarp();
    if (p.accumulate) {
      for (int i = lane; i < span; i += 32) values[int64_t(base) + i] += st[i];
      if (valid) rhs[r] += rhs_val;
    } else {
      for (int i = lane; i < span; i += 32) values[int64_t(base) + i] = st[i];
      if (valid) rhs[r] = rhs_val;
    }
    __syncwarp();
  }
}

template <typename T, int DIM>
static int launch_darcy(const DarcyParams& p, int source_mode, cudaStream_t stream) {
  const int block = 32 * kDarcyWarps;
  const int grid = grid_for(ceil_div(p.n_rows, 32 * kDarcyWarps), 1, 8);
  switch (source_mode) {
    case NFEM_COEF_NONE: darcy_rows_kernel<T, DIM, NFEM_COEF_NONE><<<grid, block, 0, stream>>>(p); break;
    case NFEM_COEF_CELL: darcy_rows_kernel<T, DIM, NFEM_COEF_CELL><<<grid, block, 0, stream>>>(p); break;
    case NFEM_COEF_QPOINT: darcy_rows_kernel<T, DIM, NFEM_COEF_QPOINT><<<grid, block, 0, stream>>>(p); break;
    default: return NFEM_ERR_INVALID_ARG;
  }
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_darcy_rt1p0_assemble(int dim, int value_type, int64_t n_cells, int64_t n_rows,
                                         const double* points, const float* points_split,
                                         const int32_t* cell_vertices, const int32_t* flux_dofs, int64_t p_base,
                                         const uint8_t* sign_mask, const void* kappa, const void* source,
                                         int source_mode, const double* qweights, int n_qp,
                                         const int32_t* row_pairs, const uint32_t* pair_codes,
                                         const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                                         int32_t* dev_status, void* stream_) {
  (void)flux_dofs;
  (void)p_base;
  (void)n_cells;
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_rows < 0)
    return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  if (!cell_vertices || !sign_mask || !kappa || !row_pairs || !pair_codes || !row_ptr || !values || !rhs)
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F64 && !points) return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F32 && !points_split) return NFEM_ERR_INVALID_ARG;
  if (source_mode != NFEM_COEF_NONE && !source) return NFEM_ERR_INVALID_ARG;
  if (source_mode == NFEM_COEF_QPOINT && (!qweights || n_qp < 1 || n_qp > 32)) return NFEM_ERR_INVALID_ARG;
  if (dim == 3 && (reinterpret_cast<uintptr_t>(cell_vertices) & 15)) return NFEM_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(row_pairs) & 7) || (reinterpret_cast<uintptr_t>(pair_codes) & 7))
    return NFEM_ERR_INVALID_ARG;
  DarcyParams p;
  p.n_rows = n_rows;
  p.points = points;
  p.split = points_split;
  p.cv = cell_vertices;
  p.sign = sign_mask;
  p.kappa = kappa;
  p.source = source;
  p.pairs = row_pairs;
  p.pair_codes = pair_codes;
  p.row_ptr = row_ptr;
  p.values = values;
  p.rhs = rhs;
  p.status = dev_status;
  p.accumulate = accumulate != 0;
  p.n_qp = source_mode == NFEM_COEF_QPOINT ? n_qp : 0;
  for (int i = 0; i < 32; ++i) p.qw[i] = (i < p.n_qp) ? qweights[i] : 0.0;
  if (value_type == NFEM_F64)
    return dim == 3 ? launch_darcy<double, 3>(p, source_mode, stream) : launch_darcy<double, 2>(p, source_mode, stream);
  return dim == 3 ? launch_darcy<float, 3>(p, source_mode, stream) : launch_darcy<float, 2>(p, source_mode, stream);
}
