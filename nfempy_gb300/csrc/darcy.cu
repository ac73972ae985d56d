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
// then stored with coalesced writes (its 16-byte-aligned middle by one TMA
// bulk copy).  Every CSR value and residual entry is written exactly once:
// no atomics, no zero-fill pass, deterministic sums.  With a record
// workspace a cell pass first evaluates each cell's metric terms once, and
// the row pass reads those records instead of the vertices (two-pass form).
#include <algorithm>
#include <vector>

#include "df64.cuh"
#include "nfem_common.cuh"

namespace nfem {

#ifndef NFEM_DARCY_WARPS
#define NFEM_DARCY_WARPS 4
#endif
constexpr int kDarcyWarps = NFEM_DARCY_WARPS;  // warps per block of the row-owner kernel
// minimum resident blocks per SM asked of the register allocator (FP32
// kernels: 10 x 128 threads -> 48 registers, 62 % warps active; FP64 keeps
// its registers).  Measured at 64^3 x 6: 4 warps x 10 blocks 98.2 us,
// 8 x 5 99.2 us, 16 x 2 110 us, 4 x 12 (40 registers, spills) 177 us.
#ifndef NFEM_DARCY_MIN_BLOCKS
#define NFEM_DARCY_MIN_BLOCKS 10
#endif
constexpr int kDarcyMaxRow = 16;
// 2: both incidences of a row in straight-line code (their loads may
// overlap); 1: one after the other (fewer live registers)
#ifndef NFEM_DARCY_INC_UNROLL
#define NFEM_DARCY_INC_UNROLL 2
#endif
constexpr int kDarcyIncUnroll = NFEM_DARCY_INC_UNROLL;

struct DarcyParams {
  int64_t n_rows;
  int64_t n_cells;
  int64_t p_base;
  const int32_t* chunk_rows;
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
  void* rec;  // per-cell records of the two-pass path (NULL: single pass)
  const int64_t* fixed;  // FP64 tetrahedra: nfem_points_fixed64 records (NULL: FP64 edge subtraction)
  int lattice;           // FP64 tetrahedra: exact integer records for lattice cells (lattice_record)
  int prow;              // the cell pass writes each cell's pressure row (pressure_row); the row pass skips them
  int64_t rp_off;        // FP64 tetrahedra: r_p of record slot s at ((double*)rec)[rp_off + s]
  int32_t* bad;          // FP32 records: [0] count, [4 ..] cells left to darcy_refine_kernel (NULL: none)
  // Work ranges of one launch: the cell pass covers cells [cell_begin,
  // cell_end); the row pass covers the rows [row_f0, row_f1) and then
  // [row_q0, row_q1) (flux rows and pressure rows of one cell slice, or all
  // rows in one range).  ring_shift >= 0: the records live in a ring of
  // three slices of 2^ring_shift cells (see rec_index).
  int64_t cell_begin, cell_end;
  int64_t row_f0, row_f1, row_q0, row_q1;
  int ring_shift;
};

// Position of cell c's record: c itself, or its place in the ring of three
// slices of 2^ring_shift cells that the overlapped assembly keeps in L2.
__device__ __forceinline__ int64_t rec_index(const DarcyParams& p, int64_t c) {
  if (p.ring_shift < 0) return c;
  const int64_t s = c >> p.ring_shift;
  return ((s % 3) << p.ring_shift) | (c & ((int64_t(1) << p.ring_shift) - 1));
}

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

// FP32: one packed 16-byte record per vertex (nfem_points_split).  The edges
// are left in units of the record's scale s (a power of two): every product
// of the metric, the determinant and the element row then carries an exact
// power of s, folded in once per incidence (element_row), which gives the
// same rounded values as scaling each edge component.
__device__ __forceinline__ void cell_edges_of(const DarcyParams& p, const int4 v, float (&J)[3][3]) {
  const float4 r0 = packed_point(p.split, v.x), r1 = packed_point(p.split, v.y), r2 = packed_point(p.split, v.z),
               r3 = packed_point(p.split, v.w);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    J[0][d] = packed_diff(r1, r0, d, 1.f);
    J[1][d] = packed_diff(r2, r0, d, 1.f);
    J[2][d] = packed_diff(r3, r0, d, 1.f);
  }
}
template <>
__device__ __forceinline__ void cell_edges<float, 3>(const DarcyParams& p, int32_t c, float (&J)[3][3]) {
  cell_edges_of(p, __ldg(reinterpret_cast<const int4*>(p.cv) + c), J);
}

template <>
__device__ __forceinline__ void cell_edges<float, 2>(const DarcyParams& p, int32_t c, float (&J)[2][3]) {
  const int32_t* vp = p.cv + int64_t(c) * 3;
  const float4 r0 = packed_point(p.split, __ldg(vp)), r1 = packed_point(p.split, __ldg(vp + 1)),
               r2 = packed_point(p.split, __ldg(vp + 2));
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    J[0][d] = packed_diff(r1, r0, d, 1.f);
    J[1][d] = packed_diff(r2, r0, d, 1.f);
  }
}

// Unit of the edges cell_edges returns: the packed records' scale in FP32,
// 1 in FP64 (plain coordinates).
template <typename T>
__device__ __forceinline__ T edge_unit(const DarcyParams& p);
template <>
__device__ __forceinline__ float edge_unit<float>(const DarcyParams& p) {
  return packed_lo_scale(p.split);
}
template <>
__device__ __forceinline__ double edge_unit<double>(const DarcyParams&) {
  return 1.0;
}

// 1 / v: correctly rounded reciprocal (no division sequence) in FP32, exact
// division in FP64
__device__ __forceinline__ float recip(float v) { return __frcp_rn(v); }
__device__ __forceinline__ double recip(double v) { return 1.0 / v; }

template <typename T, int DIM>
__device__ __forceinline__ T abs_det(const T (&J)[DIM][3], const T (&G)[DIM][DIM]) {
  if constexpr (DIM == 3) {
    T d = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    return d < T(0) ? -d : d;
  } else {
    // |e_0 x e_1| from the edges (not sqrt(G00 G11 - G01^2), whose
    // difference loses a relative eps / q^2 on thin triangles against
    // eps / q here)
    (void)G;
    const T x = J[0][1] * J[1][2] - J[0][2] * J[1][1], y = J[0][2] * J[1][0] - J[0][0] * J[1][2],
            z = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    return sqrt(x * x + y * y + z * z);
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
  int32_t c;  // the cell (for the FP64 |det J| of badly shaped cells)
};

// Badly shaped cells in FP32.  |det J| from FP32 edges carries a relative
// error of a few ulps divided by the cell's shape quality
//   q = |det J| / (|e_0| ... |e_{DIM-1}|)   (q^2 for the 2-D sqrt form),
// which reaches 1e-5 near q ~ 1e-2 (flat or needle cells in general
// orientation); and an edge shorter than 2^20 units of the fixed-point
// records carries a relative error above 2^-21 from their rounding, which
// |det J| inherits in proportion.  In the two-pass assembly the cell pass
// leaves cells with q < 0.1 or an edge below 2^20 units to a follow-up
// launch over their list (darcy_refine_kernel),
// which takes their |det J| in FP64: from the FP64 points when the caller
// passed them (exactly rounded edge differences), else from the 32-bit
// fixed-point records (exact integer differences); their records and
// pressure rows are then formed as for any other cell.  The opt-in one-pass,
// cell-chunk and sliced forms keep FP32.  In edge units, like abs_det.
constexpr float kSliverQ = 0.1f;
constexpr float kShortEdge2 = 1099511627776.0f;  // (2^20 edge units)^2

template <int DIM>
__device__ __noinline__ float refine_det(const DarcyParams& p, int32_t c) {
  int vs[DIM + 1];
  if constexpr (DIM == 3) {
    const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
    vs[0] = v.x;
    vs[1] = v.y;
    vs[2] = v.z;
    vs[3] = v.w;
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) vs[k] = __ldg(p.cv + int64_t(c) * 3 + k);
  }
  double e[DIM][3];
  double unit = 1.0;  // edge units per FP64 coordinate unit
  if (p.points) {
    unit = 1.0 / double(packed_lo_scale(p.split));
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        e[k][d] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - __ldg(p.points + int64_t(vs[0]) * 3 + d);
  } else {
    const float4 r0 = packed_point(p.split, vs[0]);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const float4 r = packed_point(p.split, vs[k + 1]);
      e[k][0] = double(int64_t(__float_as_int(r.x)) - __float_as_int(r0.x));
      e[k][1] = double(int64_t(__float_as_int(r.y)) - __float_as_int(r0.y));
      e[k][2] = double(int64_t(__float_as_int(r.z)) - __float_as_int(r0.z));
    }
  }
  double det;
  if constexpr (DIM == 3) {
    det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
          e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
    det *= unit * unit * unit;
  } else {
    const double x = e[0][1] * e[1][2] - e[0][2] * e[1][1], y = e[0][2] * e[1][0] - e[0][0] * e[1][2],
                 z = e[0][0] * e[1][1] - e[0][1] * e[1][0];
    det = sqrt(x * x + y * y + z * z) * unit * unit;
  }
  return float(det < 0.0 ? -det : det);
}

// |det J| of tetrahedron c in FP64 from the FP64 points (exactly rounded
// edge differences, hardware FP64 arithmetic): the FP64 path's badly shaped
// cells, where double-float cancellation in the triple product would exceed
// FP64's own error (a few ulps over q, like the reference's QR).
__device__ __noinline__ double refine_det64(const DarcyParams& p, int64_t c) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const int vs[4] = {v.x, v.y, v.z, v.w};
  double e[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      e[k][d] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - __ldg(p.points + int64_t(vs[0]) * 3 + d);
  const double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                     e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) + e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
  return det < 0.0 ? -det : det;
}

// The cell's shape quality q from its FP32 metric, by reciprocal square
// roots (the edge units put |e|^6 beyond the FP32 range)
template <int DIM>
__device__ __forceinline__ float shape_quality(float det, const float (&G)[DIM][DIM]) {
  float q = det * rsqrtf(G[0][0]) * rsqrtf(G[1][1]);
  if constexpr (DIM == 3) q *= rsqrtf(G[2][2]);
  return q;
}

// vpre: the cell's vertex ids already loaded (FP32 tetrahedra), or NULL
template <typename T, int DIM, int SRC>
__device__ __forceinline__ void load_incidence(const DarcyParams& p, int32_t c, bool need_geo,
                                               Incidence<T, DIM>& x, const int4* vpre = nullptr) {
  const T* kappa = static_cast<const T*>(p.kappa);
  const T* src = static_cast<const T*>(p.source);
  x.m = __ldg(p.sign + c);
  x.c = c;
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
  check_positive(p.status, x.kap);
  check_finite(p.status, x.src);
  if (need_geo) {
    if constexpr (sizeof(T) == 4 && DIM == 3) {
      if (vpre)
        cell_edges_of(p, *vpre, x.J);
      else
        cell_edges<T, DIM>(p, c, x.J);
    } else {
      cell_edges<T, DIM>(p, c, x.J);
    }
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
  // G = J^T J only where it is used: the flux rows, and the 2-D |det J|
  T G[DIM][DIM];
  auto metric = [&]() {
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int j = 0; j < DIM; ++j) G[i][j] = x.J[i][0] * x.J[j][0] + x.J[i][1] * x.J[j][1] + x.J[i][2] * x.J[j][2];
  };
  if (DIM == 2 || a < NF) metric();
  // G and det are in edge units u: G = u^2 G_true, det = u^DIM det_true; the
  // flux entries are kappa2 / (kap det_true) * u^2 (bracket in edge units)
  const T u = edge_unit<T>(p);
  T det = T(1), det_true = T(1);
  if (need_geo) {
    det = abs_det<T, DIM>(x.J, G);
    if (!(det > T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
    det_true = DIM == 3 ? det * (u * u * u) : det * (u * u);
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
    const T scale = T(C::kappa2) * recip(x.kap * (DIM == 3 ? det * u : det));
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
    if constexpr (SRC == NFEM_COEF_CELL) rhs_val += -det_true * T(C::area) * x.src;
    if constexpr (SRC == NFEM_COEF_QPOINT) rhs_val += -det_true * x.src;
  }
}

// The flux x flux block of a cell's element matrix, rows a < NF at
// M[a * 4 + b] (the same expressions as element_row, evaluated once for the
// whole matrix), and the residual entry of its pressure row.
template <typename T, int DIM, int SRC>
__device__ __forceinline__ T cell_matrix(const DarcyParams& p, const Incidence<T, DIM>& x, T* M) {
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
  const T det = abs_det<T, DIM>(x.J, G);  // edge units, as in element_row
  if (!(det > T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
  const T u = edge_unit<T>(p);
  const T det_true = DIM == 3 ? det * (u * u * u) : det * (u * u);
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
  const T scale = T(C::kappa2) * recip(x.kap * (DIM == 3 ? det * u : det));
#pragma unroll
  for (int a = 0; a < NF; ++a) {
    const T gma = a > 0 ? R[a - 1] * T(C::f1) : T(0);
#pragma unroll
    for (int b = a; b < NF; ++b) {
      const T gmb = b > 0 ? R[b - 1] * T(C::f1) : T(0);
      const T gv = (a > 0 && b > 0) ? G[a - 1][b - 1] * T(C::area) : T(0);
      const T v = scale * sg[a] * sg[b] * (tgs - gma - gmb + gv);
      M[a * 4 + b] = v;
      if (b != a) M[b * 4 + a] = v;
    }
  }
  if constexpr (SRC == NFEM_COEF_CELL) return -det_true * T(C::area) * x.src;
  if constexpr (SRC == NFEM_COEF_QPOINT) return -det_true * x.src;
  return T(0);
}

// ------------------------------------------------------------------ two-pass form
// Pass 1, one thread per cell (coalesced): the metric G = J^T J, the scale
// kappa^2 / (kappa |det J|) and the pressure row's residual entry r_p,
// evaluated once per cell instead of once per (row, cell) incidence, with
// element_row's operations and rounding.  FP32 records (one 32-byte sector):
//   3-D: [G11, G12, G13, scale | G22, G23, G33, r_p]
//   2-D: [G11, G12, G22, scale | r_p, 0, 0, 0]
// FP64 records also carry the row sums R of G and S = tr G + sum G (the
// FP64 units are scarce here, FP32 ones are not):
//   3-D: [S, R1, R2, R3 | G11, G12, G13, scale | G22, G23, G33, r_p]
//   2-D: [S, R1, R2, G11 | G12, G22, scale, r_p]
// Pass 2 is the row-owner kernel reading these records in place of the
// vertices; it forms the rest of the row in element_row's expressions and
// order, so that both forms round (and contract) alike.
template <typename T, int DIM>
struct RecLayout {
  static constexpr bool sums = sizeof(T) == 8;           // R and S stored
  static constexpr int n = (sums && DIM == 3) ? 12 : 8;  // words per cell
  static constexpr int rp = n - 1 - ((!sums && DIM == 2) ? 3 : 0);  // r_p position
  static constexpr int scale = sums ? (DIM == 3 ? 7 : 6) : 3;
  static constexpr int g0 = sums ? (DIM == 3 ? 4 : 3) : 0;  // first G word
};

// Pressure row p_base + c of cell c, written by the cell pass when p.prow
// is set: its one incidence is the cell's local DoF NF, its values are the
// orientation signs of the flux columns and 0 on the diagonal (record_row /
// final_row for a == NF), its residual entry r_p.  Consecutive cells own
// consecutive rows, so a warp's stores cover one contiguous stretch, and
// the row pass then covers the flux rows only (it no longer reads every
// record a second time for r_p).  A row other than the one incidence of
// NLOC columns that nfem_pattern_pairs makes sets NFEM_ERR_PATTERN.
// The pattern words of a pressure row, loaded when its cell's iteration
// starts so that their latency overlaps the cell's arithmetic.
struct PRowIn {
  int2 pr;
  uint32_t code, m;
  int32_t b0, b1;
};
__device__ __forceinline__ PRowIn load_prow(const DarcyParams& p, int64_t c) {
  PRowIn in;
  if (p.prow) {
    const int64_t r = p.p_base + c;
    in.pr = __ldg(reinterpret_cast<const int2*>(p.pairs) + r);
    in.code = __ldg(reinterpret_cast<const uint2*>(p.pair_codes) + r).x;
    in.b0 = __ldg(p.row_ptr + r);
    in.b1 = __ldg(p.row_ptr + r + 1);
    in.m = __ldg(p.sign + c);
  } else {
    in.pr = make_int2(-1, -1);
    in.code = in.m = 0u;
    in.b0 = in.b1 = 0;
  }
  return in;
}
// +-1 with the given sign, by bits
__device__ __forceinline__ double unit_signed(bool neg, double) {
  return __longlong_as_double(static_cast<long long>(0x3FF0000000000000ull | (static_cast<uint64_t>(neg) << 63)));
}
__device__ __forceinline__ float unit_signed(bool neg, float) {
  return __uint_as_float(0x3F800000u | (static_cast<uint32_t>(neg) << 31));
}

template <typename T, int DIM>
__device__ __forceinline__ void pressure_row(const DarcyParams& p, int64_t c, T rp, const PRowIn& in) {
  constexpr int NF = DIM + 1, NLOC = DIM + 2;
  using C = DarcyConst<T, DIM>;
  const int64_t r = p.p_base + c;
  if (in.pr.x != int32_t(c) * NLOC + NF || in.pr.y >= 0 || in.b1 - in.b0 != NLOC) {
    set_status(p.status, NFEM_ERR_PATTERN);
    return;
  }
  T* v = static_cast<T*>(p.values) + in.b0;
  T* rhs = static_cast<T*>(p.rhs);
  T val[NLOC];
  int pos[NLOC];
#pragma unroll
  for (int b = 0; b < NLOC; ++b) {
    const bool neg = b < NF && ((((in.m >> b) & 1u) != 0) != (C::sigma(b < NF ? b : 0) < T(0)));
    val[b] = b < NF ? unit_signed(neg, T(0)) : T(0);
    pos[b] = min(int((in.code >> (4 * b)) & 15u), NLOC - 1);
  }
  if (p.accumulate) {
#pragma unroll
    for (int b = 0; b < NLOC; ++b) v[pos[b]] += val[b];
    rhs[r] += rp;
  } else {
#pragma unroll
    for (int b = 0; b < NLOC; ++b) v[pos[b]] = val[b];
    rhs[r] = rp;
  }
}

// Record of cell c from its loaded incidence (see the layout above), and
// its pressure row when p.prow is set.  det_in > 0: |det J| (edge units)
// already formed in FP64 by the follow-up launch of badly shaped cells.
template <typename T, int DIM, int SRC>
__device__ __forceinline__ void write_record(const DarcyParams& p, int64_t c, const Incidence<T, DIM>& x, T u,
                                             const PRowIn& prow, T det_in = T(0)) {
  using L = RecLayout<T, DIM>;
  constexpr int NW = L::n;
  using C = DarcyConst<T, DIM>;
  T* rec = static_cast<T*>(p.rec);
  T G[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) G[i][j] = x.J[i][0] * x.J[j][0] + x.J[i][1] * x.J[j][1] + x.J[i][2] * x.J[j][2];
  T det = det_in;
  if (!(det > T(0))) {
    det = abs_det<T, DIM>(x.J, G);
    if constexpr (sizeof(T) == 4) {
      T g_min = G[0][0] < G[1][1] ? G[0][0] : G[1][1];
      if constexpr (DIM == 3) g_min = g_min < G[2][2] ? g_min : G[2][2];
      if (p.bad && det > T(0) && (shape_quality<DIM>(det, G) < kSliverQ || g_min < kShortEdge2)) {
        // left to darcy_refine_kernel (FP64 |det J|): no record, no pressure row here
        const int32_t k = atomicAdd(p.bad, 1);
        p.bad[4 + k] = int32_t(c);
        return;
      }
    }
  }
  if (!(det > T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
  const T det_true = DIM == 3 ? det * (u * u * u) : det * (u * u);
  const T scale = T(C::kappa2) * recip(x.kap * (DIM == 3 ? det * u : det));
  T rp = T(0);
  if constexpr (SRC == NFEM_COEF_CELL) rp = -det_true * T(C::area) * x.src;
  if constexpr (SRC == NFEM_COEF_QPOINT) rp = -det_true * x.src;
  T w[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) w[k] = T(0);
  if constexpr (L::sums) {
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
    w[0] = trG + sumG;
#pragma unroll
    for (int i = 0; i < DIM; ++i) w[1 + i] = R[i];
  }
  if constexpr (DIM == 3) {
    w[L::g0 + 0] = G[0][0];
    w[L::g0 + 1] = G[0][1];
    w[L::g0 + 2] = G[0][2];
    w[L::g0 + 4] = G[1][1];
    w[L::g0 + 5] = G[1][2];
    w[L::g0 + 6] = G[2][2];
  } else {
    w[L::g0 + 0] = G[0][0];
    w[L::g0 + 1] = G[0][1];
    w[L::g0 + 2] = G[1][1];
  }
  w[L::scale] = scale;
  w[L::rp] = rp;
  // 16-byte stores: a record never straddles a 32-byte sector per store
  const int64_t ri = rec_index(p, c);
  if constexpr (sizeof(T) == 4) {
    float4* out = reinterpret_cast<float4*>(rec + ri * NW);
#pragma unroll
    for (int k = 0; k < NW / 4; ++k) out[k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  } else {
    double2* out = reinterpret_cast<double2*>(rec + ri * NW);
#pragma unroll
    for (int k = 0; k < NW / 2; ++k) out[k] = make_double2(w[2 * k], w[2 * k + 1]);
  }
  if (p.prow) pressure_row<T, DIM>(p, c, rp, prow);
}

// One cell per thread and iteration (two in flight per thread measured
// slower: 100.8 against 96.0 us for the whole FP32 assembly at 64^3 x 6).
// Thread `t` of `nt` takes cells cell_begin + t, + nt, ... (the body of the
// cell-pass kernel and of the cell-pass blocks of the slice kernel).
template <typename T, int DIM, int SRC>
__device__ __forceinline__ void records_cells(const DarcyParams& p, int64_t t, int64_t nt) {
  const T u = edge_unit<T>(p);
  if constexpr (sizeof(T) == 4 && DIM == 3) {
    // the next cell's vertex ids one iteration ahead (as in the FP64 pass)
    const int4* __restrict__ cv4 = reinterpret_cast<const int4*>(p.cv);
    int4 v_next = p.cell_begin + t < p.cell_end ? __ldg(cv4 + p.cell_begin + t) : make_int4(0, 0, 0, 0);
    for (int64_t c = p.cell_begin + t; c < p.cell_end; c += nt) {
      const int4 v = v_next;
      if (c + nt < p.cell_end) v_next = __ldg(cv4 + c + nt);
      const PRowIn prow = load_prow(p, c);
      Incidence<T, DIM> x;
      load_incidence<T, DIM, SRC>(p, int32_t(c), true, x, &v);
      write_record<T, DIM, SRC>(p, c, x, u, prow);
    }
  } else {
    for (int64_t c = p.cell_begin + t; c < p.cell_end; c += nt) {
      const PRowIn prow = load_prow(p, c);
      Incidence<T, DIM> x;
      load_incidence<T, DIM, SRC>(p, int32_t(c), true, x);
      write_record<T, DIM, SRC>(p, c, x, u, prow);
    }
  }
}

template <typename T, int DIM, int SRC>
__global__ void __launch_bounds__(512) darcy_records_kernel(const DarcyParams p) {
  records_cells<T, DIM, SRC>(p, blockIdx.x * int64_t(blockDim.x) + threadIdx.x, int64_t(gridDim.x) * blockDim.x);
}

// The FP32 cells the cell pass left (shape quality below kSliverQ): |det J|
// in FP64, then the record and pressure row as in the cell pass.  The count
// is read on the device, so the launch needs no host round trip.
template <int DIM, int SRC>
__global__ void darcy_refine_kernel(const DarcyParams p) {
  const int32_t n = p.bad[0];
  const float u = edge_unit<float>(p);
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t c = p.bad[4 + i];
    const PRowIn prow = load_prow(p, c);
    Incidence<float, DIM> x;
    load_incidence<float, DIM, SRC>(p, c, true, x);
    write_record<float, DIM, SRC>(p, c, x, u, prow, refine_det<DIM>(p, c));
  }
}

// ------------------------------------------------------------------ FP64 tetrahedra
// FP64 records of tetrahedra hold the finished flux block, evaluated once
// per cell in double-float arithmetic on the FP32 pipes (df64.cuh) and
// packed into FP64 words by integer operations; only the nine edge
// subtractions run on the FP64 units.  Layout: 10 doubles (80 bytes) per
// record slot,
//   [U00, U01, U02, U03, U11, U12, U13, U22, U23, U33],
// and the pressure row's r_p in a region of its own after all slots
// (p.rp_off doubles from the start), which the row pass reads only when
// the cell pass has not written the pressure rows itself.
// U_ab = T120_ab / (30 kappa |det J|) without the orientation signs, with
//   T120_ab = (tr G + sum G) - 5 (R_a + R_b) + 20 G_ab,
// R_0 = 0, G_0b = 0 and R_a, G_ab (a, b >= 1) the row sums and entries of
// G = J^T J for the edges a - 1, b - 1: 120 times element_row's bracket
// tgs - gma - gmb + gv, so U_ab = scale * bracket with scale = 4 / (kappa
// |det J|).  The row pass applies the signs by flipping sign bits and adds
// the two incidences of a face's diagonal (its only FP64 operation).

// position of U_ab (= U_ba) in the record: the upper triangle row by row
__host__ __device__ constexpr int final_idx(int a, int b) {
  return (a < b ? a : b) * 4 - (a < b ? a : b) * ((a < b ? a : b) - 1) / 2 + (a < b ? b - a : a - b);
}
constexpr int kFinalWords = 10;

// Lattice cells.  With the fixed-point points, a cell's edge components
// e (exact 64-bit integers) are often all multiples of a common power of
// two 2^k with quotients n = e / 2^k below 2^11 in magnitude (every cell of
// a mesh on a dyadic grid, such as an n^3 cube with n a power of two, or a
// graded one whose cells span at most 2^11 steps of their own grid).  Then
// G = n n^T, the row sums, every T120_ab (|T120| < 186 * 2^22 < 2^31) and
// det (< 3 * 2^34) are exact in integer arithmetic, and the only rounding
// left is the one factor V = 1 / (30 kappa |det|):
//   U_ab = T120_ab * V * 2^(shift - k - e_kappa - e_det)
// with kappa = m_kappa 2^e_kappa, |det| = m_det 2^e_det (m in [1, 2)) and
// V = 1 / (30 m_kappa m_det) in double-float, turned into the 64-bit
// FP64 factor vs = V 2^(shift - k - e_kappa - e_det).  Each FP64 word is
// then the exact integer T120_ab (converted by bits) times vs: one FP64
// multiply, within one ulp of T120_ab vs (the FP64 pipe runs these beside
// the integer work; forming the product in 64-bit integer arithmetic took
// about a third more instructions per cell).  The same quantities as the double-float path,
// with fewer roundings and a fraction of its instructions.  (Keeping the
// integers in the record and forming the words in the row pass instead
// measured slower: the row pass needs 16 words per cell against 10 here,
// and it is the pass bound by memory latency and issue together.)
constexpr int kLatticeBits = 11;

__device__ __forceinline__ bool lattice_cell(const int64_t (&e)[3][3], int& k) {
  // trailing zeros of |x| and x agree; x ^ (x >> 63) is |x| or |x| - 1
  uint64_t o = 0, m = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o |= static_cast<uint64_t>(e[i][d]);
      m |= static_cast<uint64_t>(e[i][d] ^ (e[i][d] >> 63));
    }
  if (o == 0) return false;  // degenerate: the double-float path reports it
  k = __ffsll(static_cast<long long>(o)) - 1;
  return (m >> k) < (uint64_t(1) << kLatticeBits);
}

// Writes the record (and pressure row) of lattice cell c and returns true,
// or returns false without writing when a record word would leave the
// normal FP64 range (the double-float path then takes the cell).
template <int SRC>
__device__ __forceinline__ bool lattice_record(const DarcyParams& p, int64_t c, const int64_t (&e)[3][3], int k,
                                               int shift, double kap, dfloat F, const PRowIn& prow) {
  int32_t n[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int d = 0; d < 3; ++d) n[i][d] = static_cast<int32_t>(e[i][d] >> k);
  int32_t G[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) G[i][j] = n[i][0] * n[j][0] + n[i][1] * n[j][1] + n[i][2] * n[j][2];
  const int64_t cr0 = int64_t(n[1][1] * n[2][2] - n[1][2] * n[2][1]);
  const int64_t cr1 = int64_t(n[1][2] * n[2][0] - n[1][0] * n[2][2]);
  const int64_t cr2 = int64_t(n[1][0] * n[2][1] - n[1][1] * n[2][0]);
  const int64_t det = n[0][0] * cr0 + n[0][1] * cr1 + n[0][2] * cr2;
  const uint64_t adet = static_cast<uint64_t>(det < 0 ? -det : det);
  // m_det, m_kappa in [1, 2) and their binary exponents
  const int e_det = 63 - df_clz64(adet);
  const uint64_t kb = static_cast<uint64_t>(__double_as_longlong(kap));
  const int e_kap = int((kb >> 52) & 0x7ff) - 1023;
  // V = 1 / (30 m_kappa m_det) as the normalised 64-bit factor vq in [2^63, 2^64)
  const dfloat mdet = df_from_i64(static_cast<int64_t>(adet), e_det);
  const dfloat mkap = df_from_double(__longlong_as_double(static_cast<long long>((kb & 0xFFFFFFFFFFFFFull) |
                                                                                  (1023ull << 52))));
  // V 2^ex as one FP64 number (V in (1/120, 1/30]); every word T120 V 2^ex
  // with |T120| < 2^31 then stays a normal FP64 number
  const int ex = shift - k - e_kap - e_det;
  if (adet != 0 && (ex < -1010 || ex > 990)) return false;
  if (adet == 0) set_status(p.status, NFEM_ERR_DEGENERATE);
  const double vs = df_to_double_scaled(df_recip(df_mul_f(df_mul(mkap, mdet), 30.f)), ex);
  const int32_t R[3] = {G[0][0] + G[0][1] + G[0][2], G[0][1] + G[1][1] + G[1][2], G[0][2] + G[1][2] + G[2][2]};
  const int32_t S = G[0][0] + G[1][1] + G[2][2] + R[0] + R[1] + R[2];
  // T120 in record order, converted and stored two words at a time
  auto t120 = [&](int a, int b) -> int32_t {
    if (a == 0) return b == 0 ? S : S - 5 * R[b - 1];
    return S - 5 * (R[a - 1] + R[b - 1]) + 20 * G[a - 1][b - 1];
  };
  // the exact integer as FP64 (by bits), times vs: one FP64 multiply per word
  auto word = [&](int a, int b) { return df_i32_to_double(t120(a, b)) * vs; };
  const int64_t slot = rec_index(p, c);
  double2* o = reinterpret_cast<double2*>(static_cast<double*>(p.rec) + slot * kFinalWords);
  o[0] = make_double2(word(0, 0), word(0, 1));
  o[1] = make_double2(word(0, 2), word(0, 3));
  o[2] = make_double2(word(1, 1), word(1, 2));
  o[3] = make_double2(word(1, 3), word(2, 2));
  o[4] = make_double2(word(2, 3), word(3, 3));
  // r_p = -|det J| F = -(m_det F) 2^(e_det + 3 (k - shift))
  const double rp =
      (SRC == NFEM_COEF_NONE) ? 0.0 : df_to_double_scaled(df_neg(df_mul(mdet, F)), e_det + 3 * (k - shift));
  if (p.prow)
    pressure_row<double, 3>(p, c, rp, prow);
  else
    static_cast<double*>(p.rec)[p.rp_off + slot] = rp;
  return true;
}

// Record (and pressure row) of cell c, whose vertex ids v were loaded.
template <int SRC>
__device__ __forceinline__ void record_df_cell(const DarcyParams& p, int64_t c, const int4 v) {
  const double* __restrict__ kappa = static_cast<const double*>(p.kappa);
  const double* __restrict__ src = static_cast<const double*>(p.source);
  double* __restrict__ rec = static_cast<double*>(p.rec);
  const int vs[3] = {v.y, v.z, v.w};
  const PRowIn prow = load_prow(p, c);
  // coefficient checks on the bit patterns
  const double kap = __ldg(kappa + c);
  if (!df_bits_positive(kap)) set_status(p.status, df_bits_finite(kap) ? NFEM_ERR_DOMAIN : NFEM_ERR_NONFINITE);
  dfloat F = df_make(0.f);  // the source integrated over the reference cell
  if constexpr (SRC == NFEM_COEF_CELL) {
    const double s = __ldg(src + c);
    if (!df_bits_finite(s)) set_status(p.status, NFEM_ERR_NONFINITE);
    // 1/6 as a double-float constant (its FP32 part and the remainder)
    constexpr float kSixthHi = float(1.0 / 6.0);
    constexpr float kSixthLo = float(1.0 / 6.0 - double(kSixthHi));
    F = df_mul(df_from_double(s), dfloat{kSixthHi, kSixthLo});
  }
  if constexpr (SRC == NFEM_COEF_QPOINT) {
    double f = 0.0;
#pragma unroll 4
    for (int q = 0; q < 32; ++q)
      if (q < p.n_qp) f += p.qw[q] * __ldg(src + c * p.n_qp + q);
    if (!df_bits_finite(f)) set_status(p.status, NFEM_ERR_NONFINITE);
    F = df_from_double(f);
  }
  dfloat E[3][3];  // E[k][d]: edge k, component d
  if (p.fixed) {
    // exact integer differences of the fixed-point records
    const int shift = int(__ldg(p.fixed));
    const longlong2* Rp = reinterpret_cast<const longlong2*>(p.fixed);
    const longlong2 a0 = __ldg(Rp + 2 * (int64_t(v.x) + 1)), a1 = __ldg(Rp + 2 * (int64_t(v.x) + 1) + 1);
    int64_t e[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const longlong2 b0 = __ldg(Rp + 2 * (int64_t(vs[k]) + 1)), b1 = __ldg(Rp + 2 * (int64_t(vs[k]) + 1) + 1);
      e[k][0] = b0.x - a0.x;
      e[k][1] = b0.y - a0.y;
      e[k][2] = b1.x - a1.x;
    }
    int k2 = 0;
    if (p.lattice && lattice_cell(e, k2) && lattice_record<SRC>(p, c, e, k2, shift, kap, F, prow)) return;
    // converted by integer operations (no FP64 instruction)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) E[k][d] = df_from_i64(e[k][d], shift);
  } else {  // exactly rounded FP64 differences
    double x0[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) x0[d] = __ldg(p.points + int64_t(v.x) * 3 + d);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) E[k][d] = df_from_double(__ldg(p.points + int64_t(vs[k]) * 3 + d) - x0[d]);
  }
  const float one[3] = {1.f, 1.f, 1.f};
  // G = E E^T (edges as rows)
  dfloat G[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) G[i][j] = df_dot<3>(E[i], E[j], one);
  // |det J| = |E0 . (E1 x E2)|
  dfloat cr[3];
  {
    const float pm[2] = {1.f, -1.f};
    const dfloat a0[2] = {E[1][1], E[1][2]}, b0[2] = {E[2][2], E[2][1]};
    const dfloat a1[2] = {E[1][2], E[1][0]}, b1[2] = {E[2][0], E[2][2]};
    const dfloat a2[2] = {E[1][0], E[1][1]}, b2[2] = {E[2][1], E[2][0]};
    cr[0] = df_dot<2>(a0, b0, pm);
    cr[1] = df_dot<2>(a1, b1, pm);
    cr[2] = df_dot<2>(a2, b2, pm);
  }
  dfloat det = df_abs(df_dot<3>(E[0], cr, one));
  // a badly shaped cell: |det J| in FP64 from the points (df_dot's error
  // over the shape quality would exceed FP64's own)
  if (det.hi > 0.f && det.hi * rsqrtf(G[0][0].hi) * rsqrtf(G[1][1].hi) * rsqrtf(G[2][2].hi) < kSliverQ)
    det = df_from_double(refine_det64(p, c));
  if (!(det.hi > 0.f)) set_status(p.status, NFEM_ERR_DEGENERATE);
  // row sums R_i, S = tr G + sum G
  dfloat R[3];
  R[0] = df_add(df_add(G[0][0], G[0][1]), G[0][2]);
  R[1] = df_add(df_add(G[0][1], G[1][1]), G[1][2]);
  R[2] = df_add(df_add(G[0][2], G[1][2]), G[2][2]);
  const dfloat trG = df_add(df_add(G[0][0], G[1][1]), G[2][2]);
  const dfloat S = df_add(trG, df_add(df_add(R[0], R[1]), R[2]));
  // W = 1 / (30 kappa |det J|)
  const dfloat W = df_recip(df_mul_f(df_mul(df_from_double(kap), det), 30.f));
  dfloat R5[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) R5[i] = df_mul_f(R[i], 5.f);
  double out[kFinalWords];
  out[0] = df_to_double(df_mul(W, S));
#pragma unroll
  for (int b = 1; b < 4; ++b) out[b] = df_to_double(df_mul(W, df_sub(S, R5[b - 1])));
#pragma unroll
  for (int a = 1; a < 4; ++a)
#pragma unroll
    for (int b = a; b < 4; ++b) {
      const dfloat t = df_add(df_sub(S, df_add(R5[a - 1], R5[b - 1])), df_mul_f(G[a - 1][b - 1], 20.f));
      out[final_idx(a, b)] = df_to_double(df_mul(W, t));
    }
  const double rp = (SRC == NFEM_COEF_NONE) ? 0.0 : df_to_double(df_neg(df_mul(det, F)));
  const int64_t slot = rec_index(p, c);
  double2* o = reinterpret_cast<double2*>(rec + slot * kFinalWords);
#pragma unroll
  for (int k = 0; k < kFinalWords / 2; ++k) o[k] = make_double2(out[2 * k], out[2 * k + 1]);
  if (p.prow)
    pressure_row<double, 3>(p, c, rp, prow);
  else
    rec[p.rp_off + slot] = rp;
}

template <int SRC>
__device__ __forceinline__ void records_df_cells(const DarcyParams& p, int64_t t, int64_t nt) {
  // the next cell's vertex ids are loaded one iteration ahead, so the point
  // gathers that depend on them start without waiting for that load
  const int4* __restrict__ cv4 = reinterpret_cast<const int4*>(p.cv);
  int4 v_next = p.cell_begin + t < p.cell_end ? __ldg(cv4 + p.cell_begin + t) : make_int4(0, 0, 0, 0);
  for (int64_t c = p.cell_begin + t; c < p.cell_end; c += nt) {
    const int4 v = v_next;
    if (c + nt < p.cell_end) v_next = __ldg(cv4 + c + nt);
    record_df_cell<SRC>(p, c, v);
  }
}

#ifndef NFEM_DF_MIN_BLOCKS
#define NFEM_DF_MIN_BLOCKS 4
#endif
template <int SRC>
__global__ void __launch_bounds__(256, NFEM_DF_MIN_BLOCKS) darcy_records_df_kernel(const DarcyParams p) {
  records_df_cells<SRC>(p, blockIdx.x * int64_t(blockDim.x) + threadIdx.x, int64_t(gridDim.x) * blockDim.x);
}

// Flips the sign of x when neg (a sign-bit operation, no FP64 instruction).
__device__ __forceinline__ double flip_sign(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ (static_cast<long long>(neg) << 63));
}

// Row a of the cell in record slot `slot` from its finished FP64 record:
// the four U_ab with the orientation signs, the divergence column, and the
// pressure row's r_p.
template <bool COH>
__device__ __forceinline__ double rec_load(const double* ptr) {
  if constexpr (COH)
    return __ldcg(ptr);
  else
    return __ldg(ptr);
}

template <bool COH = false>
__device__ __forceinline__ void final_row(const DarcyParams& p, int64_t slot, uint32_t m, int a, double (&vals)[5],
                                          double& rhs_val) {
  using C = DarcyConst<double, 3>;
  const double* rec = static_cast<const double*>(p.rec);
  const double* r = rec + slot * kFinalWords;
  bool neg[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) neg[i] = (((m >> i) & 1u) != 0) != (C::sigma(i) < 0.0);  // sg_i < 0
  if (a < 4) {
    bool na = neg[0];
#pragma unroll
    for (int i = 1; i < 4; ++i) na = (a == i) ? neg[i] : na;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      // index of U_ab in the record without local-memory tables
      int idx = final_idx(0, b);
#pragma unroll
      for (int i = 1; i < 4; ++i) idx = (a == i) ? final_idx(i, b) : idx;
      vals[b] = flip_sign(rec_load<COH>(r + idx), na != neg[b]);
    }
    vals[4] = na ? 1.0 : -1.0;  // -sg_a
  } else {
#pragma unroll
    for (int b = 0; b < 4; ++b) vals[b] = neg[b] ? -1.0 : 1.0;
    vals[4] = 0.0;
    rhs_val += rec_load<COH>(rec + p.rp_off + slot);
  }
}

// Record words of cell c (vector loads: the record is 16-byte aligned); a
// pressure row (full == false) needs only the chunk holding r_p.
template <typename T, int DIM>
__device__ __forceinline__ void load_record(const T* __restrict__ rec, int32_t c, bool full,
                                            T (&w)[RecLayout<T, DIM>::n]) {
  using L = RecLayout<T, DIM>;
  constexpr int NW = L::n;
  if constexpr (sizeof(T) == 4) {
    const float4* q = reinterpret_cast<const float4*>(rec + int64_t(c) * NW);
#pragma unroll
    for (int k = 0; k < NW / 4; ++k) {
      if (!full && k != L::rp / 4) continue;
      const float4 v = __ldg(q + k);
      w[4 * k] = v.x;
      w[4 * k + 1] = v.y;
      w[4 * k + 2] = v.z;
      w[4 * k + 3] = v.w;
    }
  } else {
    const double2* q = reinterpret_cast<const double2*>(rec + int64_t(c) * NW);
#pragma unroll
    for (int k = 0; k < NW / 2; ++k) {
      if (!full && k != L::rp / 2) continue;
      const double2 v = __ldg(q + k);
      w[2 * k] = v.x;
      w[2 * k + 1] = v.y;
    }
  }
}

// Row a of cell c's element matrix from its record (element_row's values).
template <typename T, int DIM>
__device__ __forceinline__ void record_row(const T (&w)[RecLayout<T, DIM>::n], uint32_t m, int a,
                                           T (&vals)[DIM + 2], T& rhs_val) {
  using L = RecLayout<T, DIM>;
  constexpr int NF = DIM + 1;
  using C = DarcyConst<T, DIM>;
  T sg[NF];
#pragma unroll
  for (int i = 0; i < NF; ++i) sg[i] = ((m >> i) & 1u) ? -C::sigma(i) : C::sigma(i);
  if (a < NF) {
    T G[DIM][DIM];
    if constexpr (DIM == 3) {
      G[0][0] = w[L::g0]; G[0][1] = w[L::g0 + 1]; G[0][2] = w[L::g0 + 2];
      G[1][0] = G[0][1]; G[1][1] = w[L::g0 + 4]; G[1][2] = w[L::g0 + 5];
      G[2][0] = G[0][2]; G[2][1] = G[1][2]; G[2][2] = w[L::g0 + 6];
    } else {
      G[0][0] = w[L::g0]; G[0][1] = w[L::g0 + 1];
      G[1][0] = G[0][1]; G[1][1] = w[L::g0 + 2];
    }
    const T scale = w[L::scale];
    // element_row's expressions from here on
    T R[DIM];
    T S;
    if constexpr (L::sums) {
#pragma unroll
      for (int i = 0; i < DIM; ++i) R[i] = w[1 + i];
      S = w[0];
    } else {
      T trG = T(0), sumG = T(0);
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        R[i] = T(0);
#pragma unroll
        for (int j = 0; j < DIM; ++j) R[i] += G[i][j];
        trG += G[i][i];
        sumG += R[i];
      }
      S = trG + sumG;
    }
    const T tgs = S * T(C::f2);
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
    rhs_val += w[L::rp];
  }
}

// Bulk (TMA) store of a warp's staged CSR segment: one elected lane copies
// the 16-byte-aligned middle of the segment from shared to global memory;
// the lanes store the unaligned head and tail.  Both addresses and the size
// are multiples of 16 bytes (checked by the caller).
#ifndef NFEM_DARCY_BULK
#define NFEM_DARCY_BULK 1
#endif
__device__ __forceinline__ void bulk_store_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(static_cast<uint32_t>(__cvta_generic_to_shared(ssrc))), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// the staged source of every committed bulk store has been read
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// every committed bulk store has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

struct RowHead {
  int2 pr;
  uint2 cd;
};

__device__ __forceinline__ RowHead load_head(const DarcyParams& p, int64_t r, int64_t end) {
  RowHead h;
  if (r < end) {
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

// Block `rank` of `n_blocks` row blocks (kDarcyWarps warps each) writes the
// 32-row chunks rank * kDarcyWarps + warp, + n_blocks * kDarcyWarps, ...;
// st is the warp's staging buffer of 32 * kDarcyMaxRow values.
// One 32-row chunk [rb, re) (rows beyond re idle) with its lanes' head
// words h, row_ptr of the lane's row rpl and of the row after the chunk
// rpe; st is the warp's staging buffer.  COH reads the records through L2
// only (records written by other blocks of the same launch).
template <typename T, int DIM, int SRC, bool REC, bool COH = false>
__device__ __forceinline__ void process_chunk(const DarcyParams& p, T* st, int64_t rb, int64_t re, const RowHead h,
                                              int32_t rpl, int32_t rpe, bool bulk) {
  constexpr int NLOC = DIM + 2;
  constexpr int VEC = 16 / int(sizeof(T));  // values per 16 bytes
  const int lane = threadIdx.x & 31;
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  const int64_t r0 = rb;
  const int64_t r = r0 + lane;
  const bool valid = r < re;
  const int32_t base = __shfl_sync(0xffffffffu, rpl, 0);

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
  // row lengths and offsets inside the chunk straight from row_ptr
  // every lane takes part in the shuffle; lane 31 then uses the chunk end
  const int32_t rp_down = __shfl_down_sync(0xffffffffu, rpl, 1);
  const int32_t rpn = lane == 31 ? rpe : rp_down;
  const int len = valid ? rpn - rpl : 0;
  // staging index q of global entry base - sh + q: the bulk store's middle
  // is 16-byte aligned in both memories
  const int sh = bulk ? (base & (VEC - 1)) : 0;
  const int off = rpl - base + sh;
  const int span = rpe - base;
  if (span + sh > 32 * kDarcyMaxRow || span < 0) {  // rows of at most 16 entries fit
    if (lane == 0) set_status(p.status, NFEM_ERR_PATTERN);
    return;
  }
  const bool two = on[0] && on[1];
  const int pos_a0 = int((code[0] >> (4 * a[0])) & 15u), pos_a1 = int((code[1] >> (4 * a[1])) & 15u);
  // Two cells of a conforming simplicial mesh share exactly one column of a
  // face row (the face itself): then the row has 2 NLOC - 1 entries and
  // each is stored once, the diagonal summed in a register.  A warp with
  // any other layout zero-fills its image and adds every contribution.
  const bool simple = !on[0] || (two ? (len == 2 * NLOC - 1 && pos_a0 == pos_a1) : (len == NLOC));
  const bool direct = __all_sync(0xffffffffu, simple);
  if (!direct) {
    for (int i = lane; i < span; i += 32) st[sh + i] = T(0);
    __syncwarp();
  }
  constexpr int kCap = 32 * kDarcyMaxRow - 1;
  T rhs_val = T(0), diag = T(0);
#pragma unroll kDarcyIncUnroll
  for (int t = 0; t < 2; ++t) {
    if (on[t]) {
      T v[NLOC];
      if constexpr (REC && sizeof(T) == 8 && DIM == 3) {
        final_row<COH>(p, rec_index(p, c[t]), __ldg(p.sign + c[t]), a[t], v, rhs_val);
      } else if constexpr (REC) {
        T w[RecLayout<T, DIM>::n];
        load_record<T, DIM>(static_cast<const T*>(p.rec), int32_t(rec_index(p, c[t])), a[t] < DIM + 1, w);
        record_row<T, DIM>(w, __ldg(p.sign + c[t]), a[t], v, rhs_val);
      } else {
        Incidence<T, DIM> x;
        load_incidence<T, DIM, SRC>(p, c[t], geo[t], x);
        element_row<T, DIM, SRC>(p, x, a[t], geo[t], v, rhs_val);
      }
      const uint32_t cd = code[t];
      const int at = a[t];
      if (direct) {
        // the first incidence stores all its entries; the second stores its
        // own and overwrites the shared diagonal with the sum (one add)
        T d = T(0);
#pragma unroll
        for (int b = 0; b < NLOC; ++b) d = (b == at) ? v[b] : d;
        const T dsum = t == 1 ? d + diag : d;
#pragma unroll
        for (int b = 0; b < NLOC; ++b) {
          // codes index inside the row (< 16 entries); the clamp keeps a
          // corrupted code inside this warp's staging buffer
          const int idx = min(off + int((cd >> (4 * b)) & 15u), kCap);
          st[idx] = (b == at) ? dsum : v[b];
        }
        if (t == 0) diag = d;
      } else {
#pragma unroll
        for (int b = 0; b < NLOC; ++b) st[min(off + int((cd >> (4 * b)) & 15u), kCap)] += v[b];
      }
    }
  }
  __syncwarp();
  if (p.accumulate) {
    for (int i = lane; i < span; i += 32) values[int64_t(base) + i] += st[sh + i];
    if (valid) rhs[r] += rhs_val;
  } else {
    const int qe = sh + span;
    const int q0 = (sh + VEC - 1) & ~(VEC - 1), q1 = qe & ~(VEC - 1);
    T* gseg = values + (int64_t(base) - sh);  // global address of staging index 0
    if (bulk && q1 > q0) {
      if (lane == 0) bulk_store_s2g(gseg + q0, st + q0, uint32_t(q1 - q0) * uint32_t(sizeof(T)));
      if (lane < q0 - sh) gseg[sh + lane] = st[sh + lane];             // head: < VEC entries
      if (lane >= 16 && lane - 16 < qe - q1) gseg[q1 + lane - 16] = st[q1 + lane - 16];  // tail
    } else {
      for (int i = lane; i < span; i += 32) values[int64_t(base) + i] = st[sh + i];
    }
    if (valid) rhs[r] = rhs_val;
  }
  __syncwarp();
}

template <typename T, int DIM, int SRC, bool REC>
__device__ __forceinline__ void rows_body(const DarcyParams& p, T* st, int64_t rank, int64_t n_blocks) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* values = static_cast<T*>(p.values);
  // chunks of 32 rows: first over [row_f0, row_f1), then over [row_q0, row_q1)
  const int64_t nfc = (p.row_f1 - p.row_f0 + 31) / 32, nqc = (p.row_q1 - p.row_q0 + 31) / 32;
  const int64_t n_chunks = nfc + nqc;
  const int64_t jstride = n_blocks * kDarcyWarps;
  auto chunk_range = [&](int64_t j, int64_t& rb, int64_t& re) {
    if (j < nfc) {
      rb = p.row_f0 + 32 * j;
      re = p.row_f1;
    } else if (j < n_chunks) {
      rb = p.row_q0 + 32 * (j - nfc);
      re = p.row_q1;
    } else {
      rb = re = p.n_rows;
    }
  };
  int64_t j = rank * kDarcyWarps + warp;
  int64_t rb, re;
  chunk_range(j, rb, re);
  // row_ptr of the lane's row and of the row after the chunk (clamped to the range end)
  auto rp_at = [&](int64_t r, int64_t e) { return __ldg(p.row_ptr + (r < e ? r : e)); };
  RowHead head = load_head(p, rb + lane, re);
  int32_t rp_lane = rp_at(rb + lane, re), rp_end = rp_at(rb + 32, re);
  const bool bulk = NFEM_DARCY_BULK && !p.accumulate && (reinterpret_cast<uintptr_t>(values) & 15) == 0;
  for (; j < n_chunks; j += jstride) {
    if (bulk) {  // the staging buffer is free once the last bulk store has read it
      if (lane == 0) bulk_wait_read();
      __syncwarp();
    }
    const int64_t rbc = rb, rec_ = re;
    const RowHead h = head;
    const int32_t rpl = rp_lane, rpe = rp_end;
    // prefetch the next chunk of this warp (overlaps its latency with this one)
    chunk_range(j + jstride, rb, re);
    head = load_head(p, rb + lane, re);
    rp_lane = rp_at(rb + lane, re);
    rp_end = rp_at(rb + 32, re);
    process_chunk<T, DIM, SRC, REC>(p, st, rbc, rec_, h, rpl, rpe, bulk);
  }
  if (bulk && lane == 0) bulk_wait_all();
}

template <typename T, int DIM, int SRC, bool REC = false>
__global__ void __launch_bounds__(32 * kDarcyWarps,
                                  (sizeof(T) == 4 || (REC && DIM == 3)) ? NFEM_DARCY_MIN_BLOCKS : 1)
    darcy_rows_kernel(const DarcyParams p) {
  __shared__ __align__(16) T stage[kDarcyWarps][32 * kDarcyMaxRow];
  rows_body<T, DIM, SRC, REC>(p, stage[threadIdx.x >> 5], blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ slices
// One launch of the overlapped assembly of tetrahedra: the blocks of every
// group of four split into rec_quarters blocks running the cell pass over
// [cell_begin, cell_end) (the records of a later slice, compute bound) and
// 4 - rec_quarters blocks writing the rows of the current slice from
// records made by earlier launches (bandwidth bound), so the two passes run
// side by side on every SM.  No block waits for another.
template <typename T, int SRC>
__global__ void __launch_bounds__(32 * kDarcyWarps, sizeof(T) == 4 ? NFEM_DARCY_MIN_BLOCKS : 1)
    darcy_slice_kernel(const DarcyParams p, int rec_quarters) {
  __shared__ __align__(16) T stage[kDarcyWarps][32 * kDarcyMaxRow];
  const int64_t group = blockIdx.x >> 2, n_groups = gridDim.x >> 2;
  const int sub = int(blockIdx.x & 3);
  if (sub < rec_quarters) {
    const int64_t rank = group * rec_quarters + sub, nb = n_groups * rec_quarters;
    const int64_t t = rank * blockDim.x + threadIdx.x, nt = nb * blockDim.x;
    if constexpr (sizeof(T) == 8)
      records_df_cells<SRC>(p, t, nt);
    else
      records_cells<T, 3, SRC>(p, t, nt);
  } else {
    const int64_t rank = group * (4 - rec_quarters) + (sub - rec_quarters), nb = n_groups * (4 - rec_quarters);
    rows_body<T, 3, NFEM_COEF_NONE, true>(p, stage[threadIdx.x >> 5], rank, nb);
  }
}

// ------------------------------------------------------------------ cell chunks
// Cell-chunk variant of the same assembly, one chunk of 32 consecutive cells
// per warp.  Rows are numbered by first appearance, so the flux rows whose
// first incidence lies in the chunk are consecutive (the chunk row table),
// and so are the pressure rows of its cells.  Per chunk the warp:
//  (1) evaluates its 32 cells' element matrices once (lane = cell, coalesced
//      per-cell loads) into its shared-memory slice;
//  (2) queues the flux rows' second incidences that lie in a cell outside
//      the chunk (neighbours in a later row or layer of the mesh) and
//  (3) evaluates them densely, one per lane;
//  (4) writes the pressure rows and flux rows from shared memory, staged and
//      stored coalesced as in the row-owner kernel.
// Warps are independent (no block barriers).  Each value is written once and
// the queue order does not affect any value.
constexpr int kChunkWarps = 8;
constexpr int kChunkThreads = 32 * kChunkWarps;
constexpr int kMStride = 17;  // words per cell: odd, so the cells of a warp spread over the banks
constexpr int kQMax = 64;     // queued incidences per chunk; more are evaluated in the row pass
static_assert(NFEM_DARCY_CHUNK_CELLS == 32, "one warp per chunk");

template <typename T, int DIM>
struct WarpChunk {
  T M[32 * kMStride];          // rows a < NF of each cell's flux x flux block at a * 4 + b
  T rp[32];                    // residual entry of each cell's pressure row
  uint32_t sg[32];             // orientation masks
  T qv[kQMax * (DIM + 2)];     // values of the queued incidences
  int32_t qocc[kQMax];         // their occurrences (cell * NLOC + local)
  int16_t slot[4 * 32];        // queue slot per flux row of the chunk: -1 local, -2 not queued
  T stage[32 * kDarcyMaxRow];  // row images
};

// rows [first, last) of the warp's chunk (cells [c0, c0 + nk))
template <typename T, int DIM, int SRC>
__device__ __forceinline__ void warp_chunk_rows(const DarcyParams& p, WarpChunk<T, DIM>& w, int64_t first,
                                                int64_t last, int64_t c0, int64_t nk, bool is_flux) {
  constexpr int NF = DIM + 1, NLOC = DIM + 2;
  using C = DarcyConst<T, DIM>;
  const int lane = threadIdx.x & 31;
  T* st = w.stage;
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  constexpr int kCap = 32 * kDarcyMaxRow - 1;
  for (int64_t r0 = first; r0 < last; r0 += 32) {
    const int64_t r = r0 + lane;
    const bool valid = r < last;
    const RowHead h = load_head(p, valid ? r : p.n_rows, p.n_rows);
    // row lengths and offsets from row_ptr (every lane joins the shuffles)
    const int32_t rpl = __ldg(p.row_ptr + (r < p.n_rows ? r : p.n_rows));
    const int32_t rpe = __ldg(p.row_ptr + (r0 + 32 < last ? r0 + 32 : last));
    const int32_t base = __shfl_sync(0xffffffffu, rpl, 0);
    const int32_t rp_down = __shfl_down_sync(0xffffffffu, rpl, 1);
    const int occ[2] = {h.pr.x, h.pr.y};
    const uint32_t code[2] = {h.cd.x, h.cd.y};
    int32_t c[2];
    int a[2];
    bool on[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      on[t] = occ[t] >= 0;
      c[t] = on[t] ? occ[t] / NLOC : 0;
      a[t] = on[t] ? occ[t] - c[t] * NLOC : 0;
    }
    const int q1 = (is_flux && valid && on[1]) ? int(w.slot[r - first]) : -1;
    const int32_t rpn = lane == 31 ? rpe : rp_down;
    const int len = valid ? rpn - rpl : 0;
    const int off = rpl - base;
    const int span = rpe - base;
    if (span > 32 * kDarcyMaxRow || span < 0) {
      if (lane == 0) set_status(p.status, NFEM_ERR_PATTERN);
      continue;
    }
    const bool two = on[0] && on[1];
    const int pos_a0 = int((code[0] >> (4 * a[0])) & 15u), pos_a1 = int((code[1] >> (4 * a[1])) & 15u);
    const bool simple = !on[0] || (two ? (len == 2 * NLOC - 1 && pos_a0 == pos_a1) : (len == NLOC));
    const bool direct = __all_sync(0xffffffffu, simple);
    if (!direct) {
      for (int i = lane; i < span; i += 32) st[i] = T(0);
      __syncwarp();
    }
    T rhs_val = T(0), diag = T(0);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (on[t]) {
        T v[NLOC];
        const int64_t lc = int64_t(c[t]) - c0;
        const int qs = t == 1 ? q1 : -1;
        if (qs >= 0) {
#pragma unroll
          for (int b = 0; b < NLOC; ++b) v[b] = w.qv[qs * NLOC + b];
        } else if (lc >= 0 && lc < nk) {
          const uint32_t m = w.sg[lc];
          if (a[t] < NF) {
            const T* Mr = w.M + lc * kMStride + a[t] * 4;
#pragma unroll
            for (int b = 0; b < NF; ++b) v[b] = Mr[b];
            T sga = C::sigma(0);
#pragma unroll
            for (int i = 1; i < NF; ++i) sga = (a[t] == i) ? C::sigma(i) : sga;
            sga = ((m >> a[t]) & 1u) ? -sga : sga;
            v[NF] = -sga;
          } else {
#pragma unroll
            for (int b = 0; b < NF; ++b) v[b] = ((m >> b) & 1u) ? -C::sigma(b) : C::sigma(b);
            v[NF] = T(0);
            rhs_val += w.rp[lc];
          }
        } else {  // a second incidence the queue did not hold (or a chunk-table mismatch)
          Incidence<T, DIM> x;
          const bool geo = (a[t] < NF) || (SRC != 0);
          load_incidence<T, DIM, SRC>(p, c[t], geo, x);
          element_row<T, DIM, SRC>(p, x, a[t], geo, v, rhs_val);
        }
        const uint32_t cd = code[t];
        const int at = a[t];
        if (direct) {
          T d = T(0);
#pragma unroll
          for (int b = 0; b < NLOC; ++b) d = (b == at) ? v[b] : d;
#pragma unroll
          for (int b = 0; b < NLOC; ++b) {
            const int idx = min(off + int((cd >> (4 * b)) & 15u), kCap);
            st[idx] = (t == 1 && b == at) ? v[b] + diag : v[b];
          }
          if (t == 0) diag = d;
        } else {
#pragma unroll
          for (int b = 0; b < NLOC; ++b) st[min(off + int((cd >> (4 * b)) & 15u), kCap)] += v[b];
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

template <typename T, int DIM, int SRC>
__global__ void __launch_bounds__(kChunkThreads) darcy_cells_kernel(const DarcyParams p) {
  constexpr int NF = DIM + 1, NLOC = DIM + 2;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int lane = threadIdx.x & 31;
  WarpChunk<T, DIM>& w = reinterpret_cast<WarpChunk<T, DIM>*>(dsm)[threadIdx.x >> 5];
  const int64_t n_chunks = (p.n_cells + 31) / 32;
  const int64_t n_warps = int64_t(gridDim.x) * kChunkWarps;
  for (int64_t k = int64_t(blockIdx.x) * kChunkWarps + (threadIdx.x >> 5); k < n_chunks; k += n_warps) {
    const int64_t c0 = k * 32;
    const int64_t nk = min(int64_t(32), p.n_cells - c0);
    const int32_t f0 = __ldg(p.chunk_rows + k);
    const int32_t f1 = __ldg(p.chunk_rows + k + 1);
    // (1) element matrices, lane = cell
    if (lane < nk) {
      Incidence<T, DIM> x;
      load_incidence<T, DIM, SRC>(p, int32_t(c0 + lane), true, x);
      w.rp[lane] = cell_matrix<T, DIM, SRC>(p, x, w.M + lane * kMStride);
      w.sg[lane] = x.m;
    }
    // every cell opens at most NF flux rows; anything else is a table mismatch
    const bool rows_ok = f1 >= f0 && f1 - f0 <= NF * nk;
    if (!rows_ok && lane == 0) set_status(p.status, NFEM_ERR_PATTERN);
    // (2) queue the out-of-chunk second incidences
    int nq = 0;
    if (rows_ok) {
      for (int64_t rb = f0; rb < f1; rb += 32) {
        const int64_t r = rb + lane;
        int32_t occ = -1;
        if (r < f1) {
          occ = __ldg(p.pairs + 2 * r + 1);
          if (occ >= 0 && occ / NLOC < c0 + nk) occ = -1;
        }
        const unsigned want = __ballot_sync(0xffffffffu, occ >= 0);
        const int s = nq + __popc(want & ((1u << lane) - 1u));
        if (r < f1) {
          int16_t q = -1;
          if (occ >= 0) {
            if (s < kQMax) {
              w.qocc[s] = occ;
              q = int16_t(s);
            } else {
              q = -2;
            }
          }
          w.slot[r - f0] = q;
        }
        nq += __popc(want);
      }
    }
    nq = min(nq, kQMax);
    __syncwarp();
    // (3) the queue, one incidence per lane
    for (int i = lane; i < nq; i += 32) {
      const int32_t occ = w.qocc[i];
      const int32_t c = occ / NLOC;
      const int a = occ - c * NLOC;
      Incidence<T, DIM> x;
      const bool geo = (a < NF) || (SRC != 0);
      load_incidence<T, DIM, SRC>(p, c, geo, x);
      T v[NLOC], unused = T(0);
      element_row<T, DIM, SRC>(p, x, a, geo, v, unused);
#pragma unroll
      for (int b = 0; b < NLOC; ++b) w.qv[i * NLOC + b] = v[b];
    }
    __syncwarp();
    // (4) pressure rows, then flux rows
    warp_chunk_rows<T, DIM, SRC>(p, w, p.p_base + c0, p.p_base + c0 + nk, c0, nk, false);
    if (rows_ok) warp_chunk_rows<T, DIM, SRC>(p, w, f0, f1, c0, nk, true);
    __syncwarp();
  }
}

// One resident wave: blocks per SM from the occupancy calculator (queried
// once per kernel instance), times the SM count, capped by the work.
template <typename T, int DIM, int SRC, bool REC>
static int launch_darcy_rows(const DarcyParams& p, cudaStream_t stream) {
  const int block = 32 * kDarcyWarps;
  static const int per_sm = [] {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, darcy_rows_kernel<T, DIM, SRC, REC>, 32 * kDarcyWarps,
                                                      0) != cudaSuccess ||
        n < 1)
      n = 4;
    return n;
  }();
  const int64_t chunks = ceil_div(p.row_f1 - p.row_f0, 32) + ceil_div(p.row_q1 - p.row_q0, 32);
  const int tuned = knob(NFEM_KNOB_DARCY_ROWS_BLOCKS_PER_SM);
  const int grid = grid_for(ceil_div(chunks, kDarcyWarps), 1, tuned > 0 && tuned < per_sm ? tuned : per_sm);
  darcy_rows_kernel<T, DIM, SRC, REC><<<grid, block, 0, stream>>>(p);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// The cell pass over [cell_begin, cell_end): one thread per cell and
// iteration, the grid sized to the blocks the SMs hold at once (the
// occupancy of the kernel as built), so a grid-stride launch runs as one
// wave with no partly filled second one.
template <typename K>
static int resident_blocks(K kernel, int block) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, 0) != cudaSuccess || n < 1) n = 1;
  return n;
}

template <typename T, int DIM, int SRC>
static void launch_cell_pass(const DarcyParams& p, cudaStream_t stream) {
  const int64_t nc = p.cell_end - p.cell_begin;
  if (nc <= 0) return;
  const int cb = knob(NFEM_KNOB_DARCY_CELLS_BLOCK) > 0 ? knob(NFEM_KNOB_DARCY_CELLS_BLOCK) : 256;
  if constexpr (sizeof(T) == 8 && DIM == 3) {
    const int cbd = cb < 256 ? cb : 256;  // the double-float kernel is built for blocks of at most 256
    static int per_sm[3] = {0, 0, 0};     // blocks of 64, 128, 256 threads
    const int slot = cbd == 256 ? 2 : (cbd == 128 ? 1 : 0);
    if (!per_sm[slot]) per_sm[slot] = resident_blocks(darcy_records_df_kernel<SRC>, cbd);
    // two resident waves of blocks: at 64^3 x 6 the lattice cells take the same
    // time as with one wave (0.159 ms per step) and double-float cells 1.8 %
    // less; one block per 256 cells is 1.5 % slower on lattice cells
#ifndef NFEM_DF_GRID_SCALE
#define NFEM_DF_GRID_SCALE 2
#endif
    darcy_records_df_kernel<SRC><<<grid_for(nc, cbd, per_sm[slot] * NFEM_DF_GRID_SCALE), cbd, 0, stream>>>(p);
  } else {
    static int per_sm[4] = {0, 0, 0, 0};  // blocks of 64, 128, 256, 512 threads
    const int slot = cb == 512 ? 3 : (cb == 256 ? 2 : (cb == 128 ? 1 : 0));
    if (!per_sm[slot]) per_sm[slot] = resident_blocks(darcy_records_kernel<T, DIM, SRC>, cb);
    if constexpr (sizeof(T) == 4) {
      if (p.bad) cudaMemsetAsync(p.bad, 0, sizeof(int32_t), stream);
    }
    darcy_records_kernel<T, DIM, SRC><<<grid_for(nc, cb, per_sm[slot]), cb, 0, stream>>>(p);
    if constexpr (sizeof(T) == 4) {
      if (p.bad) darcy_refine_kernel<DIM, SRC><<<grid_for(nc, 128, 1), 128, 0, stream>>>(p);
    }
  }
}

// Single pass (the row kernel evaluates every incidence from the vertices)
// or, with the record workspace, the cell pass (records and the pressure
// rows) followed by the row pass over the flux rows and any rows after the
// pressure rows.
template <typename T, int DIM, int SRC>
static int launch_darcy_src(const DarcyParams& p_in, cudaStream_t stream) {
  if (!p_in.rec) return launch_darcy_rows<T, DIM, SRC, false>(p_in, stream);
  DarcyParams p = p_in;
  if (p.p_base >= 0 && p.p_base + p.n_cells <= p.n_rows) {
    p.prow = 1;
    p.row_f0 = 0;
    p.row_f1 = p.p_base;
    p.row_q0 = p.p_base + p.n_cells;
    p.row_q1 = p.n_rows;
  }
  launch_cell_pass<T, DIM, SRC>(p, stream);
  NFEM_CHECK_LAUNCH();
  return launch_darcy_rows<T, DIM, NFEM_COEF_NONE, true>(p, stream);
}

// One pass of the two-pass assembly over a range: pass 1 the cell records of
// [cell_begin, cell_end); pass 2 the rows [row_f0, row_f1) and [row_q0,
// row_q1) from records already formed (the caller orders the passes, e.g.
// records and rows of consecutive cell slices on two streams).
template <typename T, int DIM, int SRC>
static int launch_darcy_pass(const DarcyParams& p, int pass, cudaStream_t stream) {
  if (pass == 1) {
    launch_cell_pass<T, DIM, SRC>(p, stream);
    NFEM_CHECK_LAUNCH();
    return NFEM_OK;
  }
  if (p.row_f1 <= p.row_f0 && p.row_q1 <= p.row_q0) return NFEM_OK;
  return launch_darcy_rows<T, DIM, NFEM_COEF_NONE, true>(p, stream);
}

// The overlapped assembly: K = ceil(T / S) slices of S = 2^shift cells,
// K + 1 launches.  Launch 0 forms the records of slices 0 and 1; launch
// k + 1 writes the rows of slice k (its flux rows [F_k, F_k+1) and pressure
// rows) while forming the records of slice k + 2.  A row's cells lie in its
// slice or the next (the host checks lookahead < S), whose records earlier
// launches made; records of slice k + 2 take the ring place of slice k - 1,
// whose rows the previous launch wrote.
template <typename T, int SRC>
static int launch_darcy_sliced(DarcyParams p, int shift, const int64_t* flux_begin, int rec_quarters,
                               cudaStream_t stream) {
  static const int per_sm = [] {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, darcy_slice_kernel<T, SRC>, 32 * kDarcyWarps, 0) !=
            cudaSuccess ||
        n < 1)
      n = 4;
    return n;
  }();
  const int64_t S = int64_t(1) << shift, T_ = p.n_cells, K = ceil_div(T_, S);
  int grid = grid_for(int64_t(1) << 40, 1, per_sm);
  grid = grid < 4 ? 4 : grid & ~3;
  p.prow = 1;  // the cell blocks write the pressure rows of their cells
  for (int64_t l = 0; l <= K; ++l) {
    const int64_t k = l - 1;  // slice whose rows this launch writes
    p.cell_begin = l == 0 ? 0 : std::min((l + 1) * S, T_);
    p.cell_end = std::min((l == 0 ? 2 : l + 2) * S, T_);
    if (k >= 0) {
      p.row_f0 = flux_begin[k];
      p.row_f1 = flux_begin[k + 1];
      p.row_q0 = p.row_q1 = 0;
    } else {
      p.row_f0 = p.row_f1 = p.row_q0 = p.row_q1 = 0;
    }
    const bool has_rec = p.cell_end > p.cell_begin, has_rows = k >= 0;
    if (!has_rec && !has_rows) continue;
    const int q = !has_rows ? 4 : (!has_rec ? 0 : rec_quarters);
    darcy_slice_kernel<T, SRC><<<grid, 32 * kDarcyWarps, 0, stream>>>(p, q);
    NFEM_CHECK_LAUNCH();
  }
  return NFEM_OK;
}

template <typename T, int DIM, int SRC>
static int launch_darcy_chunks(const DarcyParams& p, cudaStream_t stream) {
  constexpr size_t smem = sizeof(WarpChunk<T, DIM>) * kChunkWarps;
  static const int per_sm = [] {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(darcy_cells_kernel<T, DIM, SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem)) != cudaSuccess)
      return -1;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, darcy_cells_kernel<T, DIM, SRC>, kChunkThreads, smem) !=
            cudaSuccess ||
        n < 1)
      n = 1;
    return n;
  }();
  if (per_sm < 0) return NFEM_ERR_CUDA;
  const int grid = grid_for(ceil_div(p.n_cells, 32 * kChunkWarps), 1, per_sm);
  darcy_cells_kernel<T, DIM, SRC><<<grid, kChunkThreads, smem, stream>>>(p);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

template <typename T, int DIM>
static int launch_darcy(const DarcyParams& p, int source_mode, cudaStream_t stream) {
  if (p.chunk_rows) {
    switch (source_mode) {
      case NFEM_COEF_NONE: return launch_darcy_chunks<T, DIM, NFEM_COEF_NONE>(p, stream);
      case NFEM_COEF_CELL: return launch_darcy_chunks<T, DIM, NFEM_COEF_CELL>(p, stream);
      case NFEM_COEF_QPOINT: return launch_darcy_chunks<T, DIM, NFEM_COEF_QPOINT>(p, stream);
      default: return NFEM_ERR_INVALID_ARG;
    }
  }
  switch (source_mode) {
    case NFEM_COEF_NONE: return launch_darcy_src<T, DIM, NFEM_COEF_NONE>(p, stream);
    case NFEM_COEF_CELL: return launch_darcy_src<T, DIM, NFEM_COEF_CELL>(p, stream);
    case NFEM_COEF_QPOINT: return launch_darcy_src<T, DIM, NFEM_COEF_QPOINT>(p, stream);
    default: return NFEM_ERR_INVALID_ARG;
  }
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_darcy_workspace_bytes(int dim, int value_type, int64_t n_cells, size_t* bytes) {
  if (!bytes || (dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_cells < 0)
    return NFEM_ERR_INVALID_ARG;
  // FP32: 8 words per cell, then the list of badly shaped cells (a count
  // and one index per cell); FP64: 10 + 1 (tetrahedra: the words, then r_p)
  // or 8 (triangles)
  *bytes = value_type == NFEM_F64 ? size_t(n_cells) * (dim == 3 ? 11 : 8) * 8
                                  : size_t(n_cells) * 8 * 4 + (size_t(n_cells) + 4) * 4;
  return NFEM_OK;
}

static int darcy_build(DarcyParams& p, int dim, int value_type, int64_t n_cells, int64_t n_rows,
                                         const double* points, const float* points_split,
                                         const int32_t* cell_vertices, const int32_t* flux_dofs, int64_t p_base,
                                         const uint8_t* sign_mask, const void* kappa, const void* source,
                                         int source_mode, const double* qweights, int n_qp,
                                         const int32_t* row_pairs, const uint32_t* pair_codes,
                                         const int32_t* row_ptr, const int32_t* chunk_rows, void* values,
                                         void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                                         int32_t* dev_status) {
  (void)flux_dofs;
  if ((dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_rows < 0)
    return NFEM_ERR_INVALID_ARG;
  if (!cell_vertices || !sign_mask || !kappa || !row_pairs || !pair_codes || !row_ptr || !values || !rhs)
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F64 && !points) return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F32 && (!points_split || (reinterpret_cast<uintptr_t>(points_split) & 15)))
    return NFEM_ERR_INVALID_ARG;
  if (source_mode != NFEM_COEF_NONE && !source) return NFEM_ERR_INVALID_ARG;
  if (source_mode == NFEM_COEF_QPOINT && (!qweights || n_qp < 1 || n_qp > 32)) return NFEM_ERR_INVALID_ARG;
  if (dim == 3 && (reinterpret_cast<uintptr_t>(cell_vertices) & 15)) return NFEM_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(row_pairs) & 7) || (reinterpret_cast<uintptr_t>(pair_codes) & 7))
    return NFEM_ERR_INVALID_ARG;
  if (chunk_rows && (n_cells < 1 || p_base < 0 || p_base + n_cells != n_rows)) return NFEM_ERR_INVALID_ARG;
  p.n_rows = n_rows;
  p.n_cells = n_cells;
  p.p_base = p_base;
  p.chunk_rows = chunk_rows;
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
  p.rec = nullptr;
  p.rp_off = 0;
  p.bad = nullptr;
  p.fixed = nullptr;
  p.lattice = knob(NFEM_KNOB_DARCY_F64_RECORDS) == 0;
  p.prow = 0;
  p.cell_begin = 0;
  p.cell_end = n_cells;
  p.row_f0 = 0;
  p.row_f1 = n_rows;
  p.row_q0 = p.row_q1 = 0;
  p.ring_shift = -1;
  if (value_type == NFEM_F64 && points_split) {
    if (reinterpret_cast<uintptr_t>(points_split) & 15) return NFEM_ERR_INVALID_ARG;
    p.fixed = reinterpret_cast<const int64_t*>(points_split);
  }
  if (workspace && !chunk_rows) {
    size_t need = 0;
    nfem_darcy_workspace_bytes(dim, value_type, n_cells, &need);
    if (workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 15) || n_cells < 0)
      return NFEM_ERR_WORKSPACE;
    p.rec = workspace;
    p.rp_off = kFinalWords * n_cells;
    if (value_type == NFEM_F32) p.bad = reinterpret_cast<int32_t*>(static_cast<float*>(workspace) + int64_t(n_cells) * 8);
  }
  return NFEM_OK;
}

extern "C" int nfem_darcy_rt1p0_assemble(int dim, int value_type, int64_t n_cells, int64_t n_rows,
                                         const double* points, const float* points_split,
                                         const int32_t* cell_vertices, const int32_t* flux_dofs, int64_t p_base,
                                         const uint8_t* sign_mask, const void* kappa, const void* source,
                                         int source_mode, const double* qweights, int n_qp,
                                         const int32_t* row_pairs, const uint32_t* pair_codes,
                                         const int32_t* row_ptr, const int32_t* chunk_rows, void* values,
                                         void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                                         int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_rows < 0)
    return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  DarcyParams p;
  const int rc = darcy_build(p, dim, value_type, n_cells, n_rows, points, points_split, cell_vertices, flux_dofs,
                             p_base, sign_mask, kappa, source, source_mode, qweights, n_qp, row_pairs, pair_codes,
                             row_ptr, chunk_rows, values, rhs, accumulate, workspace, workspace_bytes, dev_status);
  if (rc) return rc;
  if (value_type == NFEM_F64)
    return dim == 3 ? launch_darcy<double, 3>(p, source_mode, stream) : launch_darcy<double, 2>(p, source_mode, stream);
  return dim == 3 ? launch_darcy<float, 3>(p, source_mode, stream) : launch_darcy<float, 2>(p, source_mode, stream);
}

extern "C" int nfem_darcy_rt1p0_assemble_pass(int dim, int value_type, int64_t n_cells, int64_t n_rows,
                                              const double* points, const float* points_split,
                                              const int32_t* cell_vertices, int64_t p_base,
                                              const uint8_t* sign_mask, const void* kappa, const void* source,
                                              int source_mode, const double* qweights, int n_qp,
                                              const int32_t* row_pairs, const uint32_t* pair_codes,
                                              const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                                              void* workspace, size_t workspace_bytes, int pass, int64_t cell_begin,
                                              int64_t cell_end, int64_t row_f0, int64_t row_f1, int64_t row_q0,
                                              int64_t row_q1, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_rows < 0 ||
      (pass != 1 && pass != 2) || !workspace)
    return NFEM_ERR_INVALID_ARG;
  if (cell_begin < 0 || cell_end > n_cells || row_f0 < 0 || row_f1 > n_rows || row_q0 < 0 || row_q1 > n_rows)
    return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  DarcyParams p;
  const int rc = darcy_build(p, dim, value_type, n_cells, n_rows, points, points_split, cell_vertices, nullptr,
                             p_base, sign_mask, kappa, source, source_mode, qweights, n_qp, row_pairs, pair_codes,
                             row_ptr, nullptr, values, rhs, accumulate, workspace, workspace_bytes, dev_status);
  if (rc) return rc;
  p.cell_begin = cell_begin;
  p.cell_end = cell_end;
  p.row_f0 = row_f0;
  p.row_f1 = row_f1;
  p.row_q0 = row_q0;
  p.row_q1 = row_q1;
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    if (dim == 3) {
      switch (source_mode) {
        case NFEM_COEF_NONE: return launch_darcy_pass<T, 3, NFEM_COEF_NONE>(p, pass, stream);
        case NFEM_COEF_CELL: return launch_darcy_pass<T, 3, NFEM_COEF_CELL>(p, pass, stream);
        case NFEM_COEF_QPOINT: return launch_darcy_pass<T, 3, NFEM_COEF_QPOINT>(p, pass, stream);
        default: return NFEM_ERR_INVALID_ARG;
      }
    }
    switch (source_mode) {
      case NFEM_COEF_NONE: return launch_darcy_pass<T, 2, NFEM_COEF_NONE>(p, pass, stream);
      case NFEM_COEF_CELL: return launch_darcy_pass<T, 2, NFEM_COEF_CELL>(p, pass, stream);
      case NFEM_COEF_QPOINT: return launch_darcy_pass<T, 2, NFEM_COEF_QPOINT>(p, pass, stream);
      default: return NFEM_ERR_INVALID_ARG;
    }
  };
  return value_type == NFEM_F64 ? run(double(0)) : run(float(0));
}

extern "C" int nfem_darcy_ring_bytes(int value_type, int slice_shift, size_t* bytes) {
  if (!bytes || (value_type != NFEM_F64 && value_type != NFEM_F32) || slice_shift < 5 || slice_shift > 30)
    return NFEM_ERR_INVALID_ARG;
  // three slices of records: 10 + 1 doubles (FP64) or 8 floats (FP32) per tetrahedron
  *bytes = size_t(3) << slice_shift;
  *bytes *= value_type == NFEM_F64 ? 11 * sizeof(double) : 8 * sizeof(float);
  return NFEM_OK;
}

extern "C" int nfem_darcy_rt1p0_assemble_sliced(int value_type, int64_t n_cells, int64_t n_rows,
                                                const double* points, const void* point_records,
                                                const int32_t* cell_vertices, int64_t p_base,
                                                const uint8_t* sign_mask, const void* kappa, const void* source,
                                                int source_mode, const double* qweights, int n_qp,
                                                const int32_t* row_pairs, const uint32_t* pair_codes,
                                                const int32_t* row_ptr, const nfem_darcy_slices* slices,
                                                void* values, void* rhs, int accumulate, void* ring,
                                                size_t ring_bytes, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n_cells < 0 || n_rows < 0 || !slices) return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  if (!cell_vertices || !sign_mask || !kappa || !row_pairs || !pair_codes || !row_ptr || !values || !rhs ||
      !slices->flux_row_begin || p_base < 0 || p_base + n_cells != n_rows)
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F32 && (!point_records || (reinterpret_cast<uintptr_t>(point_records) & 15)))
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F64 && !points && !point_records) return NFEM_ERR_INVALID_ARG;
  if (point_records && (reinterpret_cast<uintptr_t>(point_records) & 15)) return NFEM_ERR_INVALID_ARG;
  if (source_mode != NFEM_COEF_NONE && !source) return NFEM_ERR_INVALID_ARG;
  if (source_mode == NFEM_COEF_QPOINT && (!qweights || n_qp < 1 || n_qp > 32)) return NFEM_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(cell_vertices) & 15) || (reinterpret_cast<uintptr_t>(row_pairs) & 7) ||
      (reinterpret_cast<uintptr_t>(pair_codes) & 7))
    return NFEM_ERR_INVALID_ARG;
  const int shift = slices->slice_shift;
  size_t need = 0;
  if (nfem_darcy_ring_bytes(value_type, shift, &need) != NFEM_OK) return NFEM_ERR_INVALID_ARG;
  if (!ring || ring_bytes < need || (reinterpret_cast<uintptr_t>(ring) & 15)) return NFEM_ERR_WORKSPACE;
  // every row's cells must lie in its slice or the next one
  if (slices->lookahead_cells < 0 || int64_t(slices->lookahead_cells) >= (int64_t(1) << shift))
    return NFEM_ERR_UNSUPPORTED;
  const int q = slices->record_quarters;
  if (q < 1 || q > 3) return NFEM_ERR_INVALID_ARG;
  const int64_t K = ceil_div(n_cells, int64_t(1) << shift);
  const int64_t* F = slices->flux_row_begin;
  if (F[0] != 0 || F[K] != p_base) return NFEM_ERR_INVALID_ARG;
  for (int64_t k = 0; k < K; ++k)
    if (F[k + 1] < F[k]) return NFEM_ERR_INVALID_ARG;
  DarcyParams p;
  p.n_rows = n_rows;
  p.n_cells = n_cells;
  p.p_base = p_base;
  p.chunk_rows = nullptr;
  p.points = points;
  p.split = value_type == NFEM_F32 ? static_cast<const float*>(point_records) : nullptr;
  p.fixed = value_type == NFEM_F64 ? static_cast<const int64_t*>(point_records) : nullptr;
  p.lattice = knob(NFEM_KNOB_DARCY_F64_RECORDS) == 0;
  p.prow = 0;
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
  p.rec = ring;
  p.bad = nullptr;  // the overlapped form keeps FP32 |det J| for every cell
  p.rp_off = int64_t(kFinalWords) * (int64_t(3) << shift);
  p.ring_shift = shift;
  if (value_type == NFEM_F64) {
    switch (source_mode) {
      case NFEM_COEF_NONE: return launch_darcy_sliced<double, NFEM_COEF_NONE>(p, shift, F, q, stream);
      case NFEM_COEF_CELL: return launch_darcy_sliced<double, NFEM_COEF_CELL>(p, shift, F, q, stream);
      case NFEM_COEF_QPOINT: return launch_darcy_sliced<double, NFEM_COEF_QPOINT>(p, shift, F, q, stream);
      default: return NFEM_ERR_INVALID_ARG;
    }
  }
  switch (source_mode) {
    case NFEM_COEF_NONE: return launch_darcy_sliced<float, NFEM_COEF_NONE>(p, shift, F, q, stream);
    case NFEM_COEF_CELL: return launch_darcy_sliced<float, NFEM_COEF_CELL>(p, shift, F, q, stream);
    case NFEM_COEF_QPOINT: return launch_darcy_sliced<float, NFEM_COEF_QPOINT>(p, shift, F, q, stream);
    default: return NFEM_ERR_INVALID_ARG;
  }
}

// ------------------------------------------------------------------ Dirichlet
// LaplaceDualWeakFormBCDirichlet (src/weak_forms/laplace_dual_weak_form.py:90-154):
// on a boundary facet the RT1 function of that face has the constant normal
// component sgn / |F| (sgn = +1 when its oriented normal points out of the
// cell), so r_f = sgn * |det J_F| / |F| * sum_q w_q p_D(x_q), and
// |det J_F| / |F| = 1 / |reference facet| (2 on triangles, 1 on intervals).
namespace nfem {
template <typename T, int DIM>
__global__ void darcy_dirichlet_kernel(int64_t n_facets, const int32_t* __restrict__ focc,
                                       const uint8_t* __restrict__ sign, const int32_t* __restrict__ cd, int ld,
                                       int dof_offset, int dof_stride, T scale,
                                       const T* __restrict__ pd, int nq, const double qw0, const double qw1,
                                       const double qw2, const double qw3, T* __restrict__ rhs) {
  using C = DarcyConst<T, DIM>;
  const double qw[4] = {qw0, qw1, qw2, qw3};
  for (int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; f < n_facets; f += int64_t(gridDim.x) * blockDim.x) {
    const int32_t occ = focc[f];
    const int32_t c = occ / (DIM + 1);
    const int i = occ - c * (DIM + 1);
    const uint32_t m = sign[c];
    T sg = C::sigma(i);
    if ((m >> i) & 1u) sg = -sg;
    T acc = T(0);
    for (int q = 0; q < nq; ++q) acc += T(qw[q]) * pd[f * nq + q];
    const T inv_ref = DIM == 3 ? T(2) : T(1);
    rhs[cd[int64_t(c) * ld + dof_offset + i * dof_stride]] += scale * sg * inv_ref * acc;
  }
}
}  // namespace nfem

static int rt1_dirichlet(int dim, int value_type, int64_t n_facets, const int32_t* facet_occ,
                         const uint8_t* sign_mask, const int32_t* cell_dofs, int ld, int dof_offset, int dof_stride,
                         double scale, const void* pd_q, const double* qweights, int n_qp, void* rhs,
                         cudaStream_t stream) {
  if ((dim != 2 && dim != 3) || (value_type != NFEM_F64 && value_type != NFEM_F32) || n_facets < 0 ||
      n_qp < 1 || n_qp > 4 || !qweights || dof_offset < 0 || dof_stride < 1 ||
      ld < dof_offset + dim * dof_stride + 1)
    return NFEM_ERR_INVALID_ARG;
  if (n_facets == 0) return NFEM_OK;
  if (!facet_occ || !sign_mask || !cell_dofs || !pd_q || !rhs) return NFEM_ERR_INVALID_ARG;
  double w[4] = {0, 0, 0, 0};
  for (int q = 0; q < n_qp; ++q) w[q] = qweights[q];
  const int g = grid_for(n_facets, 256);
#define NFEM_DIRICHLET(T, D)                                                                                        \
  darcy_dirichlet_kernel<T, D><<<g, 256, 0, stream>>>(n_facets, facet_occ, sign_mask, cell_dofs, ld, dof_offset,   \
                                                      dof_stride, T(scale), (const T*)pd_q, n_qp, w[0], w[1],      \
                                                      w[2], w[3], (T*)rhs)
  if (value_type == NFEM_F64) {
    if (dim == 3) NFEM_DIRICHLET(double, 3); else NFEM_DIRICHLET(double, 2);
  } else {
    if (dim == 3) NFEM_DIRICHLET(float, 3); else NFEM_DIRICHLET(float, 2);
  }
#undef NFEM_DIRICHLET
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_darcy_rt1_dirichlet(int dim, int value_type, int64_t n_facets, const int32_t* facet_occ,
                                        const uint8_t* sign_mask, const int32_t* cell_dofs, int ld,
                                        const void* pd_q, const double* qweights, int n_qp, void* rhs,
                                        void* stream_) {
  return rt1_dirichlet(dim, value_type, n_facets, facet_occ, sign_mask, cell_dofs, ld, 0, 1, 1.0, pd_q, qweights,
                       n_qp, rhs, (cudaStream_t)stream_);
}

extern "C" int nfem_rt1_dirichlet_rows(int dim, int value_type, int64_t n_facets, const int32_t* facet_occ,
                                       const uint8_t* sign_mask, const int32_t* cell_dofs, int ld, int dof_offset,
                                       int dof_stride, double scale, const void* pd_q, const double* qweights,
                                       int n_qp, void* rhs, void* stream_) {
  return rt1_dirichlet(dim, value_type, n_facets, facet_occ, sign_mask, cell_dofs, ld, dof_offset, dof_stride, scale,
                       pd_q, qweights, n_qp, rhs, (cudaStream_t)stream_);
}

// ------------------------------------------------------------------ L2 error
// l2_error (src/postprocess/l2_error_post_processor.py:7-63) for the RT1 x P0
// solution: err_u^2 = sum_cells sum_q |det J| w_q |u(x_q) - u_h(x_q)|^2 (vector
// branch :41-59), err_p^2 likewise with p_h = alpha_p (Lagrange branch
// :35-40).  FP64; per-block partials added in a fixed order.
namespace nfem {
struct L2Params {
  int64_t n_cells;
  const double* points;
  const int32_t* cv;
  const uint8_t* sign;
  const int32_t* cd;
  int ld;
  const double* alpha;
  const double* ue;  // [T, Q, dim]
  const double* pe;  // [T, Q]
  int nq;
  double qp[8][3];
  double qw[8];
  double* partial;   // [2, gridDim.x]
};

template <int DIM>
__global__ void darcy_l2_kernel(const L2Params p) {
  using C = DarcyConst<double, DIM>;
  __shared__ double sh[2][32];
  double eu = 0.0, ep = 0.0;
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < p.n_cells; c += int64_t(gridDim.x) * blockDim.x) {
    double x0[3], J[3][DIM];
    const int32_t v0 = p.cv[c * (DIM + 1)];
#pragma unroll
    for (int d = 0; d < 3; ++d) x0[d] = p.points[int64_t(v0) * 3 + d];
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const int32_t vk = p.cv[c * (DIM + 1) + k + 1];
#pragma unroll
      for (int d = 0; d < 3; ++d) J[d][k] = p.points[int64_t(vk) * 3 + d] - x0[d];
    }
    double det;
    if (DIM == 3) {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      det = fabs(det);
    } else {
      double g00 = 0, g01 = 0, g11 = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        g00 += J[d][0] * J[d][0];
        g01 += J[d][0] * J[d][DIM - 1];
        g11 += J[d][DIM - 1] * J[d][DIM - 1];
      }
      det = sqrt(g00 * g11 - g01 * g01);
    }
    const uint32_t m = p.sign[c];
    double a[DIM + 1];
#pragma unroll
    for (int i = 0; i <= DIM; ++i) {
      double sg = C::sigma(i);
      if ((m >> i) & 1u) sg = -sg;
      a[i] = sg * p.alpha[p.cd[c * p.ld + i]];
    }
    const double ap = p.alpha[p.cd[c * p.ld + DIM + 1]];
    const double kap = DIM == 3 ? 2.0 : 1.0;
    for (int q = 0; q < p.nq; ++q) {
      // uh = (1/|det|) J sum_i a_i kappa (xhat - vhat_i)
      double ref[DIM];
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i <= DIM; ++i) s += a[i] * kap * (p.qp[q][k] - (i == k + 1 ? 1.0 : 0.0));
        ref[k] = s;
      }
      double du2 = 0.0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double uh = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) uh += J[d][k] * ref[k];
        uh /= det;
        const double diff = p.ue[(c * p.nq + q) * DIM + d] - uh;
        du2 += diff * diff;
      }
      const double dp = p.pe[c * p.nq + q] - ap;
      eu += det * p.qw[q] * du2;
      ep += det * p.qw[q] * dp * dp;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    eu += __shfl_down_sync(0xffffffffu, eu, o);
    ep += __shfl_down_sync(0xffffffffu, ep, o);
  }
  if (lane == 0) { sh[0][warp] = eu; sh[1][warp] = ep; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double su = 0, sp = 0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) { su += sh[0][w]; sp += sh[1][w]; }
    p.partial[blockIdx.x] = su;
    p.partial[gridDim.x + blockIdx.x] = sp;
  }
}

__global__ void l2_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partial[threadIdx.x * nb + b];
    out[threadIdx.x] = sqrt(s);
  }
}
}  // namespace nfem

extern "C" int nfem_darcy_l2_error(int dim, int64_t n_cells, const double* points, const int32_t* cell_vertices,
                                   const uint8_t* sign_mask, const int32_t* cell_dofs, int ld, const double* alpha,
                                   const double* u_exact_q, const double* p_exact_q, const double* qpoints,
                                   const double* qweights, int n_qp, double* errors, void* workspace,
                                   size_t workspace_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  const int nb = 304;
  if ((dim != 2 && dim != 3) || n_cells < 0 || n_qp < 1 || n_qp > 8 || !qpoints || !qweights || !errors ||
      ld < dim + 2)
    return NFEM_ERR_INVALID_ARG;
  if (!workspace || workspace_bytes < size_t(2 * nb) * sizeof(double)) return NFEM_ERR_WORKSPACE;
  if (n_cells > 0 && (!points || !cell_vertices || !sign_mask || !cell_dofs || !alpha || !u_exact_q || !p_exact_q))
    return NFEM_ERR_INVALID_ARG;
  L2Params p;
  p.n_cells = n_cells;
  p.points = points;
  p.cv = cell_vertices;
  p.sign = sign_mask;
  p.cd = cell_dofs;
  p.ld = ld;
  p.alpha = alpha;
  p.ue = u_exact_q;
  p.pe = p_exact_q;
  p.nq = n_qp;
  for (int q = 0; q < 8; ++q) {
    p.qw[q] = q < n_qp ? qweights[q] : 0.0;
    for (int k = 0; k < 3; ++k) p.qp[q][k] = (q < n_qp && k < dim) ? qpoints[q * dim + k] : 0.0;
  }
  p.partial = (double*)workspace;
  if (dim == 3) darcy_l2_kernel<3><<<nb, 256, 0, stream>>>(p);
  else darcy_l2_kernel<2><<<nb, 256, 0, stream>>>(p);
  l2_final<<<1, 32, 0, stream>>>(p.partial, nb, errors);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

namespace nfem {

// ------------------------------------------------------------------ fused
// One persistent launch of the two-pass FP64 assembly of tetrahedra, the
// cell pass and the row pass side by side on every SM.  The work items are
// record chunks (32 consecutive cells: their records and pressure rows) and
// row chunks (32 consecutive flux rows), in the order of a schedule built
// once per pattern (nfem_darcy_fused_plan) that puts every row chunk after
// the record chunks of the cells its rows touch, plus a lead.  Warp w of
// the W resident warps takes items w, w + W, w + 2W, ... in turn:
//   record chunk: each lane forms one cell's record and pressure row; after
//                 a warp barrier lane 0 publishes the chunk's flag (release);
//   row chunk:    each lane waits (acquire, bounded) for the flags of the
//                 record chunks of its row's cells, then the warp writes the
//                 rows, reading the records through L2 only.
// Records are read back shortly after they are written, from L2, instead of
// after the whole cell pass, and no block-wide barrier couples the warps.
// The launch is cooperative, so all W warps are resident; an item waits only
// for items earlier in the schedule, each taken by a running warp whose own
// waits point further back, so every wait ends.  One that still runs out of
// polls sets NFEM_ERR_TIMEOUT and the warp goes on (its values are then not
// valid).
constexpr int kFusedThreads = 256;
constexpr int kFusedWarps = kFusedThreads / 32;
constexpr uint32_t kFusedPolls = 1u << 22;
#ifndef NFEM_FUSED_MIN_BLOCKS
#define NFEM_FUSED_MIN_BLOCKS 4
#endif

// Plan layout (int32 words): [0] items, [1] record chunks, [2] row chunks,
// [3] 0; then the last record chunk each row chunk touches; then the
// schedule (item >= 0: record chunk; item < 0: row chunk ~item); then,
// 16-byte aligned, one flag per record chunk, zeroed before each launch.
struct FusedLayout {
  int64_t rec_chunks, row_chunks, items, sync_word, words;
};
static FusedLayout fused_layout(int64_t n_cells, int64_t p_base) {
  FusedLayout L;
  L.rec_chunks = ceil_div(n_cells, int64_t(32));
  L.row_chunks = ceil_div(p_base, int64_t(32));
  L.items = L.rec_chunks + L.row_chunks;
  L.sync_word = (4 + L.row_chunks + L.items + 3) & ~int64_t(3);
  L.words = L.sync_word + L.rec_chunks;
  return L;
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* ptr) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* ptr, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(ptr), "r"(v) : "memory");
}
__device__ __forceinline__ void wait_flag(const DarcyParams& p, const uint32_t* flag) {
  uint32_t polls = 0;
  while (ld_acquire_gpu(flag) == 0u) {
    if (++polls >= kFusedPolls) {
      set_status(p.status, NFEM_ERR_TIMEOUT);
      return;
    }
    __nanosleep(32);
  }
}

template <int SRC>
__global__ void __launch_bounds__(kFusedThreads, NFEM_FUSED_MIN_BLOCKS)
    darcy_fused_kernel(const DarcyParams p, const int32_t* __restrict__ plan, uint32_t* flags) {
  __shared__ __align__(16) double stage[kFusedWarps][32 * kDarcyMaxRow];
  const int64_t n_items = plan[0];
  const int32_t* sched = plan + 4 + plan[2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t W = int64_t(gridDim.x) * kFusedWarps;
  const int4* __restrict__ cv4 = reinterpret_cast<const int4*>(p.cv);
  const bool bulk = NFEM_DARCY_BULK && !p.accumulate && (reinterpret_cast<uintptr_t>(p.values) & 15) == 0;
  double* st = stage[warp];
  auto rp_at = [&](int64_t r, int64_t e) { return __ldg(p.row_ptr + (r < e ? r : e)); };
  for (int64_t q = int64_t(blockIdx.x) * kFusedWarps + warp; q < n_items; q += W) {
    const int it = __ldg(sched + q);
    if (it >= 0) {
      const int64_t c = int64_t(it) * 32 + lane;
      if (c < p.n_cells) record_df_cell<SRC>(p, c, __ldg(cv4 + c));
      __syncwarp();
      if (lane == 0) {
        __threadfence();
        st_release_gpu(flags + it, 1u);
      }
    } else {
      const int64_t rb = p.row_f0 + int64_t(~it) * 32, re = p.row_f1;
      const RowHead h = load_head(p, rb + lane, re);
      const int32_t rpl = rp_at(rb + lane, re), rpe = rp_at(rb + 32, re);
      // (a cell beyond the plan's record chunks means the pattern is not the
      // one the plan was built from)
      const int32_t n_rec = plan[1];
      const int occ[2] = {h.pr.x, h.pr.y};
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        if (occ[t] < 0) continue;
        const int32_t k = occ[t] / 5 / 32;
        if (k < n_rec)
          wait_flag(p, flags + k);
        else
          set_status(p.status, NFEM_ERR_PATTERN);
      }
      if (bulk) {  // the staging buffer is free once the last bulk store has read it
        if (lane == 0) bulk_wait_read();
      }
      __syncwarp();
      process_chunk<double, 3, NFEM_COEF_NONE, true, true>(p, st, rb, re, h, rpl, rpe, bulk);
    }
  }
  if (bulk && lane == 0) bulk_wait_all();
}

// The last record chunk that each row chunk's rows touch (-1: none).
__global__ void fused_chunk_range_kernel(const int2* __restrict__ pairs, int64_t p_base, int64_t n_row_chunks,
                                         int32_t* __restrict__ hi_out) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  int hi = -1;
  if (r < p_base) {
    const int2 pr = pairs[r];
    if (pr.x >= 0) hi = max(hi, pr.x / 5 / 32);
    if (pr.y >= 0) hi = max(hi, pr.y / 5 / 32);
  }
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0 && (r >> 5) < n_row_chunks) hi_out[r >> 5] = hi;
}

template <int SRC>
static int fused_resident_blocks() {
  static int n = 0;
  if (!n) n = resident_blocks(darcy_fused_kernel<SRC>, kFusedThreads);
  return n;
}

template <int SRC>
static int launch_fused(const DarcyParams& p, const int32_t* plan, uint32_t* flags, int64_t items,
                        cudaStream_t stream) {
  const int grid = grid_for(items * 32, kFusedThreads, fused_resident_blocks<SRC>());
  void* args[] = {const_cast<DarcyParams*>(&p), const_cast<int32_t**>(&plan), &flags};
  NFEM_TRY_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(darcy_fused_kernel<SRC>), dim3(grid),
                                            dim3(kFusedThreads), args, 0, stream));
  return NFEM_OK;
}

}  // namespace nfem

extern "C" int nfem_darcy_fused_plan_bytes(int64_t n_cells, int64_t p_base, size_t* bytes) {
  if (!bytes || n_cells < 0 || p_base < 0) return NFEM_ERR_INVALID_ARG;
  if (n_cells > int64_t(INT32_MAX) / 5) return NFEM_ERR_OVERFLOW;
  *bytes = size_t(fused_layout(n_cells, p_base).words) * sizeof(int32_t);
  return NFEM_OK;
}

extern "C" int nfem_darcy_fused_plan(const int32_t* row_pairs, int64_t n_cells, int64_t p_base, int lead_chunks,
                                     void* plan, size_t plan_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  size_t need = 0;
  const int rc = nfem_darcy_fused_plan_bytes(n_cells, p_base, &need);
  if (rc) return rc;
  if (!plan || plan_bytes < need || (reinterpret_cast<uintptr_t>(plan) & 15) || lead_chunks < 0 ||
      (p_base > 0 && !row_pairs) || (reinterpret_cast<uintptr_t>(row_pairs) & 7))
    return NFEM_ERR_INVALID_ARG;
  const FusedLayout L = fused_layout(n_cells, p_base);
  int32_t* d = static_cast<int32_t*>(plan);
  std::vector<int32_t> h(size_t(L.sync_word), 0);
  if (L.row_chunks > 0) {
    fused_chunk_range_kernel<<<unsigned(ceil_div(L.row_chunks * 32, int64_t(256))), 256, 0, stream>>>(
        reinterpret_cast<const int2*>(row_pairs), p_base, L.row_chunks, d + 4);
    NFEM_CHECK_LAUNCH();
    NFEM_TRY_CUDA(cudaMemcpyAsync(h.data() + 4, d + 4, size_t(L.row_chunks) * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, stream));
    NFEM_TRY_CUDA(cudaStreamSynchronize(stream));
  }
  // every row chunk after the record chunks it touches plus the lead
  // (default: half the warps the GPU holds at once, so the record chunks a
  // row chunk needs were taken about one round of all warps earlier)
  const int64_t warps = int64_t(grid_for(int64_t(1) << 40, 1, fused_resident_blocks<NFEM_COEF_CELL>())) * kFusedWarps;
  const int64_t lead = lead_chunks > 0 ? lead_chunks : std::max<int64_t>(1, warps / 2);
  int32_t* sched = h.data() + 4 + L.row_chunks;
  int64_t q = 0, next_rec = 0;
  for (int64_t j = 0; j < L.row_chunks; ++j) {
    const int64_t hi = h[4 + j];
    if (hi >= L.rec_chunks) return NFEM_ERR_PATTERN;
    const int64_t upto = std::min<int64_t>(L.rec_chunks - 1, hi + lead);
    while (next_rec <= upto) sched[q++] = int32_t(next_rec++);
    sched[q++] = ~int32_t(j);
  }
  while (next_rec < L.rec_chunks) sched[q++] = int32_t(next_rec++);
  h[0] = int32_t(L.items);
  h[1] = int32_t(L.rec_chunks);
  h[2] = int32_t(L.row_chunks);
  NFEM_TRY_CUDA(cudaMemcpyAsync(d, h.data(), size_t(L.sync_word) * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
  NFEM_TRY_CUDA(cudaStreamSynchronize(stream));
  return NFEM_OK;
}

extern "C" int nfem_darcy_rt1p0_assemble_fused(int64_t n_cells, int64_t n_rows, const double* points,
                                               const void* point_records, const int32_t* cell_vertices,
                                               int64_t p_base, const uint8_t* sign_mask, const void* kappa,
                                               const void* source, int source_mode, const double* qweights, int n_qp,
                                               const int32_t* row_pairs, const uint32_t* pair_codes,
                                               const int32_t* row_ptr, void* plan, size_t plan_bytes, void* values,
                                               void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                                               int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0 || n_rows < 0 || p_base < 0 || p_base + n_cells != n_rows) return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  size_t need = 0;
  int rc = nfem_darcy_fused_plan_bytes(n_cells, p_base, &need);
  if (rc) return rc;
  if (!plan || plan_bytes < need || (reinterpret_cast<uintptr_t>(plan) & 15)) return NFEM_ERR_INVALID_ARG;
  DarcyParams p;
  rc = darcy_build(p, 3, NFEM_F64, n_cells, n_rows, points, static_cast<const float*>(point_records), cell_vertices,
                   nullptr, p_base, sign_mask, kappa, source, source_mode, qweights, n_qp, row_pairs, pair_codes,
                   row_ptr, nullptr, values, rhs, accumulate, workspace, workspace_bytes, dev_status);
  if (rc) return rc;
  if (!p.rec) return NFEM_ERR_WORKSPACE;
  const FusedLayout L = fused_layout(n_cells, p_base);
  int32_t* words = static_cast<int32_t*>(plan);
  p.prow = 1;
  p.row_f0 = 0;
  p.row_f1 = p_base;
  p.row_q0 = p.row_q1 = 0;
  uint32_t* flags = reinterpret_cast<uint32_t*>(words + L.sync_word);
  NFEM_TRY_CUDA(cudaMemsetAsync(flags, 0, size_t(L.rec_chunks) * sizeof(uint32_t), stream));
  switch (source_mode) {
    case NFEM_COEF_NONE: rc = launch_fused<NFEM_COEF_NONE>(p, words, flags, L.items, stream); break;
    case NFEM_COEF_CELL: rc = launch_fused<NFEM_COEF_CELL>(p, words, flags, L.items, stream); break;
    case NFEM_COEF_QPOINT: rc = launch_fused<NFEM_COEF_QPOINT>(p, words, flags, L.items, stream); break;
    default: return NFEM_ERR_INVALID_ARG;
  }
  if (rc) return rc;
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
