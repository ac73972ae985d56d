// Mixed Cosserat elasticity (3-D): element integrals + CSR scatter.
//
// Reference: LCEDualWeakForm.evaluate_form_vectorized
// (src/weak_forms/lce_dual_weak_form.py:410-648).  Fields s (RT1, three rows
// of the stress), m (RT1, three rows of the couple stress), u (P0^3), t (P0^3),
// local order s, m, u, t, basis-major / component-minor.  With
// Phi_ij = int psi_i psi_j^T (3 x 3) of the oriented, Piola-mapped RT1
// functions:
//   (s,s)[(i,c),(j,d)] = tr(Phi_ij) delta_cd (1/(4 mu) + 1/(4 kappa))
//                      + Phi_ij[d][c] (1/(4 mu) - 1/(4 kappa)) - vf Phi_ij[c][d],
//     vf = lambda / (2 mu (2 mu + 3 lambda));  (m,m) the same with the
//     couple-stress parameters, scaled by 1/l;
//   (t,s)[c,(j,d)] = M(v_j)[c][d], v_j = int psi_j, M(v) = [[0, vz, -vy],
//     [-vz, 0, vx], [vy, -vx, 0]]  (the asymmetry coupling, :531-580), and its
//     transpose in (s,t);
//   (u,s)[c,(j,d)] = delta_cd int div psi_j, (t,m) likewise, and transposes;
//   r[u_c] = -int f_c, r[t_c] = -int f_{3+c}  (alpha = 0).
// Closed forms on affine cells: Phi_ij = sg_i sg_j J Psihat_ij J^T / |det J|,
// v_j = sg_j J mhat_j, int div psi_j = sg_j divhat_j, sg = orientation signs.
//
// GPU design: the node-row owner of the vector P2 kernel (elasticity.cu):
// the CSR has 3 x 3 blocks (every field has three components), one warp owns
// a node's three rows, one 10-lane group per incidence, lane b evaluates the
// 3 x 3 block of local node b; group images summed in a fixed order.
#include <string.h>

#include <cmath>

#include <mutex>

#include "nfem_common.cuh"

namespace nfem {

constexpr int kCosDegMax = 32;
constexpr int kCosWarps = 4;

__constant__ double c_Psi[4 * 4 * 9];
__constant__ double c_mhat[4 * 3];
__constant__ double c_divhat[4];

static double h_Psi[144], h_mhat[12], h_divhat[4];
static bool h_cos_set = false;
static std::mutex h_cos_mutex;

static int upload_cos_tables(const double* Psi, const double* mhat, const double* divhat, cudaStream_t s) {
  std::lock_guard<std::mutex> lock(h_cos_mutex);
  if (h_cos_set && !memcmp(Psi, h_Psi, sizeof(h_Psi)) && !memcmp(mhat, h_mhat, sizeof(h_mhat)) &&
      !memcmp(divhat, h_divhat, sizeof(h_divhat)))
    return NFEM_OK;
  memcpy(h_Psi, Psi, sizeof(h_Psi));
  memcpy(h_mhat, mhat, sizeof(h_mhat));
  memcpy(h_divhat, divhat, sizeof(h_divhat));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_Psi, h_Psi, sizeof(h_Psi), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_mhat, h_mhat, sizeof(h_mhat), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaMemcpyToSymbolAsync(c_divhat, h_divhat, sizeof(h_divhat), 0, cudaMemcpyHostToDevice, s));
  NFEM_TRY_CUDA(cudaStreamSynchronize(s));
  h_cos_set = true;
  return NFEM_OK;
}

struct CosParams {
  int64_t n_nodes;
  int64_t n_cells;
  void* geom;  // [n_cells][12]: J (row-major, 9), |det J|, orientation mask (as bits), pad
  int64_t row0;
  const double* points;
  const float* split;
  const int32_t* cv;
  const uint8_t* sign;
  const double* par;  // host copy in the struct below
  double mu_s, kappa_s, lam_s, mu_o, kappa_o, lam_o, l;
  const void* force;  // [n_cells, 6] or NULL
  const int32_t* inc_ptr;
  const int32_t* inc;
  const uint8_t* codes;
  const int32_t* row_ptr;
  void* values;
  void* rhs;
  int accumulate;
  int32_t* status;
  // LCEScaledRieszMapWeakForm instead of the dual form: block-diagonal by
  // field, compliance without the 1/l of the couple stress, plus the
  // div-div term of every s row and (times l^2 for a constant l) every m row,
  // and the P0 mass on u and t; no coupling blocks, no load
  int riesz;
  // local DoFs per cell: 30 (s, m, u, t) or 18 (s, u, t: the linear
  // elasticity layout of LERieszMapWeakForm, no couple stress)
  int n_loc;
};

// block kind of local node x: 0..3 s faces, 4..7 m faces, 8 u, 9 t
__device__ __forceinline__ int cos_kind(int n_loc, int x) { return n_loc == 30 ? x : (x < 4 ? x : x + 4); }

template <typename T>
__device__ __forceinline__ void cos_edges(const CosParams& p, int32_t c, T (&J)[3][3]);

template <>
__device__ __forceinline__ void cos_edges<double>(const CosParams& p, int32_t c, double (&J)[3][3]) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p.cv) + c);
  const int vs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      J[d][k] = __ldg(p.points + int64_t(vs[k + 1]) * 3 + d) - __ldg(p.points + int64_t(vs[0]) * 3 + d);
}

template <>
__device__ __forceinline__ void cos_edges<float>(const CosParams& p, int32_t c, float (&J)[3][3]) {
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

template <typename T>
__device__ __forceinline__ T cos_det(const T (&J)[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// Badly shaped cells in FP32: det J from FP32 edges carries a relative error
// of a few ulps over the shape quality q = |det J| / (|e_0| |e_1| |e_2|), and
// an edge shorter than 2^20 units of the fixed-point records a relative error
// above 2^-21 from their rounding; cells with q < 0.1 or such an edge take J
// and det J in FP64, from the FP64 points when the caller passed them, else
// from the fixed-point records' exact integer differences, rounded to FP32
// once at the end.
constexpr float kCosSliverQ = 0.1f;

__device__ __noinline__ float cos_refine(const CosParams& p, int32_t c, float (&Jf)[3][3]) {
  double J[3][3];
  if (p.points) {
    cos_edges<double>(p, c, J);
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
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) Jf[i][k] = float(J[i][k]);
  return float(cos_det<double>(J));
}

// Per-cell geometry once per cell (each cell is read by the rows of its ten
// nodes): J, |det J| and the orientation mask.
template <typename T>
__global__ void cos_geom_kernel(const CosParams p) {
  T* out = static_cast<T*>(p.geom);
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < p.n_cells;
       c += int64_t(gridDim.x) * blockDim.x) {
    T J[3][3];
    cos_edges<T>(p, int32_t(c), J);
    T det = cos_det<T>(J);
    if constexpr (sizeof(T) == 4) {
      const T n0 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
      const T n1 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
      const T n2 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
      const T q = (det < T(0) ? -det : det) * rsqrtf(n0) * rsqrtf(n1) * rsqrtf(n2);
      const float s = packed_lo_scale(p.split) * 1048576.0f;  // 2^20 units
      if (q < T(kCosSliverQ) || fminf(n0, fminf(n1, n2)) < s * s) det = cos_refine(p, int32_t(c), J);
    }
    if (!(det != T(0))) set_status(p.status, NFEM_ERR_DEGENERATE);
    T g[12];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) g[i * 3 + k] = J[i][k];
    g[9] = det < T(0) ? -det : det;
    g[10] = T(__ldg(p.sign + c));
    g[11] = T(0);
#pragma unroll
    for (int k = 0; k < 12; ++k) out[c * 12 + k] = g[k];
  }
}

template <typename T>
__device__ __forceinline__ void cos_load_geom(const CosParams& p, int32_t c, T (&J)[3][3], T& adet, uint32_t& m) {
  T g[12];
  if constexpr (sizeof(T) == 4) {
    const float4* q = static_cast<const float4*>(p.geom) + int64_t(c) * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 v = __ldg(q + k);
      g[4 * k] = v.x;
      g[4 * k + 1] = v.y;
      g[4 * k + 2] = v.z;
      g[4 * k + 3] = v.w;
    }
  } else {
    const double2* q = static_cast<const double2*>(p.geom) + int64_t(c) * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const double2 v = __ldg(q + k);
      g[2 * k] = v.x;
      g[2 * k + 1] = v.y;
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) J[i][k] = g[i * 3 + k];
  adet = g[9];
  m = uint32_t(g[10]);
}

// 3 x 3 block between local nodes a (row) and b (column); node kinds:
// 0..3 s-faces, 4..7 m-faces, 8 u, 9 t.
template <typename T>
struct CosTables {
  T Psi[4 * 4 * 9];
  T mhat[12];
  T divhat[4];
};

template <typename T>
__device__ __forceinline__ void cos_block(const CosParams& p, const CosTables<T>& tb, const T (&J)[3][3], T adet,
                                          uint32_t m, int a, int b, T (&K)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) K[i][j] = T(0);
  const bool as = a < 4, am = a >= 4 && a < 8, au = a == 8, at = a == 9;
  const bool bs = b < 4, bm = b >= 4 && b < 8, bu = b == 8, bt = b == 9;
  const int fa = a & 3, fb = b & 3;
  const T sga = ((m >> fa) & 1u) ? T(-1) : T(1);
  const T sgb = ((m >> fb) & 1u) ? T(-1) : T(1);
  if (p.riesz) {
    if ((as && bs) || (am && bm)) {
      const T* Ps = tb.Psi + (fa * 4 + fb) * 9;
      T PJ[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int q = 0; q < 3; ++q)
          PJ[k][q] = Ps[k * 3 + 0] * J[q][0] + Ps[k * 3 + 1] * J[q][1] + Ps[k * 3 + 2] * J[q][2];
      T Phi[3][3];
      const T sc = sga * sgb / adet;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) Phi[c][d] = sc * (J[c][0] * PJ[0][d] + J[c][1] * PJ[1][d] + J[c][2] * PJ[2][d]);
      const T tr = Phi[0][0] + Phi[1][1] + Phi[2][2];
      const T mu = as ? T(p.mu_s) : T(p.mu_o), ka = as ? T(p.kappa_s) : T(p.kappa_o), la = as ? T(p.lam_s) : T(p.lam_o);
      const T cin = T(0.25) / mu + T(0.25) / ka;
      const T cout = T(0.25) / mu - T(0.25) / ka;
      const T vf = la / (T(2) * mu * (T(2) * mu + T(3) * la));
      // int div psi_a div psi_b = sga sgb divhat_a divhat_b / (|That| |det J|), |That| = 1/6
      const T dd = (as ? T(1) : T(p.l) * T(p.l)) * sga * sgb * tb.divhat[fa] * tb.divhat[fb] * T(6) / adet;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) K[c][d] = (c == d ? tr * cin + dd : T(0)) + Phi[d][c] * cout - vf * Phi[c][d];
    } else if ((au && bu) || (at && bt)) {
#pragma unroll
      for (int c = 0; c < 3; ++c) K[c][c] = adet * T(1.0 / 6.0);
    }
    return;
  }
  if ((as && bs) || (am && bm)) {
    // Phi = sga sgb J Psihat_ab J^T / |det|
    const T* Ps = tb.Psi + (fa * 4 + fb) * 9;
    T PJ[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int q = 0; q < 3; ++q)
        PJ[k][q] = Ps[k * 3 + 0] * J[q][0] + Ps[k * 3 + 1] * J[q][1] + Ps[k * 3 + 2] * J[q][2];
    T Phi[3][3];
    const T sc = sga * sgb / adet;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) Phi[c][d] = sc * (J[c][0] * PJ[0][d] + J[c][1] * PJ[1][d] + J[c][2] * PJ[2][d]);
    const T tr = Phi[0][0] + Phi[1][1] + Phi[2][2];
    T mu, ka, la, scale;
    if (as) { mu = T(p.mu_s); ka = T(p.kappa_s); la = T(p.lam_s); scale = T(1); }
    else { mu = T(p.mu_o); ka = T(p.kappa_o); la = T(p.lam_o); scale = T(1) / T(p.l); }
    const T cin = T(0.25) / mu + T(0.25) / ka;
    const T cout = T(0.25) / mu - T(0.25) / ka;
    const T vf = la / (T(2) * mu * (T(2) * mu + T(3) * la));
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) K[c][d] = scale * ((c == d ? tr * cin : T(0)) + Phi[d][c] * cout - vf * Phi[c][d]);
  } else if ((at && bs) || (as && bt)) {
    const int f = at ? fb : fa;
    const T sg = at ? sgb : sga;
    T v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      v[k] = sg * (J[k][0] * tb.mhat[f * 3 + 0] + J[k][1] * tb.mhat[f * 3 + 1] + J[k][2] * tb.mhat[f * 3 + 2]);
    T M[3][3] = {{T(0), v[2], -v[1]}, {-v[2], T(0), v[0]}, {v[1], -v[0], T(0)}};
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) K[c][d] = at ? M[c][d] : M[d][c];
  } else if ((au && bs) || (as && bu) || (at && bm) || (am && bt)) {
    const int f = (au || at) ? fb : fa;
    const T sg = (au || at) ? sgb : sga;
    const T val = sg * tb.divhat[f];
#pragma unroll
    for (int c = 0; c < 3; ++c) K[c][c] = val;
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * kCosWarps) cosserat_rows_kernel(const CosParams p) {
  // per warp, per group: rows i = 0..2 of the node, one 4-wide slot per node
  // column (components j = 0..2 and a pad), so a 3 x 3 block is added with
  // three 16-byte read-modify-writes
  __shared__ __align__(16) T img[kCosWarps][2][3 * kCosDegMax * 4];
  // reference tables read with per-lane indices: shared, not constant, memory
  __shared__ CosTables<T> tb;
  for (int i = threadIdx.x; i < 144; i += blockDim.x) tb.Psi[i] = T(c_Psi[i]);
  if (threadIdx.x < 12) tb.mhat[threadIdx.x] = T(c_mhat[threadIdx.x]);
  if (threadIdx.x < 4) tb.divhat[threadIdx.x] = T(c_divhat[threadIdx.x]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / 10, b = lane - 10 * (lane / 10);
  const T* force = static_cast<const T*>(p.force);
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  for (int64_t v = int64_t(blockIdx.x) * kCosWarps + warp; v < p.n_nodes; v += int64_t(gridDim.x) * kCosWarps) {
    const int64_t r0 = p.row0 + 3 * v;
    const int32_t base = __ldg(p.row_ptr + r0);
    const int len = __ldg(p.row_ptr + r0 + 1) - base;
    const int32_t kb = __ldg(p.inc_ptr + r0), ke = __ldg(p.inc_ptr + r0 + 1);
    if (len > 3 * kCosDegMax || len < 3 || len % 3 != 0 || ke - kb > 2) {
      if (lane == 0) set_status(p.status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    const int deg = len / 3;
    for (int q = lane; q < 2 * 3 * deg; q += 32) {
      T* slot = (q < 3 * deg ? img[warp][0] : img[warp][1]) + (q < 3 * deg ? q : q - 3 * deg) * 4;
      Slot4<T> z;
      z.zero();
      z.store(slot);
    }
    __syncwarp();
    T rhs_acc[3] = {T(0), T(0), T(0)};
    const int32_t k = kb + g;
    if (lane < 20 && k < ke && b < p.n_loc / 3) {
      const int32_t occ = __ldg(p.inc + k);
      const int32_t c = occ / p.n_loc;
      const int a = cos_kind(p.n_loc, (occ - c * p.n_loc) / 3);
      // node position inside the row; the clamp keeps a corrupted code in
      // this node's image (a valid one is < deg)
      const int pos = min(int(__ldg(p.codes + int64_t(k) * 16 + b)), deg - 1);
      T J[3][3], adet;
      uint32_t m;
      cos_load_geom<T>(p, c, J, adet, m);
      T K[3][3];
      cos_block<T>(p, tb, J, adet, m, a, cos_kind(p.n_loc, b), K);
      T* im = img[warp][g];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T* slot = im + (i * deg + pos) * 4;
        Slot4<T> s4;
        s4.load(slot);
#pragma unroll
        for (int j = 0; j < 3; ++j) s4[j] += K[i][j];
        s4.store(slot);
      }
      if (b == 0 && force && (a == 8 || a == 9)) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
          rhs_acc[i] = -adet * T(1.0 / 6.0) * __ldg(force + int64_t(c) * 6 + (a == 8 ? 0 : 3) + i);
      }
    }
    __syncwarp();
    // combine the two group images in a fixed order: one (row i, column) slot per lane
    for (int q = lane; q < 3 * deg; q += 32) {
      Slot4<T> s0, s1;
      s0.load(img[warp][0] + q * 4);
      s1.load(img[warp][1] + q * 4);
      const int i = q / deg, pos = q - i * deg;
      T* out = values + int64_t(base) + i * len + 3 * pos;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T sum = s0[j] + s1[j];
        if (p.accumulate) out[j] += sum; else out[j] = sum;
      }
    }
    T r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = __shfl_sync(0xffffffffu, rhs_acc[i], 0) + __shfl_sync(0xffffffffu, rhs_acc[i], 10);
    if (lane < 3 && rhs) {
      const T rv = lane == 0 ? r[0] : (lane == 1 ? r[1] : r[2]);
      if (p.accumulate) rhs[r0 + lane] += rv; else rhs[r0 + lane] = rv;
    }
    __syncwarp();
  }
}

// Register form of the node rows (as elasticity_rows_reg_kernel): lane L
// owns node column L of the row (deg <= 32), the two groups evaluate the
// blocks of the row's (at most two) incidences, and each block reaches the
// owner of its column by nine warp shuffles.  No shared-memory image; every
// block added by its owner in incidence order (bitwise deterministic).
__device__ __forceinline__ int cos_code_match(uint4 cw, int col) {
  const uint32_t rep = 0x01010101u * uint32_t(col);
  const uint32_t m0 = __vcmpeq4(cw.x, rep), m1 = __vcmpeq4(cw.y, rep), m2 = __vcmpeq4(cw.z, rep) & 0x0000ffffu;
  if (m0) return (__ffs(m0) - 1) >> 3;
  if (m1) return 4 + ((__ffs(m1) - 1) >> 3);
  if (m2) return 8 + ((__ffs(m2) - 1) >> 3);
  return -1;
}

template <typename T>
__global__ void __launch_bounds__(32 * kCosWarps) cosserat_rows_reg_kernel(const CosParams p) {
  __shared__ CosTables<T> tb;
  for (int i = threadIdx.x; i < 144; i += blockDim.x) tb.Psi[i] = T(c_Psi[i]);
  if (threadIdx.x < 12) tb.mhat[threadIdx.x] = T(c_mhat[threadIdx.x]);
  if (threadIdx.x < 4) tb.divhat[threadIdx.x] = T(c_divhat[threadIdx.x]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / 10, b = lane - 10 * (lane / 10);
  const T* force = static_cast<const T*>(p.force);
  T* values = static_cast<T*>(p.values);
  T* rhs = static_cast<T*>(p.rhs);
  const uint4* codes4 = reinterpret_cast<const uint4*>(p.codes);
  for (int64_t v = int64_t(blockIdx.x) * kCosWarps + warp; v < p.n_nodes; v += int64_t(gridDim.x) * kCosWarps) {
    const int64_t r0 = p.row0 + 3 * v;
    const int32_t base = __ldg(p.row_ptr + r0);
    const int len = __ldg(p.row_ptr + r0 + 1) - base;
    const int32_t kb = __ldg(p.inc_ptr + r0), ke = __ldg(p.inc_ptr + r0 + 1);
    if (len > 3 * kCosDegMax || len < 3 || len % 3 != 0 || ke - kb > 2) {
      if (lane == 0) set_status(p.status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    const int deg = len / 3;
    T K[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) K[i][j] = T(0);
    T rhs_acc[3] = {T(0), T(0), T(0)};
    const int32_t k = kb + g;
    if (lane < 20 && k < ke && b < p.n_loc / 3) {
      const int32_t occ = __ldg(p.inc + k);
      const int32_t c = occ / p.n_loc;
      const int a = cos_kind(p.n_loc, (occ - c * p.n_loc) / 3);
      T J[3][3], adet;
      uint32_t m;
      cos_load_geom<T>(p, c, J, adet, m);
      cos_block<T>(p, tb, J, adet, m, a, cos_kind(p.n_loc, b), K);
      if (b == 0 && force && (a == 8 || a == 9)) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
          rhs_acc[i] = -adet * T(1.0 / 6.0) * __ldg(force + int64_t(c) * 6 + (a == 8 ? 0 : 3) + i);
      }
    }
    T acc[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) acc[e] = T(0);
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
      if (kb + gg >= ke) break;  // warp-uniform
      const uint4 cw = __ldg(codes4 + (kb + gg));
      const int src = lane < deg ? cos_code_match(cw, lane) : -1;
      const int from = src >= 0 ? 10 * gg + src : lane;
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const T val = __shfl_sync(0xffffffffu, K[e / 3][e % 3], from);
        if (src >= 0) acc[e] += val;
      }
    }
    if (lane < deg) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T* out = values + int64_t(base) + i * len + 3 * lane;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (p.accumulate) out[j] += acc[i * 3 + j]; else out[j] = acc[i * 3 + j];
        }
      }
    }
    T r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = __shfl_sync(0xffffffffu, rhs_acc[i], 0) + __shfl_sync(0xffffffffu, rhs_acc[i], 10);
    if (lane < 3 && rhs) {
      const T rv = lane == 0 ? r[0] : (lane == 1 ? r[1] : r[2]);
      if (p.accumulate) rhs[r0 + lane] += rv; else rhs[r0 + lane] = rv;
    }
  }
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_cosserat_workspace_bytes(int value_type, int64_t n_cells, size_t* bytes) {
  if (!bytes || n_cells < 0 || (value_type != NFEM_F64 && value_type != NFEM_F32)) return NFEM_ERR_INVALID_ARG;
  *bytes = size_t(n_cells) * 12 * (value_type == NFEM_F64 ? sizeof(double) : sizeof(float));
  return NFEM_OK;
}

static int cosserat_launch(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0, const double* points,
                           const float* points_split, const int32_t* cell_vertices, const uint8_t* sign_mask,
                           const double* params7, const void* force, const double* ref_Psi, const double* ref_mhat,
                           const double* ref_divhat, const int32_t* inc_ptr, const int32_t* inc,
                           const uint8_t* node_codes, const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                           void* workspace, size_t workspace_bytes, int32_t* dev_status, void* stream_, int riesz,
                           int n_loc = 30) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0) return NFEM_ERR_INVALID_ARG;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n_nodes < 0 || row0 < 0 || !params7)
    return NFEM_ERR_INVALID_ARG;
  if (n_nodes == 0) return NFEM_OK;
  if (!cell_vertices || !sign_mask || !ref_Psi || !ref_mhat || !ref_divhat || !inc_ptr || !inc || !node_codes ||
      !row_ptr || !values || (!rhs && !riesz))
    return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F64 && !points) return NFEM_ERR_INVALID_ARG;
  if (value_type == NFEM_F32 && (!points_split || (reinterpret_cast<uintptr_t>(points_split) & 15)))
    return NFEM_ERR_INVALID_ARG;
  if (reinterpret_cast<uintptr_t>(cell_vertices) & 15) return NFEM_ERR_INVALID_ARG;
  // the material is one set of host constants: checked here (lambda may be
  // negative down to -2 mu / 3; the moduli mu, kappa and the length l not)
  for (int k = 0; k < 7; ++k)
    if (!std::isfinite(params7[k])) return NFEM_ERR_NONFINITE;
  if (!(params7[1] > 0) || !(params7[2] > 0) || !(params7[4] > 0) || !(params7[5] > 0) || !(params7[6] > 0))
    return NFEM_ERR_DOMAIN;
  int rc = upload_cos_tables(ref_Psi, ref_mhat, ref_divhat, stream);
  if (rc) return rc;
  CosParams p;
  p.n_nodes = n_nodes;
  p.row0 = row0;
  p.points = points;
  p.split = points_split;
  p.cv = cell_vertices;
  p.sign = sign_mask;
  p.par = nullptr;
  p.lam_s = params7[0];
  p.mu_s = params7[1];
  p.kappa_s = params7[2];
  p.lam_o = params7[3];
  p.mu_o = params7[4];
  p.kappa_o = params7[5];
  p.l = params7[6];
  p.force = force;
  p.inc_ptr = inc_ptr;
  p.inc = inc;
  p.codes = node_codes;
  p.row_ptr = row_ptr;
  p.values = values;
  p.rhs = rhs;
  p.accumulate = accumulate != 0;
  p.status = dev_status;
  p.riesz = riesz;
  p.n_loc = n_loc;
  const size_t vb = value_type == NFEM_F64 ? sizeof(double) : sizeof(float);
  if (!workspace || workspace_bytes < size_t(n_cells) * 12 * vb || (reinterpret_cast<uintptr_t>(workspace) & 15))
    return NFEM_ERR_WORKSPACE;
  p.n_cells = n_cells;
  p.geom = workspace;
  const int grid = grid_for(ceil_div(n_nodes, kCosWarps), 1, 8);
  // shared-memory images (the default: 0.346 against 0.353 ms at 24^3 x 6) or
  // register accumulation (knob 2)
  const bool reg = knob(NFEM_KNOB_ELAS_ROWS) == 2;
  if (value_type == NFEM_F64) {
    cos_geom_kernel<double><<<grid_for(n_cells, 256), 256, 0, stream>>>(p);
    if (reg)
      cosserat_rows_reg_kernel<double><<<grid, 32 * kCosWarps, 0, stream>>>(p);
    else
      cosserat_rows_kernel<double><<<grid, 32 * kCosWarps, 0, stream>>>(p);
  } else {
    cos_geom_kernel<float><<<grid_for(n_cells, 256), 256, 0, stream>>>(p);
    if (reg)
      cosserat_rows_reg_kernel<float><<<grid, 32 * kCosWarps, 0, stream>>>(p);
    else
      cosserat_rows_kernel<float><<<grid, 32 * kCosWarps, 0, stream>>>(p);
  }
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}


extern "C" int nfem_cosserat_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                      const double* points, const float* points_split, const int32_t* cell_vertices,
                                      const uint8_t* sign_mask, const double* params7, const void* force,
                                      const double* ref_Psi, const double* ref_mhat, const double* ref_divhat,
                                      const int32_t* inc_ptr, const int32_t* inc, const uint8_t* node_codes,
                                      const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                                      void* workspace, size_t workspace_bytes, int32_t* dev_status,
                                      void* stream) {
  return cosserat_launch(value_type, n_cells, n_nodes, row0, points, points_split, cell_vertices, sign_mask, params7,
                         force, ref_Psi, ref_mhat, ref_divhat, inc_ptr, inc, node_codes, row_ptr, values, rhs,
                         accumulate, workspace, workspace_bytes, dev_status, stream, 0);
}

extern "C" int nfem_cosserat_riesz_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                            const double* points, const float* points_split,
                                            const int32_t* cell_vertices, const uint8_t* sign_mask,
                                            const double* params7, const double* ref_Psi, const double* ref_mhat,
                                            const double* ref_divhat, const int32_t* inc_ptr, const int32_t* inc,
                                            const uint8_t* node_codes, const int32_t* row_ptr, void* values,
                                            int accumulate, void* workspace, size_t workspace_bytes,
                                            int32_t* dev_status, void* stream) {
  return cosserat_launch(value_type, n_cells, n_nodes, row0, points, points_split, cell_vertices, sign_mask, params7,
                         nullptr, ref_Psi, ref_mhat, ref_divhat, inc_ptr, inc, node_codes, row_ptr, values, nullptr,
                         accumulate, workspace, workspace_bytes, dev_status, stream, 1);
}

extern "C" int nfem_le_dual_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                     const double* points, const float* points_split, const int32_t* cell_vertices,
                                     const uint8_t* sign_mask, double lambda_, double mu, const void* force,
                                     const double* ref_Psi, const double* ref_mhat, const double* ref_divhat,
                                     const int32_t* inc_ptr, const int32_t* inc, const uint8_t* node_codes,
                                     const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                                     void* workspace, size_t workspace_bytes, int32_t* dev_status, void* stream) {
  // the Cosserat dual form over the 18-DoF layout with kappa = mu: the
  // compliance weighs the symmetric and skew parts alike (1/(2 mu)), and the
  // (t, s) and (u, s) couplings are the same operators
  const double par[7] = {lambda_, mu, mu, lambda_, mu, mu, 1.0};
  return cosserat_launch(value_type, n_cells, n_nodes, row0, points, points_split, cell_vertices, sign_mask, par,
                         force, ref_Psi, ref_mhat, ref_divhat, inc_ptr, inc, node_codes, row_ptr, values, rhs,
                         accumulate, workspace, workspace_bytes, dev_status, stream, 0, 18);
}

extern "C" int nfem_le_riesz_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                      const double* points, const float* points_split,
                                      const int32_t* cell_vertices, const uint8_t* sign_mask, double lambda_,
                                      double mu, const double* ref_Psi, const double* ref_mhat,
                                      const double* ref_divhat, const int32_t* inc_ptr, const int32_t* inc,
                                      const uint8_t* node_codes, const int32_t* row_ptr, void* values,
                                      int accumulate, void* workspace, size_t workspace_bytes,
                                      int32_t* dev_status, void* stream) {
  // the stress block of the Cosserat Riesz map with kappa = mu (equal weights
  // 1/(2 mu) on the symmetric and skew parts: 1/(4 mu) + 1/(4 kappa) = 1/(2 mu),
  // 1/(4 mu) - 1/(4 kappa) = 0) is the linear-elastic compliance; the
  // couple-stress parameters are unused by the 18-DoF layout
  const double par[7] = {lambda_, mu, mu, lambda_, mu, mu, 1.0};
  return cosserat_launch(value_type, n_cells, n_nodes, row0, points, points_split, cell_vertices, sign_mask, par,
                         nullptr, ref_Psi, ref_mhat, ref_divhat, inc_ptr, inc, node_codes, row_ptr, values, nullptr,
                         accumulate, workspace, workspace_bytes, dev_status, stream, 1, 18);
}
