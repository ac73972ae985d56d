// Post-processing norms of one field of a product space on affine simplices.
//
// Reference: l2_error (src/postprocess/l2_error_post_processor.py:7-63: the
// Lagrange branch :35-40 compares components 0..dim-1, the vector branch
// :41-59 the rows of an RT field), div_error (:185-238), div_scaled_error
// (:240-306) and, with no discrete solution, l2_norm / div_norm
// (src/postprocess/solution_norms_post_processor.py:7-80).  Per cell
//   err^2 += sum_q |det J| w_q |e(x_q) - u_h(x_q)|^2
// with u_h from the cell's DoFs (basis-major, component-minor from
// dof_offset in the cell's row of cell_dofs):
//   Lagrange value   u_h,c = sum_a phihat_a(q) alpha_(a,c),  c < n_cmp
//   RT1 value        u_h,c = J (sum_i s_i psihat_i(q) alpha_(i,c)) / |det J|
//                    (row c of the field, its first n_cmp physical components)
//   RT1 divergence   div_h,c = sum_i s_i divhat_i alpha_(i,c) / |det J|
//   RT1 scaled div.  div_h,c = sum_i s_i (grad l . psi_i + l divhat_i /
//                    |det J|) alpha_(i,c), l and grad l at the points
// with s_i the orientation sign of the cell (sign_mask bit i: negated) and
// psihat, divhat the reference tables of the caller (they carry the
// reference normal convention).  FP64 throughout; one thread per cell, block
// partials added in a fixed order, so the result is deterministic.
#include "nfem_common.cuh"

namespace nfem {

constexpr int kNormMaxQ = 32;
constexpr int kNormMaxPhi = 10;
constexpr int kNormMaxComp = 3;
constexpr int kNormBlocks = 304;  // 2 x 152 SMs

struct NormParams {
  int dim, family, quantity;
  int64_t n_cells;
  const double* points;
  const int32_t* cv;
  const uint8_t* sign;
  const int32_t* cd;
  int ld, dof_offset, n_phi, n_comp, n_cmp, n_qp;
  const double* alpha;  // NULL: the exact field's own norm
  const double* exact;
  const double* gamma;       // [T, Q] (scaled divergence)
  const double* grad_gamma;  // [T, Q, dim]
  double* partial;
  double qw[kNormMaxQ];
  double tab[kNormMaxQ * kNormMaxPhi * 3];  // Lagrange [Q][n_phi]; RT1 [Q][n_phi][dim]
  double divhat[kNormMaxPhi];
};

template <int DIM>
__global__ void __launch_bounds__(256) field_error_kernel(const NormParams p) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < p.n_cells;
       c += int64_t(gridDim.x) * blockDim.x) {
    // J[d][k] = x_{k+1,d} - x_{0,d}
    double J[3][DIM];
    const int32_t v0 = __ldg(p.cv + c * (DIM + 1));
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const int32_t vk = __ldg(p.cv + c * (DIM + 1) + k + 1);
#pragma unroll
      for (int d = 0; d < 3; ++d) J[d][k] = __ldg(p.points + int64_t(vk) * 3 + d) - __ldg(p.points + int64_t(v0) * 3 + d);
    }
    double det;
    if constexpr (DIM == 3) {
      det = fabs(J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]));
    } else {
      double g00 = 0, g01 = 0, g11 = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        g00 += J[d][0] * J[d][0];
        g01 += J[d][0] * J[d][1];
        g11 += J[d][1] * J[d][1];
      }
      det = sqrt(g00 * g11 - g01 * g01);
    }
    const uint32_t m = p.family == 1 ? __ldg(p.sign + c) : 0u;
    // local coefficients alpha_(a, comp)
    double a[kNormMaxPhi][kNormMaxComp];
    for (int i = 0; i < p.n_phi; ++i)
      for (int k = 0; k < p.n_comp; ++k) {
        double v = 0.0;
        if (p.alpha) v = p.alpha[p.cd[c * p.ld + p.dof_offset + i * p.n_comp + k]];
        if (p.family == 1 && ((m >> i) & 1u)) v = -v;  // orientation sign
        a[i][k] = v;
      }
    for (int q = 0; q < p.n_qp; ++q) {
      double e2 = 0.0;
      // exact values per point: Lagrange [n_cmp]; RT1 values [n_comp][n_cmp]; divergences [n_comp]
      const int stride = p.family == 0 ? p.n_cmp : (p.quantity == 0 ? p.n_comp * p.n_cmp : p.n_comp);
      const double* ex = p.exact + (c * p.n_qp + q) * int64_t(stride);
      if (p.family == 0) {  // Lagrange values, components 0..n_cmp-1
        for (int k = 0; k < p.n_cmp; ++k) {
          double uh = 0.0;
          for (int i = 0; i < p.n_phi; ++i) uh += p.tab[q * p.n_phi + i] * a[i][k];
          const double d = ex[k] - uh;
          e2 += d * d;
        }
      } else if (p.quantity == 0) {  // RT1 rows: Piola-mapped values
        for (int k = 0; k < p.n_comp; ++k) {
          double ref[DIM];
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            double s = 0.0;
            for (int i = 0; i < p.n_phi; ++i) s += p.tab[(q * p.n_phi + i) * DIM + j] * a[i][k];
            ref[j] = s;
          }
          for (int d = 0; d < p.n_cmp; ++d) {
            double uh = 0.0;
#pragma unroll
            for (int j = 0; j < DIM; ++j) uh += J[d][j] * ref[j];
            const double diff = ex[k * p.n_cmp + d] - uh / det;
            e2 += diff * diff;
          }
        }
      } else {  // RT1 row divergences (optionally scaled by l)
        double gl[DIM], l = 1.0;
        if (p.quantity == 2) {
          l = p.gamma[c * p.n_qp + q];
#pragma unroll
          for (int j = 0; j < DIM; ++j) gl[j] = p.grad_gamma[(c * p.n_qp + q) * DIM + j];
        }
        for (int k = 0; k < p.n_comp; ++k) {
          double dv = 0.0;
          for (int i = 0; i < p.n_phi; ++i) {
            double t = l * p.divhat[i] / det;
            if (p.quantity == 2) {
              // grad l . psi_i with psi_i = J psihat_i / |det J|
              double g = 0.0;
#pragma unroll
              for (int j = 0; j < DIM; ++j) {
                double pj = 0.0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) pj += J[d][j] * gl[d];
                g += pj * p.tab[(q * p.n_phi + i) * DIM + j];
              }
              t += g / det;
            }
            dv += t * a[i][k];
          }
          const double diff = ex[k] - dv;
          e2 += diff * diff;
        }
      }
      acc += det * p.qw[q] * e2;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) sh[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    p.partial[blockIdx.x] = s;
  }
}

__global__ void field_error_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partial[b];
    *out = sqrt(s);
  }
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_field_error_workspace_bytes(size_t* bytes) {
  if (!bytes) return NFEM_ERR_INVALID_ARG;
  *bytes = size_t(kNormBlocks) * sizeof(double);
  return NFEM_OK;
}

extern "C" int nfem_field_error(int dim, int family, int quantity, int64_t n_cells, const double* points,
                                const int32_t* cell_vertices, const uint8_t* sign_mask, const int32_t* cell_dofs,
                                int ld, int dof_offset, int n_phi, int n_comp, int n_cmp, const double* alpha,
                                const double* exact_q, const double* gamma_q, const double* grad_gamma_q,
                                const double* ref_table, const double* ref_div, const double* qweights, int n_qp,
                                double* result, void* workspace, size_t workspace_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((dim != 2 && dim != 3) || (family != 0 && family != 1) || quantity < 0 || quantity > 2 || n_cells < 0 ||
      n_qp < 1 || n_qp > kNormMaxQ || n_phi < 1 || n_phi > kNormMaxPhi || n_comp < 1 || n_comp > kNormMaxComp ||
      n_cmp < 1 || !ref_table || !qweights || !result || dof_offset < 0 || ld < dof_offset + n_phi * n_comp)
    return NFEM_ERR_INVALID_ARG;
  if (family == 0 && (quantity != 0 || n_cmp > n_comp)) return NFEM_ERR_INVALID_ARG;
  if (family == 1 && (n_phi != dim + 1 || (quantity == 0 && n_cmp > 3) || (quantity > 0 && !ref_div)))
    return NFEM_ERR_INVALID_ARG;
  if (quantity == 2 && (!gamma_q || !grad_gamma_q)) return NFEM_ERR_INVALID_ARG;
  if (n_cells > 0 && (!points || !cell_vertices || !cell_dofs || !exact_q || (family == 1 && !sign_mask)))
    return NFEM_ERR_INVALID_ARG;
  if (!workspace || workspace_bytes < size_t(kNormBlocks) * sizeof(double)) return NFEM_ERR_WORKSPACE;
  NormParams p;
  p.dim = dim;
  p.family = family;
  p.quantity = quantity;
  p.n_cells = n_cells;
  p.points = points;
  p.cv = cell_vertices;
  p.sign = sign_mask;
  p.cd = cell_dofs;
  p.ld = ld;
  p.dof_offset = dof_offset;
  p.n_phi = n_phi;
  p.n_comp = n_comp;
  p.n_cmp = n_cmp;
  p.n_qp = n_qp;
  p.alpha = alpha;
  p.exact = exact_q;
  p.gamma = gamma_q;
  p.grad_gamma = grad_gamma_q;
  p.partial = static_cast<double*>(workspace);
  for (int q = 0; q < kNormMaxQ; ++q) p.qw[q] = q < n_qp ? qweights[q] : 0.0;
  const int width = family == 0 ? 1 : dim;
  for (int k = 0; k < kNormMaxQ * kNormMaxPhi * 3; ++k) p.tab[k] = k < n_qp * n_phi * width ? ref_table[k] : 0.0;
  for (int i = 0; i < kNormMaxPhi; ++i) p.divhat[i] = (ref_div && i < n_phi) ? ref_div[i] : 0.0;
  if (dim == 3)
    field_error_kernel<3><<<kNormBlocks, 256, 0, stream>>>(p);
  else
    field_error_kernel<2><<<kNormBlocks, 256, 0, stream>>>(p);
  NFEM_CHECK_LAUNCH();
  field_error_final<<<1, 32, 0, stream>>>(p.partial, kNormBlocks, result);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
