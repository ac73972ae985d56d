// K6: the learned preconditioner's network - forward, backward and Adam.
//
// No reference counterpart: nfempy has no learned component.  The network
// is x -> relu(W1 x + b1) -> relu(W2 h1 + b2) -> W3 h2 + b3 with weights
// W_l [out, in] row-major in one flat parameter vector
//   [W1 | b1 | W2 | b2 | W3 | b3]
// and batch-major activations [batch, features].  Inference reads BF16
// weights (FP32 accumulation); training keeps FP32 master weights and
// refreshes the BF16 copy after every Adam step.
//
// GEMM: 64 x 64 output tiles, 16-deep K slices staged in shared memory, each
// of 256 threads owns a 4 x 4 register tile; operand transposes are template
// flags; the epilogue fuses the bias, the ReLU, and the ReLU mask of the
// backward pass.
#include <cuda_bf16.h>

#include "nfem_common.cuh"

namespace nfem {

constexpr int kBM = 64, kBN = 64, kBK = 16;

template <typename T>
__device__ __forceinline__ float ld_as_float(const T* p) {
  if constexpr (sizeof(T) == 2) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
  } else {
    return float(*p);
  }
}

// C[m, n] = sum_k A(m, k) B(k, n) (+ bias[n]); optional ReLU; optional mask
// (C *= mask[m, n] > 0).  A(m, k) = TA ? A[k * lda + m] : A[m * lda + k];
// B(k, n) = TB ? B[n * ldb + k] : B[k * ldb + n].
template <typename TAe, typename TBe, bool TA, bool TB>
__global__ void __launch_bounds__(256)
    gemm_kernel(int M, int N, int K, const TAe* __restrict__ A, int lda, const TBe* __restrict__ B, int ldb,
                float* __restrict__ C, int ldc, const float* __restrict__ bias, int relu,
                const float* __restrict__ mask, int ldm) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += kBK) {
    // A tile: kBM x kBK = 1024 values, 4 per thread
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + q * 256;
      int mm, kk;
      if (TA) { mm = idx % kBM; kk = idx / kBM; } else { kk = idx % kBK; mm = idx / kBK; }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TA ? ld_as_float(A + int64_t(gk) * lda + gm) : ld_as_float(A + int64_t(gm) * lda + gk);
      As[kk][mm] = v;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + q * 256;
      int nn, kk;
      if (TB) { kk = idx % kBK; nn = idx / kBK; } else { nn = idx % kBN; kk = idx / kBN; }
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < K) v = TB ? ld_as_float(B + int64_t(gn) * ldb + gk) : ld_as_float(B + int64_t(gk) * ldb + gn);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[gn];
      if (relu) v = fmaxf(v, 0.f);
      if (mask && !(mask[int64_t(gm) * ldm + gn] > 0.f)) v = 0.f;
      C[int64_t(gm) * ldc + gn] = v;
    }
  }
}

template <typename TAe, typename TBe, bool TA, bool TB>
static int gemm(int M, int N, int K, const TAe* A, int lda, const TBe* B, int ldb, float* C, int ldc,
                const float* bias, int relu, const float* mask, int ldm, cudaStream_t s) {
  if (M <= 0 || N <= 0) return NFEM_OK;
  dim3 grid(unsigned(ceil_div(N, kBN)), unsigned(ceil_div(M, kBM)));
  gemm_kernel<TAe, TBe, TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu, mask, ldm);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// dY = (Y - T) / batch; loss partials per block (sum of squares)
__global__ void loss_grad_kernel(int64_t n, const float* __restrict__ y, const float* __restrict__ t, float inv_b,
                                 float* __restrict__ dy, double* __restrict__ partial) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = d * inv_b;
    acc += double(d) * double(d);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) sh[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += sh[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void loss_final_kernel(const double* __restrict__ partial, int nb, double scale, double* __restrict__ loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += partial[b];
    *loss = scale * s;
  }
}

// g[n] = sum_m D[m, n] (deterministic column sums)
__global__ void colsum_kernel(int M, int N, const float* __restrict__ D, float* __restrict__ g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float acc = 0.f;
  for (int m = 0; m < M; ++m) acc += D[int64_t(m) * N + n];
  g[n] = acc;
}

__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                            __nv_bfloat16* __restrict__ pb) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void to_bf16_kernel(int64_t n, const float* __restrict__ p, __nv_bfloat16* __restrict__ pb) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    pb[i] = __float2bfloat16_rn(p[i]);
}

struct MlpLayout {
  int in, h1, h2, out;
  int64_t oW1, ob1, oW2, ob2, oW3, ob3, total;
};

static bool layout(const int32_t* dims, MlpLayout& L) {
  if (!dims) return false;
  L.in = dims[0]; L.h1 = dims[1]; L.h2 = dims[2]; L.out = dims[3];
  if (L.in < 1 || L.h1 < 1 || L.h2 < 1 || L.out < 1) return false;
  L.oW1 = 0;
  L.ob1 = L.oW1 + int64_t(L.h1) * L.in;
  L.oW2 = L.ob1 + L.h1;
  L.ob2 = L.oW2 + int64_t(L.h2) * L.h1;
  L.oW3 = L.ob2 + L.h2;
  L.ob3 = L.oW3 + int64_t(L.out) * L.h2;
  L.total = L.ob3 + L.out;
  return true;
}

template <typename WT>
static int forward_t(const MlpLayout& L, const WT* P, const float* Pf, int64_t B, const float* x, float* h1, float* h2,
                     float* y, cudaStream_t s) {
  // biases always read from the FP32 copy when present (they are tiny)
  const float* b1 = Pf ? Pf + L.ob1 : nullptr;
  const float* b2 = Pf ? Pf + L.ob2 : nullptr;
  const float* b3 = Pf ? Pf + L.ob3 : nullptr;
  int rc = gemm<float, WT, false, true>(int(B), L.h1, L.in, x, L.in, P + L.oW1, L.in, h1, L.h1, b1, 1, nullptr, 0, s);
  if (rc) return rc;
  rc = gemm<float, WT, false, true>(int(B), L.h2, L.h1, h1, L.h1, P + L.oW2, L.h1, h2, L.h2, b2, 1, nullptr, 0, s);
  if (rc) return rc;
  return gemm<float, WT, false, true>(int(B), L.out, L.h2, h2, L.h2, P + L.oW3, L.h2, y, L.out, b3, 0, nullptr, 0, s);
}

template <typename WT>
static int backward_t(const MlpLayout& L, const WT* P, int64_t B, const float* x, const float* h1, const float* h2,
                      const float* y, const float* t, float* G, float* work, double* loss, cudaStream_t s) {
  float* dy = work;                       // [B, out]
  float* dz2 = dy + B * L.out;            // [B, h2]
  float* dz1 = dz2 + B * L.h2;            // [B, h1]
  const int64_t used = B * (int64_t(L.out) + L.h2 + L.h1);
  double* partial = reinterpret_cast<double*>(work + used + (used & 1));
  const int nb = 256;
  loss_grad_kernel<<<nb, 256, 0, s>>>(B * L.out, y, t, 1.f / float(B), dy, partial);
  if (loss) loss_final_kernel<<<1, 32, 0, s>>>(partial, nb, 0.5 / double(B), loss);
  NFEM_CHECK_LAUNCH();
  int rc;
  // layer 3
  rc = gemm<float, float, true, false>(L.out, L.h2, int(B), dy, L.out, h2, L.h2, G + L.oW3, L.h2, nullptr, 0, nullptr, 0, s);
  if (rc) return rc;
  colsum_kernel<<<unsigned(ceil_div(L.out, 128)), 128, 0, s>>>(int(B), L.out, dy, G + L.ob3);
  rc = gemm<float, WT, false, false>(int(B), L.h2, L.out, dy, L.out, P + L.oW3, L.h2, dz2, L.h2, nullptr, 0, h2, L.h2, s);
  if (rc) return rc;
  // layer 2
  rc = gemm<float, float, true, false>(L.h2, L.h1, int(B), dz2, L.h2, h1, L.h1, G + L.oW2, L.h1, nullptr, 0, nullptr, 0, s);
  if (rc) return rc;
  colsum_kernel<<<unsigned(ceil_div(L.h2, 128)), 128, 0, s>>>(int(B), L.h2, dz2, G + L.ob2);
  rc = gemm<float, WT, false, false>(int(B), L.h1, L.h2, dz2, L.h2, P + L.oW2, L.h1, dz1, L.h1, nullptr, 0, h1, L.h1, s);
  if (rc) return rc;
  // layer 1
  rc = gemm<float, float, true, false>(L.h1, L.in, int(B), dz1, L.h1, x, L.in, G + L.oW1, L.in, nullptr, 0, nullptr, 0, s);
  if (rc) return rc;
  colsum_kernel<<<unsigned(ceil_div(L.h1, 128)), 128, 0, s>>>(int(B), L.h1, dz1, G + L.ob1);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_mlp_param_count(const int32_t* dims, int64_t* count) {
  MlpLayout L;
  if (!count || !layout(dims, L)) return NFEM_ERR_INVALID_ARG;
  *count = L.total;
  return NFEM_OK;
}

extern "C" int nfem_mlp_backward_workspace_bytes(const int32_t* dims, int64_t batch, size_t* bytes) {
  MlpLayout L;
  if (!bytes || batch < 1 || !layout(dims, L)) return NFEM_ERR_INVALID_ARG;
  *bytes = size_t(batch) * (L.out + L.h2 + L.h1 + 1) * sizeof(float) + 256 * sizeof(double) + 64;
  return NFEM_OK;
}

extern "C" int nfem_mlp_forward(const int32_t* dims, int weight_type, const void* params, const float* params_f32,
                                int64_t batch, const float* x, float* h1, float* h2, float* y, void* stream) {
  MlpLayout L;
  if (!layout(dims, L) || batch < 0 || batch > INT32_MAX || !params || !x || !h1 || !h2 || !y)
    return NFEM_ERR_INVALID_ARG;
  if (batch == 0) return NFEM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (weight_type == NFEM_F32)
    return forward_t<float>(L, (const float*)params, params_f32 ? params_f32 : (const float*)params, batch, x, h1, h2,
                            y, s);
  if (weight_type == NFEM_BF16) {
    if (!params_f32) return NFEM_ERR_INVALID_ARG;
    return forward_t<__nv_bfloat16>(L, (const __nv_bfloat16*)params, params_f32, batch, x, h1, h2, y, s);
  }
  return NFEM_ERR_INVALID_ARG;
}

extern "C" int nfem_mlp_backward(const int32_t* dims, int weight_type, const void* params, int64_t batch,
                                 const float* x, const float* h1, const float* h2, const float* y,
                                 const float* target, float* grads, void* workspace, size_t workspace_bytes,
                                 double* loss, void* stream) {
  MlpLayout L;
  if (!layout(dims, L) || batch < 1 || batch > INT32_MAX || !params || !x || !h1 || !h2 || !y || !target || !grads)
    return NFEM_ERR_INVALID_ARG;
  size_t need = 0;
  nfem_mlp_backward_workspace_bytes(dims, batch, &need);
  if (!workspace || workspace_bytes < need) return NFEM_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  float* work = (float*)workspace;
  if (weight_type == NFEM_F32)
    return backward_t<float>(L, (const float*)params, batch, x, h1, h2, y, target, grads, work, loss, s);
  if (weight_type == NFEM_BF16)
    return backward_t<__nv_bfloat16>(L, (const __nv_bfloat16*)params, batch, x, h1, h2, y, target, grads, work, loss, s);
  return NFEM_ERR_INVALID_ARG;
}

extern "C" int nfem_adam_step(int64_t n, float* params, const float* grads, float* m, float* v, float lr, float beta1,
                              float beta2, float eps, int step, void* params_bf16, void* stream) {
  if (n < 0 || step < 1 || (n > 0 && (!params || !grads || !m || !v))) return NFEM_ERR_INVALID_ARG;
  if (n == 0) return NFEM_OK;
  const float bc1 = 1.f - powf(beta1, float(step));
  const float bc2 = 1.f - powf(beta2, float(step));
  adam_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, params, grads, m, v, lr, beta1, beta2, eps, bc1,
                                                                  bc2, (__nv_bfloat16*)params_bf16);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_to_bf16(int64_t n, const float* x, void* out, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return NFEM_ERR_INVALID_ARG;
  if (n == 0) return NFEM_OK;
  to_bf16_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, x, (__nv_bfloat16*)out);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
