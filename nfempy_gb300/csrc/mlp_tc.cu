// K6b: inference of the learned preconditioner's network on the 5th-generation
// tensor cores (tcgen05 + TMEM), one fused kernel for the three layers.
//
// No reference counterpart: nfempy has no learned component.  Network and
// parameter layout as in mlp.cu: y = W3 relu(W2 relu(W1 x + b1) + b2) + b3,
// weights [out, in] row-major in one flat vector [W1 | b1 | W2 | b2 | W3 | b3],
// BF16 weights (the inference copy), FP32 biases.  This kernel covers the
// shape the preconditioner uses: in <= 16 features, two hidden layers of
// width 256, one output.
//
// Per tile of 128 rows (faces):
//   1. the tile's inputs, rounded to BF16 and padded to K = 16, are stored
//      into the A1 operand in shared memory;
//   2. layer 1 on the tensor cores: one tcgen05.mma (kind::f16, BF16 x BF16
//      -> FP32, M = 128, N = 256, K = 16) from A1 and the resident padded W1
//      into TMEM columns 0..255, committed to an mbarrier;
//   3. epilogue 1: each warp reads its 32 TMEM lanes (rows) and 128 columns
//      with tcgen05.ld, adds b1, applies the ReLU and stores BF16 into the
//      A2 operand;
//   4. layer 2: 16 tcgen05.mma (K = 16 each) from A2 and the resident W2
//      into TMEM columns 256..511, committed to the mbarrier;
//   5. epilogue 2: tcgen05.ld, + b2, ReLU, the dot with W3; the two column
//      halves of a row meet in shared memory and the row's output is
//      written once.
// The grid is persistent (one CTA per SM, W1 and W2 loaded once per CTA).
//
// Shared-memory operands use the canonical no-swizzle K-major layout of the
// UMMA descriptors: 8-row x 16-byte core matrices, the 16-byte K chunks of
// a row group adjacent (leading byte offset 128 B), row groups (K / 8) * 128
// bytes apart (stride byte offset), so element (row, k) of a K-wide BF16
// operand lives at (row % 8) * 16 + (row / 8) * (K / 8) * 128 + (k % 8) * 2
// + (k / 8) * 128.
#include <cuda_bf16.h>

#include "nfem_common.cuh"
#include "tc_common.cuh"

namespace nfem {
namespace {

constexpr int kTM = 128;        // rows per tile (MMA M)
constexpr int kH = 256;         // hidden width (MMA N, and the K extent of layer 2)
constexpr int kInMax = 16;      // input features (layer 1 K, zero-padded)
constexpr int kThreads = 256;
constexpr uint32_t kTmemCols = 512;  // layer 1 in columns 0..255, layer 2 in 256..511
constexpr uint32_t kRowGroupBytes = (kH / 8) * 128;       // 4096: row-group stride of A2 and W2
constexpr uint32_t kRowGroupBytes1 = (kInMax / 8) * 128;  // 256: row-group stride of A1 and W1

constexpr size_t kOffA = 0;                                  // A2 [128 x 256] BF16
constexpr size_t kOffB = kOffA + size_t(kTM) * kH * 2;       // W2 [256 x 256] BF16, 65536
constexpr size_t kOffA1 = kOffB + size_t(kH) * kH * 2;       // A1 [128 x 16] BF16, 196608
constexpr size_t kOffW1 = kOffA1 + size_t(kTM) * kInMax * 2;  // W1 [256 x 16] BF16, 200704
constexpr size_t kOffB1 = kOffW1 + size_t(kH) * kInMax * 2;   // 208896
constexpr size_t kOffB2 = kOffB1 + kH * 4;
constexpr size_t kOffW3 = kOffB2 + kH * 4;
constexpr size_t kOffPart = kOffW3 + kH * 4;
constexpr size_t kOffBar = kOffPart + kTM * 4;
constexpr size_t kOffSlot = kOffBar + 8;
constexpr size_t kOffFlag = kOffSlot + 4;
constexpr size_t kSmemBytes = kOffFlag + 4 + 1024;  // + alignment slack

// Instruction descriptor: BF16 x BF16 -> FP32, M 128, N 256, both K-major.
constexpr uint32_t kIdesc = tc::idesc(tc::kTypeBF16, 128, 256);

__device__ __forceinline__ uint32_t operand_offset(int row, int k) {
  return uint32_t((row & 7) * 16 + (row >> 3) * kRowGroupBytes + (k & 7) * 2 + (k >> 3) * 128);
}
__device__ __forceinline__ uint32_t operand1_offset(int row, int k) {
  return uint32_t((row & 7) * 16 + (row >> 3) * kRowGroupBytes1 + (k & 7) * 2 + (k >> 3) * 128);
}

// Thread 0 issues nothing else while it waits: a bounded poll of the
// mbarrier phase, NFEM_ERR_TIMEOUT and the flag when it runs out.
__device__ __forceinline__ void wait_commit(uint32_t bar, uint32_t parity, int32_t* status, volatile int32_t* flag) {
  if (!tc::wait_commit(bar, parity, status)) *flag = 1;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(kThreads, 1)
    mlp_infer_tc_kernel(int64_t n_rows, int n_in, const __nv_bfloat16* __restrict__ W1,
                        const float* __restrict__ b1, const __nv_bfloat16* __restrict__ W2,
                        const float* __restrict__ b2, const __nv_bfloat16* __restrict__ W3,
                        const float* __restrict__ b3p, const float* __restrict__ x, float* __restrict__ y,
                        int32_t* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem + kOffA;
  uint8_t* sB = smem + kOffB;
  uint8_t* sA1 = smem + kOffA1;
  uint8_t* sW1 = smem + kOffW1;
  float* sb1 = reinterpret_cast<float*>(smem + kOffB1);
  float* sb2 = reinterpret_cast<float*>(smem + kOffB2);
  float* sw3 = reinterpret_cast<float*>(smem + kOffW3);
  float* spart = reinterpret_cast<float*>(smem + kOffPart);
  uint64_t* sbar = reinterpret_cast<uint64_t*>(smem + kOffBar);
  uint32_t* sslot = reinterpret_cast<uint32_t*>(smem + kOffSlot);
  volatile int32_t* sflag = reinterpret_cast<volatile int32_t*>(smem + kOffFlag);
  const int t = threadIdx.x, warp = t >> 5;

  // resident operands: W2 and the zero-padded W1 in the canonical layout,
  // biases and W3 in FP32.  W2 staging: lane l of warp-step w takes row
  // 8 (w % 32) + l % 8 and K chunk 4 (w / 32) + l / 8, so each group of
  // eight lanes stores one whole 128-byte core matrix line (no bank
  // conflict beyond the four wavefronts of 512 bytes) and reads 64
  // contiguous bytes of a row
  const bool w2_aligned = (reinterpret_cast<uintptr_t>(W2) & 15) == 0;
  for (int idx = t; idx < kH * (kH / 8); idx += kThreads) {
    const int l = idx & 31, w = idx >> 5;
    const int n = (w & 31) * 8 + (l & 7), kc = (w >> 5) * 4 + (l >> 3);
    uint4 v;
    if (w2_aligned) {
      v = __ldg(reinterpret_cast<const uint4*>(W2 + size_t(n) * kH + kc * 8));
    } else {
      const uint16_t* src = reinterpret_cast<const uint16_t*>(W2) + size_t(n) * kH + kc * 8;
      v.x = src[0] | (uint32_t(src[1]) << 16);
      v.y = src[2] | (uint32_t(src[3]) << 16);
      v.z = src[4] | (uint32_t(src[5]) << 16);
      v.w = src[6] | (uint32_t(src[7]) << 16);
    }
    *reinterpret_cast<uint4*>(sB + operand_offset(n, kc * 8)) = v;
  }
  for (int idx = t; idx < kH * 2; idx += kThreads) {
    const int n = idx & (kH - 1), kc = idx >> 8;
    uint16_t e[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = kc * 8 + q;
      e[q] = k < n_in ? reinterpret_cast<const uint16_t*>(W1)[size_t(n) * n_in + k] : uint16_t(0);
    }
    *reinterpret_cast<uint4*>(sW1 + operand1_offset(n, kc * 8)) =
        make_uint4(e[0] | (uint32_t(e[1]) << 16), e[2] | (uint32_t(e[3]) << 16), e[4] | (uint32_t(e[5]) << 16),
                   e[6] | (uint32_t(e[7]) << 16));
  }
  for (int j = t; j < kH; j += kThreads) {
    sb1[j] = b1[j];
    sb2[j] = b2[j];
    sw3[j] = __bfloat162float(W3[j]);
  }
  const float b3 = *b3p;
  if (t == 0) {
    tc::bar_init(tc::smem_u32(sbar));
    *sflag = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_u32(sslot), kTmemCols);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *sslot;
  const uint32_t bar = tc::smem_u32(sbar);
  const uint32_t a_base = tc::smem_u32(sA), b_base = tc::smem_u32(sB);
  const uint32_t a1_base = tc::smem_u32(sA1), w1_base = tc::smem_u32(sW1);

  const int r = t & (kTM - 1), half = t >> 7;
  const int quarter = warp & 3, chalf = warp >> 2;  // TMEM lanes 32 quarter.., columns 128 chalf..
  const uint32_t lane_base = uint32_t(quarter * 32) << 16;
  const int64_t n_tiles = (n_rows + kTM - 1) / kTM;
  uint32_t parity = 0;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t row = tile * kTM + r;
    // ---- inputs -> A1: thread half h stores K chunk h of its row
    {
      float xv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = half * 8 + q;
        xv[q] = (row < n_rows && k < n_in) ? __ldg(x + row * n_in + k) : 0.f;
      }
      *reinterpret_cast<uint4*>(sA1 + operand1_offset(r, half * 8)) =
          make_uint4(pack_bf16x2(xv[0], xv[1]), pack_bf16x2(xv[2], xv[3]), pack_bf16x2(xv[4], xv[5]),
                     pack_bf16x2(xv[6], xv[7]));
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- layer 1 (tensor cores): one MMA, K = 16
    if (t == 0) {
      tc::mma_f16(tmem, tc::smem_desc(a1_base, 128, kRowGroupBytes1), tc::smem_desc(w1_base, 128, kRowGroupBytes1), kIdesc,
                  0u);
      tc::commit(bar);
      wait_commit(bar, parity, status, sflag);
    }
    parity ^= 1u;
    __syncthreads();
    if (*sflag) break;
    tc::fence_after_sync();
    // ---- epilogue 1: + b1, ReLU, BF16 -> A2
#pragma unroll 1
    for (int c0 = 0; c0 < kH / 2; c0 += 32) {
      uint32_t v[32];
      const int cb = chalf * (kH / 2) + c0;
      tc::tmem_ld32(tmem + lane_base + uint32_t(cb), v);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t pk[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = q * 8 + 2 * e;
          pk[e] = pack_bf16x2(fmaxf(__uint_as_float(v[i]) + sb1[cb + i], 0.f),
                              fmaxf(__uint_as_float(v[i + 1]) + sb1[cb + i + 1], 0.f));
        }
        *reinterpret_cast<uint4*>(sA + operand_offset(r, cb + q * 8)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- layer 2 (tensor cores): 16 MMAs of K = 16 (two 16-byte K chunks each)
    if (t == 0) {
#pragma unroll 1
      for (int ks = 0; ks < kH / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(a_base + ks * 256, 128, kRowGroupBytes);
        const uint64_t bd = tc::smem_desc(b_base + ks * 256, 128, kRowGroupBytes);
        tc::mma_f16(tmem + uint32_t(kH), ad, bd, kIdesc, ks > 0 ? 1u : 0u);
      }
      tc::commit(bar);
      wait_commit(bar, parity, status, sflag);
    }
    parity ^= 1u;
    __syncthreads();
    if (*sflag) break;
    tc::fence_after_sync();
    // ---- epilogue 2: + b2, ReLU, . W3
    float acc = 0.f;
#pragma unroll 1
    for (int c0 = 0; c0 < kH / 2; c0 += 32) {
      uint32_t v[32];
      const int cb = chalf * (kH / 2) + c0;
      tc::tmem_ld32(tmem + lane_base + uint32_t(kH + cb), v);
#pragma unroll
      for (int i = 0; i < 32; ++i) acc = fmaf(fmaxf(__uint_as_float(v[i]) + sb2[cb + i], 0.f), sw3[cb + i], acc);
    }
    if (chalf == 1) spart[r] = acc;
    tc::fence_before_sync();
    __syncthreads();
    if (chalf == 0 && row < n_rows) y[row] = acc + spart[r] + b3;
  }
  // free the tensor memory (every MMA has completed: its commit was waited for)
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

}  // namespace
}  // namespace nfem

using namespace nfem;

extern "C" int nfem_mlp_infer_tc(const int32_t* dims, const void* params, const float* params_f32, int64_t batch,
                                 const float* x, float* y, int32_t* dev_status, void* stream) {
  if (!dims || !params || !params_f32 || batch < 0 || (batch > 0 && (!x || !y))) return NFEM_ERR_INVALID_ARG;
  const int n_in = dims[0], h1 = dims[1], h2 = dims[2], n_out = dims[3];
  if (n_in < 1 || h1 < 1 || h2 < 1 || n_out < 1) return NFEM_ERR_INVALID_ARG;
  if (n_in > kInMax || h1 != kH || h2 != kH || n_out != 1) return NFEM_ERR_UNSUPPORTED;
  if (batch == 0) return NFEM_OK;
  const int64_t oW1 = 0, ob1 = oW1 + int64_t(h1) * n_in, oW2 = ob1 + h1, ob2 = oW2 + int64_t(h2) * h1;
  const int64_t oW3 = ob2 + h2, ob3 = oW3 + h2;
  cudaStream_t s = (cudaStream_t)stream;
  auto kern = mlp_infer_tc_kernel;
  NFEM_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes)));
  int dev = 0, n_sm = 0;
  NFEM_TRY_CUDA(cudaGetDevice(&dev));
  NFEM_TRY_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t n_tiles = (batch + kTM - 1) / kTM;
  const int grid = int(n_tiles < n_sm ? n_tiles : n_sm);
  const __nv_bfloat16* P = reinterpret_cast<const __nv_bfloat16*>(params);
  kern<<<grid, kThreads, kSmemBytes, s>>>(batch, n_in, P + oW1, params_f32 + ob1, P + oW2, params_f32 + ob2,
                                          P + oW3, params_f32 + ob3, x, y, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
