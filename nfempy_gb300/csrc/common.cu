// ABI helpers, device prefix scan, coordinate split, launch knobs.
#include <atomic>
#include <mutex>

#include "nfem_common.cuh"

namespace nfem {

static int g_num_sms = 0;

static std::atomic<int> g_knobs[NFEM_KNOB_COUNT];

int knob(int key) { return (key >= 0 && key < NFEM_KNOB_COUNT) ? g_knobs[key].load(std::memory_order_relaxed) : 0; }

int grid_for(int64_t n_items, int block, int blocks_per_sm) {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
  }
  int64_t need = ceil_div(n_items, block);
  int64_t cap = int64_t(g_num_sms) * blocks_per_sm;
  if (need < 1) need = 1;
  return int(need < cap ? need : cap);
}

// ---------------------------------------------------------------- scan
// Three passes over tiles of kScanTile counts: tile sums, a single-block scan
// of the tile sums, then per-tile scans offset by the scanned sums.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* smem, int64_t* total) {
  // warp-level inclusive scan, then scan of warp totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int64_t w = lane < nw ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) smem[lane] = w;
  }
  __syncthreads();
  int64_t warp_prefix = warp > 0 ? smem[warp - 1] : 0;
  if (total) *total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  __shared__ int64_t smem[32];
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + int64_t(k) * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  int64_t total;
  block_exclusive_scan(s, smem, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_sums_single(int64_t* __restrict__ sums, int64_t n_tiles, int64_t* __restrict__ out_total) {
  __shared__ int64_t smem[32];
  int64_t carry = 0;
  for (int64_t b = 0; b < n_tiles; b += blockDim.x) {
    int64_t i = b + threadIdx.x;
    int64_t v = i < n_tiles ? sums[i] : 0;
    int64_t total;
    int64_t ex = block_exclusive_scan(v, smem, &total);
    if (i < n_tiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void scan_tiles(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ sums,
                           int64_t* __restrict__ out) {
  __shared__ int64_t smem[32];
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  // each thread owns kScanItems consecutive items
  int32_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + int64_t(threadIdx.x) * kScanItems + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int64_t ex = block_exclusive_scan(s, smem, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + int64_t(threadIdx.x) * kScanItems + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
}

size_t scan_workspace_bytes(int64_t n) {
  int64_t tiles = ceil_div(n > 0 ? n : 1, kScanTile);
  return align256(size_t(tiles) * sizeof(int64_t)) + 256;
}

int exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes,
                       cudaStream_t stream) {
  if (n < 0 || !out) return NFEM_ERR_INVALID_ARG;
  if (ws_bytes < scan_workspace_bytes(n) || !ws) return NFEM_ERR_WORKSPACE;
  if (n == 0) {
    NFEM_TRY_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), stream));
    return NFEM_OK;
  }
  int64_t tiles = ceil_div(n, kScanTile);
  if (tiles > INT32_MAX) return NFEM_ERR_OVERFLOW;
  int64_t* sums = reinterpret_cast<int64_t*>(ws);
  scan_tile_sums<<<unsigned(tiles), kScanThreads, 0, stream>>>(in, n, sums);
  NFEM_CHECK_LAUNCH();
  scan_sums_single<<<1, 1024, 0, stream>>>(sums, tiles, out + n);
  NFEM_CHECK_LAUNCH();
  scan_tiles<<<unsigned(tiles), kScanThreads, 0, stream>>>(in, n, sums, out);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ------------------------------------------------- scan without allocation
// Scratch for nfem_exclusive_scan_noalloc: one int64 per tile of kScanTile
// counts.  A file-scope device array exists once per device that loads the
// library and stays resident until the process exits.
constexpr int64_t kNoAllocMaxTiles = 16384;
constexpr int64_t kNoAllocMaxCounts = kNoAllocMaxTiles * kScanTile;  // 67,108,864
static __device__ __align__(256) int64_t g_noalloc_scan_scratch[kNoAllocMaxTiles];

// Device address of g_noalloc_scan_scratch, looked up once per device.  In
// host code the symbol's name is only a host-side stand-in and must never be
// handed to a kernel; cudaGetSymbolAddress gives the real device address.
// The cached address is valid for the lifetime of the device's primary
// context: a cudaDeviceReset in this process destroys that context (the
// module is loaded again on next use, possibly at another address), so the
// no-allocation scan must not be called after a device reset.
constexpr int kMaxDevices = 64;
static int64_t* g_noalloc_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(int64_t** out) {
  int dev = 0;
  NFEM_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return NFEM_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_scratch_ptr[dev]) {
    int64_t* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scan_scratch);
    if (e != cudaSuccess || !ptr) return NFEM_ERR_CUDA;
    g_noalloc_scratch_ptr[dev] = ptr;
  }
  *out = g_noalloc_scratch_ptr[dev];
  return NFEM_OK;
}

// ---------------------------------------------------------------- split
// Packed fixed-point point records (format in nfem_common.cuh).  Three launches: per-block
// bounding boxes, one thread folding them into the header record (centre and
// lo_scale), then the records.  The per-block boxes are parked in the output
// buffer's point records, which the last launch overwrites.
constexpr int kSplitBlocks = 152;

__global__ void bbox_partial_kernel(const double* __restrict__ p, int64_t n, double* __restrict__ part) {
  double mn[3], mx[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    mn[k] = 1.0 / 0.0;
    mx[k] = -1.0 / 0.0;
  }
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double x = p[i * 3 + k];
      mn[k] = fmin(mn[k], x);
      mx[k] = fmax(mx[k], x);
    }
  __shared__ double sh[32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmax(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sh[warp][k] = mn[k];
      sh[warp][3 + k] = mx[k];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int k = threadIdx.x;
    double v = sh[0][k];
    for (int w = 1; w < int(blockDim.x >> 5); ++w) v = k < 3 ? fmin(v, sh[w][k]) : fmax(v, sh[w][k]);
    part[blockIdx.x * 6 + k] = v;
  }
}

// One block: fold nb partial boxes (or, when nb == 0, the points
// themselves) into the header record.  scale = 2^(e - 30) with
// |point - c| < 2^e, so the fixed-point coordinates stay below 2^30.
__global__ void split_header_kernel(const double* __restrict__ part, int nb, const double* __restrict__ p,
                                    int64_t n, float4* __restrict__ out) {
  __shared__ double sh[6][256];
  double mn[3], mx[3];
  for (int k = 0; k < 3; ++k) {
    mn[k] = 1.0 / 0.0;
    mx[k] = -1.0 / 0.0;
  }
  if (nb > 0) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
      for (int k = 0; k < 3; ++k) {
        mn[k] = fmin(mn[k], part[b * 6 + k]);
        mx[k] = fmax(mx[k], part[b * 6 + 3 + k]);
      }
  } else {
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
      for (int k = 0; k < 3; ++k) {
        mn[k] = fmin(mn[k], p[i * 3 + k]);
        mx[k] = fmax(mx[k], p[i * 3 + k]);
      }
  }
  for (int k = 0; k < 3; ++k) {
    sh[k][threadIdx.x] = mn[k];
    sh[3 + k][threadIdx.x] = mx[k];
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; ++k) {
        sh[k][threadIdx.x] = fmin(sh[k][threadIdx.x], sh[k][threadIdx.x + w]);
        sh[3 + k][threadIdx.x] = fmax(sh[3 + k][threadIdx.x], sh[3 + k][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  float c[3];
  double ext = 0.0;
  for (int k = 0; k < 3; ++k) {
    c[k] = n > 0 ? __double2float_rn(0.5 * (sh[k][0] + sh[3 + k][0])) : 0.0f;
    ext = fmax(ext, fmax(fabs(sh[k][0] - double(c[k])), fabs(sh[3 + k][0] - double(c[k]))));
  }
  int e = 0;
  frexp(ext, &e);  // ext < 2^e
  e = max(e, -96);
  out[0] = make_float4(float(ldexp(1.0, e - 30)), c[0], c[1], c[2]);
}

__global__ void split_points_kernel(const double* __restrict__ p, int64_t n, float4* __restrict__ out) {
  const float4 hd = out[0];
  const double inv = 1.0 / double(hd.x);
  const double c[3] = {double(hd.y), double(hd.z), double(hd.w)};
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    int q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double t = rint((p[i * 3 + k] - c[k]) * inv);
      q[k] = int(fmax(-1073741823.0, fmin(1073741823.0, t)));  // |q| < 2^30
    }
    out[1 + i] = make_float4(__int_as_float(q[0]), __int_as_float(q[1]), __int_as_float(q[2]), 0.0f);
  }
}

// ---------------------------------------------------------------- copies
// Copy through the SMs (16-byte vectors, grid-stride).  Between device memory
// and pinned host memory this runs over the chip-to-chip link with every SM
// issuing loads and stores, rather than through one copy engine.
__global__ void copy16_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, int64_t n16) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n16; i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}

__global__ void copy1_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}

}  // namespace nfem

using namespace nfem;

// Device-side address of p: device memory as is, pinned host memory through
// its mapping; anything else (pageable host memory) is refused.
static int device_address(const void* p, const void** out) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return NFEM_ERR_INVALID_ARG;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    *out = p;
    return NFEM_OK;
  }
  if (at.type == cudaMemoryTypeHost && at.devicePointer) {
    *out = at.devicePointer;
    return NFEM_OK;
  }
  return NFEM_ERR_INVALID_ARG;
}

extern "C" int nfem_copy_bytes(const void* src_, void* dst_, size_t bytes, void* stream_) {
  if (bytes == 0) return NFEM_OK;
  if (!src_ || !dst_) return NFEM_ERR_INVALID_ARG;
  const void* src = nullptr;
  const void* dstc = nullptr;
  if (device_address(src_, &src) != NFEM_OK || device_address(dst_, &dstc) != NFEM_OK) return NFEM_ERR_INVALID_ARG;
  void* dst = const_cast<void*>(dstc);
  cudaStream_t stream = (cudaStream_t)stream_;
  const uintptr_t a = reinterpret_cast<uintptr_t>(src), b = reinterpret_cast<uintptr_t>(dst);
  if (((a | b) & 15) == 0) {
    const int64_t n16 = int64_t(bytes / 16);
    if (n16 > 0)
      copy16_kernel<<<grid_for(n16, 256, 4), 256, 0, stream>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst),
                                                              n16);
    const int64_t tail = int64_t(bytes - size_t(n16) * 16);
    if (tail > 0)
      copy1_kernel<<<1, 32, 0, stream>>>(static_cast<const uint8_t*>(src) + n16 * 16,
                                         static_cast<uint8_t*>(dst) + n16 * 16, tail);
  } else {
    copy1_kernel<<<grid_for(int64_t(bytes), 256, 4), 256, 0, stream>>>(static_cast<const uint8_t*>(src),
                                                                      static_cast<uint8_t*>(dst), int64_t(bytes));
  }
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_abi_version(void) { return 1; }

extern "C" int nfem_knob_set(int key, int value) {
  switch (key) {
    case NFEM_KNOB_DARCY_ROWS_BLOCKS_PER_SM:
      if (value < 0 || value > 32) return NFEM_ERR_INVALID_ARG;
      break;
    case NFEM_KNOB_DARCY_CELLS_BLOCK:
      if (value != 0 && value != 128 && value != 256 && value != 512) return NFEM_ERR_INVALID_ARG;
      break;
    case NFEM_KNOB_ELAS_WARPS:
      if (value != 0 && value != 2 && value != 4 && value != 8) return NFEM_ERR_INVALID_ARG;
      break;
    case NFEM_KNOB_ELAS_ROWS:
      if (value < 0 || value > 3) return NFEM_ERR_INVALID_ARG;
      break;
    case NFEM_KNOB_COARSE_TC:
      if (value < 0 || value > 2) return NFEM_ERR_INVALID_ARG;
      break;
    case NFEM_KNOB_DARCY_F64_RECORDS:
      if (value < 0 || value > 1) return NFEM_ERR_INVALID_ARG;
      break;
    default:
      return NFEM_ERR_INVALID_ARG;
  }
  g_knobs[key].store(value, std::memory_order_relaxed);
  return NFEM_OK;
}

extern "C" int nfem_knob_get(int key, int* value) {
  if (!value || key < 0 || key >= NFEM_KNOB_COUNT) return NFEM_ERR_INVALID_ARG;
  *value = g_knobs[key].load(std::memory_order_relaxed);
  return NFEM_OK;
}

extern "C" const char* nfem_status_string(int s) {
  switch (s) {
    case NFEM_OK: return "ok";
    case NFEM_ERR_INVALID_ARG: return "invalid argument";
    case NFEM_ERR_CUDA: return "CUDA runtime error";
    case NFEM_ERR_WORKSPACE: return "workspace too small";
    case NFEM_ERR_OVERFLOW: return "size does not fit the index type";
    case NFEM_ERR_CAPACITY: return "per-row buffer or hash table full";
    case NFEM_ERR_PATTERN: return "assembled row disagrees with the CSR pattern";
    case NFEM_ERR_UNSUPPORTED: return "unsupported configuration";
    case NFEM_ERR_NOT_CONVERGED: return "Krylov iteration cap reached";
    case NFEM_ERR_BREAKDOWN: return "Krylov breakdown";
    case NFEM_ERR_NONFINITE: return "non-finite value";
    case NFEM_ERR_DEGENERATE: return "degenerate cell (|det J| == 0)";
    case NFEM_ERR_DOMAIN: return "coefficient outside its domain (kappa <= 0 or mu <= 0)";
    case NFEM_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    default: return "unknown status";
  }
}

extern "C" int nfem_scan_workspace_bytes(int64_t n, size_t* bytes) {
  if (!bytes || n < 0) return NFEM_ERR_INVALID_ARG;
  *bytes = scan_workspace_bytes(n);
  return NFEM_OK;
}

extern "C" int nfem_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, void* ws,
                                   size_t ws_bytes, void* stream) {
  if (n > 0 && !counts) return NFEM_ERR_INVALID_ARG;
  return exclusive_scan_i32(counts, n, offsets, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int nfem_points_split(const double* points, int64_t n_points, float* out, void* stream_) {
  if (n_points < 0 || !out || (n_points > 0 && !points)) return NFEM_ERR_INVALID_ARG;
  if (n_points > INT32_MAX) return NFEM_ERR_OVERFLOW;
  if (reinterpret_cast<uintptr_t>(out) & 15) return NFEM_ERR_INVALID_ARG;
  cudaStream_t stream = (cudaStream_t)stream_;
  float4* rec = reinterpret_cast<float4*>(out);
  // partial boxes (6 doubles per block) live in records 1.. until the last launch
  const int nb = int(n_points / 3 < kSplitBlocks ? n_points / 3 : kSplitBlocks);
  double* part = reinterpret_cast<double*>(rec + 1);
  if (nb > 0) bbox_partial_kernel<<<nb, 256, 0, stream>>>(points, n_points, part);
  split_header_kernel<<<1, 256, 0, stream>>>(part, nb, points, n_points, rec);
  if (n_points > 0) split_points_kernel<<<grid_for(n_points, 256), 256, 0, stream>>>(points, n_points, rec);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ---------------------------------------------------------------- fixed64
// Exact 64-bit fixed-point records for the FP64 assembly of tetrahedra:
// x = q * 2^-shift with shift = 1084 - (biased exponent of max |x|), so
// |q| < 2^62 and no centring: q holds every bit of x at or above 2^-shift
// (all of them for |x| >= 2^-10 max |x|, otherwise x is rounded to within
// 2^-62 max |x|), and an edge q1 - q0 is an exact integer difference.
__global__ void absmax_bits_kernel(const double* __restrict__ p, int64_t n3, unsigned long long* __restrict__ out) {
  unsigned long long m = 0ull;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n3; i += int64_t(gridDim.x) * blockDim.x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(p[i])) & 0x7FFFFFFFFFFFFFFFull;
    m = b > m ? b : m;  // ordered like |x| for non-negative finite values
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// header record: shift from the maximum parked in rec[1] by absmax_bits_kernel
__global__ void fixed64_header_kernel(int64_t* __restrict__ rec) {
  const unsigned long long amax = static_cast<unsigned long long>(rec[1]);
  const int e = int((amax >> 52) & 0x7ff);
  rec[0] = amax == 0ull ? 0 : 1084 - e;
  rec[1] = rec[2] = rec[3] = 0;
}

__global__ void fixed64_points_kernel(const double* __restrict__ p, int64_t n, int64_t* __restrict__ rec) {
  const int shift = int(rec[0]);
  for (int64_t v = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; v < n; v += int64_t(gridDim.x) * blockDim.x) {
    longlong2* out = reinterpret_cast<longlong2*>(rec + 4 * (v + 1));
    out[0] = make_longlong2(__double2ll_rn(scalbn(p[3 * v], shift)), __double2ll_rn(scalbn(p[3 * v + 1], shift)));
    out[1] = make_longlong2(__double2ll_rn(scalbn(p[3 * v + 2], shift)), 0);
  }
}

extern "C" int nfem_points_fixed64(const double* points, int64_t n_points, int64_t* records, void* stream_) {
  if (n_points < 0 || !records || (n_points > 0 && !points)) return NFEM_ERR_INVALID_ARG;
  if (n_points > INT32_MAX) return NFEM_ERR_OVERFLOW;
  if (reinterpret_cast<uintptr_t>(records) & 15) return NFEM_ERR_INVALID_ARG;
  cudaStream_t stream = (cudaStream_t)stream_;
  NFEM_TRY_CUDA(cudaMemsetAsync(records, 0, 4 * sizeof(int64_t), stream));
  if (n_points > 0)
    absmax_bits_kernel<<<grid_for(3 * n_points, 256), 256, 0, stream>>>(
        points, 3 * n_points, reinterpret_cast<unsigned long long*>(records + 1));
  fixed64_header_kernel<<<1, 1, 0, stream>>>(records);
  if (n_points > 0) fixed64_points_kernel<<<grid_for(n_points, 256), 256, 0, stream>>>(points, n_points, records);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_exclusive_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, void* stream) {
  if (n < 0 || !offsets || (n > 0 && !counts)) return NFEM_ERR_INVALID_ARG;
  if (n > kNoAllocMaxCounts) return NFEM_ERR_CAPACITY;
  int64_t* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    NFEM_TRY_CUDA(cudaMemsetAsync(offsets, 0, sizeof(int64_t), st));
    return NFEM_OK;
  }
  // The same three passes as nfem_exclusive_scan.  Every tile sum the later
  // passes read is written by the first pass of the same call, so whatever a
  // previous call left in the scratch needs no clearing.
  const int64_t tiles = ceil_div(n, kScanTile);
  scan_tile_sums<<<unsigned(tiles), kScanThreads, 0, st>>>(counts, n, scratch);
  NFEM_CHECK_LAUNCH();
  scan_sums_single<<<1, 1024, 0, st>>>(scratch, tiles, offsets + n);
  NFEM_CHECK_LAUNCH();
  scan_tiles<<<unsigned(tiles), kScanThreads, 0, st>>>(counts, n, scratch, offsets);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
