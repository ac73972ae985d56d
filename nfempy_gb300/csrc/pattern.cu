// K0: CSR sparsity pattern of the element cliques ("pattern A") and row
// incidence lists.
//
// Reference behaviour: every entry of every element matrix is added to a
// PETSc AIJ matrix with setValue(addv=True) (src/assembly/ScatterFormData.py:5-11),
// so the pattern is the union of the cliques cell_dofs x cell_dofs with
// columns sorted per row, explicit zeros kept.
//
// GPU design: a counting sort builds, per row, the list of (cell, local)
// occurrences of that DoF (sorted per row for determinism).  One warp per
// row then gathers the DoFs of every incident cell into shared memory,
// bitonic-sorts them and counts / writes the distinct ones.  Row lengths go
// through an exclusive scan to give row_ptr.
#include "nfem_common.cuh"

namespace nfem {

constexpr int kRowCap = 2048;        // candidates per row (warp shared buffer)
constexpr int kWarpsPerBlock = 4;

__global__ void count_rows(const int32_t* __restrict__ cd, int64_t n_cells, int n_loc, int ld, int64_t n_rows,
                           int32_t* __restrict__ counts, int32_t* status) {
  const int64_t n = n_cells * n_loc;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / n_loc;
    const int a = int(o - c * n_loc);
    int32_t r = cd[c * ld + a];
    if (r < 0 || r >= n_rows) { set_status(status, NFEM_ERR_INVALID_ARG); continue; }
    atomicAdd(counts + r, 1);
  }
}

__global__ void to_i32(const int64_t* __restrict__ in, int64_t n, int32_t* __restrict__ out,
                       int32_t* __restrict__ out2, int32_t* status) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    int64_t v = in[i];
    if (v > INT32_MAX) set_status(status, NFEM_ERR_OVERFLOW);
    out[i] = int32_t(v);
    if (out2) out2[i] = int32_t(v);
  }
}

__global__ void fill_incidence(const int32_t* __restrict__ cd, int64_t n_cells, int n_loc, int ld, int64_t n_rows,
                               int32_t* __restrict__ cursor, int32_t* __restrict__ inc) {
  const int64_t n = n_cells * n_loc;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / n_loc;
    const int a = int(o - c * n_loc);
    int32_t r = cd[c * ld + a];
    if (r < 0 || r >= n_rows) continue;
    int32_t pos = atomicAdd(cursor + r, 1);
    inc[pos] = int32_t(c * n_loc + a);
  }
}

__global__ void sort_incidence(const int32_t* __restrict__ inc_ptr, int64_t n_rows, int32_t* __restrict__ inc) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t b = inc_ptr[r], e = inc_ptr[r + 1];
    for (int32_t i = b + 1; i < e; ++i) {
      int32_t x = inc[i];
      int32_t j = i - 1;
      while (j >= b && inc[j] > x) {
        inc[j + 1] = inc[j];
        --j;
      }
      inc[j + 1] = x;
    }
  }
}

// Gathers and sorts the candidate columns of row r into buf; returns the count
// (or -1 when over capacity).  Called by a full warp.
__device__ int warp_row_candidates(const int32_t* __restrict__ cd, int n_loc, int ld,
                                   const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc, int64_t r,
                                   int32_t* buf) {
  const int lane = threadIdx.x & 31;
  const int32_t b = inc_ptr[r], e = inc_ptr[r + 1];
  const int m = (e - b) * n_loc;
  if (m > kRowCap) return -1;
  for (int i = lane; i < m; i += 32) {
    const int k = i / n_loc;
    const int j = i - k * n_loc;
    const int32_t occ = inc[b + k];
    const int32_t c = occ / n_loc;
    buf[i] = cd[int64_t(c) * ld + j];
  }
  int P = 1;
  while (P < m) P <<= 1;
  for (int i = m + lane; i < P; i += 32) buf[i] = INT32_MAX;
  __syncwarp();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          int32_t x = buf[i], y = buf[ixj];
          bool up = (i & k) == 0;
          if ((x > y) == up) {
            buf[i] = y;
            buf[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
  }
  return m;
}

__global__ void row_lengths(const int32_t* __restrict__ cd, int n_loc, int ld, int64_t n_rows,
                            const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                            int32_t* __restrict__ row_len, int32_t* status) {
  __shared__ int32_t sbuf[kWarpsPerBlock][kRowCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* buf = sbuf[warp];
  for (int64_t r = int64_t(blockIdx.x) * kWarpsPerBlock + warp; r < n_rows; r += int64_t(gridDim.x) * kWarpsPerBlock) {
    int m = warp_row_candidates(cd, n_loc, ld, inc_ptr, inc, r, buf);
    if (m < 0) {
      if (lane == 0) { set_status(status, NFEM_ERR_CAPACITY); row_len[r] = 0; }
      __syncwarp();
      continue;
    }
    int cnt = 0;
    for (int i0 = 0; i0 < m; i0 += 32) {
      int i = i0 + lane;
      bool is_new = i < m && (i == 0 || buf[i] != buf[i - 1]);
      cnt += __popc(__ballot_sync(0xffffffffu, is_new));
    }
    if (lane == 0) row_len[r] = cnt;
    __syncwarp();
  }
}

__global__ void row_cols(const int32_t* __restrict__ cd, int n_loc, int ld, int64_t n_rows,
                         const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                         const int32_t* __restrict__ row_ptr, int32_t* __restrict__ col_idx, int32_t* status) {
  __shared__ int32_t sbuf[kWarpsPerBlock][kRowCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* buf = sbuf[warp];
  for (int64_t r = int64_t(blockIdx.x) * kWarpsPerBlock + warp; r < n_rows; r += int64_t(gridDim.x) * kWarpsPerBlock) {
    int m = warp_row_candidates(cd, n_loc, ld, inc_ptr, inc, r, buf);
    if (m < 0) {
      if (lane == 0) set_status(status, NFEM_ERR_CAPACITY);
      __syncwarp();
      continue;
    }
    const int32_t base = row_ptr[r], len = row_ptr[r + 1] - row_ptr[r];
    int pos = 0;
    for (int i0 = 0; i0 < m; i0 += 32) {
      int i = i0 + lane;
      bool is_new = i < m && (i == 0 || buf[i] != buf[i - 1]);
      unsigned bal = __ballot_sync(0xffffffffu, is_new);
      int my = pos + __popc(bal & ((1u << lane) - 1u));
      if (is_new && my < len) col_idx[base + my] = buf[i];
      pos += __popc(bal);
    }
    if (lane == 0 && pos != len) set_status(status, NFEM_ERR_PATTERN);
    __syncwarp();
  }
}

__global__ void slot_kernel(const int32_t* __restrict__ cd, int64_t n_cells, int n_loc, int ld,
                            const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                            int32_t* __restrict__ slots, int32_t* status) {
  const int64_t n = n_cells * n_loc;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / n_loc;
    const int a = int(o - c * n_loc);
    const int32_t r = cd[c * ld + a];
    const int32_t b0 = row_ptr[r], b1 = row_ptr[r + 1];
    for (int b = 0; b < n_loc; ++b) {
      const int32_t col = cd[c * ld + b];
      int32_t lo = b0, hi = b1;
      while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (col_idx[mid] < col) lo = mid + 1; else hi = mid;
      }
      if (lo >= b1 || col_idx[lo] != col) { set_status(status, NFEM_ERR_PATTERN); lo = -1; }
      slots[o * n_loc + b] = lo;
    }
  }
}

// Per incidence entry (row r, cell c, local a): the position of each of the
// cell's columns b inside row r, relative to row_ptr[r], 4 bits per b.
__global__ void local_codes_kernel(const int32_t* __restrict__ cd, int n_loc, int ld, int64_t n_rows,
                                   const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                   const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                                   uint32_t* __restrict__ codes, int32_t* status) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t b0 = row_ptr[r], b1 = row_ptr[r + 1];
    if (b1 - b0 > 16) { set_status(status, NFEM_ERR_UNSUPPORTED); continue; }
    for (int32_t k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k) {
      const int32_t occ = inc[k];
      const int32_t c = occ / n_loc;
      uint32_t code = 0;
      for (int b = 0; b < n_loc; ++b) {
        const int32_t col = cd[int64_t(c) * ld + b];
        int32_t lo = b0, hi = b1;
        while (lo < hi) {
          int32_t mid = (lo + hi) >> 1;
          if (col_idx[mid] < col) lo = mid + 1; else hi = mid;
        }
        if (lo >= b1 || col_idx[lo] != col) set_status(status, NFEM_ERR_PATTERN);
        code |= uint32_t(lo - b0) << (4 * b);
      }
      codes[k] = code;
    }
  }
}

// Fixed-stride incidence layout for rows with at most two incidences:
// pairs[r] = (occ0, occ1) with -1 for absent, pair_codes[r] = (code0, code1).
__global__ void pairs_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                             const uint32_t* __restrict__ codes, int64_t n_rows, int2* __restrict__ pairs,
                             uint2* __restrict__ pair_codes, int32_t* status) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t b = inc_ptr[r], e = inc_ptr[r + 1];
    if (e - b > 2) set_status(status, NFEM_ERR_UNSUPPORTED);
    int2 pr = make_int2(-1, -1);
    uint2 cd = make_uint2(0u, 0u);
    if (e > b) { pr.x = inc[b]; cd.x = codes[b]; }
    if (e > b + 1) { pr.y = inc[b + 1]; cd.y = codes[b + 1]; }
    pairs[r] = pr;
    pair_codes[r] = cd;
  }
}

static size_t pattern_bytes(int64_t n_rows) {
  size_t b = 0;
  b += align256(size_t(n_rows) * 4) * 3;                 // counts, cursor, row_len
  b += align256(size_t(n_rows + 1) * 8) * 2;             // 64-bit offsets
  b += align256(scan_workspace_bytes(n_rows));
  b += align256(sizeof(int32_t)) + align256(sizeof(int64_t));
  return b + 2048;
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_pattern_workspace_bytes(int64_t n_cells, int n_loc, int64_t n_rows, size_t* bytes) {
  if (!bytes || n_cells < 0 || n_loc < 1 || n_rows < 0) return NFEM_ERR_INVALID_ARG;
  *bytes = pattern_bytes(n_rows);
  return NFEM_OK;
}

extern "C" int nfem_pattern_rows(const int32_t* cd, int64_t n_cells, int n_loc, int ld, int64_t n_rows, void* ws,
                                 size_t ws_bytes, int32_t* inc_ptr, int32_t* inc, int32_t* row_ptr,
                                 int64_t* nnz_host, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0 || n_loc < 1 || ld < n_loc || n_rows < 0 || !inc_ptr || !row_ptr || !nnz_host ||
      (n_cells > 0 && (!cd || !inc)))
    return NFEM_ERR_INVALID_ARG;
  if (n_cells * n_loc >= INT32_MAX || n_rows >= INT32_MAX) return NFEM_ERR_OVERFLOW;
  if (!ws || ws_bytes < pattern_bytes(n_rows)) return NFEM_ERR_WORKSPACE;
  Carver cw{reinterpret_cast<char*>(ws), 0, ws_bytes};
  int32_t* counts = cw.take<int32_t>(n_rows);
  int32_t* cursor = cw.take<int32_t>(n_rows);
  int32_t* row_len = cw.take<int32_t>(n_rows);
  int64_t* off = cw.take<int64_t>(n_rows + 1);
  int64_t* off2 = cw.take<int64_t>(n_rows + 1);
  size_t sws_b = scan_workspace_bytes(n_rows);
  void* sws = cw.take<char>(sws_b);
  int32_t* status = cw.take<int32_t>(1);
  if (!cw.ok()) return NFEM_ERR_WORKSPACE;
  const int B = 256;
  NFEM_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), stream));
  NFEM_TRY_CUDA(cudaMemsetAsync(counts, 0, size_t(n_rows) * 4, stream));
  if (n_cells > 0) {
    count_rows<<<grid_for(n_cells * n_loc, B), B, 0, stream>>>(cd, n_cells, n_loc, ld, n_rows, counts, status);
    NFEM_CHECK_LAUNCH();
  }
  int rc = exclusive_scan_i32(counts, n_rows, off, sws, sws_b, stream);
  if (rc) return rc;
  to_i32<<<grid_for(n_rows + 1, B), B, 0, stream>>>(off, n_rows + 1, inc_ptr, nullptr, status);
  to_i32<<<grid_for(n_rows, B), B, 0, stream>>>(off, n_rows, cursor, nullptr, status);
  NFEM_CHECK_LAUNCH();
  if (n_cells > 0) {
    fill_incidence<<<grid_for(n_cells * n_loc, B), B, 0, stream>>>(cd, n_cells, n_loc, ld, n_rows, cursor, inc);
    sort_incidence<<<grid_for(n_rows, B), B, 0, stream>>>(inc_ptr, n_rows, inc);
    NFEM_CHECK_LAUNCH();
  }
  if (n_rows > 0) {
    row_lengths<<<grid_for(ceil_div(n_rows, kWarpsPerBlock), 1, 16), 32 * kWarpsPerBlock, 0,
                  stream>>>(cd, n_loc, ld, n_rows, inc_ptr, inc, row_len, status);
    NFEM_CHECK_LAUNCH();
  }
  rc = exclusive_scan_i32(row_len, n_rows, off2, sws, sws_b, stream);
  if (rc) return rc;
  to_i32<<<grid_for(n_rows + 1, B), B, 0, stream>>>(off2, n_rows + 1, row_ptr, nullptr, status);
  NFEM_CHECK_LAUNCH();
  int64_t nnz = 0;
  int32_t h_status = 0;
  NFEM_TRY_CUDA(cudaMemcpyAsync(&nnz, off2 + n_rows, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
  NFEM_TRY_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
  NFEM_TRY_CUDA(cudaStreamSynchronize(stream));
  if (dev_status && h_status) NFEM_TRY_CUDA(cudaMemcpy(dev_status, &h_status, 4, cudaMemcpyHostToDevice));
  *nnz_host = nnz;
  return h_status;
}

extern "C" int nfem_pattern_cols(const int32_t* cd, int64_t n_cells, int n_loc, int ld, int64_t n_rows,
                                 const int32_t* inc_ptr, const int32_t* inc, const int32_t* row_ptr,
                                 int32_t* col_idx, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0 || n_loc < 1 || ld < n_loc || n_rows < 0 || !inc_ptr || !row_ptr) return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  row_cols<<<grid_for(ceil_div(n_rows, kWarpsPerBlock), 1, 16), 32 * kWarpsPerBlock, 0, stream>>>(
      cd, n_loc, ld, n_rows, inc_ptr, inc, row_ptr, col_idx, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_pattern_local_codes(const int32_t* cd, int64_t n_cells, int n_loc, int ld, int64_t n_rows,
                                       const int32_t* inc_ptr, const int32_t* inc, const int32_t* row_ptr,
                                       const int32_t* col_idx, uint32_t* codes, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_loc < 1 || n_loc > 8 || ld < n_loc || n_rows < 0 || n_cells < 0) return NFEM_ERR_INVALID_ARG;
  if (n_rows > 0 && (!cd || !inc_ptr || !inc || !row_ptr || !col_idx || !codes)) return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  local_codes_kernel<<<grid_for(n_rows, 256), 256, 0, stream>>>(cd, n_loc, ld, n_rows, inc_ptr, inc, row_ptr, col_idx,
                                                                codes, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_pattern_pairs(const int32_t* inc_ptr, const int32_t* inc, const uint32_t* codes,
                                  int64_t n_rows, int32_t* pairs, uint32_t* pair_codes, int32_t* dev_status,
                                  void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_rows < 0 || (n_rows > 0 && (!inc_ptr || !inc || !codes || !pairs || !pair_codes)))
    return NFEM_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(pairs) & 7) || (reinterpret_cast<uintptr_t>(pair_codes) & 7))
    return NFEM_ERR_INVALID_ARG;
  if (n_rows == 0) return NFEM_OK;
  pairs_kernel<<<grid_for(n_rows, 256), 256, 0, stream>>>(inc_ptr, inc, codes, n_rows, reinterpret_cast<int2*>(pairs),
                                                          reinterpret_cast<uint2*>(pair_codes), dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// Cell-chunk row table for the mixed RT1 x P0 layout.  Rows [0, p_base) are
// flux rows numbered by first appearance, so the first incidence's cell is
// non-decreasing along them; chunk_rows[k] = the first flux row whose first
// cell is >= k * chunk_cells (chunk_rows[n_chunks] = p_base).  Rows
// [p_base, p_base + n_cells) must be the pressure rows of cells 0.. in order.
// Any other layout sets NFEM_ERR_UNSUPPORTED.
__global__ void chunk_rows_kernel(const int2* __restrict__ pairs, int64_t n_rows, int n_loc, int64_t p_base,
                                  int64_t n_cells, int chunk_cells, int64_t n_chunks, int32_t* __restrict__ chunk_rows,
                                  int32_t* status) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x) {
    const int2 pr = pairs[r];
    if (r >= p_base) {
      const int64_t c = r - p_base;
      if (pr.x != int32_t(c * n_loc + n_loc - 1) || pr.y != -1) set_status(status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    if (pr.x < 0) {
      set_status(status, NFEM_ERR_UNSUPPORTED);
      continue;
    }
    const int64_t k = (pr.x / n_loc) / chunk_cells;
    int64_t kp = -1;
    if (r > 0) {
      const int2 q = pairs[r - 1];
      kp = q.x < 0 ? k : (q.x / n_loc) / chunk_cells;
      if (kp > k) set_status(status, NFEM_ERR_UNSUPPORTED);
    }
    for (int64_t j = kp + 1; j <= k && j <= n_chunks; ++j) chunk_rows[j] = int32_t(r);
    if (r == p_base - 1)
      for (int64_t j = k + 1; j <= n_chunks; ++j) chunk_rows[j] = int32_t(p_base);
  }
}

extern "C" int nfem_pattern_darcy_chunks(const int32_t* pairs, int64_t n_rows, int n_loc, int64_t p_base,
                                         int64_t n_cells, int32_t* chunk_rows, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_rows < 0 || n_loc < 2 || p_base < 0 || n_cells < 0 || !chunk_rows || (n_rows > 0 && !pairs))
    return NFEM_ERR_INVALID_ARG;
  if (reinterpret_cast<uintptr_t>(pairs) & 7) return NFEM_ERR_INVALID_ARG;
  if (p_base + n_cells != n_rows || n_rows >= INT32_MAX) return NFEM_ERR_UNSUPPORTED;
  const int64_t n_chunks = ceil_div(n_cells, NFEM_DARCY_CHUNK_CELLS);
  if (p_base == 0) {
    NFEM_TRY_CUDA(cudaMemsetAsync(chunk_rows, 0, size_t(n_chunks + 1) * sizeof(int32_t), stream));
  }
  if (n_rows == 0) return NFEM_OK;
  chunk_rows_kernel<<<grid_for(n_rows, 256), 256, 0, stream>>>(reinterpret_cast<const int2*>(pairs), n_rows, n_loc,
                                                               p_base, n_cells, NFEM_DARCY_CHUNK_CELLS, n_chunks,
                                                               chunk_rows, dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_pattern_slots(const int32_t* cd, int64_t n_cells, int n_loc, int ld, const int32_t* row_ptr,
                                  const int32_t* col_idx, int32_t* slots, int32_t* dev_status, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n_cells < 0 || n_loc < 1 || ld < n_loc || (n_cells > 0 && (!cd || !row_ptr || !col_idx || !slots)))
    return NFEM_ERR_INVALID_ARG;
  if (n_cells * n_loc * n_loc >= INT64_MAX / 4) return NFEM_ERR_OVERFLOW;
  if (n_cells == 0) return NFEM_OK;
  slot_kernel<<<grid_for(n_cells * n_loc, 256), 256, 0, stream>>>(cd, n_cells, n_loc, ld, row_ptr, col_idx, slots,
                                                                  dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ------------------------------------------------------------ generic scatter
// Element matrices and residuals evaluated elsewhere (a weak form the device
// does not implement, evaluated cell by cell on the host like the
// reference's scatter_form_data) added into the CSR pattern: one thread per
// (element, a, b) entry, the column found by binary search in the row, an
// atomic add (the order of the additions into one entry may vary).
namespace nfem {
template <typename T>
__global__ void scatter_elements_kernel(int64_t n_el, int n_loc, const int32_t* __restrict__ dofs,
                                        const T* __restrict__ jel, const T* __restrict__ rel,
                                        const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                        int64_t n_rows, T* __restrict__ values, T* __restrict__ rhs,
                                        int32_t* status) {
  const int64_t nn = int64_t(n_loc) * n_loc;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n_el * nn;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t el = e / nn;
    const int a = int((e / n_loc) % n_loc), b = int(e % n_loc);
    const int32_t row = dofs[el * n_loc + a], col = dofs[el * n_loc + b];
    if (row < 0 || col < 0 || row >= n_rows || col >= n_rows) {
      set_status(status, NFEM_ERR_INVALID_ARG);
      continue;
    }
    if (jel) {
      int32_t lo = rp[row], hi = rp[row + 1];
      const int32_t end = hi;
      while (lo < hi) {  // at most log2(row length) steps
        const int32_t mid = (lo + hi) >> 1;
        if (ci[mid] < col) lo = mid + 1; else hi = mid;
      }
      if (lo < end && ci[lo] == col)
        atomicAdd(values + lo, jel[e]);
      else
        set_status(status, NFEM_ERR_PATTERN);
    }
    if (rel && b == 0) atomicAdd(rhs + row, rel[el * n_loc + a]);
  }
}
}  // namespace nfem

extern "C" int nfem_scatter_elements(int value_type, int64_t n_el, int n_loc, const int32_t* dofs,
                                     const void* j_el, const void* r_el, const int32_t* row_ptr,
                                     const int32_t* col_idx, int64_t n_rows, void* values, void* rhs,
                                     int32_t* dev_status, void* stream) {
  using namespace nfem;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n_el < 0 || n_loc < 1 || n_rows < 0)
    return NFEM_ERR_INVALID_ARG;
  if (n_el == 0) return NFEM_OK;
  if (!dofs || (j_el && (!row_ptr || !col_idx || !values)) || (r_el && !rhs)) return NFEM_ERR_INVALID_ARG;
  const int64_t work = n_el * int64_t(n_loc) * n_loc;
  const int g = grid_for(work, 256);
  cudaStream_t s = (cudaStream_t)stream;
  if (value_type == NFEM_F64)
    scatter_elements_kernel<double><<<g, 256, 0, s>>>(n_el, n_loc, dofs, (const double*)j_el, (const double*)r_el,
                                                      row_ptr, col_idx, n_rows, (double*)values, (double*)rhs,
                                                      dev_status);
  else
    scatter_elements_kernel<float><<<g, 256, 0, s>>>(n_el, n_loc, dofs, (const float*)j_el, (const float*)r_el,
                                                     row_ptr, col_idx, n_rows, (float*)values, (float*)rhs,
                                                     dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

// ------------------------------------------------------------ single entries
// (row, col, value) triples added into the CSR pattern: the batched form of
// PETSc's Mat.setValue(row, col, value, addv=True) that the reference's
// scatter calls once per entry (src/assembly/ScatterFormData.py:5-11).
namespace nfem {
template <typename T>
__global__ void csr_add_coo_kernel(int64_t n, const int32_t* __restrict__ rows, const int32_t* __restrict__ cols,
                                   const double* __restrict__ vals, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ ci, int64_t n_rows, T* __restrict__ values,
                                   int32_t* status) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    const int32_t row = rows[e], col = cols[e];
    if (row < 0 || col < 0 || row >= n_rows || col >= n_rows) {
      set_status(status, NFEM_ERR_INVALID_ARG);
      continue;
    }
    int32_t lo = rp[row], hi = rp[row + 1];
    const int32_t end = hi;
    while (lo < hi) {
      const int32_t mid = (lo + hi) >> 1;
      if (ci[mid] < col) lo = mid + 1; else hi = mid;
    }
    if (lo < end && ci[lo] == col)
      atomicAdd(values + lo, T(vals[e]));
    else
      set_status(status, NFEM_ERR_PATTERN);
  }
}
}  // namespace nfem

extern "C" int nfem_csr_add_entries(int value_type, int64_t n, const int32_t* rows, const int32_t* cols,
                                    const double* vals, const int32_t* row_ptr, const int32_t* col_idx,
                                    int64_t n_rows, void* values, int32_t* dev_status, void* stream) {
  using namespace nfem;
  if ((value_type != NFEM_F64 && value_type != NFEM_F32) || n < 0 || n_rows < 0) return NFEM_ERR_INVALID_ARG;
  if (n == 0) return NFEM_OK;
  if (!rows || !cols || !vals || !row_ptr || !col_idx || !values) return NFEM_ERR_INVALID_ARG;
  const int g = grid_for(n, 256);
  cudaStream_t s = (cudaStream_t)stream;
  if (value_type == NFEM_F64)
    csr_add_coo_kernel<double><<<g, 256, 0, s>>>(n, rows, cols, vals, row_ptr, col_idx, n_rows, (double*)values,
                                                 dev_status);
  else
    csr_add_coo_kernel<float><<<g, 256, 0, s>>>(n, rows, cols, vals, row_ptr, col_idx, n_rows, (float*)values,
                                                dev_status);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
