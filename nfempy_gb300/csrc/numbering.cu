// K0: entity numbering in first-appearance order, orientation flags, DoF map.
//
// Reference behaviour (nfempy): Mesh.build_conformal_mesh gives each distinct
// sorted vertex tuple a global entity (src/mesh/mesh.py:239-339);
// MeshTopology lists the entities of each dimension in the order they first
// appear while walking the cells and their local sub-entities
// (src/mesh/mesh.py:639-681, src/mesh/mesh_topology.py:28-35), and DoFMap
// numbers DoFs in that order (src/spaces/dof_map.py:38-129).
//
// GPU design: one occurrence per (cell, local sub-entity).  Occurrences are
// inserted into an open-addressing hash table keyed by the packed sorted
// vertex tuple whose value is the minimum occurrence index (atomicMin), i.e.
// the first appearance.  An occurrence is "first" when it holds that minimum;
// an exclusive scan over the first-flags gives each entity its rank, and every
// occurrence reads the rank of its entity's first occurrence.  No sort.
#include "nfem_common.cuh"

namespace nfem {

__constant__ int8_t c_sub[2][4][6][3];  // [cell_dim-2][entity_dim][local][vertex]
__constant__ int8_t c_nsub[2][4];

static const int8_t h_sub[2][4][6][3] = {
    // triangle
    {{{0}, {1}, {2}},
     {{1, 2}, {0, 2}, {0, 1}},
     {{0, 1, 2}},
     {}},
    // tetrahedron
    {{{0}, {1}, {2}, {3}},
     {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}},
     {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}},
     {{0, 1, 2}}}};
static const int8_t h_nsub[2][4] = {{3, 3, 1, 0}, {4, 6, 4, 1}};

static bool g_tables_ready = false;
static int upload_tables() {
  if (g_tables_ready) return NFEM_OK;
  NFEM_TRY_CUDA(cudaMemcpyToSymbol(c_sub, h_sub, sizeof(h_sub)));
  NFEM_TRY_CUDA(cudaMemcpyToSymbol(c_nsub, h_nsub, sizeof(h_nsub)));
  g_tables_ready = true;
  return NFEM_OK;
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

__device__ __forceinline__ void sort3(int32_t& a, int32_t& b, int32_t& c) {
  int32_t t;
  if (a > b) { t = a; a = b; b = t; }
  if (b > c) { t = b; b = c; c = t; }
  if (a > b) { t = a; a = b; b = t; }
}

// key of a sorted tuple (+1 so that 0 marks an empty slot)
__device__ __forceinline__ uint64_t pack_key(const int32_t* v, int k) {
  if (k == 2) {
    int32_t a = min(v[0], v[1]), b = max(v[0], v[1]);
    return ((uint64_t(uint32_t(a)) << 32) | uint64_t(uint32_t(b))) + 1ULL;
  }
  int32_t a = v[0], b = v[1], c = v[2];
  sort3(a, b, c);
  return ((uint64_t(a) << 42) | (uint64_t(b) << 21) | uint64_t(c)) + 1ULL;
}

// Inserts key with value `val` (atomicMin).  Returns the slot or -1 if full.
__device__ __forceinline__ int64_t hash_insert_min(uint64_t* keys, int32_t* vals, uint64_t mask,
                                                   uint64_t key, int32_t val) {
  uint64_t h = mix64(key) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    unsigned long long k = keys[h];
    if (k == 0ULL) {
      unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(keys + h), 0ULL,
                                          (unsigned long long)key);
      k = prev == 0ULL ? (unsigned long long)key : prev;
    }
    if (k == key) {
      atomicMin(vals + h, val);
      return int64_t(h);
    }
    h = (h + 1) & mask;
  }
  return -1;
}

__device__ __forceinline__ int64_t hash_find(const uint64_t* keys, uint64_t mask, uint64_t key) {
  uint64_t h = mix64(key) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    uint64_t k = keys[h];
    if (k == key) return int64_t(h);
    if (k == 0ULL) return -1;
    h = (h + 1) & mask;
  }
  return -1;
}

__global__ void fill_i32(int32_t* p, int64_t n, int32_t v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

// vertices: first[v] = min occurrence
__global__ void vertex_first(const int32_t* __restrict__ cv, int64_t n_cells, int nv,
                             int64_t n_points, int32_t* __restrict__ first, int32_t* status) {
  const int64_t n = n_cells * nv;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    int32_t v = cv[o];
    if (v < 0 || v >= n_points) { set_status(status, NFEM_ERR_INVALID_ARG); continue; }
    atomicMin(first + v, int32_t(o));
  }
}

__global__ void vertex_flags(const int32_t* __restrict__ cv, int64_t n_cells, int nv, int64_t n_points,
                             const int32_t* __restrict__ first, int32_t* __restrict__ is_first,
                             int32_t* __restrict__ first_occ) {
  const int64_t n = n_cells * nv;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    int32_t v = cv[o];
    int32_t f = (v >= 0 && v < n_points) ? first[v] : int32_t(o);
    first_occ[o] = f;
    is_first[o] = (f == int32_t(o));
  }
}

__global__ void entity_insert(const int32_t* __restrict__ cv, int64_t n_cells, int nv, int cdi, int ed,
                              uint64_t* keys, int32_t* vals, uint64_t mask, int32_t* status) {
  const int ne = c_nsub[cdi][ed];
  const int k = ed + 1;
  const int64_t n = n_cells * ne;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / ne;
    const int e = int(o - c * ne);
    int32_t v[3];
    for (int j = 0; j < k; ++j) v[j] = cv[c * nv + c_sub[cdi][ed][e][j]];
    if (hash_insert_min(keys, vals, mask, pack_key(v, k), int32_t(o)) < 0) set_status(status, NFEM_ERR_CAPACITY);
  }
}

__global__ void entity_flags(const int32_t* __restrict__ cv, int64_t n_cells, int nv, int cdi, int ed,
                             const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals, uint64_t mask,
                             int32_t* __restrict__ is_first, int32_t* __restrict__ first_occ, int32_t* status) {
  const int ne = c_nsub[cdi][ed];
  const int k = ed + 1;
  const int64_t n = n_cells * ne;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / ne;
    const int e = int(o - c * ne);
    int32_t v[3];
    for (int j = 0; j < k; ++j) v[j] = cv[c * nv + c_sub[cdi][ed][e][j]];
    int64_t h = hash_find(keys, mask, pack_key(v, k));
    int32_t f = h >= 0 ? vals[h] : int32_t(o);
    if (h < 0) set_status(status, NFEM_ERR_CAPACITY);
    first_occ[o] = f;
    is_first[o] = (f == int32_t(o));
  }
}

__global__ void gather_rank(const int32_t* __restrict__ first_occ, const int64_t* __restrict__ scan, int64_t n,
                            int32_t* __restrict__ rank) {
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x)
    rank[o] = int32_t(scan[first_occ[o]]);
}

__global__ void facet_insert(const int32_t* __restrict__ facets, int64_t n_facets, int k, uint64_t* keys,
                             int32_t* vals, uint64_t mask, int32_t* status) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_facets; i += int64_t(gridDim.x) * blockDim.x) {
    int32_t v[3];
    for (int j = 0; j < k; ++j) v[j] = facets[i * k + j];
    if (hash_insert_min(keys, vals, mask, pack_key(v, k), int32_t(i)) < 0) set_status(status, NFEM_ERR_CAPACITY);
  }
}

// bit0 = reflected, bit1 = tagged (facets of the cells only)
__global__ void facet_flags(const int32_t* __restrict__ cv, int64_t n_cells, int nv, int cdi,
                            const int32_t* __restrict__ facets, int facets_first, const uint64_t* __restrict__ bkeys,
                            const int32_t* __restrict__ bvals, uint64_t bmask, int has_b,
                            uint8_t* __restrict__ flags) {
  const int ed = cdi + 1;  // cell_dim - 1
  const int ne = c_nsub[cdi][ed];
  const int k = ed + 1;
  const int64_t n = n_cells * ne;
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = o / ne;
    const int e = int(o - c * ne);
    int32_t v[3];
    for (int j = 0; j < k; ++j) v[j] = cv[c * nv + c_sub[cdi][ed][e][j]];
    int64_t h = has_b ? hash_find(bkeys, bmask, pack_key(v, k)) : -1;
    const bool tagged = h >= 0;
    bool reflected;
    if (k == 2) {
      // stored order: the boundary line's file order if that block came
      // first, otherwise sorted (src/mesh/mesh.py:137-167, :226-229)
      int32_t s0 = min(v[0], v[1]), s1 = max(v[0], v[1]);
      if (tagged && facets_first) {
        int32_t fi = bvals[h];
        s0 = facets[int64_t(fi) * 2 + 0];
        s1 = facets[int64_t(fi) * 2 + 1];
      }
      reflected = !(v[0] == s0 && v[1] == s1);
    } else {
      int inv = int(v[0] > v[1]) + int(v[0] > v[2]) + int(v[1] > v[2]);
      reflected = (inv & 1) != 0;
    }
    flags[o] = uint8_t((reflected ? 1 : 0) | (tagged ? 2 : 0));
  }
}

__global__ void rt1_mask_kernel(const uint8_t* __restrict__ flags, int64_t n_cells, int nf, int dim3,
                                uint8_t* __restrict__ mask) {
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < n_cells; c += int64_t(gridDim.x) * blockDim.x) {
    uint8_t m = 0;
    for (int i = 0; i < nf; ++i) {
      uint8_t f = flags[c * nf + i];
      bool neg = (f & 1) != 0;
      // boundary faces with local index 1 or 3 are forced to reflection
      // (src/basis/permute_and_transform.py:102-105)
      if (dim3 && (f & 2) && (i == 1 || i == 3)) neg = true;
      if (neg) m |= uint8_t(1u << i);
    }
    mask[c] = m;
  }
}

struct DofBlocks {
  nfem_dof_block b[NFEM_MAX_DOF_BLOCKS];
  int n;
};

__global__ void compose_kernel(int64_t n_cells, DofBlocks blocks, int32_t* __restrict__ out, int ld,
                               int32_t* status) {
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < n_cells; c += int64_t(gridDim.x) * blockDim.x) {
    int col = 0;
    for (int bi = 0; bi < blocks.n; ++bi) {
      const nfem_dof_block& b = blocks.b[bi];
      for (int e = 0; e < b.n_ent; ++e) {
        int64_t r = b.occ_rank ? int64_t(b.occ_rank[c * b.n_ent + e]) : c;
        int64_t first = b.base + r * b.width;
        for (int j = 0; j < b.width; ++j) {
          int64_t d = first + j;
          if (d > INT32_MAX) set_status(status, NFEM_ERR_OVERFLOW);
          out[c * ld + col++] = int32_t(d);
        }
      }
    }
  }
}

static uint64_t next_pow2(uint64_t x) {
  uint64_t p = 1024;
  while (p < x) p <<= 1;
  return p;
}

struct NumberingPlan {
  int64_t n_occ;
  uint64_t cap, bcap;
};

static NumberingPlan plan_for(int64_t n_cells, int cell_dim, int entity_dim, int64_t n_facets) {
  NumberingPlan p;
  p.n_occ = n_cells * h_nsub[cell_dim - 2][entity_dim];
  p.cap = entity_dim == 0 ? 0 : next_pow2(uint64_t(2 * p.n_occ));
  p.bcap = n_facets > 0 ? next_pow2(uint64_t(2 * n_facets)) : 0;
  return p;
}

static size_t numbering_bytes(const NumberingPlan& p, int64_t n_points) {
  size_t b = 0;
  b += align256(size_t(p.n_occ) * 4) * 2;             // is_first, first_occ
  b += align256(size_t(p.n_occ + 1) * 8);             // scan out
  b += align256(scan_workspace_bytes(p.n_occ));       // scan workspace
  b += align256(size_t(n_points) * 4);                // vertex first
  b += align256(size_t(p.cap) * 8) + align256(size_t(p.cap) * 4);
  b += align256(size_t(p.bcap) * 8) + align256(size_t(p.bcap) * 4);
  b += align256(sizeof(int32_t));                     // status
  return b + 4096;
}

}  // namespace nfem

using namespace nfem;

extern "C" int nfem_numbering_workspace_bytes(int64_t n_cells, int cell_dim, int entity_dim, int64_t n_points,
                                              int64_t n_facets, size_t* bytes) {
  if (!bytes || n_cells < 0 || cell_dim < 2 || cell_dim > 3 || entity_dim < 0 || entity_dim >= cell_dim ||
      n_points < 0 || n_facets < 0)
    return NFEM_ERR_INVALID_ARG;
  *bytes = numbering_bytes(plan_for(n_cells, cell_dim, entity_dim, n_facets), n_points);
  return NFEM_OK;
}

extern "C" int nfem_number_entities(const int32_t* cv, int64_t n_cells, int cell_dim, int entity_dim,
                                    int64_t n_points, const int32_t* facets, int64_t n_facets, int facets_first,
                                    void* ws, size_t ws_bytes, int32_t* occ_rank, uint8_t* flags,
                                    int64_t* n_entities_out, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (cell_dim < 2 || cell_dim > 3 || entity_dim < 0 || entity_dim >= cell_dim || n_cells < 0 || !occ_rank ||
      !n_entities_out || (n_cells > 0 && !cv) || (n_facets > 0 && !facets))
    return NFEM_ERR_INVALID_ARG;
  if (entity_dim == 2 && n_points >= (int64_t(1) << 21)) return NFEM_ERR_UNSUPPORTED;
  if (n_points >= INT32_MAX) return NFEM_ERR_OVERFLOW;
  NumberingPlan p = plan_for(n_cells, cell_dim, entity_dim, n_facets);
  if (p.n_occ >= INT32_MAX) return NFEM_ERR_OVERFLOW;
  if (!ws || ws_bytes < numbering_bytes(p, n_points)) return NFEM_ERR_WORKSPACE;
  int rc = upload_tables();
  if (rc) return rc;
  const int nv = cell_dim + 1, cdi = cell_dim - 2;
  Carver cv_ws{reinterpret_cast<char*>(ws), 0, ws_bytes};
  int32_t* is_first = cv_ws.take<int32_t>(p.n_occ);
  int32_t* first_occ = cv_ws.take<int32_t>(p.n_occ);
  int64_t* scan = cv_ws.take<int64_t>(p.n_occ + 1);
  size_t scan_ws_bytes = scan_workspace_bytes(p.n_occ);
  void* scan_ws = cv_ws.take<char>(scan_ws_bytes);
  int32_t* vfirst = cv_ws.take<int32_t>(n_points);
  uint64_t* keys = cv_ws.take<uint64_t>(p.cap);
  int32_t* vals = cv_ws.take<int32_t>(p.cap);
  uint64_t* bkeys = cv_ws.take<uint64_t>(p.bcap);
  int32_t* bvals = cv_ws.take<int32_t>(p.bcap);
  int32_t* status = cv_ws.take<int32_t>(1);
  if (!cv_ws.ok()) return NFEM_ERR_WORKSPACE;
  NFEM_TRY_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), stream));
  const int B = 256;
  if (p.n_occ == 0) {
    NFEM_TRY_CUDA(cudaMemsetAsync(n_entities_out, 0, sizeof(int64_t), stream));
    return NFEM_OK;
  }
  if (entity_dim == 0) {
    fill_i32<<<grid_for(n_points, B), B, 0, stream>>>(vfirst, n_points, INT32_MAX);
    vertex_first<<<grid_for(p.n_occ, B), B, 0, stream>>>(cv, n_cells, nv, n_points, vfirst, status);
    vertex_flags<<<grid_for(p.n_occ, B), B, 0, stream>>>(cv, n_cells, nv, n_points, vfirst, is_first, first_occ);
  } else {
    NFEM_TRY_CUDA(cudaMemsetAsync(keys, 0, p.cap * sizeof(uint64_t), stream));
    fill_i32<<<grid_for(int64_t(p.cap), B), B, 0, stream>>>(vals, int64_t(p.cap), INT32_MAX);
    entity_insert<<<grid_for(p.n_occ, B), B, 0, stream>>>(cv, n_cells, nv, cdi, entity_dim, keys, vals, p.cap - 1,
                                                          status);
    entity_flags<<<grid_for(p.n_occ, B), B, 0, stream>>>(cv, n_cells, nv, cdi, entity_dim, keys, vals, p.cap - 1,
                                                         is_first, first_occ, status);
  }
  NFEM_CHECK_LAUNCH();
  rc = exclusive_scan_i32(is_first, p.n_occ, scan, scan_ws, scan_ws_bytes, stream);
  if (rc) return rc;
  gather_rank<<<grid_for(p.n_occ, B), B, 0, stream>>>(first_occ, scan, p.n_occ, occ_rank);
  NFEM_CHECK_LAUNCH();
  NFEM_TRY_CUDA(cudaMemcpyAsync(n_entities_out, scan + p.n_occ, sizeof(int64_t), cudaMemcpyDeviceToDevice, stream));
  if (flags && entity_dim == cell_dim - 1) {
    int has_b = n_facets > 0;
    if (has_b) {
      NFEM_TRY_CUDA(cudaMemsetAsync(bkeys, 0, p.bcap * sizeof(uint64_t), stream));
      fill_i32<<<grid_for(int64_t(p.bcap), B), B, 0, stream>>>(bvals, int64_t(p.bcap), INT32_MAX);
      facet_insert<<<grid_for(n_facets, B), B, 0, stream>>>(facets, n_facets, cell_dim, bkeys, bvals, p.bcap - 1,
                                                            status);
    }
    facet_flags<<<grid_for(p.n_occ, B), B, 0, stream>>>(cv, n_cells, nv, cdi, facets, facets_first, bkeys, bvals,
                                                        has_b ? p.bcap - 1 : 0, has_b, flags);
    NFEM_CHECK_LAUNCH();
  }
  int32_t h_status = 0;
  NFEM_TRY_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
  NFEM_TRY_CUDA(cudaStreamSynchronize(stream));
  return h_status;
}

extern "C" int nfem_rt1_sign_mask(const uint8_t* flags, int64_t n_cells, int cell_dim, uint8_t* mask, void* stream) {
  if (cell_dim < 2 || cell_dim > 3 || n_cells < 0 || (n_cells > 0 && (!flags || !mask))) return NFEM_ERR_INVALID_ARG;
  if (n_cells == 0) return NFEM_OK;
  rt1_mask_kernel<<<grid_for(n_cells, 256), 256, 0, (cudaStream_t)stream>>>(flags, n_cells, cell_dim + 1,
                                                                            cell_dim == 3, mask);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}

extern "C" int nfem_compose_cell_dofs(int64_t n_cells, int n_blocks, const nfem_dof_block* blocks, int32_t* cell_dofs,
                                      int ld, void* stream) {
  if (n_blocks < 1 || n_blocks > NFEM_MAX_DOF_BLOCKS || !blocks || n_cells < 0 || (n_cells > 0 && !cell_dofs))
    return NFEM_ERR_INVALID_ARG;
  DofBlocks db;
  db.n = n_blocks;
  int width = 0;
  for (int i = 0; i < n_blocks; ++i) {
    db.b[i] = blocks[i];
    if (blocks[i].n_ent < 0 || blocks[i].width < 0 || blocks[i].base < 0) return NFEM_ERR_INVALID_ARG;
    if (blocks[i].n_ent > 0 && blocks[i].width > 0 && !blocks[i].occ_rank && blocks[i].n_ent != 1)
      return NFEM_ERR_INVALID_ARG;
    width += blocks[i].n_ent * blocks[i].width;
  }
  if (ld < width) return NFEM_ERR_INVALID_ARG;
  if (n_cells == 0) return NFEM_OK;
  compose_kernel<<<grid_for(n_cells, 256), 256, 0, (cudaStream_t)stream>>>(n_cells, db, cell_dofs, ld, nullptr);
  NFEM_CHECK_LAUNCH();
  return NFEM_OK;
}
