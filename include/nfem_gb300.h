/*
 * nfem_gb300.h - C ABI of the GB300 finite-element assembly-and-solve path.
 *
 * Every entry point is `extern "C"`, takes plain device pointers, sizes and a
 * cudaStream_t (passed as void*), never allocates device memory unless its
 * comment says so, never throws, and returns an nfem_status.  Kernels are
 * asynchronous on `stream`; conditions detected on the device (a row whose
 * merged length disagrees with the pattern, a full hash table, a Krylov
 * breakdown) are written to an optional device `int32_t* dev_status` word
 * (first nonzero code wins) that the caller reads after synchronising.
 *
 * Index conventions: cell-to-vertex, cell-to-DoF, CSR row_ptr and col_idx are
 * int32 (sizes are checked against 2^31 - 1); point coordinates are FP64
 * [n_points, 3] row-major like the reference's mesh.points.
 *
 * Each declaration names the reference interface it replaces (paths are
 * inside the nfempy project).
 */
#ifndef NFEM_GB300_H
#define NFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  NFEM_OK = 0,
  NFEM_ERR_INVALID_ARG = 1,   /* bad pointer / size / enum */
  NFEM_ERR_CUDA = 2,          /* a CUDA runtime call or launch failed */
  NFEM_ERR_WORKSPACE = 3,     /* workspace smaller than the query returned */
  NFEM_ERR_OVERFLOW = 4,      /* a size does not fit the index type */
  NFEM_ERR_CAPACITY = 5,      /* a per-row buffer or hash table is full */
  NFEM_ERR_PATTERN = 6,       /* assembled row disagrees with the CSR pattern */
  NFEM_ERR_UNSUPPORTED = 7,   /* configuration not implemented */
  NFEM_ERR_NOT_CONVERGED = 8, /* Krylov iteration cap reached */
  NFEM_ERR_BREAKDOWN = 9,     /* Krylov breakdown (zero or non-finite denominator) */
  NFEM_ERR_NONFINITE = 10,    /* NaN / Inf detected in an input or residual */
  NFEM_ERR_DEGENERATE = 11,   /* a cell with |det J| == 0 */
  NFEM_ERR_DOMAIN = 12,       /* a coefficient outside its domain (kappa <= 0, mu <= 0) */
  NFEM_ERR_TIMEOUT = 13       /* a bounded device-side wait ran out */
} nfem_status;

typedef enum { NFEM_F64 = 0, NFEM_F32 = 1, NFEM_BF16 = 2 } nfem_value_type;

/* Coefficient sampling modes for per-cell data arrays. */
typedef enum {
  NFEM_COEF_NONE = 0,      /* absent (treated as zero) */
  NFEM_COEF_CELL = 1,      /* one value per cell, [n_cells] */
  NFEM_COEF_QPOINT = 2     /* one value per quadrature point, [n_cells, n_qp] */
} nfem_coef_mode;

/* ------------------------------------------------------------------ misc */
int nfem_abi_version(void);
const char* nfem_status_string(int status);

/* Launch knobs: process-wide launch shapes that an autotuner may set
 * (nfempy_gb300.autotune times candidates and caches the best per GPU and
 * workload).  No reference counterpart.  0 restores the built-in choice.
 *   NFEM_KNOB_DARCY_ROWS_BLOCKS_PER_SM   resident blocks per SM of the Darcy
 *                                        row pass (0: the occupancy maximum)
 *   NFEM_KNOB_DARCY_CELLS_BLOCK          threads per block of the Darcy cell
 *                                        pass: 128, 256 (0) or 512
 *   NFEM_KNOB_ELAS_WARPS                 warps per block of the elasticity
 *                                        node rows with shared images: 2, 4 (0) or 8
 *   NFEM_KNOB_ELAS_ROWS                  elasticity and Cosserat node rows: 1
 *                                        shared-memory row images, 2 register
 *                                        accumulation by warp shuffles, 3
 *                                        (elasticity) registers for rows of at
 *                                        most 32 node columns and images for
 *                                        longer rows; 0 the built-in choice
 *                                        (shared-memory images)
 *   NFEM_KNOB_COARSE_TC                  trailing updates of the dense coarse
 *                                        inverse: 0 tensor cores (3xTF32) from
 *                                        512 aggregates on, 1 CUDA cores, 2
 *                                        tensor cores from 128 on
 *   NFEM_KNOB_DARCY_F64_RECORDS          FP64 Darcy records of tetrahedra: 0
 *                                        exact integer arithmetic for lattice
 *                                        cells (edges that are multiples of a
 *                                        common power of two with quotients
 *                                        below 2^20) and double-float for the
 *                                        others, 1 double-float for every cell
 * nfem_knob_set returns NFEM_ERR_INVALID_ARG for an unknown key or value. */
typedef enum {
  NFEM_KNOB_DARCY_ROWS_BLOCKS_PER_SM = 0,
  NFEM_KNOB_DARCY_CELLS_BLOCK = 1,
  NFEM_KNOB_ELAS_WARPS = 2,
  NFEM_KNOB_ELAS_ROWS = 3,
  NFEM_KNOB_COARSE_TC = 4,
  NFEM_KNOB_DARCY_F64_RECORDS = 5,
  NFEM_KNOB_COUNT = 6
} nfem_knob;
int nfem_knob_set(int key, int value);
int nfem_knob_get(int key, int* value);

/* Exclusive prefix sum of n int32 counts into n + 1 int64 offsets. */
int nfem_scan_workspace_bytes(int64_t n, size_t* bytes);
int nfem_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets,
                        void* workspace, size_t workspace_bytes, void* stream);

/* The same scan for callers that cannot allocate device memory: code that
 * runs while a CUDA graph is being captured (cudaMalloc is not a capturable
 * operation), or inside a host framework that owns all device memory through
 * its own pool allocator and forbids raw allocations.  No counterpart in the
 * reference.  The scan's scratch (one int64 per 4096 counts) is a fixed
 * device array inside the library, so n is limited to 67,108,864 counts
 * (NFEM_ERR_CAPACITY above that).  The first call on a device looks up that
 * array's device address; make that first call before any stream capture.
 * All calls on a device share the one array: calls whose kernels overlap on
 * the GPU (different streams, or different host threads without ordering)
 * race and must be serialised by the caller.  The looked-up address lives
 * as long as the device's primary context: do not call this scan after a
 * cudaDeviceReset in the same process.  Allocates nothing. */
int nfem_exclusive_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets,
                                void* stream);

/* --------------------------------------- K0: entity numbering (a1, a2, a8)
 * Replaces Mesh.build_conformal_mesh + insert_* (src/mesh/mesh.py:125-339),
 * the first-appearance entity order of MeshTopology
 * (src/mesh/mesh_topology.py:16-35 via src/mesh/mesh.py:639-681) and the
 * orientation checks of src/basis/permute_and_transform.py:8-107.
 *
 * For every (cell, local sub-entity of dimension entity_dim) occurrence,
 * writes the rank of its global entity in first-appearance order over the
 * cells (cells in the given order, sub-entities in the reference's local
 * order).  entity_dim must be 0, 1 or 2 and < cell_dim.  When entity_dim ==
 * cell_dim - 1 and `flags` is non-NULL, also writes per occurrence:
 *   bit0 = reflected  (2-D: local edge order differs from the stored edge
 *                      order; 3-D: the face's global tags are an odd
 *                      permutation of sorted order)
 *   bit1 = tagged     (the facet appears in the boundary facet block)
 * `facets` [n_facets, cell_dim] are the tagged lower-dimensional cells in file
 * order; facets_first != 0 means that block precedes the cells in the file
 * (it then fixes the stored node order of those edges).
 * n_entities_out is a device int64.
 */
int nfem_numbering_workspace_bytes(int64_t n_cells, int cell_dim, int entity_dim,
                                   int64_t n_points, int64_t n_facets, size_t* bytes);
int nfem_number_entities(const int32_t* cell_vertices, int64_t n_cells, int cell_dim,
                         int entity_dim, int64_t n_points, const int32_t* facets,
                         int64_t n_facets, int facets_first, void* workspace,
                         size_t workspace_bytes, int32_t* occ_rank, uint8_t* flags,
                         int64_t* n_entities_out, void* stream);

/* Packs the RT1 orientation sign of each local facet into one byte per cell
 * (bit i set = basis function i negated), applying the reference rule
 * (src/basis/permute_and_transform.py:57-107 for 3-D, :8-35 for 2-D). */
int nfem_rt1_sign_mask(const uint8_t* facet_flags, int64_t n_cells, int cell_dim,
                       uint8_t* sign_mask, void* stream);

/* ------------------------------------------------------ K0: DoF map (a3, a4)
 * Replaces DoFMap.build_entity_maps / destination_indices
 * (src/spaces/dof_map.py:38-146) and ProductSpace.destination_indexes
 * (src/spaces/product_space.py:147-170).  Blocks are concatenated in order;
 * block b contributes, for each local entity e < n_ent and j < width, the DoF
 * base + rank(c, e) * width + j (rank = cell index when occ_rank is NULL). */
typedef struct {
  const int32_t* occ_rank; /* [n_cells, n_ent] or NULL for the cell block */
  int32_t n_ent;           /* local entities of this dimension per cell */
  int32_t width;           /* e_dofs * n_comp */
  int64_t base;            /* first global DoF of the block */
} nfem_dof_block;

#define NFEM_MAX_DOF_BLOCKS 16
int nfem_compose_cell_dofs(int64_t n_cells, int n_blocks, const nfem_dof_block* blocks,
                           int32_t* cell_dofs, int ld, void* stream);

/* ------------------------------------------------ K0: CSR pattern (a15)
 * Replaces the sparsity that PETSc builds from the per-entry setValue calls
 * of src/assembly/ScatterFormData.py:5-11 ("pattern A": every entry of every
 * element clique, zeros included, columns sorted per row).
 *
 * Step 1 (rows): row incidence lists (cell * n_loc + local, sorted per row)
 * and row lengths.  inc_ptr [n_rows + 1], inc [n_cells * n_loc] (int32),
 * row_ptr [n_rows + 1] (int32).  *nnz_host receives the total (the call
 * synchronises on `stream` to read it back).
 * Step 2 (cols): col_idx [nnz].
 * Optional slot map: slots [n_cells, n_loc, n_loc] = position of each element
 * entry in the CSR value array. */
int nfem_pattern_workspace_bytes(int64_t n_cells, int n_loc, int64_t n_rows, size_t* bytes);
int nfem_pattern_rows(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int ld,
                      int64_t n_rows, void* workspace, size_t workspace_bytes,
                      int32_t* inc_ptr, int32_t* inc, int32_t* row_ptr,
                      int64_t* nnz_host, int32_t* dev_status, void* stream);
int nfem_pattern_cols(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int ld,
                      int64_t n_rows, const int32_t* inc_ptr, const int32_t* inc,
                      const int32_t* row_ptr, int32_t* col_idx, int32_t* dev_status,
                      void* stream);
int nfem_pattern_slots(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int ld,
                       const int32_t* row_ptr, const int32_t* col_idx, int32_t* slots,
                       int32_t* dev_status, void* stream);

/* Compressed slot map for short rows: per incidence entry k of row r (cell c,
 * local a), codes[k] packs, 4 bits per local column b (n_loc <= 8, rows of at
 * most 16 entries), the position of cell_dofs[c, b] inside row r relative to
 * row_ptr[r].  Used by the row-owner assembly kernels. */
int nfem_pattern_local_codes(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int ld,
                             int64_t n_rows, const int32_t* inc_ptr, const int32_t* inc,
                             const int32_t* row_ptr, const int32_t* col_idx, uint32_t* codes,
                             int32_t* dev_status, void* stream);

/* Fixed-stride form of the incidence lists for rows with at most two
 * incidences (mixed RT1 x P0 spaces): pairs [n_rows, 2] = the (cell * n_loc +
 * local) occurrences of each row or -1, pair_codes [n_rows, 2] = their slot
 * codes.  Returns NFEM_ERR_UNSUPPORTED (through dev_status) for longer lists. */
int nfem_pattern_pairs(const int32_t* inc_ptr, const int32_t* inc, const uint32_t* codes,
                       int64_t n_rows, int32_t* pairs, uint32_t* pair_codes,
                       int32_t* dev_status, void* stream);

/* Exact 64-bit fixed-point point records for the FP64 assembly of
 * tetrahedra: records [1 + n_points, 4] int64, 16-byte aligned.  Record 0 =
 * (shift, 0, 0, 0); record v + 1 = (qx, qy, qz, 0) with q = x * 2^shift
 * rounded to the nearest integer and shift = 1084 - (biased FP64 exponent
 * of max |x|), so |q| < 2^62.  No centring: q holds every bit of x at or
 * above 2^-shift, and an edge vector q1 - q0 is an exact integer difference
 * (accurate to 2^-62 max |x|), which the FP64 kernels turn into
 * double-float values with integer operations.  No reference counterpart
 * (device data layout). */
int nfem_points_fixed64(const double* points, int64_t n_points, int64_t* records, void* stream);

/* Adds element matrices j_el [n_el, n_loc, n_loc] and residuals r_el
 * [n_el, n_loc] (either may be NULL) of value_type into the CSR values and
 * rhs at the rows / columns dofs [n_el, n_loc]: the generic path of
 * scatter_form_data / scatter_interface_form_data /
 * scatter_time_dependent_form_data (src/assembly/ScatterFormData.py:5-79)
 * for weak forms evaluated outside the library.  Atomic additions (the
 * order of the additions into one entry may vary); an entry outside the
 * pattern sets NFEM_ERR_PATTERN, a DoF outside [0, n_rows)
 * NFEM_ERR_INVALID_ARG, in dev_status. */
int nfem_scatter_elements(int value_type, int64_t n_el, int n_loc, const int32_t* dofs,
                          const void* j_el, const void* r_el, const int32_t* row_ptr,
                          const int32_t* col_idx, int64_t n_rows, void* values, void* rhs,
                          int32_t* dev_status, void* stream);

/* Adds n (row, col, value) triples (values FP64, converted to value_type)
 * into the CSR values: Mat.setValue(row, col, value, addv=True) batched
 * (src/assembly/ScatterFormData.py:5-11).  Atomic; an entry outside the
 * pattern sets NFEM_ERR_PATTERN, a row or column outside [0, n_rows)
 * NFEM_ERR_INVALID_ARG, in dev_status. */
int nfem_csr_add_entries(int value_type, int64_t n, const int32_t* rows, const int32_t* cols,
                         const double* vals, const int32_t* row_ptr, const int32_t* col_idx,
                         int64_t n_rows, void* values, int32_t* dev_status, void* stream);

/* Copies `bytes` from src to dst with a kernel (16-byte vectors when both are
 * 16-byte aligned).  Either pointer may be pinned host memory mapped into the
 * device address space (cudaHostAlloc), so results reach the host without a
 * copy engine; pageable host memory is refused (NFEM_ERR_INVALID_ARG).  No
 * reference counterpart (host I/O helper). */
int nfem_copy_bytes(const void* src, void* dst, size_t bytes, void* stream);

/* Cells per entry of the cell-chunk row table of the mixed Darcy layout. */
#define NFEM_DARCY_CHUNK_CELLS 32

/* Cell-chunk row table for nfem_darcy_rt1p0_assemble: chunk_rows
 * [ceil(n_cells / NFEM_DARCY_CHUNK_CELLS) + 1], entry k = the first flux row
 * whose first incidence lies in a cell >= k * NFEM_DARCY_CHUNK_CELLS.  Needs
 * the first-appearance layout of a mixed RT1 x P0 space: flux rows
 * [0, p_base), then one pressure row per cell in cell order
 * (n_rows = p_base + n_cells); anything else returns NFEM_ERR_UNSUPPORTED
 * (directly or through dev_status). */
int nfem_pattern_darcy_chunks(const int32_t* pairs, int64_t n_rows, int n_loc, int64_t p_base,
                              int64_t n_cells, int32_t* chunk_rows, int32_t* dev_status,
                              void* stream);

/* Packs FP64 points into 16-byte fixed-point records so FP32 kernels form
 * cell edge vectors with one load per vertex, an exact integer difference
 * and no FP64 arithmetic.  points_split: [1 + n_points, 4] 32-bit words,
 * 16-byte aligned.  Record 0 = (scale, cx, cy, cz) as floats; record v + 1 =
 * (qx, qy, qz, 0) as int32, q = round((x - c) / scale), c the bounding-box
 * centre, scale = 2^(e - 30) for a half-extent below 2^e (|q| < 2^30).  Edge
 * vectors carry an absolute error below scale: a relative error below
 * 1e-9 x (cells across the mesh). */
int nfem_points_split(const double* points, int64_t n_points, float* points_split,
                      void* stream);

/* --------------------------- K1-K4: mixed Darcy RT1 x P0 (a6-a10, a15)
 * Replaces LaplaceDualWeakForm.evaluate_form
 * (src/weak_forms/laplace_dual_weak_form.py:10-86) for every cell together
 * with the scatter of src/assembly/ScatterFormData.py:5-25: writes the CSR
 * values of the global Jacobian (pattern from nfem_pattern_*) and the global
 * residual at alpha = 0, r = -int f w on pressure rows, 0 on flux rows.
 *
 * Geometry: affine simplices, contravariant Piola with |det J|, orientation
 * signs from nfem_rt1_sign_mask.  kappa is one value per cell; source is per
 * cell or per quadrature point of the rule `2*1+1` (collapsed Gauss-Jacobi,
 * 4 points on triangles, 8 on tetrahedra; ordering as in the reference).
 * value_type selects FP64 (coordinates `points`) or FP32 (coordinates
 * `points_split` from nfem_points_split); kappa/source/values/rhs then have
 * that type.  For FP64 tetrahedra with the record workspace, `points_split`
 * may instead carry the int64 records of nfem_points_fixed64 (cast to
 * const float*): the cell pass then forms its edges from them with no FP64
 * instruction; NULL keeps FP64 subtraction of `points`.  flux_dofs [n_cells, dim + 1] are the RT1 DoFs, the pressure DoF
 * of cell c is p_base + c.  qweights (host, n_qp entries) are the reference
 * quadrature weights, read only when source_mode == NFEM_COEF_QPOINT.
 * row_pairs/pair_codes come from nfem_pattern_rows, nfem_pattern_local_codes and
 * nfem_pattern_pairs with cell_dofs = [flux_dofs | p_base + c].  accumulate == 0 overwrites
 * values/rhs (the first form of an assembly pass, like a zeroed PETSc Mat
 * and residual); accumulate != 0 adds to them (setValue(addv=True)).  Each CSR value and residual entry is written once
 * (no atomics, deterministic).  chunk_rows (optional, from
 * nfem_pattern_darcy_chunks with the same p_base) selects the cell-chunk
 * kernel: each warp evaluates the element matrices of 32 consecutive cells
 * once and writes the rows whose first incidence lies there; NULL selects
 * the row-owner kernel, which evaluates every incidence of a row on its own.
 * Both give the same values up to rounding. */
int nfem_darcy_rt1p0_assemble(int dim, int value_type, int64_t n_cells, int64_t n_rows,
                              const double* points, const float* points_split,
                              const int32_t* cell_vertices, const int32_t* flux_dofs,
                              int64_t p_base, const uint8_t* sign_mask,
                              const void* kappa, const void* source, int source_mode,
                              const double* qweights, int n_qp,
                              const int32_t* row_pairs, const uint32_t* pair_codes,
                              const int32_t* row_ptr, const int32_t* chunk_rows,
                              void* values, void* rhs, int accumulate,
                              void* workspace, size_t workspace_bytes,
                              int32_t* dev_status, void* stream);
/* Record workspace of the two-pass row-owner assembly: with workspace !=
 * NULL (and chunk_rows == NULL) a cell pass first evaluates, once per cell,
 * the metric terms all rows of the cell's element matrix are made of
 * (G = J^T J, the scale and the pressure row's residual entry: 8 FP32 words
 * per cell; FP64 triangles add the row sums of G, 8 words; FP64 tetrahedra
 * keep the ten distinct entries of the flux block and the residual entry,
 * 11 words) and the row pass reads them in place of the vertices; the
 * values agree with the one pass to rounding (the same expressions, fused
 * alike or not).  The cell pass also writes each cell's pressure row
 * (row p_base + c).  FP32 cells of poor shape quality (|det J| below 0.1
 * times the product of their edge lengths from vertex 0) are finished by a
 * second launch that takes |det J| in FP64 from `points` (or from the
 * fixed-point records when `points` is NULL); the FP32 workspace holds
 * their list (4 bytes per cell and 16).  NULL: one pass that evaluates every (row, cell) incidence from the
 * vertices.  The workspace is 16-byte aligned, of at least this size. */
int nfem_darcy_workspace_bytes(int dim, int value_type, int64_t n_cells, size_t* bytes);

/* One pass of the two-pass assembly over a range (workspace required):
 * pass 1 forms the cell records of [cell_begin, cell_end); pass 2 writes the
 * rows [row_f0, row_f1) and [row_q0, row_q1) from records already formed.
 * The caller orders the passes, e.g. the records of consecutive cell slices
 * on one stream and the rows of each slice on a second stream once the
 * records of every cell its rows touch are done (each row written once, as
 * by nfem_darcy_rt1p0_assemble). */
int nfem_darcy_rt1p0_assemble_pass(int dim, int value_type, int64_t n_cells, int64_t n_rows,
                                   const double* points, const float* points_split,
                                   const int32_t* cell_vertices, int64_t p_base, const uint8_t* sign_mask,
                                   const void* kappa, const void* source, int source_mode,
                                   const double* qweights, int n_qp, const int32_t* row_pairs,
                                   const uint32_t* pair_codes, const int32_t* row_ptr, void* values,
                                   void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                                   int pass, int64_t cell_begin, int64_t cell_end, int64_t row_f0,
                                   int64_t row_f1, int64_t row_q0, int64_t row_q1, int32_t* dev_status,
                                   void* stream);

/* Overlapped form of nfem_darcy_rt1p0_assemble for tetrahedra (same
 * reference interface, same values up to rounding): the mesh is cut into
 * K = ceil(n_cells / 2^slice_shift) slices of consecutive cells and the
 * assembly runs as K + 1 launches on `stream`, each writing the rows of one
 * slice while a quarter-share of its blocks forms the cell records of the
 * slice two ahead.  The records live in `ring` (three slices, from
 * nfem_darcy_ring_bytes), small enough to stay in L2, so the cell pass and
 * the row pass overlap and the records never travel to HBM and back.
 * Needs the first-appearance layout of a mixed RT1 x P0 space (flux rows
 * [0, p_base), pressure row p_base + c of cell c), the pairs / pair_codes /
 * row_ptr of nfem_pattern_pairs, and a host plan:
 *   flux_row_begin [K + 1] (host): first flux row whose first incidence
 *     lies in slice k (the chunk table of nfem_pattern_darcy_chunks at the
 *     slice starts), flux_row_begin[K] = p_base;
 *   lookahead_cells: the largest (second incidence cell - first incidence
 *     cell) over the flux rows, which must be below 2^slice_shift
 *     (NFEM_ERR_UNSUPPORTED otherwise);
 *   record_quarters (1..3): quarters of the blocks of a launch that form
 *     records while the others write rows.
 * point_records: nfem_points_split records (FP32) or nfem_points_fixed64
 * records (FP64; NULL: FP64 subtraction of `points`). */
typedef struct {
  int32_t slice_shift;
  int32_t lookahead_cells;
  int32_t record_quarters;
  const int64_t* flux_row_begin;
} nfem_darcy_slices;
int nfem_darcy_ring_bytes(int value_type, int slice_shift, size_t* bytes);
int nfem_darcy_rt1p0_assemble_sliced(int value_type, int64_t n_cells, int64_t n_rows,
                                     const double* points, const void* point_records,
                                     const int32_t* cell_vertices, int64_t p_base,
                                     const uint8_t* sign_mask, const void* kappa, const void* source,
                                     int source_mode, const double* qweights, int n_qp,
                                     const int32_t* row_pairs, const uint32_t* pair_codes,
                                     const int32_t* row_ptr, const nfem_darcy_slices* slices,
                                     void* values, void* rhs, int accumulate, void* ring,
                                     size_t ring_bytes, int32_t* dev_status, void* stream);

/* Fused form of nfem_darcy_rt1p0_assemble for FP64 tetrahedra (same
 * reference interface, LaplaceDualWeakForm.evaluate_form
 * src/weak_forms/laplace_dual_weak_form.py:10-86 with the scatter of
 * src/assembly/ScatterFormData.py:5-25; bitwise the values of the two-pass
 * form): one persistent cooperative launch whose warps take record chunks
 * (32 cells: records and pressure rows) and row chunks (32 flux rows) in
 * the order of a plan, each row chunk after the record chunks of the cells
 * it touches, so records are read back from L2 soon after they are
 * written.  A row chunk waits (bounded) for its record chunks' flags; a
 * wait that runs out sets NFEM_ERR_TIMEOUT.
 * nfem_darcy_fused_plan builds the plan once per pattern (it reads
 * row_pairs, synchronises `stream` and copies one word per row chunk to the
 * host); lead_chunks > 0 sets how many record chunks run ahead of the rows
 * (0: half the warps the GPU holds at once).  The plan also holds the
 * chunk flags that each assembly zeroes, so one plan serves one assembly
 * at a time.  Requires n_rows = p_base + n_cells and
 * the record workspace of nfem_darcy_workspace_bytes(3, NFEM_F64, ...);
 * point_records may carry nfem_points_fixed64 records or be NULL. */
int nfem_darcy_fused_plan_bytes(int64_t n_cells, int64_t p_base, size_t* bytes);
int nfem_darcy_fused_plan(const int32_t* row_pairs, int64_t n_cells, int64_t p_base, int lead_chunks,
                          void* plan, size_t plan_bytes, void* stream);
int nfem_darcy_rt1p0_assemble_fused(int64_t n_cells, int64_t n_rows, const double* points,
                                    const void* point_records, const int32_t* cell_vertices,
                                    int64_t p_base, const uint8_t* sign_mask, const void* kappa,
                                    const void* source, int source_mode, const double* qweights, int n_qp,
                                    const int32_t* row_pairs, const uint32_t* pair_codes,
                                    const int32_t* row_ptr, void* plan, size_t plan_bytes, void* values,
                                    void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                                    int32_t* dev_status, void* stream);

/* Replaces LaplaceDualWeakFormBCDirichlet.evaluate_form
 * (src/weak_forms/laplace_dual_weak_form.py:90-154) with its scatter: adds
 * int_F p_D (psi_f . n) to the residual entry of each boundary facet's flux
 * DoF.  facet_occ [n_facets] = cell * (dim + 1) + local face of the facet's
 * cell; pd_q [n_facets, n_qp] = p_D at the facet quadrature points (rule of
 * order 3 on the facet, n_qp <= 4, weights qweights on the host).  Each
 * boundary facet's DoF belongs to one facet: plain additions, deterministic. */
int nfem_darcy_rt1_dirichlet(int dim, int value_type, int64_t n_facets, const int32_t* facet_occ,
                             const uint8_t* sign_mask, const int32_t* cell_dofs, int ld,
                             const void* pd_q, const double* qweights, int n_qp, void* rhs,
                             void* stream);

/* The same facet term for one row of an RT1 field inside a larger layout:
 * the face DoF of local face i is cell_dofs[c * ld + dof_offset + i *
 * dof_stride], and scale multiplies the term.  Replaces
 * LCEDualWeakFormBCDirichlet.evaluate_form
 * (src/weak_forms/lce_dual_weak_form.py:651-756): per component c of the
 * stress (couple stress) field, dof_offset = field start + c, dof_stride = 3,
 * scale = -1, pd_q = the c-th component of u_D (t_D). */
int nfem_rt1_dirichlet_rows(int dim, int value_type, int64_t n_facets, const int32_t* facet_occ,
                            const uint8_t* sign_mask, const int32_t* cell_dofs, int ld, int dof_offset,
                            int dof_stride, double scale, const void* pd_q, const double* qweights, int n_qp,
                            void* rhs, void* stream);

/* Replaces l2_error (src/postprocess/l2_error_post_processor.py:7-63) for a
 * mixed Darcy RT1 x P0 solution alpha (FP64): errors[0] = ||u - u_h||_L2,
 * errors[1] = ||p - p_h||_L2 (device doubles), with the exact fields sampled
 * at the quadrature points, u_exact_q [n_cells, n_qp, dim], p_exact_q
 * [n_cells, n_qp]; qpoints [n_qp, dim] / qweights [n_qp] on the host.
 * workspace >= 2 * 304 doubles.  FP64 throughout, fixed-order reduction. */
int nfem_darcy_l2_error(int dim, int64_t n_cells, const double* points,
                        const int32_t* cell_vertices, const uint8_t* sign_mask,
                        const int32_t* cell_dofs, int ld, const double* alpha,
                        const double* u_exact_q, const double* p_exact_q, const double* qpoints,
                        const double* qweights, int n_qp, double* errors, void* workspace,
                        size_t workspace_bytes, void* stream);

/* Replaces l2_error (src/postprocess/l2_error_post_processor.py:7-63),
 * div_error (:185-238), div_scaled_error (:240-306) and, with alpha == NULL,
 * l2_norm / div_norm (src/postprocess/solution_norms_post_processor.py:7-78)
 * for one field of a product space on affine simplices, FP64:
 * *result (device double) = sqrt(sum_cells sum_q |det J| w_q |e - u_h|^2).
 * family: 0 Lagrange (ref_table [n_qp, n_phi] values), 1 RT1 (ref_table
 * [n_qp, n_phi, dim] reference values with the reference normal signs,
 * ref_div [n_phi] their divergences; cell signs from sign_mask).
 * quantity: 0 values (exact_q [T, n_qp, n_cmp] for Lagrange, components
 * 0..n_cmp-1; [T, n_qp, n_comp, n_cmp] for the rows of an RT1 field),
 * 1 divergence of each RT1 row (exact_q [T, n_qp, n_comp]), 2 the scaled
 * divergence grad l . psi + l div psi (gamma_q [T, n_qp], grad_gamma_q
 * [T, n_qp, dim]).  The field's local DoFs start at dof_offset in each row
 * of cell_dofs (basis-major, component-minor).  n_qp <= 32, n_phi <= 10,
 * n_comp <= 3.  Block partials added in a fixed order (deterministic). */
int nfem_field_error_workspace_bytes(size_t* bytes);
int nfem_field_error(int dim, int family, int quantity, int64_t n_cells, const double* points,
                     const int32_t* cell_vertices, const uint8_t* sign_mask, const int32_t* cell_dofs,
                     int ld, int dof_offset, int n_phi, int n_comp, int n_cmp, const double* alpha,
                     const double* exact_q, const double* gamma_q, const double* grad_gamma_q,
                     const double* ref_table, const double* ref_div, const double* qweights, int n_qp,
                     double* result, void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------- vector P2 linear elasticity (a12, a13, a15)
 * Replaces LEPrimalWeakForm.evaluate_form
 * (src/weak_forms/le_primal_weak_form.py:10-129) for every tetrahedron, with
 * the scatter of src/assembly/ScatterFormData.py:5-25: the CSR values of the
 * global Jacobian and the residual at alpha = 0 (r = +int f . phi).  One
 * field, 3 components, DoF = row0 + 3 * node + component.  lambda and mu are
 * per cell, force per cell [n_cells, 3] or NULL.  ref_S [10*10*3*3]
 * (int dhat_k phihat_a dhat_l phihat_b) and ref_m [10] (int phihat_a) are the
 * exact reference-tetrahedron tables (host arrays).  max_node_degree = the
 * largest number of node columns of any node row (row length / 3; <= 255),
 * or 0 for the library bound of 96: it sizes the shared-memory row images.
 * Row owner, each value written once, deterministic. */
int nfem_pattern_node_codes(const int32_t* cell_dofs, int64_t n_cells, int n_loc, int n_comp,
                            int64_t row0, int64_t n_rows, const int32_t* inc_ptr,
                            const int32_t* inc, const int32_t* row_ptr, const int32_t* col_idx,
                            uint8_t* node_codes, int32_t* dev_status, void* stream);
/* Workspace of nfem_elasticity_p2_assemble: the per-cell geometry
 * (J^-1, lambda |det J|, mu |det J|, |det J|), 12 values of value_type per
 * cell, evaluated once per cell before the node rows read it. */
int nfem_elasticity_p2_workspace_bytes(int value_type, int64_t n_cells, size_t* bytes);
int nfem_elasticity_p2_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                const double* points, const float* points_split,
                                const int32_t* cell_vertices, const void* lambda_,
                                const void* mu, const void* force, const double* ref_S,
                                const double* ref_m, const int32_t* inc_ptr, const int32_t* inc,
                                const uint8_t* node_codes, const int32_t* row_ptr,
                                int max_node_degree, void* values, void* rhs, int accumulate,
                                void* workspace, size_t workspace_bytes, int32_t* dev_status,
                                void* stream);
/* Replaces LEPrimalWeakFormBCDirichlet.evaluate_form
 * (src/weak_forms/le_primal_weak_form.py:131-177) with u_D = 0: adds
 * beta * int_F phi_a phi_b to every component's (a, b) entry of the boundary
 * facets' rows.  facet_dofs [n_facets, 18] in facet P2 order, facet_vertices
 * [n_facets, 3]; ref_Mf [6*6] the reference-triangle P2 mass matrix.
 * Accumulates with atomics (the order of additions into a row may vary). */
int nfem_elasticity_p2_penalty(int value_type, int64_t n_facets, const int32_t* facet_dofs,
                               const int32_t* facet_vertices, const double* points, double beta,
                               const double* ref_S, const double* ref_m, const double* ref_Mf,
                               const int32_t* row_ptr, const int32_t* col_idx, void* values,
                               int32_t* dev_status, void* stream);

/* ------------------------------- mixed Cosserat elasticity, 3-D (a14)
 * Replaces LCEDualWeakForm.evaluate_form_vectorized
 * (src/weak_forms/lce_dual_weak_form.py:410-648) for every tetrahedron with
 * the scatter: fields s (RT1 x 3), m (RT1 x 3), u (P0 x 3), t (P0 x 3), DoF =
 * row0 + 3 * node + component.  params7 = {lambda_s, mu_s, kappa_s,
 * lambda_o, mu_o, kappa_o, l} (host), force [n_cells, 6] (f_u, f_t) or
 * NULL; ref_Psi [4*4*3*3] = int psihat_i psihat_j^T, ref_mhat [4*3] =
 * int psihat_i, ref_divhat [4] = int div psihat_i on the reference
 * tetrahedron (host).  Row owner over node rows, each value written once. */
/* Workspace of nfem_cosserat_assemble: the per-cell geometry (J, |det J|,
 * orientation), 12 values of value_type per cell. */
int nfem_cosserat_workspace_bytes(int value_type, int64_t n_cells, size_t* bytes);
int nfem_cosserat_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                           const double* points, const float* points_split,
                           const int32_t* cell_vertices, const uint8_t* sign_mask,
                           const double* params7, const void* force, const double* ref_Psi,
                           const double* ref_mhat, const double* ref_divhat,
                           const int32_t* inc_ptr, const int32_t* inc,
                           const uint8_t* node_codes, const int32_t* row_ptr, void* values,
                           void* rhs, int accumulate, void* workspace, size_t workspace_bytes,
                           int32_t* dev_status, void* stream);

/* Replaces LCEScaledRieszMapWeakForm.evaluate_form_vectorized
 * (src/weak_forms/lce_scaled_riesz_map_weak_form.py:415-598), the
 * preconditioning operator the Cosserat driver assembles
 * (examples/cosserat_elasticity/mfe_cosserat_elasticity_example_3.py:189-240),
 * into the CSR pattern of the dual form (its blocks are a subset): per field
 * block-diagonal; (s,s) the stress compliance plus (div tau_i, div tau_j) of
 * every row, (m,m) the couple-stress compliance plus l^2 (div v_i, div v_j)
 * (a constant length l = params7[6]; a varying l is not supported), (u,u)
 * and (t,t) the P0 mass.  Arguments as nfem_cosserat_assemble, no load. */
int nfem_cosserat_riesz_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                                 const double* points, const float* points_split,
                                 const int32_t* cell_vertices, const uint8_t* sign_mask,
                                 const double* params7, const double* ref_Psi, const double* ref_mhat,
                                 const double* ref_divhat, const int32_t* inc_ptr, const int32_t* inc,
                                 const uint8_t* node_codes, const int32_t* row_ptr, void* values,
                                 int accumulate, void* workspace, size_t workspace_bytes,
                                 int32_t* dev_status, void* stream);

/* -------------------------------------------- K5 + K7: Krylov solve (a17)
 * Replaces the PETSc KSP solves of the drivers
 * (examples/md_elliptic_scalar/md_elliptic_scalar.py:343-363,
 * examples/cauchy_elasticity/cg_elasticity_example_1.py:159-170,
 * examples/cosserat_elasticity/mfe_cosserat_elasticity_example_3.py:256-297):
 * solves A x = b to ||b - A x||_2 / ||b||_2 <= rtol with the residual always
 * evaluated in FP64 on the FP64 matrix, inner flexible GMRES(restart) in FP32
 * on the FP32 copy of the same matrix (iterative refinement). */
typedef struct {
  int64_t n_rows;
  const int32_t* row_ptr;
  const int32_t* col_idx;
  const void* values;
  int value_type; /* nfem_value_type */
} nfem_csr;

typedef enum {
  NFEM_PC_NONE = 0,
  NFEM_PC_JACOBI = 1,      /* point Jacobi: diag_inv [n_rows] */
  NFEM_PC_CELL_BLOCK = 2,  /* cell-patch block Jacobi (weighted additive Schwarz over
                              the element cliques): cell_dofs [n_cells, n_loc],
                              block_inv [n_cells, n_loc, n_loc], row incidences */
  NFEM_PC_TWO_LEVEL = 3,   /* NFEM_PC_CELL_BLOCK smoother followed by a Galerkin coarse
                              correction (see nfem_two_level) */
  NFEM_PC_NODE_BLOCK = 4   /* nfem_solve_ir_pcg only: inverses of the 3 x 3 diagonal
                              blocks of the nodes of a vector field (DoF = 3 node + c) */
} nfem_pc_kind;

/* Two-level preconditioner: z = B v, then z += P Ac^-1 P^T (v - A z), with B
 * the cell-block Jacobi, P the prolongation from n_agg aggregates of cells
 * (pressure DoF of a cell -> its aggregate with weight 1; flux row f -> the
 * aggregates of the pressure columns of row f with weight -w_f * sum of the
 * row's entries in that aggregate's columns, so rows of faces interior to an
 * aggregate vanish) and Ac = P^T A P formed exactly (Galerkin) and inverted
 * densely.  w [n_rows] are the flux-extension weights: 1/|a_ff| is the
 * classical choice; the learned preconditioner predicts them with the network.
 * All arrays are caller-owned; the coarse correction also needs the FP32
 * matrix (a32 in nfem_precond). */
typedef struct {
  int64_t p_base;            /* pressure DoF of cell c is p_base + c */
  int32_t n_agg;
  const int32_t* cell_agg;   /* [n_cells] aggregate of each cell */
  const float* w;            /* [n_rows] flux-extension weights */
  const int32_t* p_agg;      /* [n_rows, 2] aggregates of each row's P entries, -1 = none */
  float* p_val;              /* [n_rows, 2] filled by nfem_precond_setup */
  int64_t pt_nnz;
  const int32_t* pt_ptr;     /* [n_agg + 1] CSR of P^T, rows ascending in each list */
  const int32_t* pt_row;     /* [pt_nnz] */
  const int32_t* pt_slot;    /* [pt_nnz] index 2 * row + slot into p_val */
  float* pt_val;             /* [pt_nnz] filled by nfem_precond_setup */
  double* ac;                /* [n_agg, n_agg] Galerkin coarse matrix (blocks: [ac_entries]) */
  double* gj;                /* [n_agg, 2 n_agg] Gauss-Jordan scratch (blocks: unused, may be NULL) */
  float* ac_inv;             /* [n_agg, n_agg] (blocks: [ac_entries]) */
  float* work;               /* [64 + n_rows + 2 n_agg] */
  /* Block-diagonal coarse matrix (n_blocks > 0): a batch of independent
   * problems assembled as one disjoint union has no coupling between the
   * aggregates of different problems, so Ac is stored, inverted and applied
   * block by block.  The aggregates of block b are blk_ptr[b] ..
   * blk_ptr[b + 1] - 1; block b's s_b x s_b entries (row-major) start at
   * blk_off[b] in ac and ac_inv.  A nonzero of A coupling two blocks is
   * an error (NFEM_ERR_INVALID_ARG in the device status).  n_blocks = 0 keeps
   * the dense n_agg x n_agg layout and leaves the fields below unread. */
  int32_t n_blocks;
  int32_t blk_max;           /* largest s_b, at most NFEM_COARSE_BLOCK_MAX */
  int64_t ac_entries;        /* blk_off[n_blocks] */
  const int32_t* blk_ptr;    /* [n_blocks + 1] */
  const int64_t* blk_off;    /* [n_blocks + 1] */
  const int32_t* agg_blk;    /* [n_agg] block of each aggregate */
  /* Optional product A P of the FP32 matrix and the prolongation (CSR,
   * columns = aggregates).  With it the preconditioner also returns A z for
   * the z it computes, as (v - r) + (A P) e from the residual r = v - A z_s
   * of its smoother step and the coarse correction e, and the Krylov solver
   * skips its own SpMV with A.  ap_ptr [n_rows + 1] and ap_col [ap_nnz] come
   * from nfem_two_level_ap_pattern; nfem_precond_setup fills ap_val [ap_nnz]
   * from the FP32 matrix (a32 in nfem_precond).  ap_ptr == NULL: not used. */
  int64_t ap_nnz;
  const int32_t* ap_ptr;
  const int32_t* ap_col;
  float* ap_val;
  /* Cycle: omega (> 0; 0 means 1) damps the cell-block smoother, z = omega B v;
   * post_smooth != 0 adds z += omega B (v - A z) after the coarse correction
   * (a symmetric two-level cycle: one more smoother apply and SpMV per
   * application, fewer Krylov iterations). */
  float omega;
  int32_t post_smooth;
} nfem_two_level;

#define NFEM_COARSE_BLOCK_MAX 1024

typedef struct {
  int kind;
  int n_loc;
  int64_t n_cells;
  const int32_t* cell_dofs;
  const int32_t* inc_ptr;
  const int32_t* inc;
  float* block_inv;
  float* diag_inv;
  /* Optional weighted inner product for the flexible GMRES: W^1/2 and W^-1/2
   * [n_rows] filled by nfem_precond_setup (which then needs setup_scratch,
   * 2 * n_rows doubles).  W balances the flux and pressure rows of saddle-point
   * systems: W_i = sqrt(s_i^2 c_i^2), s_i^2 = 1/|a_ii| (or the inverse Schur
   * diagonal sum_j a_ij^2/|a_jj| where a_ii = 0), c_i^2 = squared column norm
   * of the preconditioner.  NULL = Euclidean inner product. */
  float* wsqrt;
  float* winvsqrt;
  double* setup_scratch;
  const nfem_two_level* two_level; /* NFEM_PC_TWO_LEVEL only (host pointer) */
  const nfem_csr* a32;             /* FP32 matrix, NFEM_PC_TWO_LEVEL only (host pointer) */
  /* Optional (host pointer): the cell-block smoother (times the two-level
   * omega) stored in A's CSR pattern, FP32 values [nnz] filled by
   * nfem_precond_setup; row_ptr and col_idx must be A64's.  With it each
   * smoother application is one SpMV.  NULL: applied cell block by cell
   * block. */
  const nfem_csr* smoother;
} nfem_precond;

typedef struct {
  double rtol;        /* FP64 relative residual target */
  double inner_rtol;  /* reduction asked of each FP32 inner solve */
  int restart;        /* GMRES restart length, 1..128 */
  int max_inner;      /* cap on total inner iterations */
  int max_outer;      /* cap on refinement steps */
  float* snapshots;   /* optional [max_snapshots, n_rows] FP32: the iterate after
                         every restart cycle (training data for the learned
                         preconditioner); NULL = none */
  int max_snapshots;
  int no_graphs;      /* 0: from the second restart cycle on, the cycle's steps
                         are replayed as one CUDA graph; 1: launched one by one */
  /* Schedule (no reference counterpart).  schedule_mode 1 records, into the
   * host array schedule [schedule_capacity], the launch schedule this solve
   * took: {n_outer, then per refinement step: n_cycles, then the steps of
   * each cycle}; schedule[0] = -1 when it did not fit.  schedule_mode 2
   * replays a recorded schedule without any host synchronisation (the call
   * can be captured into a CUDA graph with the assembly before it): the same
   * launches, the step counts taken from the schedule rather than from the
   * device, no nested cycle graphs; the FP64 relative residual
   * ||b - A x|| / ||b|| after the last step is written to the device double
   * relres_out, which the caller checks (a system whose solve needs more
   * steps than recorded ends above rtol there).  info then holds the
   * recorded counts. */
  int32_t* schedule;
  int schedule_capacity;
  int schedule_mode;
  double* relres_out;
} nfem_solve_params;

typedef struct {
  int inner_iterations;
  int outer_iterations;
  double initial_relres;
  double final_relres;
  int status;
  int n_snapshots;
} nfem_solve_info;

/* y = A x (FP32 or FP64 matrix and vectors) */
int nfem_spmv(int value_type, int64_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
              const void* values, const void* x, void* y, void* stream);
/* r = b - A x in FP64 */
int nfem_residual_f64(int64_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
                      const double* values, const double* x, const double* b, double* r,
                      void* stream);
/* Builds the preconditioner data from the FP64 matrix (block inverses in
 * FP64 Gauss-Jordan, stored FP32). */
int nfem_precond_setup(const nfem_precond* pc, const nfem_csr* A64, int32_t* dev_status,
                       void* stream);
/* Pattern of A P (see nfem_two_level.ap_ptr) from the pattern of A and the
 * aggregates of P (L->p_agg).  ap_col == NULL: counts the distinct aggregates
 * of each row into the offsets ap_ptr [n_rows + 1] and returns their total in
 * *nnz_host (synchronises `stream`).  Otherwise fills ap_col [*nnz_host],
 * ascending in each row, for the ap_ptr of the first call.  Rows with more
 * than 64 distinct aggregates report NFEM_ERR_CAPACITY. */
int nfem_two_level_ap_workspace_bytes(int64_t n_rows, size_t* bytes);
int nfem_two_level_ap_pattern(const nfem_csr* A, const nfem_two_level* L, void* workspace,
                              size_t workspace_bytes, int32_t* ap_ptr, int32_t* ap_col,
                              int64_t* nnz_host, int32_t* dev_status, void* stream);
int nfem_precond_apply(const nfem_precond* pc, int64_t n, const float* v, float* z, void* stream);
int nfem_solve_workspace_bytes(int64_t n_rows, int restart, size_t* bytes);
/* Synchronises on `stream` once per GMRES cycle and per refinement step. */
int nfem_solve_ir_fgmres(const nfem_csr* A64, const nfem_csr* A32, const nfem_precond* pc,
                         const double* b, double* x, const nfem_solve_params* params,
                         void* workspace, size_t workspace_bytes, nfem_solve_info* info,
                         void* stream);

/* ------------------------- mixed linear elasticity (s, u, t), 3-D */
/* Replaces LERieszMapWeakForm.evaluate_form_vectorized
 * (src/weak_forms/le_riesz_map_weak_form.py:245-360): the Riesz map of the
 * mixed linear-elastic space s (RT1 x 3), u (P0 x 3), t (P0 x 3), 18 local
 * DoFs, DoF = row0 + 3 * node + component; per stress row c the compliance
 * 1/(2 mu) int psi_i . psi_j plus int div psi_i div psi_j, minus
 * lambda / (2 mu (2 mu + 3 lambda)) int psi_i[c] psi_j[d] across rows, and
 * the P0 mass on u and t.  Constant lambda, mu (host); the Cosserat node-row
 * kernel in its Riesz mode over the 18-DoF layout.  Arguments otherwise as
 * nfem_cosserat_riesz_assemble. */
/* Replaces LEDualWeakForm.evaluate_form_vectorized
 * (src/weak_forms/le_dual_weak_form.py:354-515), the mixed linear-elastic
 * form with weakly imposed symmetry, with the scatter: the same 18-DoF
 * layout; per stress row the compliance 1/(2 mu) (psi_i . psi_j) minus
 * lambda / (2 mu (2 mu + 3 lambda)) psi_i[c] psi_j[d], the rotation
 * coupling (t, s) = the skew moments of the stress basis, the displacement
 * coupling (u, s) = int div psi_j per component, and r = -int f_u, -int f_t
 * (force [n_cells, 6] of cell means, or NULL).  Constant lambda, mu. */
int nfem_le_dual_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                          const double* points, const float* points_split, const int32_t* cell_vertices,
                          const uint8_t* sign_mask, double lambda_, double mu, const void* force,
                          const double* ref_Psi, const double* ref_mhat, const double* ref_divhat,
                          const int32_t* inc_ptr, const int32_t* inc, const uint8_t* node_codes,
                          const int32_t* row_ptr, void* values, void* rhs, int accumulate,
                          void* workspace, size_t workspace_bytes, int32_t* dev_status, void* stream);
int nfem_le_riesz_assemble(int value_type, int64_t n_cells, int64_t n_nodes, int64_t row0,
                           const double* points, const float* points_split,
                           const int32_t* cell_vertices, const uint8_t* sign_mask, double lambda_,
                           double mu, const double* ref_Psi, const double* ref_mhat,
                           const double* ref_divhat, const int32_t* inc_ptr, const int32_t* inc,
                           const uint8_t* node_codes, const int32_t* row_ptr, void* values,
                           int accumulate, void* workspace, size_t workspace_bytes,
                           int32_t* dev_status, void* stream);


/* Conjugate gradients for symmetric positive definite systems (the
 * driver's PETSc CG, examples/cauchy_elasticity/cg_elasticity_example_1.py:
 * 159-170, with a block-diagonal preconditioner in place of ICC): FP32 CG on
 * A32 inside FP64 iterative refinement on A64 until ||b - A x|| / ||b|| <=
 * rtol; each inner solve stops at inner_rtol (relative, on its own start).
 * x is overwritten (start 0 is not assumed: the first residual uses x).
 * pc_kind NFEM_PC_JACOBI (inv [n_rows] = 1 / a_ii) or NFEM_PC_NODE_BLOCK
 * (inv [n_rows / 3][9]), filled by nfem_pcg_setup from the FP64 matrix.
 * Reductions in a fixed order (deterministic).  Synchronises on `stream`
 * every 16 inner iterations and per refinement step.  A non-positive p.Ap
 * sets NFEM_ERR_BREAKDOWN. */
int nfem_pcg_setup(int pc_kind, const nfem_csr* A64, float* inv, int32_t* dev_status, void* stream);
int nfem_pcg_workspace_bytes(int64_t n_rows, size_t* bytes);
int nfem_solve_ir_pcg(const nfem_csr* A64, const nfem_csr* A32, int pc_kind, const float* inv,
                      const double* b, double* x, double rtol, double inner_rtol, int max_inner,
                      int max_outer, void* workspace, size_t workspace_bytes, nfem_solve_info* info,
                      int32_t* dev_status, void* stream);

/* ----------------------------------- K6: learned preconditioner network
 * No counterpart in the reference (nfempy has no learned component).
 * Network x -> relu(W1 x + b1) -> relu(W2 h1 + b2) -> W3 h2 + b3, dims =
 * {in, h1, h2, out}, parameters flat [W1 | b1 | W2 | b2 | W3 | b3] with
 * W_l [out, in] row-major; activations batch-major.  weight_type NFEM_BF16
 * reads BF16 weights (and biases from params_f32), FP32 accumulation. */
int nfem_mlp_param_count(const int32_t* dims, int64_t* count);
/* Inference of the same network on the tensor cores (tcgen05.mma, BF16 x
 * BF16 -> FP32 accumulators in tensor memory): y [batch] = the network's
 * output for x [batch, dims[0]], one fused persistent kernel.  params = the
 * BF16 copy, params_f32 = the FP32 master (biases).  The inputs and the
 * hidden activations after layer 1 are rounded to BF16 (the MMA operand
 * type).  Shapes other than dims = {<= 16, 256, 256, 1} return
 * NFEM_ERR_UNSUPPORTED. */
int nfem_mlp_infer_tc(const int32_t* dims, const void* params, const float* params_f32, int64_t batch,
                      const float* x, float* y, int32_t* dev_status, void* stream);
int nfem_mlp_forward(const int32_t* dims, int weight_type, const void* params,
                     const float* params_f32, int64_t batch, const float* x, float* h1,
                     float* h2, float* y, void* stream);
/* Gradients of loss = 0.5 / batch * sum ||y - target||^2 into grads (flat,
 * FP32, same layout as the parameters); loss (device double) optional. */
int nfem_mlp_backward_workspace_bytes(const int32_t* dims, int64_t batch, size_t* bytes);
int nfem_mlp_backward(const int32_t* dims, int weight_type, const void* params, int64_t batch,
                      const float* x, const float* h1, const float* h2, const float* y,
                      const float* target, float* grads, void* workspace,
                      size_t workspace_bytes, double* loss, void* stream);
/* Adam on the flat FP32 parameters; refreshes params_bf16 when non-NULL. */
int nfem_adam_step(int64_t n, float* params, const float* grads, float* m, float* v, float lr,
                   float beta1, float beta2, float eps, int step, void* params_bf16,
                   void* stream);
int nfem_to_bf16(int64_t n, const float* x, void* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NFEM_GB300_H */
