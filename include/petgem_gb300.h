/*
 * petgem_gb300 -- C ABI of the GB300 (sm_103a) forward-modelling hot path of
 * petgem: H(curl) elemental matrices -> CSR assembly -> complex Krylov solve
 * -> receiver interpolation.
 *
 * Conventions
 *   - Every pointer argument is a DEVICE pointer unless its comment says
 *     "host".  Buffers are allocated by the caller; functions that need
 *     scratch space take (workspace, workspace_bytes) and have a matching
 *     *_workspace_bytes() size query.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Index arrays are int32 unless stated; CSR row pointers are int64.
 *   - Complex arrays are interleaved (re, im) pairs: complex128 = 2 doubles,
 *     complex64 = 2 floats.
 *   - Every function returns PG_OK (0) or a negative PG_ERR_* status; it never
 *     exits the process (petgem prints and calls exit(-1),
 *     e.g. petgem/hvfem.py:284-286; here the status is returned instead).
 *     pg_last_error() gives a message for the last failure on this thread.
 *   - Calls are asynchronous on `stream` unless documented as synchronising.
 */
#ifndef PETGEM_GB300_H
#define PETGEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PG_OK = 0,
  PG_ERR_ARG = -1,           /* invalid argument (sizes, order, null pointer) */
  PG_ERR_CUDA = -2,          /* CUDA runtime error, see pg_last_error() */
  PG_ERR_WORKSPACE = -3,     /* workspace missing or too small */
  PG_ERR_UNSUPPORTED = -4,   /* e.g. basis order outside 1..6 */
  PG_ERR_DEGENERATE = -5,    /* element with det(J) == 0 or non-finite geometry */
  PG_ERR_NOT_FOUND = -6,     /* point outside every element */
  PG_ERR_NOT_CONVERGED = -7, /* Krylov solve hit max_it before rtol */
  PG_ERR_BREAKDOWN = -8,     /* Krylov breakdown (zero/denormal Arnoldi norm) */
  PG_ERR_NONFINITE = -9      /* NaN/Inf in a residual or input */
};

/* ABI version of this library (increments on incompatible changes). */
int pg_abi_version(void);
/* Message for the last failing call on the calling thread. */
const char* pg_last_error(void);

/* Measurement helper, no petgem counterpart: FP64 FMA throughput probe
 * (8 independent FMA chains per thread, 256 threads per block).
 * out: f64 [blocks * 256]; pg_fp64_probe_flops gives the flops of one launch. */
int pg_fp64_probe(double* out, int blocks, int iters, void* stream);
int64_t pg_fp64_probe_flops(int blocks, int iters);

/* Copy `bytes` from src to dst with the SMs (16-byte loads and stores; no
 * petgem counterpart: it moves results to the host).  dst may be pinned host
 * memory that the GPU maps (cudaHostAlloc'd memory under unified addressing),
 * so results stream to the host without a copy engine.  blocks: grid size
 * (0: 4 per SM).  src, dst 16-byte aligned. */
int pg_copy_bytes(const void* src, void* dst, int64_t bytes, int blocks, void* stream);

/* ------------------------------------------------------------------------
 * Reference-space integration tables
 * --------------------------------------------------------------------- */

/* Number of doubles in one orientation tuple's table for order p:
 * 12 * nd(nd+1)/2 with nd = p(p+2)(p+3)/2 (6 mass + 6 curl-curl
 * symmetric moment tables, packed upper triangle). */
int64_t pg_table_doubles(int p);

/* Workspace for pg_orientation_tuples. */
size_t pg_tuples_workspace_bytes(int64_t n_elems);

/* Distinct (edge-flag, face-code) orientation tuples of the elements.
 * eo: int8 [T*6] edge flags (0/1), fo: int8 [T*4] face codes (0..5), as
 * produced by petgem/hvfem.py:122 computeElementOrientation.
 * Out: tuple_of_elem int32 [T]; codes int32 [cap min(T, 82944)] tuple codes
 * in ascending order; n_tuples int64 [1] (device).  Deterministic. */
int pg_orientation_tuples(const int8_t* eo, const int8_t* fo, int64_t n_elems,
                          int32_t* tuple_of_elem, int32_t* codes, int64_t* n_tuples,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Tables of integrated products of reference-space shape functions and
 * curls for each tuple (the Gauss sums of petgem/hvfem.py:270-310 with the
 * element geometry factored out).  tables: f64 [n_tuples * pg_table_doubles(p)].
 * Entries below 1e-13 of their moment's largest magnitude (analytically zero
 * moments, e.g. curls of gradient-type edge functions) are stored as 0.0. */
int pg_tuple_tables(const int32_t* codes, int64_t n_tuples, int p, double* tables, void* stream);

/* ------------------------------------------------------------------------
 * Elemental matrices
 * --------------------------------------------------------------------- */

/* Batched sibling of petgem/hvfem.py:223 computeElementalMatrices.
 * Element e has vertices nodes[elemsN[4e+k]] (nodes f64 [*,3]), conductivity
 * sigma[2e] (horizontal), sigma[2e+1] (vertical), orientation tuple
 * tuple_of_elem[e] into `tables`.  Out: M, K f64 [T * nd * nd], row-major per
 * element, scaled by the SIGNED det(J) exactly as the reference.
 * status: int32 [1] device, set to PG_ERR_DEGENERATE if any det(J) is zero
 * or non-finite (left untouched otherwise; may be NULL). */
int pg_elemental_matrices(const double* nodes, const int32_t* elemsN, const double* sigma,
                          const int32_t* tuple_of_elem, const double* tables, int64_t n_elems,
                          int p, double* M, double* K, int32_t* status, void* stream);


/* ------------------------------------------------------------------------
 * Mesh topology, DOF numbering, orientation, PEC boundary (bit-exact)
 * --------------------------------------------------------------------- */

/* Workspace for pg_topology. */
size_t pg_topology_workspace_bytes(int64_t n_elems);

/* Edges and faces of a tetrahedral mesh, numbered exactly as petgem:
 * replaces petgem/mesh.py:18 computeEdges, mesh.py:56 computeFaces and
 * mesh.py:92 computeFacesEdges (with vectors.py:15 deleteDuplicateRows and
 * vectors.py:81 invConnectivity).
 * In: elemsN int32 [T*4] (0-based node ids < n_nodes <= 2^21).
 * Out: elemsE [T*6]; elemsF [T*4]; edgesNodes [cap 6T * 2] (sorted pair);
 * facesN [cap 4T * 3] (vertex order of the first occurrence); facesE
 * [cap 4T * 3]; face_nelem [cap 4T] (elements sharing each face: 1 on the
 * boundary); counts int64 [2] = (nEdges, nFaces); status int32 [1] set to
 * PG_ERR_ARG if a node id is out of range (caller zeroes it). */
int pg_topology(const int32_t* elemsN, int64_t n_elems, int64_t n_nodes, int32_t* elemsE, int32_t* elemsF,
                int32_t* edgesNodes, int32_t* facesN, int32_t* facesE, int32_t* face_nelem, int64_t* counts,
                int32_t* status, void* workspace, size_t workspace_bytes, void* stream);

/* Element-to-DOF map: replaces petgem/hvfem.py:15 computeConnectivityDOFS
 * (its dof_edges/dof_faces/dof_volume are the closed forms p*e+j,
 * nE*p + f*p(p-1) + j, nE*p + nF*p(p-1) + e*p(p-1)(p-2)/2 + j).
 * Out: dofs int32 [T * p(p+2)(p+3)/2]. */
int pg_connectivity_dofs(const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF,
                         int p, int32_t* dofs, void* stream);

/* Edge flags and face codes of every element: replaces
 * petgem/hvfem.py:122 computeElementOrientation.  Out: eo int8 [T*6],
 * fo int8 [T*4]. */
int pg_element_orientation(const int32_t* elemsN, const int32_t* elemsE, const int32_t* edgesNodes,
                           const int32_t* elemsF, const int32_t* facesE, int64_t n_elems, int8_t* eo, int8_t* fo,
                           void* stream);

/* Workspace for pg_boundary_dofs. */
size_t pg_boundary_workspace_bytes(int64_t nE, int64_t nF);

/* PEC (Dirichlet) DOF list in petgem's order: edge DOFs of boundary edges
 * (ascending edge id) then face DOFs of boundary faces (ascending face id).
 * Replaces petgem/mesh.py:149 computeBoundaryFaces, mesh.py:224
 * computeBoundaryEdges, mesh.py:280 computeBoundaries.
 * Out: bnd int32 [cap nE*p + nF*p(p-1)], n_bnd int64 [1]. */
int pg_boundary_dofs(const int32_t* face_nelem, const int32_t* facesE, int64_t nE, int64_t nF, int p, int32_t* bnd,
                     int64_t* n_bnd, void* workspace, size_t workspace_bytes, void* stream);

/* Single-function building blocks (used by the drop-in mesh entry points):
 *  - pg_faces_edges: facesE [nF*3] from elemsF/elemsE, lowest-index owner
 *    element (petgem/mesh.py:92 computeFacesEdges); owner_ws int32 [nF].
 *  - pg_face_counts: elements sharing each face (1 = boundary,
 *    petgem/mesh.py:149 computeBoundaryFaces).
 *  - pg_flag_edges_of_pairs: flags [nE] = 1 for edges whose sorted node pair
 *    appears in pairs [n_pairs*2] (petgem/mesh.py:224 computeBoundaryEdges).
 *  - pg_select_equal: ascending indices i with values[i] == target. */
int pg_faces_edges(const int32_t* elemsF, const int32_t* elemsE, int64_t n_elems, int64_t nF, int32_t* facesE,
                   int32_t* owner_ws, int32_t* status, void* stream);
int pg_face_counts(const int32_t* elemsF, int64_t n_elems, int64_t nF, int32_t* face_nelem, void* stream);
int pg_flag_edges_of_pairs(const int32_t* edgesNodes, int64_t nE, const int32_t* pairs, int64_t n_pairs,
                           int32_t* flags, void* stream);
size_t pg_select_workspace_bytes(int64_t n);
int pg_select_equal(const int32_t* values, int64_t n, int32_t target, int32_t* out, int64_t* count,
                    void* workspace, size_t workspace_bytes, void* stream);

/* Allocation-free pg_select_equal (no counterpart in the reference).  For
 * callers that cannot allocate device memory (their device memory is owned
 * by another allocator, or their request path must not allocate): the
 * scratch is a static device array inside this library, so the call makes no
 * allocation.  Limit: n <= PG_NOALLOC_MAX_N (larger n returns PG_ERR_ARG;
 * use pg_select_equal with a workspace instead).  Every GPU that loads the
 * library keeps the ~2 MB array until exit.  The first call on a device looks
 * up the array's device address with that device current; make that first
 * call before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU (concurrent streams, or several host threads) race and
 * must be serialised by the caller.  The looked-up address is kept for the
 * life of the process; after cudaDeviceReset of a device, do not call this
 * function on that device again. */
#define PG_NOALLOC_MAX_N 262144
int64_t pg_select_equal_noalloc_max_n(void);
int pg_select_equal_noalloc(const int32_t* values, int64_t n, int32_t target, int32_t* out, int64_t* count,
                            void* stream);

/* ------------------------------------------------------------------------
 * CSR pattern and value assembly (replaces petgem/parallel.py:150
 * createParallelMatrix + the Mat.setValues(ADD_VALUES)/assemblyBegin/End
 * loop of petgem/solver.py:182-235)
 * --------------------------------------------------------------------- */

/* Entities with DOFs per element: 6 (p=1), 10 (p=2), 11 (p>=3). */
int pg_pattern_local_entities(int p);

size_t pg_pattern_workspace_bytes(int64_t n_elems, int64_t nE, int64_t nF, int p);

/* Phase 1.  With nl = pg_pattern_local_entities(p), M = T*nl*nl:
 * Out: members int32 [M] (element-entity pair codes e*nl*nl + la*nl + lb,
 * grouped by global entity pair, ascending element inside a group);
 * pair_start int32 [cap M+1]; pair_colstart int32 [cap M]; rowptr int64
 * [N+1] with N = nE*p + nF*p(p-1) + T*p(p-1)(p-2)/2; counts int64 [2] =
 * (n_pairs, nnz).  Columns of every row are sorted ascending, as PETSc AIJ. */
int pg_pattern_build(const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p,
                     int32_t* members, int32_t* pair_start, int32_t* pair_colstart, int64_t* rowptr,
                     int64_t* counts, void* workspace, size_t workspace_bytes, void* stream);

/* Phase 2: column indices col int32 [nnz]. */
int pg_pattern_columns(const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                       int64_t n_pairs, const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE,
                       int64_t nF, int p, const int64_t* rowptr, int32_t* col, void* stream);

/* vals complex128 [nnz] = sum_e (K_e - i omega_mu M_e) from materialised
 * elemental matrices (pg_elemental_matrices), summed per entry in ascending
 * element order (deterministic). */
int pg_assemble_values(const double* M, const double* K, const int32_t* members, const int32_t* pair_start,
                       const int32_t* pair_colstart, int64_t n_pairs, const int32_t* elemsE, const int32_t* elemsF,
                       int64_t n_elems, int64_t nE, int64_t nF, int p, const int64_t* rowptr, double omega_mu,
                       double* vals, void* stream);

/* Per-element geometry coefficients for the fused path: coef f64 [T*12] =
 * (J J^T / det, -omega_mu * det * invJ^T diag(sh,sh,sv) invJ), 6 symmetric
 * entries each.  status int32 [1] <- PG_ERR_DEGENERATE on det(J) == 0. */
int pg_element_coefficients(const double* nodes, const int32_t* elemsN, const double* sigma, int64_t n_elems,
                            double omega_mu, double* coef, int32_t* status, void* stream);

/* The same coefficients as double-float pairs, float [T*24] = (hi, lo) per
 * value, for pg_assemble_fused_ex arithmetic 1. */
int pg_element_coefficients_df(const double* nodes, const int32_t* elemsN, const double* sigma, int64_t n_elems,
                               double omega_mu, float* coef_pairs, int32_t* status, void* stream);

size_t pg_pattern_items_workspace_bytes(int64_t n_pairs, int64_t max_items);

/* Work list of the symmetric fused assembly: for every entity pair (a, b)
 * with a <= b, one item per entry of its upper block (all na*nb entries when
 * a < b, the na(na+1)/2 upper entries when a == b), encoded (pair << 12) |
 * entry, ordered by the pair's member count (stable) so that neighbouring
 * items run equal loop trip counts; pair_partner[g] = index of the
 * transposed pair (b, a).  Synchronises the stream once (item count).
 * Out: pair_partner int32 [n_pairs]; items int64 [max_items >= count];
 * n_items int64 [1]. */
int pg_pattern_items(const int32_t* members, const int32_t* pair_start, int64_t n_pairs, const int32_t* elemsE,
                     const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p, int64_t max_items,
                     int32_t* pair_partner, int64_t* items, int64_t* n_items, void* workspace,
                     size_t workspace_bytes, void* stream);

/* Fused elemental + assembly: vals complex128 [nnz] without materialising
 * elemental matrices.  Each item sums 12 FMAs per member element (element
 * coefficients x orientation-tuple tables) in ascending element order and
 * writes the value to its slot and to the transposed slot, so A comes out
 * exactly symmetric and bitwise reproducible. */
int pg_assemble_fused(const double* coef, const int32_t* tuple_of_elem, const double* tables, const int32_t* members,
                      const int32_t* pair_start, const int32_t* pair_colstart, const int32_t* pair_partner,
                      const int64_t* items, int64_t n_items, int64_t n_pairs, const int32_t* elemsE,
                      const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p, const int64_t* rowptr,
                      double* vals, void* stream);

/* pg_assemble_fused with two options: arithmetic 0 = FP64 (coef, tables
 * are double), 1 = double-float on the FP32 pipes (coef, tables are (hi, lo)
 * float pairs from pg_to_double_float; ~2^-48 relative rounding, output
 * complex128); pec_flags (uint8 [N], from pg_pec_flags, may be NULL) applies
 * zeroRowsColumns(diag=1) while writing, replacing a pg_apply_pec pass. */
int pg_assemble_fused_ex(const void* coef, const int32_t* tuple_of_elem, const void* tables, const int32_t* members,
                         const int32_t* pair_start, const int32_t* pair_colstart, const int32_t* pair_partner,
                         const int64_t* items, int64_t n_items, int64_t n_pairs, const int32_t* elemsE,
                         const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p, const int64_t* rowptr,
                         const uint8_t* pec_flags, int arithmetic, double* vals, void* stream);

/* Assembly records: the mesh-only part of every item of the symmetric work
 * list (pg_pattern_items) resolved once per mesh, in the same order, so the
 * per-model pass (pg_assemble_records) reads one record, the pair's members,
 * the element coefficients and one table entry per member.  A record is
 * pg_assembly_record_bytes(nnz) bytes (16 while nnz < 2^31, else 24): output
 * position, transpose position, first member, meta (member count, local DOF
 * indices, transpose / PEC flags).  pec_flags (uint8 [N] from pg_pec_flags,
 * may be NULL) marks items in PEC rows or columns.  records 16-byte aligned.
 * status int32 [1] <- PG_ERR_UNSUPPORTED when a pair has > 255 members. */
int64_t pg_assembly_record_bytes(int64_t nnz);
int pg_assembly_records(const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                        const int32_t* pair_partner, const int64_t* items, int64_t n_items, const int32_t* elemsE,
                        const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p, const int64_t* rowptr,
                        int64_t nnz, const uint8_t* pec_flags, void* records, int32_t* status, void* stream);

/* Tables of pg_tuple_tables re-laid entry-major, [U][NT][12] in the order of
 * the element coefficients: doubles (arithmetic 0) or (hi, lo) float pairs
 * (arithmetic 1).  out holds U*NT*12 doubles or float pairs. */
int pg_tuple_tables_entry_major(const double* tables, int64_t n_tuples, int p, int arithmetic, void* out,
                                void* stream);

/* A values from records: arithmetic 0 = FP64 (coef from
 * pg_element_coefficients, entry-major double tables), 1 = double-float
 * (coef from pg_element_coefficients_df, entry-major pair tables); output
 * complex128 either way.  apply_pec != 0 writes zeroRowsColumns(diag=1)
 * values for the entries flagged by pg_assembly_records.  coef, tables,
 * records and vals 16-byte aligned.  Same values, bit for bit, as
 * pg_assemble_fused_ex with the same arithmetic. */
int pg_assemble_records(const void* coef, const int32_t* tuple_of_elem, const void* tables_entry_major,
                        const int32_t* members, const void* records, int64_t n_items, int64_t nnz, int p,
                        int arithmetic, int apply_pec, double* vals, void* stream);

/* out_pairs [2n] float = (hi, lo) with hi = fl32(x), lo = fl32(x - hi). */
int pg_to_double_float(const double* in, int64_t n, float* out_pairs, void* stream);

/* flags uint8 [n_dofs] = 1 on the PEC DOFs bnd [n_bnd]. */
int pg_pec_flags(const int32_t* bnd, int64_t n_bnd, int64_t n_dofs, uint8_t* flags, void* stream);

/* b[bnd[i] * nrhs + k] = 0 for every RHS k (b complex128 [N * nrhs]), the
 * RHS half of petgem's PEC (solver.py:565-567). */
int pg_pec_rhs(const int32_t* bnd, int64_t n_bnd, int nrhs, double* b, void* stream);

/* PETSc MatZeroRowsColumns(rows, diag=1) and b[rows] = 0
 * (petgem/solver.py:552-577).  b may be NULL.  flag_ws uint8 [n_dofs]. */
int pg_apply_pec(const int64_t* rowptr, const int32_t* col, double* vals, int64_t n_dofs, const int32_t* bnd,
                 int64_t n_bnd, double* b, uint8_t* flag_ws, void* stream);

/* ------------------------------------------------------------------------
 * Points: location, point-dipole source, receiver interpolation
 * --------------------------------------------------------------------- */

/* First (lowest-index) element containing each point within barycentric
 * tolerance tol, -1 if none: the brute-force find_simplex(tol=1e-12) rule of
 * petgem/preprocessing.py:414-425 and postprocessing.py:532-539.
 * pts f64 [R*3]; elem_out int32 [R]. */
int pg_locate_points(const double* nodes, const int32_t* elemsN, int64_t n_elems, const double* pts, int64_t n_pts,
                     double tol, int32_t* elem_out, void* stream);

/* b[dofs_e] += (scale_re + i scale_im) * (field . N_e(position)) for the
 * element *elem (device int32): the total-field point dipole of
 * petgem/solver.py:247-316 (scale = i omega mu).  position_host and
 * field_host are HOST double[3].  status <- PG_ERR_NOT_FOUND if *elem < 0. */
int pg_source_rhs(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo, const int32_t* dofs,
                  int p, const int32_t* elem, const double* position_host, const double* field_host,
                  double scale_re, double scale_im, double* b, int32_t* status, void* stream);

/* Receiver fields (petgem/postprocessing.py:479 fieldInterpolator):
 * fields complex128 [R*6] = (Ex,Ey,Ez,Hx,Hy,Hz), H = curl E / (i omega_mu);
 * NaN for receivers with elem < 0. */
int pg_gather_fields(const double* x, const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                     const int32_t* dofs, int p, const double* pts, const int32_t* elem, int64_t n_pts,
                     double omega_mu, double* fields, void* stream);

/* ------------------------------------------------------------------------
 * Magnetotelluric plane-wave right-hand side (petgem/solver.py:318-512).
 * The 1-D field u(z) (petgem/mt1d.py) is solved on the host between
 * pg_mt_face_z and pg_mt_rhs.
 * ---------------------------------------------------------------------- */

/* Boundary faces (one element, face_nelem from pg_topology) in ascending face
 * order with their element and local face index: petgem's
 * computeBoundaryFaces + computeBoundaryElements (mesh.py:128-221).
 * bface / belem int32 and blocal int8 hold up to n_faces entries;
 * n_bfaces int64 [1] <- the count. */
size_t pg_boundary_faces_workspace_bytes(int64_t n_faces);
int pg_boundary_faces(const int32_t* elemsF, const int32_t* face_nelem, int64_t n_elems, int64_t n_faces,
                      int32_t* bface, int32_t* belem, int8_t* blocal, int64_t* n_bfaces, void* workspace,
                      size_t workspace_bytes, void* stream);

/* computeFacePlane (mesh.py:324-429): plane int8 [n_bfaces] = bottom 0,
 * left 1, front 2, right 3, back 4, top 5 of the box bbox = {min_x, max_x,
 * min_y, max_y, min_z, max_z} (host array); centroid_z f64 [n_bfaces] = z of
 * the face centroid over the element's local face vertices (solver.py:360).
 * status int32 [1] <- PG_ERR_UNSUPPORTED for a face on no box side. */
int pg_face_planes(const double* nodes, const int32_t* elemsN, const int32_t* facesN, const int32_t* bface,
                   const int32_t* belem, const int8_t* blocal, int64_t n_bfaces, const double* bbox, int8_t* plane,
                   double* centroid_z, int32_t* status, void* stream);

/* z [n_bfaces * n_rule] of the triangle rule points (rule f64 [n_rule * 3] =
 * s, t, weight on the triangle (0,0),(1,0),(0,1)) mapped onto each boundary
 * face (transform2Dto3DInReferenceElement + getRealFromReference). */
int pg_mt_face_z(const double* nodes, const int32_t* elemsN, const int32_t* belem, const int8_t* blocal,
                 int64_t n_bfaces, const double* rule, int n_rule, double* z, void* stream);

/* Per-DOF ordered scatter plan of the boundary contributions (face f, local
 * DOF l): order int32 [n_bfaces * nd], seg_start int32 [n_bfaces * nd + 1],
 * seg_dof int32 [n_bfaces * nd], n_seg int64 [1]. */
size_t pg_mt_plan_workspace_bytes(int64_t n_bfaces, int p);
int pg_mt_plan(const int32_t* dofs, const int32_t* belem, int64_t n_bfaces, int p, int64_t n_dofs, int32_t* order,
               int32_t* seg_start, int32_t* seg_dof, int64_t* n_seg, void* workspace, size_t workspace_bytes,
               void* stream);

/* b[:, rhs] += (scale_re + i scale_im) sum_k w_k |det J_2D| ((n x N_l) x n) .
 * e_k with e_k = u[f, k] times the direction of getNeumannBCface(plane,
 * polarization) (1 = x, 2 = y); u complex128 [n_bfaces * n_rule]; b complex128
 * [N * nrhs] (RHS fastest).  Faces are added per DOF in ascending order.
 * Workspace: pg_mt_rhs_workspace_bytes(n_bfaces, p). */
size_t pg_mt_rhs_workspace_bytes(int64_t n_bfaces, int p);
int pg_mt_rhs(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo, int p,
              const int32_t* belem, const int8_t* blocal, const int8_t* plane, int64_t n_bfaces, const double* rule,
              int n_rule, const double* u, int polarization, double scale_re, double scale_im, const int32_t* order,
              const int32_t* seg_start, const int32_t* seg_dof, int64_t n_seg, double* b, int nrhs, int rhs,
              void* workspace, size_t workspace_bytes, void* stream);

/* Nodal E and H for visualisation (petgem/postprocessing.py:173-260): each
 * element evaluates E and curl E at its vertices pulled 0.01 % towards the
 * centroid; a node gets the mean over its elements (ascending element order),
 * H = curl E / (i omega mu).  fields complex128 [n_nodes, 6] (Ex..Hz); a node
 * in no element gives NaN, as petgem's 0/0 does.
 * Workspace: pg_node_fields_workspace_bytes(n_elems, n_nodes). */
size_t pg_node_fields_workspace_bytes(int64_t n_elems, int64_t n_nodes);
int pg_node_fields(const double* x, const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                   const int32_t* dofs, int p, int64_t n_elems, int64_t n_nodes, double omega_mu, double* fields,
                   void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Adjoint gradient of a receiver misfit (no petgem counterpart; built from
 * the elemental mass matrices of hvfem.py:223-316 and the interpolation of
 * postprocessing.py:566-614).
 * ---------------------------------------------------------------------- */

/* Transpose of the E part of pg_gather_fields: b[dofs_e(r)] +=
 * sum_c N^c_j(xi_r) weights[r][c] (weights complex128 [n_pts, 3]; receivers
 * with elem < 0 are skipped).  Receivers are added in order (deterministic).
 * Workspace: pg_receiver_adjoint_workspace_bytes(p, n_pts). */
size_t pg_receiver_adjoint_workspace_bytes(int p, int64_t n_pts);
int pg_receiver_adjoint(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                        const int32_t* dofs, int p, const double* pts, const int32_t* elem, int64_t n_pts,
                        const double* weights, double* b, void* workspace, size_t workspace_bytes, void* stream);

/* out[e] (complex128 [T]) = y_e^T (-omega mu M_e) x_e, with x_e = x[dofs_e],
 * y_e = y[dofs_e] and the mass coefficients of pg_element_coefficients
 * (coef[e][6..11]) against the table-major tables of pg_tuple_tables.  The
 * gradient of phi = sum |E_rx - d|^2 with respect to m_e = log10 sigma_e is
 * 2 ln(10) Im(out[e]) for x = u (forward field) and y = lambda (adjoint
 * field, A lambda = G^T conj(E_rx - d) with PEC rows zeroed). */
int pg_element_mass_bilinear(const double* coef, const int32_t* tuple_of_elem, const double* tables,
                             const int32_t* dofs, const double* x, const double* y, int64_t n_elems, int p,
                             double* out, void* stream);

/* ------------------------------------------------------------------------
 * Krylov (replaces the PETSc KSP of petgem/solver.py:584-594)
 * --------------------------------------------------------------------- */

/* y = A x, CSR with int64 row pointers; nrhs in {1,2,4,8,16,32}, vectors
 * stored row-major with the RHS index fastest. */
int pg_spmv_z(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n_rows, const double* x,
              double* y, int nrhs, void* stream);
int pg_spmv_c(const int64_t* rowptr, const int32_t* col, const float* vals, int64_t n_rows, const float* x, float* y,
              int nrhs, void* stream);

typedef struct pg_gmres_opts {
  int restart;    /* GMRES(m), 1..64 (PETSc default 30) */
  int max_it;     /* cap on Arnoldi steps */
  double rtol;    /* stop when ||b - A x|| <= rtol ||b|| (true residual, FP64) */
  int precision;  /* 0: complex128 Arnoldi; 1: complex64 Arnoldi + complex128 refinement */
  int reorth;     /* 1: classical Gram-Schmidt applied twice (CGS2) */
  /* entity block-Jacobi (block_p 1..6; 0 = diagonal Jacobi), PETSc -pc_type
   * bjacobi with one block per edge / face / element: the matrix is
   * pg_pattern_build's pattern for a mesh with block_edges edges, block_faces
   * faces and block_volumes elements at order block_p; GMRES runs on A M^-1
   * (right preconditioning, so the Arnoldi residual is the true one) with
   * M^-1 = A_aa^-1 per entity block, from A_aa = L D L^T (blocks above 12
   * DOFs stay diagonal). */
  int block_p;
  int64_t block_edges, block_faces, block_volumes;
  /* gradient correction (diagonal Jacobi, block_p 0; grad_rowptr NULL =
   * off), as in pg_cocg_opts: GMRES runs on A B with
   * B = D^-1 + G diag(G^T A G)^-1 G^T, G the map of pg_gradient_map (with
   * or without its vector P1 columns; right preconditioning; in precision
   * 1 the correction of the Arnoldi steps runs on the complex64 basis). */
  int64_t grad_cols;
  const int64_t* grad_rowptr;
  const int32_t* grad_col;
  const double* grad_val;
  const int64_t* gradt_rowptr;
  const int32_t* gradt_row;
  const double* gradt_val;
} pg_gmres_opts;

typedef struct pg_gmres_result {
  int64_t iterations; /* Arnoldi steps (max over RHS) */
  int64_t restarts;   /* cycles (= FP64 refinement steps in mixed precision) */
  double relres;      /* max over RHS of the final true relative residual */
  int status;
} pg_gmres_result;

void pg_gmres_default_opts(pg_gmres_opts* opts);
size_t pg_gmres_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_gmres_opts* opts);

/* Right-Jacobi-preconditioned restarted GMRES on A x = b with nrhs RHS
 * (b, x: complex128 [n*nrhs]; x holds the initial guess).  Synchronises the
 * stream once per restart.  result and relres_per_rhs are HOST pointers
 * (may be NULL).  Returns PG_OK, PG_ERR_NOT_CONVERGED (x holds the last
 * iterate), or an error. */
int pg_gmres(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz, const double* b,
             double* x, int nrhs, const pg_gmres_opts* opts, pg_gmres_result* result, double* relres_per_rhs,
             void* workspace, size_t workspace_bytes, void* stream);

/* COCG (conjugate orthogonal CG) for the complex-symmetric A with symmetric
 * Jacobi scaling; an additional KSP type beside GMRES for the same system
 * (petgem configures PETSc's KSP from the options file, solver.py:588).
 * precision 0: complex128 throughout; 1: complex64 matrix and SpMV with a
 * complex128 recurrence and FP64 reliable updates; 2 ("df64"): matrix and
 * recurrence in double-float (FP32 hi + lo pairs, ~48-bit mantissa) computed
 * on the FP32 pipes, FP64 reliable updates; 3 ("ir32"): FP64 iterative
 * refinement of the true residual around complex64 inner COCG solves (matrix,
 * vectors and products all complex64), each restarted from the current FP64
 * residual and run until its residual estimate has dropped by inner_rtol.
 * The true FP64 residual is checked every check_every iterations (doubling up
 * to 400; for precision 3 at every refinement step) and decides convergence. */
typedef struct pg_cocg_opts {
  int max_it;
  double rtol;
  int precision;
  int check_every;
  /* entity block-Jacobi (block_p 1..6; 0 = diagonal Jacobi): the matrix is
   * pg_pattern_build's pattern for a mesh with block_edges edges, block_faces
   * faces and block_volumes elements at order block_p (DOFs numbered entity by
   * entity); each entity's diagonal block is factored L D L^T and the solver
   * runs on S A S^T, S = D^-1/2 L^-1 (blocks above 12 DOFs stay diagonal).
   * Not used by pg_cocg_multifreq; pg_cocg_segments takes block_p from here
   * and each system's entity counts from its seg_entities argument. */
  int block_p;
  int64_t block_edges, block_faces, block_volumes;
  /* precision 3: relative residual reduction each complex64 inner solve aims
   * for (0 or outside (0, 1), the default: 1e-2, or 1e-4 with the gradient
   * correction); an inner solve stops after at most 8x the inner iterations
   * of the first refinement step (at least 1,000) */
  double inner_rtol;
  /* gradient correction (pg_cocg: precision 0, 2 or 3; pg_gmres: 0 or 1;
   * diagonal Jacobi, block_p 0; grad_rowptr NULL = off): G, n rows by grad_cols columns, and
   * its transpose from pg_gradient_map.  The preconditioner becomes
   *   B = D^-1 + G diag(G^T A G)^-1 G^T
   * (D = diag A; diag(G^T A G) is formed from A when the solve starts), which
   * adds a Jacobi step on the gradient fields that the edge Jacobi step
   * cannot reduce, and (when the map carries its vector P1 columns) one on
   * the vector-nodal fields; no petgem counterpart (petgem/solver.py:584-594
   * leaves the preconditioner to PETSc). */
  int64_t grad_cols;
  const int64_t* grad_rowptr;
  const int32_t* grad_col;
  const double* grad_val;
  const int64_t* gradt_rowptr;
  const int32_t* gradt_row;
  const double* gradt_val;
} pg_cocg_opts;

/* Discrete gradient for the COCG gradient correction (no petgem counterpart):
 * G[r, phi] = coefficient of grad(phi) on H(curl) DOF r, phi running over
 * the order-p H1 functions (p 1..3): the mesh's vertices, then (p >= 2) one
 * quadratic bubble per edge, then (p = 3) a cubic bubble per edge and one
 * per face.  Built from the mesh maps of pg_topology / pg_connectivity_dofs /
 * pg_orientation_tuples (dofs int32 [n_elems * nd], tuple_of_elem and codes
 * as pg_tuple_tables takes them) by exact L2 projection on the reference
 * element; rows follow the DOF numbering (edges, faces, volumes), entries of
 * a row are written by one owner element.  Columns with an entry in a row
 * flagged in pec_flags (uint8 [n], may be NULL) are dropped, zeros are not
 * stored.  G: g_rowptr int64 [n + 1], g_col int32, g_val f64; its transpose:
 * gt_rowptr int64 [n_cols + 1], gt_row int32 (ascending in each row), gt_val
 * f64; the entry arrays hold at most max_entries (pg_gradient_map_sizes) and
 * g_rowptr[n] = gt_rowptr[n_cols] entries are stored.  Deterministic;
 * synchronises (PG_ERR_UNSUPPORTED if a coefficient falls outside its row's
 * entity structure, i.e. the basis and the map disagree).  vector_p1 != 0
 * (p 2..3; nodes f64 [n_nodes * 3] needed) appends the vector P1 fields
 * lambda_v e_d, 3 columns per vertex (column n_grad + 3 v + d): the
 * auxiliary space of the vector-nodal correction, whose Jacobi step the
 * solvers apply together with the gradient's. */
int pg_gradient_map_sizes(int64_t n_nodes, int64_t n_edges, int64_t n_faces, int64_t n_elems, int p, int vector_p1,
                          int64_t* n_cols /* host */, int64_t* max_entries /* host */);
size_t pg_gradient_map_workspace_bytes(int64_t n_nodes, int64_t n_edges, int64_t n_faces, int64_t n_elems,
                                       int64_t n_tuples, int p, int vector_p1);
int pg_gradient_map(const double* nodes, const int32_t* elemsN, const int32_t* elemsE, const int32_t* elemsF,
                    const int32_t* dofs, const int32_t* tuple_of_elem, const int32_t* codes, int64_t n_tuples,
                    int64_t n_elems, int64_t n_nodes, int64_t n_edges, int64_t n_faces, int p, int vector_p1,
                    const uint8_t* pec_flags, int64_t* g_rowptr, int32_t* g_col, double* g_val, int64_t* gt_rowptr,
                    int32_t* gt_row, double* gt_val, void* workspace, size_t workspace_bytes, void* stream);

void pg_cocg_default_opts(pg_cocg_opts* opts);
size_t pg_cocg_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* opts);
/* Same conventions as pg_gmres (result.restarts = number of residual checks). */
int pg_cocg(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz, const double* b,
            double* x, int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result, double* relres_per_rhs,
            void* workspace, size_t workspace_bytes, void* stream);

/* Several frequencies in one double-float COCG (precision must be 2): column
 * j solves (Re A0 + i s_j Im A0) x_j = b_j, where vals = A0 = K - i omega_0 mu
 * M is assembled (PEC applied) at one frequency omega_0 and s_j = omega_j /
 * omega_0 > 0 (col_scale: host array [nrhs]).  The matrix is read once per
 * iteration for all columns; each column has its own Jacobi scaling.  b, x
 * complex128 [n * nrhs] (RHS fastest).  The gradient correction of
 * pg_cocg_opts applies, with each column's own diagonal
 * diag(G^T A_j G) = Re d + i s_j Im d, d = diag(G^T A0 G); block_p is
 * ignored.  Other arguments as pg_cocg. */
size_t pg_cocg_multifreq_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* opts /* may be NULL */);
int pg_cocg_multifreq(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                      const double* b, double* x, int nrhs, const double* col_scale, const pg_cocg_opts* opts,
                      pg_gmres_result* result, double* relres_per_rhs, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Several independent systems (meshes of different sizes, or one mesh at
 * several frequencies) in one double-float COCG (precision must be 2).  The
 * systems are stored as one block-diagonal CSR matrix: system j owns rows
 * seg_rows[j] .. seg_rows[j+1]-1 (host array [n_seg + 1], seg_rows[0] = 0,
 * seg_rows[n_seg] = n) and references only its own columns (checked).  Each
 * system keeps its own COCG scalars and convergence test, so its solution is
 * the one it would reach alone; every launch serves all systems.  With
 * opts->block_p > 0 each system gets entity block-Jacobi scaling and
 * seg_entities (host [3 * n_seg]) gives its (edges, faces, elements);
 * otherwise seg_entities may be NULL.  The gradient correction of
 * pg_cocg_opts applies with diagonal scaling; G is then block-diagonal over
 * the systems (system j's map with its rows shifted by seg_rows[j] and its
 * columns by the columns of the systems before it).  b, x complex128 [n * nrhs] (RHS
 * fastest), nrhs right-hand sides per system.  relres and its (host,
 * [n_seg * nrhs], system-major, either may be NULL) receive each system's
 * final true relative residual and iteration count; result.iterations is the
 * largest count.  Replaces, for a batch of models, one KSPSolve per model
 * (petgem/solver.py:584-594). */
size_t pg_cocg_segments_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const int64_t* seg_rows, int n_seg,
                                        const int64_t* seg_entities, const pg_cocg_opts* opts);
int pg_cocg_segments(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                     const int64_t* seg_rows, int n_seg, const int64_t* seg_entities, const double* b, double* x,
                     int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result, double* relres, int64_t* its,
                     void* workspace, size_t workspace_bytes, void* stream);
/* Host-only inspection helper, no petgem counterpart: the block map
 * pg_cocg_segments launches with (host arrays).  blk[j] .. blk[j+1]-1 are the
 * blocks of system j: with active == NULL the first map (blocks in
 * proportion to rows, at least one each); else the map after a residual
 * check with active[j] != 0 for the systems still iterating (same total, one
 * block per converged system). */
int pg_segments_block_map(const int64_t* seg_rows, int n_seg, int nrhs, const unsigned char* active, int* blk);


#ifdef __cplusplus
}
#endif
#endif /* PETGEM_GB300_H */
