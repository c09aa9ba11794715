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
 * element geometry factored out).  tables: f64 [n_tuples * pg_table_doubles(p)]. */
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

#ifdef __cplusplus
}
#endif
#endif /* PETGEM_GB300_H */
