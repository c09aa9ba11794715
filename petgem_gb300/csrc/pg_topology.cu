// Mesh topology, DOF numbering, element orientation and PEC boundary DOFs.
//
// Bit-exact restatement of petgem's numbering:
//  * edge id = lexicographic rank of the sorted vertex pair
//    (petgem/mesh.py:18-53 via vectors.py:15-64 np.unique on rows);
//  * face id = rank of the sorted vertex triple; facesN keeps the vertex
//    order of the first occurrence (mesh.py:56-89);
//  * facesE = the face's edges in the local order of the lowest-index
//    element that contains it (mesh.py:92-125, vectors.py:81-132);
//  * DOFs: edge block, face block, volume block (hvfem.py:15-98);
//  * boundary faces have one owner; boundary edges lie on boundary faces;
//    PEC DOFs = edge DOFs (ascending edge) then face DOFs (ascending face)
//    (mesh.py:149-321).
// Ranks come from a stable radix sort of integer keys, so every id, and the
// first-occurrence choice, is independent of thread scheduling.
#include "pg_common.cuh"
#include "pg_sort.cuh"

namespace {

__constant__ int kEV[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
__constant__ int kFV[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
__constant__ int kFE[4][3] = {{0, 1, 2}, {0, 4, 3}, {1, 5, 4}, {2, 5, 3}};

#define GRID_STRIDE(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_edge_keys(const int32_t* elemsN, int64_t T, int64_t nn, uint64_t* keys, int32_t* vals,
                            int32_t* status) {
  GRID_STRIDE(i, 6 * T) {
    const int64_t e = i / 6;
    const int l = (int)(i % 6);
    int64_t a = elemsN[4 * e + kEV[l][0]], b = elemsN[4 * e + kEV[l][1]];
    if (a < 0 || b < 0 || a >= nn || b >= nn) {
      *status = PG_ERR_ARG;
      a = 0;
      b = 0;
    }
    const uint64_t lo = (uint64_t)(a < b ? a : b), hi = (uint64_t)(a < b ? b : a);
    keys[i] = lo * (uint64_t)nn + hi;
    vals[i] = (int32_t)i;
  }
}

__global__ void k_face_keys(const int32_t* elemsN, int64_t T, int64_t nn, uint64_t* keys, int32_t* vals,
                            int32_t* status) {
  GRID_STRIDE(i, 4 * T) {
    const int64_t e = i / 4;
    const int l = (int)(i % 4);
    int64_t v[3];
    for (int k = 0; k < 3; ++k) {
      v[k] = elemsN[4 * e + kFV[l][k]];
      if (v[k] < 0 || v[k] >= nn) {
        *status = PG_ERR_ARG;
        v[k] = 0;
      }
    }
    // sort the triple
    if (v[0] > v[1]) { int64_t t = v[0]; v[0] = v[1]; v[1] = t; }
    if (v[1] > v[2]) { int64_t t = v[1]; v[1] = v[2]; v[2] = t; }
    if (v[0] > v[1]) { int64_t t = v[0]; v[0] = v[1]; v[1] = t; }
    keys[i] = ((uint64_t)v[0] * (uint64_t)nn + (uint64_t)v[1]) * (uint64_t)nn + (uint64_t)v[2];
    vals[i] = (int32_t)i;
  }
}

__global__ void k_group_flags(const uint64_t* keys, int64_t n, int32_t* flags) {
  GRID_STRIDE(i, n) flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_edge_assign(const uint64_t* keys, const int32_t* vals, const int32_t* excl, int64_t n, int64_t nn,
                              int32_t* elemsE, int32_t* edgesNodes) {
  GRID_STRIDE(i, n) {
    const int flag = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
    const int32_t id = excl[i] + flag - 1;
    elemsE[vals[i]] = id;
    if (flag) {
      edgesNodes[2 * (int64_t)id] = (int32_t)(keys[i] / (uint64_t)nn);
      edgesNodes[2 * (int64_t)id + 1] = (int32_t)(keys[i] % (uint64_t)nn);
    }
  }
}

__global__ void k_face_assign(const uint64_t* keys, const int32_t* vals, const int32_t* excl, int64_t n,
                              const int32_t* elemsN, const int32_t* elemsE, int32_t* elemsF, int32_t* facesN,
                              int32_t* facesE, int32_t* face_nelem) {
  GRID_STRIDE(i, n) {
    const int flag = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
    const int32_t id = excl[i] + flag - 1;
    const int32_t v = vals[i];
    elemsF[v] = id;
    atomicAdd(&face_nelem[id], 1);
    if (flag) {  // first occurrence = lowest (element, local face) index
      const int64_t e = v / 4;
      const int l = v % 4;
      for (int k = 0; k < 3; ++k) {
        facesN[3 * (int64_t)id + k] = elemsN[4 * e + kFV[l][k]];
        facesE[3 * (int64_t)id + k] = elemsE[6 * e + kFE[l][k]];
      }
    }
  }
}

__global__ void k_zero32(int32_t* a, int64_t n) { GRID_STRIDE(i, n) a[i] = 0; }

__global__ void k_store_count(const int32_t* src, int64_t* dst) { *dst = *src; }

__global__ void k_dofs(const int32_t* elemsE, const int32_t* elemsF, int64_t T, int64_t nE, int64_t nF, int p,
                       int32_t* dofs) {
  const int de = p, df = p * (p - 1), dv = p * (p - 1) * (p - 2) / 2;
  const int nd = 6 * de + 4 * df + dv;
  GRID_STRIDE(i, T * nd) {
    const int64_t e = i / nd;
    const int m = (int)(i % nd);
    int64_t d;
    if (m < 6 * de) {
      d = (int64_t)de * elemsE[6 * e + m / de] + m % de;
    } else if (m < 6 * de + 4 * df) {
      const int q = m - 6 * de;
      d = nE * de + (int64_t)df * elemsF[4 * e + q / df] + q % df;
    } else {
      d = nE * de + nF * df + e * dv + (m - 6 * de - 4 * df);
    }
    dofs[i] = (int32_t)d;
  }
}

__global__ void k_orientation(const int32_t* elemsN, const int32_t* elemsE, const int32_t* edgesNodes,
                              const int32_t* elemsF, const int32_t* facesE, int64_t T, int8_t* eo, int8_t* fo) {
  GRID_STRIDE(e, T) {
    // edges (hvfem.py:143-177): flag 1 iff the local pair is the reverse of the sorted global pair
    for (int i = 0; i < 6; ++i) {
      const int32_t g = elemsE[6 * e + i];
      const int32_t a = elemsN[4 * e + kEV[i][0]], b = elemsN[4 * e + kEV[i][1]];
      eo[6 * e + i] = (a == edgesNodes[2 * (int64_t)g + 1] && b == edgesNodes[2 * (int64_t)g]) ? 1 : 0;
    }
    // faces (hvfem.py:179-215): positions k1, k2 of local edges 0, 1 of the face in facesE
    for (int i = 0; i < 4; ++i) {
      const int32_t f = elemsF[4 * e + i];
      const int32_t e0 = elemsE[6 * e + kFE[i][0]], e1 = elemsE[6 * e + kFE[i][1]];
      int k1 = 0, k2 = 0;
      for (int k = 0; k < 3; ++k) {
        const int32_t g = facesE[3 * (int64_t)f + k];
        if (e0 == g) k1 = k + 1;
        if (e1 == g) k2 = k + 1;
      }
      const int sel = k1 * 10 + k2;
      int code = 0;
      if (sel == 12) code = 0;
      else if (sel == 31) code = 1;
      else if (sel == 23) code = 2;
      else if (sel == 32) code = 3;
      else if (sel == 13) code = 4;
      else if (sel == 21) code = 5;
      fo[4 * e + i] = (int8_t)code;
    }
  }
}

__global__ void k_boundary_flags(const int32_t* face_nelem, const int32_t* facesE, int64_t nF, int32_t* eflag,
                                 int32_t* fflag) {
  GRID_STRIDE(f, nF) {
    const int b = face_nelem[f] == 1;
    fflag[f] = b;
    if (b)
      for (int k = 0; k < 3; ++k) eflag[facesE[3 * f + k]] = 1;
  }
}

__global__ void k_boundary_edges(const int32_t* eflag_pos, const int32_t* face_nelem, const int32_t* facesE,
                                 int64_t nF, int64_t nE, int p, int32_t* eflag, int32_t* bnd) {
  // eflag still holds flags; eflag_pos the exclusive scan
  GRID_STRIDE(e, nE) {
    if (eflag[e])
      for (int j = 0; j < p; ++j) bnd[(int64_t)eflag_pos[e] * p + j] = (int32_t)((int64_t)p * e + j);
  }
}

__global__ void k_boundary_faces(const int32_t* fflag, const int32_t* fpos, const int32_t* nbe, int64_t nF,
                                 int64_t nE, int p, int32_t* bnd) {
  const int df = p * (p - 1);
  const int64_t base = (int64_t)(*nbe) * p;
  GRID_STRIDE(f, nF) {
    if (fflag[f])
      for (int j = 0; j < df; ++j) bnd[base + (int64_t)fpos[f] * df + j] = (int32_t)(nE * p + f * df + j);
  }
}

__global__ void k_boundary_count(const int32_t* nbe, const int32_t* nbf, int p, int64_t* n_bnd) {
  *n_bnd = (int64_t)(*nbe) * p + (int64_t)(*nbf) * p * (p - 1);
}

}  // namespace

extern "C" size_t pg_topology_workspace_bytes(int64_t n_elems) {
  const int64_t n = 6 * n_elems;
  return pg_align256(sizeof(uint64_t) * n) + pg_align256(sizeof(int32_t) * n) * 2 + pg::sort_workspace_bytes(n) +
         pg::scan_workspace_bytes(n) + 1024;
}

extern "C" int pg_topology(const int32_t* elemsN, int64_t n_elems, int64_t n_nodes, int32_t* elemsE,
                           int32_t* elemsF, int32_t* edgesNodes, int32_t* facesN, int32_t* facesE,
                           int32_t* face_nelem, int64_t* counts, int32_t* status, void* workspace,
                           size_t workspace_bytes, void* stream) {
  if (n_elems < 1 || n_nodes < 4 || !elemsN || !elemsE || !elemsF || !edgesNodes || !facesN || !facesE ||
      !face_nelem || !counts || !status) {
    pg_set_error("pg_topology: bad argument");
    return PG_ERR_ARG;
  }
  if (n_nodes > (1 << 21)) {
    pg_set_error("pg_topology: more than 2^21 nodes is not supported (63-bit face keys)");
    return PG_ERR_UNSUPPORTED;
  }
  if (6 * n_elems >= (1ll << 31)) {
    pg_set_error("pg_topology: too many elements");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_topology_workspace_bytes(n_elems)) {
    pg_set_error("pg_topology: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  const int64_t n6 = 6 * n_elems, n4 = 4 * n_elems;
  PgArena ar(workspace, workspace_bytes);
  uint64_t* keys = ar.take<uint64_t>(n6);
  int32_t* vals = ar.take<int32_t>(n6);
  int32_t* ids = ar.take<int32_t>(n6);
  const size_t sort_b = pg::sort_workspace_bytes(n6);
  void* sort_ws = ar.take<char>(sort_b);
  const size_t scan_b = pg::scan_workspace_bytes(n6);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(4);
  if (!keys || !vals || !ids || !sort_ws || !scan_ws || !tot) return PG_ERR_WORKSPACE;
  const unsigned g6 = pg_blocks(n6, 256), g4 = pg_blocks(n4, 256);
  int st;

  // ---- edges
  k_edge_keys<<<g6, 256, 0, s>>>(elemsN, n_elems, n_nodes, keys, vals, status);
  st = pg::sort_pairs(keys, vals, n6, pg::bits_for((uint64_t)n_nodes * n_nodes - 1), sort_ws, sort_b, s);
  if (st) { pg_set_error("pg_topology: edge sort failed"); return st; }
  k_group_flags<<<g6, 256, 0, s>>>(keys, n6, ids);
  st = pg::scan_exclusive_i32(ids, ids, n6, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_edge_assign<<<g6, 256, 0, s>>>(keys, vals, ids, n6, n_nodes, elemsE, edgesNodes);
  k_store_count<<<1, 1, 0, s>>>(tot, counts);

  // ---- faces
  k_face_keys<<<g4, 256, 0, s>>>(elemsN, n_elems, n_nodes, keys, vals, status);
  const uint64_t nn = (uint64_t)n_nodes;
  st = pg::sort_pairs(keys, vals, n4, pg::bits_for(nn * nn * nn - 1), sort_ws, sort_b, s);
  if (st) { pg_set_error("pg_topology: face sort failed"); return st; }
  k_group_flags<<<g4, 256, 0, s>>>(keys, n4, ids);
  st = pg::scan_exclusive_i32(ids, ids, n4, tot + 1, scan_ws, scan_b, s);
  if (st) return st;
  k_zero32<<<g4, 256, 0, s>>>(face_nelem, n4);
  k_face_assign<<<g4, 256, 0, s>>>(keys, vals, ids, n4, elemsN, elemsE, elemsF, facesN, facesE, face_nelem);
  k_store_count<<<1, 1, 0, s>>>(tot + 1, counts + 1);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_connectivity_dofs(const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE,
                                    int64_t nF, int p, int32_t* dofs, void* stream) {
  if (p < 1 || p > 6) {
    pg_set_error("pg_connectivity_dofs: order must be 1..6");
    return PG_ERR_UNSUPPORTED;
  }
  const int64_t total = nE * p + nF * p * (p - 1) + n_elems * (p * (p - 1) * (p - 2) / 2);
  if (n_elems < 1 || nE < 1 || nF < 1 || !elemsE || !elemsF || !dofs || total >= (1ll << 31)) {
    pg_set_error("pg_connectivity_dofs: bad argument");
    return PG_ERR_ARG;
  }
  const int64_t n = n_elems * pg_nd_elem(p);
  k_dofs<<<pg_blocks(n, 256), 256, 0, pg_stream(stream)>>>(elemsE, elemsF, n_elems, nE, nF, p, dofs);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_element_orientation(const int32_t* elemsN, const int32_t* elemsE, const int32_t* edgesNodes,
                                      const int32_t* elemsF, const int32_t* facesE, int64_t n_elems, int8_t* eo,
                                      int8_t* fo, void* stream) {
  if (n_elems < 1 || !elemsN || !elemsE || !edgesNodes || !elemsF || !facesE || !eo || !fo) {
    pg_set_error("pg_element_orientation: bad argument");
    return PG_ERR_ARG;
  }
  k_orientation<<<pg_blocks(n_elems, 256), 256, 0, pg_stream(stream)>>>(elemsN, elemsE, edgesNodes, elemsF, facesE,
                                                                        n_elems, eo, fo);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" size_t pg_boundary_workspace_bytes(int64_t nE, int64_t nF) {
  return pg_align256(sizeof(int32_t) * nE) * 2 + pg_align256(sizeof(int32_t) * nF) * 2 +
         pg::scan_workspace_bytes(nE > nF ? nE : nF) + 1024;
}

extern "C" int pg_boundary_dofs(const int32_t* face_nelem, const int32_t* facesE, int64_t nE, int64_t nF, int p,
                                int32_t* bnd, int64_t* n_bnd, void* workspace, size_t workspace_bytes,
                                void* stream) {
  if (p < 1 || p > 6 || nE < 1 || nF < 1 || !face_nelem || !facesE || !bnd || !n_bnd) {
    pg_set_error("pg_boundary_dofs: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_boundary_workspace_bytes(nE, nF)) {
    pg_set_error("pg_boundary_dofs: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  PgArena ar(workspace, workspace_bytes);
  int32_t* eflag = ar.take<int32_t>(nE);
  int32_t* epos = ar.take<int32_t>(nE);
  int32_t* fflag = ar.take<int32_t>(nF);
  int32_t* fpos = ar.take<int32_t>(nF);
  const size_t scan_b = pg::scan_workspace_bytes(nE > nF ? nE : nF);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(4);
  if (!eflag || !epos || !fflag || !fpos || !scan_ws || !tot) return PG_ERR_WORKSPACE;
  k_zero32<<<pg_blocks(nE, 256), 256, 0, s>>>(eflag, nE);
  k_boundary_flags<<<pg_blocks(nF, 256), 256, 0, s>>>(face_nelem, facesE, nF, eflag, fflag);
  int st = pg::scan_exclusive_i32(eflag, epos, nE, tot, scan_ws, scan_b, s);
  if (st) return st;
  st = pg::scan_exclusive_i32(fflag, fpos, nF, tot + 1, scan_ws, scan_b, s);
  if (st) return st;
  k_boundary_edges<<<pg_blocks(nE, 256), 256, 0, s>>>(epos, face_nelem, facesE, nF, nE, p, eflag, bnd);
  if (p >= 2) k_boundary_faces<<<pg_blocks(nF, 256), 256, 0, s>>>(fflag, fpos, tot, nF, nE, p, bnd);
  k_boundary_count<<<1, 1, 0, s>>>(tot, tot + 1, p, n_bnd);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

// ---------------------------------------------------------------------------
// Small building blocks behind the single-function mesh entry points.
namespace {

__global__ void k_owner_init(int32_t* owner, int64_t n) { GRID_STRIDE(i, n) owner[i] = 0x7fffffff; }

__global__ void k_owner_min(const int32_t* elemsF, int64_t T, int64_t nF, int32_t* owner, int32_t* status) {
  GRID_STRIDE(i, 4 * T) {
    const int32_t f = elemsF[i];
    if (f < 0 || f >= nF) { *status = PG_ERR_ARG; continue; }
    atomicMin(&owner[f], (int32_t)i);   // i = 4 e + l: lowest element, then lowest local face
  }
}

__global__ void k_faces_edges(const int32_t* owner, const int32_t* elemsE, int64_t nF, int32_t* facesE) {
  GRID_STRIDE(f, nF) {
    const int32_t v = owner[f];
    if (v == 0x7fffffff) continue;
    const int64_t e = v / 4;
    const int l = v % 4;
    for (int k = 0; k < 3; ++k) facesE[3 * f + k] = elemsE[6 * e + kFE[l][k]];
  }
}

__global__ void k_face_counts(const int32_t* elemsF, int64_t T, int64_t nF, int32_t* cnt) {
  GRID_STRIDE(i, 4 * T) {
    const int32_t f = elemsF[i];
    if (f >= 0 && f < nF) atomicAdd(&cnt[f], 1);
  }
}

// pairs (sorted node pairs) -> flag[edge id] = 1 by binary search in the
// lexicographically sorted edgesNodes table
__global__ void k_flag_pairs(const int32_t* edgesNodes, int64_t nE, const int32_t* pairs, int64_t npairs,
                             int32_t* flag) {
  GRID_STRIDE(i, npairs) {
    const int64_t a = pairs[2 * i], b = pairs[2 * i + 1];
    int64_t lo = 0, hi = nE - 1;
    while (lo <= hi) {
      const int64_t mid = (lo + hi) >> 1;
      const int64_t ma = edgesNodes[2 * mid], mb = edgesNodes[2 * mid + 1];
      if (ma == a && mb == b) { flag[mid] = 1; break; }
      if (ma < a || (ma == a && mb < b)) lo = mid + 1; else hi = mid - 1;
    }
  }
}

__global__ void k_eq_flags(const int32_t* v, int64_t n, int32_t target, int32_t* flags) {
  GRID_STRIDE(i, n) flags[i] = v[i] == target ? 1 : 0;
}

__global__ void k_compact(const int32_t* flags, const int32_t* pos, int64_t n, int32_t* out) {
  GRID_STRIDE(i, n) if (flags[i]) out[pos[i]] = (int32_t)i;
}

}  // namespace

extern "C" int pg_faces_edges(const int32_t* elemsF, const int32_t* elemsE, int64_t n_elems, int64_t nF,
                              int32_t* facesE, int32_t* owner_ws, int32_t* status, void* stream) {
  if (n_elems < 1 || nF < 1 || !elemsF || !elemsE || !facesE || !owner_ws || !status) {
    pg_set_error("pg_faces_edges: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  k_owner_init<<<pg_blocks(nF, 256), 256, 0, s>>>(owner_ws, nF);
  k_owner_min<<<pg_blocks(4 * n_elems, 256), 256, 0, s>>>(elemsF, n_elems, nF, owner_ws, status);
  k_faces_edges<<<pg_blocks(nF, 256), 256, 0, s>>>(owner_ws, elemsE, nF, facesE);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_face_counts(const int32_t* elemsF, int64_t n_elems, int64_t nF, int32_t* face_nelem, void* stream) {
  if (n_elems < 1 || nF < 1 || !elemsF || !face_nelem) {
    pg_set_error("pg_face_counts: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  PG_CUDA_TRY(cudaMemsetAsync(face_nelem, 0, sizeof(int32_t) * nF, s));
  k_face_counts<<<pg_blocks(4 * n_elems, 256), 256, 0, s>>>(elemsF, n_elems, nF, face_nelem);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_flag_edges_of_pairs(const int32_t* edgesNodes, int64_t nE, const int32_t* pairs, int64_t n_pairs,
                                      int32_t* flags, void* stream) {
  if (nE < 1 || n_pairs < 0 || !edgesNodes || !flags || (n_pairs > 0 && !pairs)) {
    pg_set_error("pg_flag_edges_of_pairs: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  PG_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int32_t) * nE, s));
  if (n_pairs > 0) k_flag_pairs<<<pg_blocks(n_pairs, 256), 256, 0, s>>>(edgesNodes, nE, pairs, n_pairs, flags);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" size_t pg_select_workspace_bytes(int64_t n) { return pg::select_workspace_bytes_for(n); }

extern "C" int pg_select_equal(const int32_t* values, int64_t n, int32_t target, int32_t* out, int64_t* count,
                               void* workspace, size_t workspace_bytes, void* stream) {
  if (n < 1 || !values || !out || !count) {
    pg_set_error("pg_select_equal: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_select_workspace_bytes(n)) {
    pg_set_error("pg_select_equal: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  PgArena ar(workspace, workspace_bytes);
  int32_t* flags = ar.take<int32_t>(n);
  int32_t* pos = ar.take<int32_t>(n);
  const size_t scan_b = pg::scan_workspace_bytes(n);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(2);
  if (!flags || !pos || !scan_ws || !tot) return PG_ERR_WORKSPACE;
  k_eq_flags<<<pg_blocks(n, 256), 256, 0, s>>>(values, n, target, flags);
  int st = pg::scan_exclusive_i32(flags, pos, n, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_compact<<<pg_blocks(n, 256), 256, 0, s>>>(flags, pos, n, out);
  k_store_count<<<1, 1, 0, s>>>(tot, count);
  PG_LAUNCH_CHECK();
  return PG_OK;
}
