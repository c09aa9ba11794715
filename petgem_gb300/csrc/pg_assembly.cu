// CSR sparsity pattern and deterministic value assembly of
//   A = sum_e P_e^T (K_e - i omega mu M_e) P_e      (petgem/solver.py:182-235)
// plus PEC rows/columns (solver.py:552-577).
//
// Pattern.  petgem inserts every element's dense nd x nd block into a PETSc
// AIJ matrix, so row r's columns are the union of the DOFs of the elements
// containing r, sorted.  DOFs are numbered entity by entity (edges, faces,
// volumes), so all rows of one entity share one column list, made of whole
// DOF blocks of the entities adjacent to it.  The builder therefore works on
// entity pairs: keys (a, b) for every pair of entities of every element
// (nl^2 per element, nl = 6/10/11 entities with DOFs for p = 1/2/>=3) are
// radix-sorted; each distinct key is one dense na x nb block of A, and the
// sorted run of equal keys lists, in ascending element order, every element
// contributing to that block.
//
// Values.  Each block is summed over its member elements in that fixed
// order (no atomics): bitwise reproducible and independent of the launch
// shape.  Two value paths exist: from materialised elemental matrices, and a
// fused path that evaluates each contribution from the element's 12
// geometry coefficients and its orientation tuple's moment tables, so the
// elemental matrices are never written to memory.
#include "pg_common.cuh"
#include "pg_df.cuh"
#include "pg_sort.cuh"

namespace {

#define GRID_STRIDE(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

struct Ent {
  int64_t nE, nF, T;
  int p, nl, de, df, dv;
  __host__ __device__ Ent(int64_t nE_, int64_t nF_, int64_t T_, int p_) : nE(nE_), nF(nF_), T(T_), p(p_) {
    de = p;
    df = p * (p - 1);
    dv = p * (p - 1) * (p - 2) / 2;
    nl = p == 1 ? 6 : (p == 2 ? 10 : 11);
  }
  __host__ __device__ int64_t count() const { return nE + nF + T; }
  // global entity id of local entity l of element e
  __device__ int64_t ent(const int32_t* elemsE, const int32_t* elemsF, int64_t e, int l) const {
    if (l < 6) return elemsE[6 * e + l];
    if (l < 10) return nE + elemsF[4 * e + (l - 6)];
    return nE + nF + e;
  }
  __host__ __device__ int nd_ent(int64_t a) const { return a < nE ? de : (a < nE + nF ? df : dv); }
  __host__ __device__ int64_t first_dof(int64_t a) const {
    if (a < nE) return a * de;
    if (a < nE + nF) return nE * de + (a - nE) * df;
    return nE * de + nF * df + (a - nE - nF) * dv;
  }
  // local DOF offset of local entity l inside the element's nd DOFs
  __host__ __device__ int local_off(int l) const {
    if (l < 6) return l * de;
    if (l < 10) return 6 * de + (l - 6) * df;
    return 6 * de + 4 * df;
  }
  __host__ __device__ int64_t ndofs() const { return nE * de + nF * df + T * dv; }
  // entity of global DOF r
  __device__ int64_t ent_of_dof(int64_t r) const {
    if (r < nE * de) return r / de;
    r -= nE * de;
    if (r < nF * df) return nE + r / df;
    r -= nF * df;
    return nE + nF + r / dv;
  }
};

__global__ void k_pair_keys(const int32_t* elemsE, const int32_t* elemsF, Ent E, uint64_t* keys, int32_t* vals) {
  const int nl2 = E.nl * E.nl;
  const uint64_t n_ent = (uint64_t)E.count();
  GRID_STRIDE(i, E.T * nl2) {
    const int64_t e = i / nl2;
    const int r = (int)(i % nl2);
    const int la = r / E.nl, lb = r % E.nl;
    const uint64_t a = (uint64_t)E.ent(elemsE, elemsF, e, la);
    const uint64_t b = (uint64_t)E.ent(elemsE, elemsF, e, lb);
    keys[i] = a * n_ent + b;
    vals[i] = (int32_t)i;
  }
}

__global__ void k_flags(const uint64_t* keys, int64_t n, int32_t* flags) {
  GRID_STRIDE(i, n) flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// per sorted position: pair id; per pair: start, a, b, nb
__global__ void k_pairs(const uint64_t* keys, const int32_t* excl, int64_t n, Ent E, int32_t* pair_start,
                        int64_t* pair_a, int32_t* pair_nb) {
  const uint64_t n_ent = (uint64_t)E.count();
  GRID_STRIDE(i, n) {
    if (i == 0 || keys[i] != keys[i - 1]) {
      const int32_t g = excl[i];
      pair_start[g] = (int32_t)i;
      pair_a[g] = (int64_t)(keys[i] / n_ent);
      pair_nb[g] = E.nd_ent((int64_t)(keys[i] % n_ent));
    }
  }
}

__global__ void k_pair_tail(const int32_t* n_pairs, int64_t M, int32_t* pair_start, int64_t* counts) {
  pair_start[*n_pairs] = (int32_t)M;
  counts[0] = *n_pairs;
}

// ent_first[a] = first pair of entity a
__global__ void k_ent_first(const int64_t* pair_a, const int32_t* n_pairs, int32_t* ent_first) {
  const int64_t np = *n_pairs;
  GRID_STRIDE(g, np) {
    if (g == 0 || pair_a[g] != pair_a[g - 1]) ent_first[pair_a[g]] = (int32_t)g;
  }
}

// colstart[g] = X[g] - X[ent_first[a]];  row length of a = X[last]+nb[last]-X[first]
__global__ void k_colstart(const int64_t* pair_a, const int32_t* X, const int32_t* pair_nb, const int32_t* ent_first,
                           const int32_t* n_pairs, int32_t* colstart, int32_t* ent_len) {
  const int64_t np = *n_pairs;
  GRID_STRIDE(g, np) {
    const int64_t a = pair_a[g];
    const int32_t x0 = X[ent_first[a]];
    colstart[g] = X[g] - x0;
    if (g == np - 1 || pair_a[g + 1] != a) ent_len[a] = X[g] + pair_nb[g] - x0;
  }
}

// row lengths into rowptr[0..N) and 0 into rowptr[N], ready for the exclusive scan
__global__ void k_rowlen(Ent E, const int32_t* ent_len, int64_t N, int64_t* rowptr) {
  GRID_STRIDE(r, N + 1) rowptr[r] = r < N ? ent_len[E.ent_of_dof(r)] : 0;
}

__global__ void k_zero_i32(int32_t* a, int64_t n) { GRID_STRIDE(i, n) a[i] = 0; }

// one warp per pair: fill the block's column indices
__global__ void k_columns(const int32_t* members, const int32_t* pair_start, const int32_t* colstart, int64_t n_pairs,
                          const int32_t* elemsE, const int32_t* elemsF, Ent E, const int64_t* rowptr, int32_t* col) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nl2 = E.nl * E.nl;
  for (int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; g < n_pairs; g += warps) {
    const int32_t m = members[pair_start[g]];
    const int64_t e = m / nl2;
    const int r = m % nl2;
    const int64_t a = E.ent(elemsE, elemsF, e, r / E.nl), b = E.ent(elemsE, elemsF, e, r % E.nl);
    const int na = E.nd_ent(a), nb = E.nd_ent(b);
    const int64_t fa = E.first_dof(a), fb = E.first_dof(b);
    const int cs = colstart[g];
    for (int t = lane; t < na * nb; t += 32) {
      const int i = t / nb, j = t % nb;
      col[rowptr[fa + i] + cs + j] = (int32_t)(fb + j);
    }
  }
}

// values from materialised M, K: warp per pair, lanes over block entries
__global__ void k_values_mk(const double* __restrict__ Mm, const double* __restrict__ Km,
                            const int32_t* __restrict__ members, const int32_t* __restrict__ pair_start,
                            const int32_t* __restrict__ colstart, int64_t n_pairs, const int32_t* elemsE,
                            const int32_t* elemsF, Ent E, int nd, const int64_t* __restrict__ rowptr, double omu,
                            double2* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nl2 = E.nl * E.nl;
  const int64_t nd2 = (int64_t)nd * nd;
  for (int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; g < n_pairs; g += warps) {
    const int32_t s0 = pair_start[g], s1 = pair_start[g + 1];
    const int32_t m0 = members[s0];
    const int64_t e0 = m0 / nl2;
    const int r0 = m0 % nl2;
    const int64_t a = E.ent(elemsE, elemsF, e0, r0 / E.nl), b = E.ent(elemsE, elemsF, e0, r0 % E.nl);
    const int na = E.nd_ent(a), nb = E.nd_ent(b);
    const int64_t fa = E.first_dof(a);
    const int cs = colstart[g];
    for (int t = lane; t < na * nb; t += 32) {
      const int i = t / nb, j = t % nb;
      double re = 0.0, im = 0.0;
      for (int32_t s = s0; s < s1; ++s) {
        const int32_t m = members[s];
        const int64_t e = m / nl2;
        const int r = m % nl2;
        const int64_t off = e * nd2 + (int64_t)(E.local_off(r / E.nl) + i) * nd + E.local_off(r % E.nl) + j;
        re += Km[off];
        im += Mm[off];
      }
      vals[rowptr[fa + i] + cs + j] = make_double2(re, -omu * im);
    }
  }
}

__device__ __forceinline__ void put_coef(double* cf, int t, double v) { cf[t] = v; }
__device__ __forceinline__ void put_coef(float2* cf, int t, double v) {
  const float h = __double2float_rn(v);
  cf[t] = make_float2(h, __double2float_rn(v - (double)h));
}

// per-element coefficients for the fused path: [cK(6) | -omega mu det S (6)],
// as doubles or as (hi, lo) double-float pairs
template <typename C>
__global__ void k_coefficients(const double* nodes, const int32_t* elemsN, const double* sigma, int64_t T, double omu,
                               C* coef, int32_t* status) {
  GRID_STRIDE(e, T) {
    double x[4][3];
    for (int v = 0; v < 4; ++v) {
      const int64_t n = elemsN[4 * e + v];
      x[v][0] = nodes[3 * n];
      x[v][1] = nodes[3 * n + 1];
      x[v][2] = nodes[3 * n + 2];
    }
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) J[r][c] = x[r + 1][c] - x[0][c];
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    C* cf = coef + 12 * e;
    if (!(det != 0.0) || !isfinite(det)) {
      *status = PG_ERR_DEGENERATE;
      for (int t = 0; t < 12; ++t) put_coef(cf, t, 0.0);
      continue;
    }
    // With adj = det inv(J) (the adjugate): cK = J J^T / det and
    // cM = -omega mu det inv^T D inv = -omega mu adj^T D adj / det, which
    // spares the nine inverse entries and the rescaling by det (GB300's FP64
    // pipe makes every operation here count); 1 / det correctly rounded.
    const double id = __drcp_rn(det);
    double adj[3][3];   // adj[c][a] = inv[c][a] * det
    adj[0][0] = c00;
    adj[1][0] = c01;
    adj[2][0] = c02;
    adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double D[3] = {sigma[2 * e], sigma[2 * e], sigma[2 * e + 1]};
    double w[3][3];     // D adj
    for (int c = 0; c < 3; ++c)
      for (int b = 0; b < 3; ++b) w[c][b] = D[c] * adj[c][b];
    const double mscale = -omu * id;
    const int pa[6] = {0, 1, 2, 0, 0, 1};
    const int pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      double s = 0.0, g = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        s = fma(adj[c][pa[t]], w[c][pb[t]], s);
        g = fma(J[pa[t]][c], J[pb[t]][c], g);
      }
      put_coef(cf, t, g * id);
      put_coef(cf, 6 + t, mscale * s);
    }
  }
}

// The per-element coefficients in double-float arithmetic on the FP32 pipes
// (the FP64 form spends ~180 FP64 operations per element, which on GB300's
// ~2 FP64 operations per clock per SM made it the second-largest kernel of an
// assembly pass).  J = x_r - x_0 is formed in FP64 (exact up to rounding of
// the difference) and split; then, with adj(J) the adjugate (inv J =
// adj / det):  cK = J J^T / det,  cM = -omega mu adj^T D adj / det.
__global__ void k_coefficients_dfa(const double* __restrict__ nodes, const int32_t* __restrict__ elemsN,
                                   const double* __restrict__ sigma, int64_t T, float omu_h, float omu_l,
                                   float2* __restrict__ coef, int32_t* __restrict__ status) {
  GRID_STRIDE(e, T) {
    double x0[3];
    dfv J[3][3];
    {
      const int64_t n0 = elemsN[4 * e];
      for (int c = 0; c < 3; ++c) x0[c] = nodes[3 * n0 + c];
      for (int r = 0; r < 3; ++r) {
        const int64_t n = elemsN[4 * e + r + 1];
        for (int c = 0; c < 3; ++c) J[r][c] = df_from_double(nodes[3 * n + c] - x0[c]);
      }
    }
    auto cross = [&](int a, int b, int c, int d, int f, int g, int h, int k) {
      // J[a][b] J[c][d] - J[f][g] J[h][k]
      return df_sum(df_mul(J[a][b], J[c][d]), df_neg(df_mul(J[f][g], J[h][k])));
    };
    dfv A[3][3];   // adjugate, inv J = A / det
    A[0][0] = cross(1, 1, 2, 2, 1, 2, 2, 1);
    A[1][0] = cross(1, 2, 2, 0, 1, 0, 2, 2);
    A[2][0] = cross(1, 0, 2, 1, 1, 1, 2, 0);
    A[0][1] = cross(0, 2, 2, 1, 0, 1, 2, 2);
    A[1][1] = cross(0, 0, 2, 2, 0, 2, 2, 0);
    A[2][1] = cross(0, 1, 2, 0, 0, 0, 2, 1);
    A[0][2] = cross(0, 1, 1, 2, 0, 2, 1, 1);
    A[1][2] = cross(0, 2, 1, 0, 0, 0, 1, 2);
    A[2][2] = cross(0, 0, 1, 1, 0, 1, 1, 0);
    const dfv det = df_sum(df_sum(df_mul(J[0][0], A[0][0]), df_mul(J[0][1], A[1][0])), df_mul(J[0][2], A[2][0]));
    float2* cf = coef + 12 * e;
    if (!(det.h != 0.f) || !isfinite(det.h)) {
      *status = PG_ERR_DEGENERATE;
      for (int t = 0; t < 12; ++t) cf[t] = make_float2(0.f, 0.f);
      continue;
    }
    const dfv id = df_rcp(det);
    const dfv sh = df_from_double(sigma[2 * e]), sv = df_from_double(sigma[2 * e + 1]);
    const dfv D[3] = {sh, sh, sv};
    dfv W[3][3];   // W[c][a] = D[c] A[c][a]
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) W[c][a] = df_mul(D[c], A[c][a]);
    const dfv m = df_neg(df_mul(dfv{omu_h, omu_l}, id));
    const int pa[6] = {0, 1, 2, 0, 0, 1};
    const int pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      dfv g = df_mul(J[pa[t]][0], J[pb[t]][0]);
      dfv s = df_mul(W[0][pa[t]], A[0][pb[t]]);
      for (int c = 1; c < 3; ++c) {
        g = df_sum(g, df_mul(J[pa[t]][c], J[pb[t]][c]));
        s = df_sum(s, df_mul(W[c][pa[t]], A[c][pb[t]]));
      }
      const dfv k = df_mul(g, id), mm = df_mul(s, m);
      cf[t] = make_float2(k.h, k.l);
      cf[6 + t] = make_float2(mm.h, mm.l);
    }
  }
}

__device__ __forceinline__ int packed_index(int j, int k, int nd) {
  if (k < j) { int t = j; j = k; k = t; }
  return j * nd - (j * (j - 1)) / 2 + (k - j);
}

__device__ __forceinline__ double2 pec_value(const uint8_t* pec, int64_t row, int64_t col, double2 v);

// ---- symmetric item lists: one item per upper entry of every pair with a <= b
__global__ void k_pair_keys_of(const int32_t* members, const int32_t* pair_start, int64_t n_pairs,
                               const int32_t* elemsE, const int32_t* elemsF, Ent E, int64_t* pair_key,
                               int32_t* n_items) {
  const int nl2 = E.nl * E.nl;
  const int64_t n_ent = E.count();
  GRID_STRIDE(g, n_pairs) {
    const int32_t m = members[pair_start[g]];
    const int64_t e = m / nl2;
    const int r = m % nl2;
    const int64_t a = E.ent(elemsE, elemsF, e, r / E.nl), b = E.ent(elemsE, elemsF, e, r % E.nl);
    pair_key[g] = a * n_ent + b;
    const int na = E.nd_ent(a), nb = E.nd_ent(b);
    n_items[g] = a < b ? na * nb : (a == b ? na * (na + 1) / 2 : 0);
  }
}

__global__ void k_partner(const int64_t* pair_key, int64_t n_pairs, Ent E, int32_t* partner) {
  const int64_t n_ent = E.count();
  GRID_STRIDE(g, n_pairs) {
    const int64_t key = pair_key[g];
    const int64_t want = (key % n_ent) * n_ent + key / n_ent;
    int64_t lo = 0, hi = n_pairs - 1, found = -1;
    while (lo <= hi) {
      const int64_t mid = (lo + hi) >> 1;
      const int64_t v = pair_key[mid];
      if (v == want) { found = mid; break; }
      if (v < want) lo = mid + 1; else hi = mid - 1;
    }
    partner[g] = (int32_t)found;
  }
}

__global__ void k_items(const int32_t* n_items, const int32_t* item_start, int64_t n_pairs, int64_t* items) {
  GRID_STRIDE(g, n_pairs) {
    const int c = n_items[g];
    const int64_t base = item_start[g];
    for (int t = 0; t < c; ++t) items[base + t] = ((int64_t)g << 12) | t;
  }
}

__global__ void k_store_i64(const int32_t* src, int64_t* dst) { *dst = *src; }

// sort key of every item: member count of its pair
__global__ void k_item_keys(const int64_t* items, const int32_t* n_items_dev, const int32_t* pair_start,
                            uint64_t* keys, int32_t* vals) {
  const int64_t n = *n_items_dev;
  GRID_STRIDE(i, n) {
    const int64_t g = items[i] >> 12;
    const int32_t c = pair_start[g + 1] - pair_start[g];
    keys[i] = (uint64_t)(c < 255 ? c : 255);
    vals[i] = (int32_t)i;
  }
}

__global__ void k_item_gather(const int64_t* items, const int32_t* n_items_dev, const int32_t* order, int64_t* out) {
  const int64_t n = *n_items_dev;
  GRID_STRIDE(i, n) out[i] = items[order[i]];
}

// fused symmetric values: one thread per item; members summed in element order,
// 12 FMAs per member; the value goes to slot (a,b) and to its transpose (b,a).
template <int P>
__global__ void __launch_bounds__(256) k_values_sym(const double* __restrict__ coef,
                                                    const int32_t* __restrict__ tuple_of_elem,
                                                    const double* __restrict__ tables,
                                                    const int32_t* __restrict__ members,
                                                    const int32_t* __restrict__ pair_start,
                                                    const int32_t* __restrict__ colstart,
                                                    const int32_t* __restrict__ partner,
                                                    const int64_t* __restrict__ items, int64_t n_items,
                                                    const int32_t* __restrict__ elemsE,
                                                    const int32_t* __restrict__ elemsF, int64_t nE, int64_t nF,
                                                    int64_t T, const int64_t* __restrict__ rowptr,
                                                    const uint8_t* __restrict__ pec, double2* __restrict__ vals) {
  constexpr int NL = P == 1 ? 6 : (P == 2 ? 10 : 11);
  constexpr int NL2 = NL * NL;
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  constexpr int NT = ND * (ND + 1) / 2;
  const Ent E(nE, nF, T, P);
  GRID_STRIDE(idx, n_items) {
    const int64_t it = items[idx];
    const int64_t g = it >> 12;
    int t = (int)(it & 4095);
    const int32_t s0 = pair_start[g], s1 = pair_start[g + 1];
    const int32_t m0 = members[s0];
    const int64_t e0 = m0 / NL2;
    const int r0 = m0 % NL2;
    const int64_t a = E.ent(elemsE, elemsF, e0, r0 / NL), b = E.ent(elemsE, elemsF, e0, r0 % NL);
    const int na = E.nd_ent(a), nb = E.nd_ent(b);
    int i, j;
    if (a != b) {
      i = t / nb;
      j = t - i * nb;
    } else {  // upper triangle of an na x na block, row by row
      i = 0;
      while (t >= na - i) { t -= na - i; ++i; }
      j = i + t;
    }
    double re = 0.0, im = 0.0;
    for (int32_t q = s0; q < s1; ++q) {
      const int32_t m = members[q];
      const int64_t e = m / NL2;
      const int r = m - (int)(e * NL2);
      const int la = r / NL, lb = r - la * NL;
      const int jl = E.local_off(la) + i, kl = E.local_off(lb) + j;
      const double* tb = tables + (int64_t)__ldg(tuple_of_elem + e) * (12 * NT) + packed_index(jl, kl, ND);
      const double* cf = coef + 12 * e;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        re = fma(__ldg(cf + k), __ldg(tb + (6 + k) * NT), re);
        im = fma(__ldg(cf + 6 + k), __ldg(tb + k * NT), im);
      }
    }
    const double2 v = make_double2(re, im);
    const int64_t fa = E.first_dof(a), fb = E.first_dof(b);
    vals[rowptr[fa + i] + colstart[g] + j] = pec_value(pec, fa + i, fb + j, v);
    if (a != b) vals[rowptr[fb + j] + colstart[partner[g]] + i] = pec_value(pec, fb + j, fa + i, v);
    else if (i != j) vals[rowptr[fa + j] + colstart[g] + i] = pec_value(pec, fa + j, fa + i, v);
  }
}


// PEC applied while writing (zeroRowsColumns(rows, diag=1), solver.py:562):
// entries in a boundary row or column become 0, the boundary diagonal 1.
__device__ __forceinline__ double2 pec_value(const uint8_t* pec, int64_t row, int64_t col, double2 v) {
  if (pec && (pec[row] | pec[col])) return make_double2(row == col && pec[row] ? 1.0 : 0.0, 0.0);
  return v;
}

// Double-float variant of k_values_sym: coefficients and tables are (hi, lo)
// FP32 pairs, the 12 products per member are double-float multiply-adds on
// the FP32 pipes; only the final conversion to complex128 uses FP64.
template <int P>
__global__ void __launch_bounds__(256) k_values_sym_df(const float2* __restrict__ coef,
                                                       const int32_t* __restrict__ tuple_of_elem,
                                                       const float2* __restrict__ tables,
                                                       const int32_t* __restrict__ members,
                                                       const int32_t* __restrict__ pair_start,
                                                       const int32_t* __restrict__ colstart,
                                                       const int32_t* __restrict__ partner,
                                                       const int64_t* __restrict__ items, int64_t n_items,
                                                       const int32_t* __restrict__ elemsE,
                                                       const int32_t* __restrict__ elemsF, int64_t nE, int64_t nF,
                                                       int64_t T, const int64_t* __restrict__ rowptr,
                                                       const uint8_t* __restrict__ pec, double2* __restrict__ vals) {
  constexpr int NL = P == 1 ? 6 : (P == 2 ? 10 : 11);
  constexpr int NL2 = NL * NL;
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  constexpr int NT = ND * (ND + 1) / 2;
  const Ent E(nE, nF, T, P);
  GRID_STRIDE(idx, n_items) {
    const int64_t it = items[idx];
    const int64_t g = it >> 12;
    int t = (int)(it & 4095);
    const int32_t s0 = pair_start[g], s1 = pair_start[g + 1];
    const int32_t m0 = members[s0];
    const int64_t e0 = m0 / NL2;
    const int r0 = m0 % NL2;
    const int64_t a = E.ent(elemsE, elemsF, e0, r0 / NL), b = E.ent(elemsE, elemsF, e0, r0 % NL);
    const int na = E.nd_ent(a), nb = E.nd_ent(b);
    int i, j;
    if (a != b) {
      i = t / nb;
      j = t - i * nb;
    } else {
      i = 0;
      while (t >= na - i) { t -= na - i; ++i; }
      j = i + t;
    }
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int32_t q = s0; q < s1; ++q) {
      const int32_t m = members[q];
      const int64_t e = m / NL2;
      const int r = m - (int)(e * NL2);
      const int la = r / NL, lb = r - la * NL;
      const int jl = E.local_off(la) + i, kl = E.local_off(lb) + j;
      const float2* tb = tables + (int64_t)__ldg(tuple_of_elem + e) * (12 * NT) + packed_index(jl, kl, ND);
      const float2* cf = coef + 12 * e;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float2 ck = __ldg(cf + k), tk = __ldg(tb + (6 + k) * NT);
        df_mac(rh, rl, ck.x, ck.y, tk.x, tk.y);
        const float2 cm = __ldg(cf + 6 + k), tm = __ldg(tb + k * NT);
        df_mac(ih, il, cm.x, cm.y, tm.x, tm.y);
      }
    }
    const double2 v = make_double2(df_to_double(rh, rl), df_to_double(ih, il));
    const int64_t fa = E.first_dof(a), fb = E.first_dof(b);
    vals[rowptr[fa + i] + colstart[g] + j] = pec_value(pec, fa + i, fb + j, v);
    if (a != b) vals[rowptr[fb + j] + colstart[partner[g]] + i] = pec_value(pec, fb + j, fa + i, v);
    else if (i != j) vals[rowptr[fa + j] + colstart[g] + i] = pec_value(pec, fa + j, fa + i, v);
  }
}

__global__ void k_to_df(const double* __restrict__ in, int64_t n, float2* __restrict__ out) {
  GRID_STRIDE(i, n) {
    const double v = in[i];
    const float h = __double2float_rn(v);
    out[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

__global__ void k_pec_rhs(const int32_t* bnd, int64_t n_bnd, int nrhs, double2* b) {
  GRID_STRIDE(i, n_bnd * nrhs) b[(int64_t)bnd[i / nrhs] * nrhs + i % nrhs] = make_double2(0.0, 0.0);
}

__global__ void k_mark_bnd(const int32_t* bnd, int64_t nb, uint8_t* flag, double2* b) {
  GRID_STRIDE(i, nb) {
    flag[bnd[i]] = 1;
    if (b) b[bnd[i]] = make_double2(0.0, 0.0);
  }
}

// zeroRowsColumns(rows, diag=1): warp per row
__global__ void k_pec(const int64_t* rowptr, const int32_t* col, double2* vals, int64_t N, const uint8_t* flag) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < N; r += warps) {
    const bool rb = flag[r] != 0;
    for (int64_t k = rowptr[r] + lane; k < rowptr[r + 1]; k += 32) {
      const int32_t c = col[k];
      if (rb) vals[k] = make_double2(c == r ? 1.0 : 0.0, 0.0);
      else if (flag[c]) vals[k] = make_double2(0.0, 0.0);
    }
  }
}

unsigned warp_grid(int64_t items) {
  int64_t blocks = (items + 7) / 8;  // 8 warps per 256-thread block
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  return (unsigned)blocks;
}

}  // namespace

extern "C" int pg_pattern_local_entities(int p) { return p == 1 ? 6 : (p == 2 ? 10 : 11); }

extern "C" size_t pg_pattern_workspace_bytes(int64_t n_elems, int64_t nE, int64_t nF, int p) {
  const int nl = pg_pattern_local_entities(p);
  const int64_t M = n_elems * nl * nl;
  const int64_t n_ent = nE + nF + n_elems;
  return pg_align256(sizeof(uint64_t) * M) + pg_align256(sizeof(int32_t) * M) /*excl*/ +
         pg_align256(sizeof(int64_t) * M) /*pair_a*/ + pg_align256(sizeof(int32_t) * M) * 2 /*nb, X*/ +
         pg_align256(sizeof(int32_t) * n_ent) * 2 + pg::sort_workspace_bytes(M) + pg::scan_workspace_bytes(M) +
         4096;
}

extern "C" int pg_pattern_build(const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE,
                                int64_t nF, int p, int32_t* members, int32_t* pair_start, int32_t* pair_colstart,
                                int64_t* rowptr, int64_t* counts, void* workspace, size_t workspace_bytes,
                                void* stream) {
  if (p < 1 || p > 6) {
    pg_set_error("pg_pattern_build: order must be 1..6");
    return PG_ERR_UNSUPPORTED;
  }
  Ent E(nE, nF, n_elems, p);
  const int64_t M = n_elems * E.nl * E.nl;
  const int64_t N = E.ndofs();
  if (n_elems < 1 || nE < 1 || nF < 1 || !elemsE || !elemsF || !members || !pair_start || !pair_colstart || !rowptr ||
      !counts || M >= (1ll << 31) || N >= (1ll << 31)) {
    pg_set_error("pg_pattern_build: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_pattern_workspace_bytes(n_elems, nE, nF, p)) {
    pg_set_error("pg_pattern_build: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  PgArena ar(workspace, workspace_bytes);
  uint64_t* keys = ar.take<uint64_t>(M);
  int32_t* excl = ar.take<int32_t>(M);
  int64_t* pair_a = ar.take<int64_t>(M);
  int32_t* pair_nb = ar.take<int32_t>(M);
  int32_t* X = ar.take<int32_t>(M);
  const int64_t n_ent = E.count();
  int32_t* ent_first = ar.take<int32_t>(n_ent);
  int32_t* ent_len = ar.take<int32_t>(n_ent);
  const size_t sort_b = pg::sort_workspace_bytes(M);
  void* sort_ws = ar.take<char>(sort_b);
  const size_t scan_b = pg::scan_workspace_bytes(M);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(8);
  if (!keys || !excl || !pair_a || !pair_nb || !X || !ent_first || !ent_len || !sort_ws || !scan_ws || !tot)
    return PG_ERR_WORKSPACE;
  const unsigned gM = pg_blocks(M, 256);
  int st;
  k_pair_keys<<<gM, 256, 0, s>>>(elemsE, elemsF, E, keys, members);
  st = pg::sort_pairs(keys, members, M, pg::bits_for((uint64_t)n_ent * (uint64_t)n_ent - 1), sort_ws, sort_b, s);
  if (st) { pg_set_error("pg_pattern_build: sort failed"); return st; }
  k_flags<<<gM, 256, 0, s>>>(keys, M, excl);
  st = pg::scan_exclusive_i32(excl, excl, M, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_pairs<<<gM, 256, 0, s>>>(keys, excl, M, E, pair_start, pair_a, pair_nb);
  k_pair_tail<<<1, 1, 0, s>>>(tot, M, pair_start, counts);
  // X = exclusive scan of nb over pairs (length n_pairs <= M; the tail beyond n_pairs is unused)
  // n_pairs is only known on the device: scan over the M-capacity prefix with zero padding.
  k_zero_i32<<<gM, 256, 0, s>>>(X, M);
  // copy nb into X's input (X reused as output of the scan)
  st = pg::scan_exclusive_i32(pair_nb, X, M, nullptr, scan_ws, scan_b, s);
  if (st) return st;
  k_ent_first<<<gM, 256, 0, s>>>(pair_a, tot, ent_first);
  k_zero_i32<<<pg_blocks(n_ent, 256), 256, 0, s>>>(ent_len, n_ent);
  k_colstart<<<gM, 256, 0, s>>>(pair_a, X, pair_nb, ent_first, tot, pair_colstart, ent_len);
  k_rowlen<<<pg_blocks(N + 1, 256), 256, 0, s>>>(E, ent_len, N, rowptr);
  st = pg::scan_exclusive_i64(rowptr, rowptr, N + 1, counts + 1, scan_ws, scan_b, s);
  if (st) return st;
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_pattern_columns(const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                                  int64_t n_pairs, const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems,
                                  int64_t nE, int64_t nF, int p, const int64_t* rowptr, int32_t* col, void* stream) {
  if (p < 1 || p > 6 || n_pairs < 1 || !members || !pair_start || !pair_colstart || !rowptr || !col) {
    pg_set_error("pg_pattern_columns: bad argument");
    return PG_ERR_ARG;
  }
  Ent E(nE, nF, n_elems, p);
  k_columns<<<warp_grid(n_pairs), 256, 0, pg_stream(stream)>>>(members, pair_start, pair_colstart, n_pairs, elemsE,
                                                               elemsF, E, rowptr, col);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_assemble_values(const double* M, const double* K, const int32_t* members, const int32_t* pair_start,
                                  const int32_t* pair_colstart, int64_t n_pairs, const int32_t* elemsE,
                                  const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF, int p,
                                  const int64_t* rowptr, double omega_mu, double* vals, void* stream) {
  if (p < 1 || p > 6 || n_pairs < 1 || !M || !K || !members || !pair_start || !pair_colstart || !rowptr || !vals) {
    pg_set_error("pg_assemble_values: bad argument");
    return PG_ERR_ARG;
  }
  Ent E(nE, nF, n_elems, p);
  k_values_mk<<<warp_grid(n_pairs), 256, 0, pg_stream(stream)>>>(M, K, members, pair_start, pair_colstart, n_pairs,
                                                                 elemsE, elemsF, E, pg_nd_elem(p), rowptr, omega_mu,
                                                                 reinterpret_cast<double2*>(vals));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_element_coefficients(const double* nodes, const int32_t* elemsN, const double* sigma,
                                       int64_t n_elems, double omega_mu, double* coef, int32_t* status,
                                       void* stream) {
  if (n_elems < 1 || !nodes || !elemsN || !sigma || !coef || !status) {
    pg_set_error("pg_element_coefficients: bad argument");
    return PG_ERR_ARG;
  }
  k_coefficients<<<pg_blocks(n_elems, 256), 256, 0, pg_stream(stream)>>>(nodes, elemsN, sigma, n_elems, omega_mu,
                                                                        coef, status);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_element_coefficients_df(const double* nodes, const int32_t* elemsN, const double* sigma,
                                          int64_t n_elems, double omega_mu, float* coef_pairs, int32_t* status,
                                          void* stream) {
  if (n_elems < 1 || !nodes || !elemsN || !sigma || !coef_pairs || !status) {
    pg_set_error("pg_element_coefficients_df: bad argument");
    return PG_ERR_ARG;
  }
  const float omu_h = (float)omega_mu;
  const float omu_l = (float)(omega_mu - (double)omu_h);
  k_coefficients_dfa<<<pg_blocks(n_elems, 256), 256, 0, pg_stream(stream)>>>(
      nodes, elemsN, sigma, n_elems, omu_h, omu_l, reinterpret_cast<float2*>(coef_pairs), status);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" size_t pg_pattern_items_workspace_bytes(int64_t n_pairs, int64_t max_items) {
  return pg_align256(sizeof(int64_t) * n_pairs) + pg_align256(sizeof(int32_t) * (n_pairs + 1)) * 2 +
         pg::scan_workspace_bytes(n_pairs + 1) + pg_align256(sizeof(uint64_t) * max_items) +
         pg_align256(sizeof(int32_t) * max_items) + pg_align256(sizeof(int64_t) * max_items) +
         pg::sort_workspace_bytes(max_items) + 1024;
}

extern "C" int pg_pattern_items(const int32_t* members, const int32_t* pair_start, int64_t n_pairs,
                                const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE, int64_t nF,
                                int p, int64_t max_items, int32_t* pair_partner, int64_t* items, int64_t* n_items,
                                void* workspace, size_t workspace_bytes, void* stream) {
  if (p < 1 || p > 6 || n_pairs < 1 || !members || !pair_start || !pair_partner || !items || !n_items) {
    pg_set_error("pg_pattern_items: bad argument");
    return PG_ERR_ARG;
  }
  if (max_items < 1 || max_items >= (1ll << 31) || !workspace ||
      workspace_bytes < pg_pattern_items_workspace_bytes(n_pairs, max_items)) {
    pg_set_error("pg_pattern_items: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  Ent E(nE, nF, n_elems, p);
  PgArena ar(workspace, workspace_bytes);
  int64_t* pair_key = ar.take<int64_t>(n_pairs);
  int32_t* cnt = ar.take<int32_t>(n_pairs + 1);
  int32_t* start = ar.take<int32_t>(n_pairs + 1);
  const size_t scan_b = pg::scan_workspace_bytes(n_pairs + 1);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(4);
  uint64_t* ikeys = ar.take<uint64_t>(max_items);
  int32_t* ivals = ar.take<int32_t>(max_items);
  int64_t* itmp = ar.take<int64_t>(max_items);
  const size_t sort_b = pg::sort_workspace_bytes(max_items);
  void* sort_ws = ar.take<char>(sort_b);
  if (!pair_key || !cnt || !start || !scan_ws || !tot || !ikeys || !ivals || !itmp || !sort_ws)
    return PG_ERR_WORKSPACE;
  const unsigned gP = pg_blocks(n_pairs, 256);
  k_pair_keys_of<<<gP, 256, 0, s>>>(members, pair_start, n_pairs, elemsE, elemsF, E, pair_key, cnt);
  k_partner<<<gP, 256, 0, s>>>(pair_key, n_pairs, E, pair_partner);
  int st = pg::scan_exclusive_i32(cnt, start, n_pairs, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_items<<<gP, 256, 0, s>>>(cnt, start, n_pairs, itmp);
  k_store_i64<<<1, 1, 0, s>>>(tot, n_items);
  // bucket items by member count (stable), so warps see uniform loop trip counts
  int32_t h_tot = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&h_tot, tot, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_tot > max_items) {
    pg_set_error("pg_pattern_items: max_items too small");
    return PG_ERR_ARG;
  }
  const unsigned gI = pg_blocks(h_tot > 0 ? h_tot : 1, 256);
  k_item_keys<<<gI, 256, 0, s>>>(itmp, tot, pair_start, ikeys, ivals);
  st = pg::sort_pairs(ikeys, ivals, h_tot, 8, sort_ws, sort_b, s);
  if (st) return st;
  k_item_gather<<<gI, 256, 0, s>>>(itmp, tot, ivals, items);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_assemble_fused(const double* coef, const int32_t* tuple_of_elem, const double* tables,
                                 const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                                 const int32_t* pair_partner, const int64_t* items, int64_t n_items, int64_t n_pairs,
                                 const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE,
                                 int64_t nF, int p, const int64_t* rowptr, double* vals, void* stream) {
  if (p < 1 || p > 6 || n_pairs < 1 || n_items < 1 || !coef || !tuple_of_elem || !tables || !members ||
      !pair_start || !pair_colstart || !pair_partner || !items || !rowptr || !vals) {
    pg_set_error("pg_assemble_fused: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  double2* v = reinterpret_cast<double2*>(vals);
  int64_t blocks = (n_items + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  const unsigned grid = (unsigned)blocks;
#define PG_SYM(P) k_values_sym<P><<<grid, 256, 0, s>>>(coef, tuple_of_elem, tables, members, pair_start, pair_colstart, \
                                                       pair_partner, items, n_items, elemsE, elemsF, nE, nF, n_elems,   \
                                                       rowptr, nullptr, v)
  switch (p) {
    case 1: PG_SYM(1); break;
    case 2: PG_SYM(2); break;
    case 3: PG_SYM(3); break;
    case 4: PG_SYM(4); break;
    case 5: PG_SYM(5); break;
    case 6: PG_SYM(6); break;
  }
#undef PG_SYM
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_apply_pec(const int64_t* rowptr, const int32_t* col, double* vals, int64_t n_dofs,
                            const int32_t* bnd, int64_t n_bnd, double* b, uint8_t* flag_ws, void* stream) {
  if (n_dofs < 1 || !rowptr || !col || !vals || !flag_ws || (n_bnd > 0 && !bnd)) {
    pg_set_error("pg_apply_pec: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  PG_CUDA_TRY(cudaMemsetAsync(flag_ws, 0, (size_t)n_dofs, s));
  if (n_bnd > 0)
    k_mark_bnd<<<pg_blocks(n_bnd, 256), 256, 0, s>>>(bnd, n_bnd, flag_ws, reinterpret_cast<double2*>(b));
  k_pec<<<warp_grid(n_dofs), 256, 0, s>>>(rowptr, col, reinterpret_cast<double2*>(vals), n_dofs, flag_ws);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_to_double_float(const double* in, int64_t n, float* out_pairs, void* stream) {
  if (n < 1 || !in || !out_pairs) {
    pg_set_error("pg_to_double_float: bad argument");
    return PG_ERR_ARG;
  }
  k_to_df<<<pg_blocks(n, 256), 256, 0, pg_stream(stream)>>>(in, n, reinterpret_cast<float2*>(out_pairs));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_pec_flags(const int32_t* bnd, int64_t n_bnd, int64_t n_dofs, uint8_t* flags, void* stream) {
  if (n_dofs < 1 || !flags || (n_bnd > 0 && !bnd)) {
    pg_set_error("pg_pec_flags: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  PG_CUDA_TRY(cudaMemsetAsync(flags, 0, (size_t)n_dofs, s));
  if (n_bnd > 0) k_mark_bnd<<<pg_blocks(n_bnd, 256), 256, 0, s>>>(bnd, n_bnd, flags, nullptr);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_pec_rhs(const int32_t* bnd, int64_t n_bnd, int nrhs, double* b, void* stream) {
  if (nrhs < 1 || !b || (n_bnd > 0 && !bnd)) {
    pg_set_error("pg_pec_rhs: bad argument");
    return PG_ERR_ARG;
  }
  if (n_bnd > 0)
    k_pec_rhs<<<pg_blocks(n_bnd * nrhs, 256), 256, 0, pg_stream(stream)>>>(bnd, n_bnd, nrhs,
                                                                           reinterpret_cast<double2*>(b));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_assemble_fused_ex(const void* coef, const int32_t* tuple_of_elem, const void* tables,
                                    const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                                    const int32_t* pair_partner, const int64_t* items, int64_t n_items,
                                    int64_t n_pairs, const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems,
                                    int64_t nE, int64_t nF, int p, const int64_t* rowptr, const uint8_t* pec_flags,
                                    int arithmetic, double* vals, void* stream) {
  if (p < 1 || p > 6 || n_pairs < 1 || n_items < 1 || !coef || !tuple_of_elem || !tables || !members ||
      !pair_start || !pair_colstart || !pair_partner || !items || !rowptr || !vals ||
      (arithmetic != 0 && arithmetic != 1)) {
    pg_set_error("pg_assemble_fused_ex: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  double2* v = reinterpret_cast<double2*>(vals);
  int64_t blocks = (n_items + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  const unsigned grid = (unsigned)blocks;
  if (arithmetic == 0) {
    const double* c = reinterpret_cast<const double*>(coef);
    const double* tb = reinterpret_cast<const double*>(tables);
#define PG_SYM64(P) k_values_sym<P><<<grid, 256, 0, s>>>(c, tuple_of_elem, tb, members, pair_start, pair_colstart, \
                                                         pair_partner, items, n_items, elemsE, elemsF, nE, nF, n_elems, \
                                                         rowptr, pec_flags, v)
    switch (p) {
      case 1: PG_SYM64(1); break;
      case 2: PG_SYM64(2); break;
      case 3: PG_SYM64(3); break;
      case 4: PG_SYM64(4); break;
      case 5: PG_SYM64(5); break;
      case 6: PG_SYM64(6); break;
    }
#undef PG_SYM64
  } else {
    const float2* c = reinterpret_cast<const float2*>(coef);
    const float2* tb = reinterpret_cast<const float2*>(tables);
#define PG_SYMDF(P) k_values_sym_df<P><<<grid, 256, 0, s>>>(c, tuple_of_elem, tb, members, pair_start, pair_colstart, \
                                                            pair_partner, items, n_items, elemsE, elemsF, nE, nF,      \
                                                            n_elems, rowptr, pec_flags, v)
    switch (p) {
      case 1: PG_SYMDF(1); break;
      case 2: PG_SYMDF(2); break;
      case 3: PG_SYMDF(3); break;
      case 4: PG_SYMDF(4); break;
      case 5: PG_SYMDF(5); break;
      case 6: PG_SYMDF(6); break;
    }
#undef PG_SYMDF
  }
  PG_LAUNCH_CHECK();
  return PG_OK;
}

// ---- assembly records: the per-mesh part of the work list resolved once ----
// One record per item of the symmetric work list, in the same order: the
// output position of the entry, the position of its transpose, the pair's
// first member and a meta word.  The per-model pass then reads the record,
// the members, each member's element coefficients and one table entry: three
// dependent loads instead of the item -> pair -> member -> entity -> rowptr
// chain.  (Records covering two columns halve the coefficient loads but need
// ~2x the registers; on GB300 the lost occupancy cost more than the loads.)
namespace {

// meta: member count (8 bits) | i (6) << 8 | j (6) << 14 | flags
constexpr uint32_t REC_HAS_T = 1u << 20;   // transpose position present
constexpr uint32_t REC_PEC_ZERO = 1u << 21;
constexpr uint32_t REC_PEC_ONE = 1u << 22;

struct ItemView {
  int64_t g, a, b, fa, fb;
  int32_t s0, s1;
  int na, nb, i, j;
};

// decode one item (pair << 12 | entry) of the symmetric work list
__device__ __forceinline__ ItemView view_item(int64_t it, const int32_t* members, const int32_t* pair_start,
                                              const int32_t* elemsE, const int32_t* elemsF, const Ent& E) {
  ItemView v;
  v.g = it >> 12;
  int t = (int)(it & 4095);
  v.s0 = pair_start[v.g];
  v.s1 = pair_start[v.g + 1];
  const int NL = E.nl, NL2 = E.nl * E.nl;
  const int32_t m0 = members[v.s0];
  const int64_t e0 = m0 / NL2;
  const int r0 = m0 % NL2;
  v.a = E.ent(elemsE, elemsF, e0, r0 / NL);
  v.b = E.ent(elemsE, elemsF, e0, r0 % NL);
  v.na = E.nd_ent(v.a);
  v.nb = E.nd_ent(v.b);
  if (v.a != v.b) {
    v.i = t / v.nb;
    v.j = t - v.i * v.nb;
  } else {
    int i = 0;
    while (t >= v.na - i) { t -= v.na - i; ++i; }
    v.i = i;
    v.j = i + t;
  }
  v.fa = E.first_dof(v.a);
  v.fb = E.first_dof(v.b);
  return v;
}

struct RecS {   // nnz < 2^31
  int32_t pos, tpos, s0;
  uint32_t meta;
};
struct RecL {
  int64_t pos, tpos;
  int32_t s0;
  uint32_t meta;
};
__device__ __forceinline__ void rec_put(RecS* r, int64_t idx, int64_t p1, int64_t p2, int32_t s0, uint32_t meta) {
  reinterpret_cast<int4*>(r)[idx] = make_int4((int32_t)p1, (int32_t)p2, s0, (int32_t)meta);
}
__device__ __forceinline__ void rec_put(RecL* r, int64_t idx, int64_t p1, int64_t p2, int32_t s0, uint32_t meta) {
  long long* q = reinterpret_cast<long long*>(r + idx);
  q[0] = p1;
  q[1] = p2;
  q[2] = (long long)(((unsigned long long)meta << 32) | (uint32_t)s0);
}
__device__ __forceinline__ void rec_get(const RecS* r, int64_t idx, int64_t& p1, int64_t& p2, int32_t& s0,
                                        uint32_t& meta) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(r) + idx);
  p1 = v.x;
  p2 = v.y;
  s0 = v.z;
  meta = (uint32_t)v.w;
}
__device__ __forceinline__ void rec_get(const RecL* r, int64_t idx, int64_t& p1, int64_t& p2, int32_t& s0,
                                        uint32_t& meta) {
  const long long* q = reinterpret_cast<const long long*>(r + idx);   // 8-byte aligned only
  p1 = __ldg(q);
  p2 = __ldg(q + 1);
  const unsigned long long w = (unsigned long long)__ldg(q + 2);
  s0 = (int32_t)(uint32_t)(w & 0xffffffffull);
  meta = (uint32_t)(w >> 32);
}

template <typename R>
__global__ void k_records(const int64_t* __restrict__ items, int64_t n_items, const int32_t* __restrict__ members,
                          const int32_t* __restrict__ pair_start, const int32_t* __restrict__ colstart,
                          const int32_t* __restrict__ partner, const int32_t* __restrict__ elemsE,
                          const int32_t* __restrict__ elemsF, Ent E, const int64_t* __restrict__ rowptr,
                          const uint8_t* __restrict__ pec, R* __restrict__ recs, int32_t* __restrict__ status) {
  GRID_STRIDE(idx, n_items) {
    const ItemView v = view_item(items[idx], members, pair_start, elemsE, elemsF, E);
    const int64_t row = v.fa + v.i, col = v.fb + v.j;
    const int64_t p1 = rowptr[row] + colstart[v.g] + v.j;
    int64_t p2 = 0;
    uint32_t meta = (uint32_t)(v.s1 - v.s0) | ((uint32_t)v.i << 8) | ((uint32_t)v.j << 14);
    if (v.a != v.b) {
      p2 = rowptr[col] + colstart[partner[v.g]] + v.i;
      meta |= REC_HAS_T;
    } else if (v.i != v.j) {
      p2 = rowptr[v.fa + v.j] + colstart[v.g] + v.i;
      meta |= REC_HAS_T;
    }
    if (v.s1 - v.s0 > 255) *status = PG_ERR_UNSUPPORTED;
    if (pec && (pec[row] | pec[col])) meta |= (row == col) ? REC_PEC_ONE : REC_PEC_ZERO;
    rec_put(recs, idx, p1, p2, v.s0, meta);
  }
}

// tables [U][12][NT] (mass R^ab, then stiffness Q^ab) -> entry-major
// [U][NT][12] ordered like the coefficients (stiffness first, then mass), as
// doubles or as (hi, lo) double-float pairs
template <typename C>
__global__ void k_tables_entry_major(const double* __restrict__ in, int64_t U, int NT, C* __restrict__ out) {
  GRID_STRIDE(x, U * NT * 12) {
    const int k = (int)(x % 12);
    const int64_t ue = x / 12;
    const int64_t u = ue / NT;
    const int en = (int)(ue - u * NT);
    const int src_k = k < 6 ? 6 + k : k - 6;
    put_coef(out + x, 0, in[(u * 12 + src_k) * NT + en]);
  }
}

template <typename C>
struct Pack12;
template <>
struct Pack12<double> {
  double2 v[6];
  __device__ __forceinline__ void load(const double* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int k = 0; k < 6; ++k) v[k] = __ldg(q + k);
  }
};
template <>
struct Pack12<float2> {
  float4 v[6];
  __device__ __forceinline__ void load(const float2* p) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int k = 0; k < 6; ++k) v[k] = __ldg(q + k);
  }
};

struct AccD {
  double re = 0.0, im = 0.0;
  __device__ __forceinline__ void mac(const Pack12<double>& c, const Pack12<double>& t) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      re = fma(c.v[k].x, t.v[k].x, re);
      re = fma(c.v[k].y, t.v[k].y, re);
      im = fma(c.v[3 + k].x, t.v[3 + k].x, im);
      im = fma(c.v[3 + k].y, t.v[3 + k].y, im);
    }
  }
  __device__ __forceinline__ double2 value() const { return make_double2(re, im); }
};
struct AccDF {
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  __device__ __forceinline__ void mac(const Pack12<float2>& c, const Pack12<float2>& t) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      df_mac(rh, rl, c.v[k].x, c.v[k].y, t.v[k].x, t.v[k].y);
      df_mac(rh, rl, c.v[k].z, c.v[k].w, t.v[k].z, t.v[k].w);
      df_mac(ih, il, c.v[3 + k].x, c.v[3 + k].y, t.v[3 + k].x, t.v[3 + k].y);
      df_mac(ih, il, c.v[3 + k].z, c.v[3 + k].w, t.v[3 + k].z, t.v[3 + k].w);
    }
  }
  __device__ __forceinline__ double2 value() const {
    return make_double2(df_to_double(rh, rl), df_to_double(ih, il));
  }
};

template <int P, typename C, typename Acc, typename R>
__global__ void __launch_bounds__(256) k_values_rec(const C* __restrict__ coef, const int32_t* __restrict__ tuple_of_elem,
                                                    const C* __restrict__ tables, const int32_t* __restrict__ members,
                                                    const R* __restrict__ recs, int64_t n_items, int apply_pec,
                                                    double2* __restrict__ vals) {
  constexpr int NL = P == 1 ? 6 : (P == 2 ? 10 : 11);
  constexpr int NL2 = NL * NL;
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  constexpr int NT = ND * (ND + 1) / 2;
  constexpr int DE = P, DF = P * (P - 1);
  GRID_STRIDE(idx, n_items) {
    int64_t p1, p2;
    int32_t s0;
    uint32_t meta;
    rec_get(recs, idx, p1, p2, s0, meta);
    double2 v;
    if (apply_pec && (meta & (REC_PEC_ZERO | REC_PEC_ONE))) {
      v = make_double2((meta & REC_PEC_ONE) ? 1.0 : 0.0, 0.0);
    } else {
      const int c = (int)(meta & 255u);
      const int i = (int)((meta >> 8) & 63u), j = (int)((meta >> 14) & 63u);
      Acc acc;
      auto entry = [&](int32_t m, const C*& cf, const C*& tb) {
        const int e = m / NL2;
        const int r = m - e * NL2;
        const int la = r / NL, lb = r - la * NL;
        const int ja = (la < 6 ? la * DE : (la < 10 ? 6 * DE + (la - 6) * DF : 6 * DE + 4 * DF)) + i;
        const int kb = (lb < 6 ? lb * DE : (lb < 10 ? 6 * DE + (lb - 6) * DF : 6 * DE + 4 * DF)) + j;
        cf = coef + 12 * (int64_t)e;
        tb = tables + ((int64_t)__ldg(tuple_of_elem + e) * NT + packed_index(ja, kb, ND)) * 12;
      };
      int32_t q = s0;
      const int32_t qe = s0 + c;
      for (; q + 1 < qe; q += 2) {
        const C *cfa, *tba, *cfb, *tbb;
        entry(__ldg(members + q), cfa, tba);
        entry(__ldg(members + q + 1), cfb, tbb);
        Pack12<C> ca, ta, cb, tbv;
        ca.load(cfa);
        ta.load(tba);
        cb.load(cfb);
        tbv.load(tbb);
        acc.mac(ca, ta);
        acc.mac(cb, tbv);
      }
      if (q < qe) {
        const C *cfa, *tba;
        entry(__ldg(members + q), cfa, tba);
        Pack12<C> ca, ta;
        ca.load(cfa);
        ta.load(tba);
        acc.mac(ca, ta);
      }
      v = acc.value();
    }
    vals[p1] = v;
    if (meta & REC_HAS_T) vals[p2] = v;
  }
}

}  // namespace

extern "C" int64_t pg_assembly_record_bytes(int64_t nnz) { return nnz < (1ll << 31) ? 16 : 24; }

extern "C" int pg_assembly_records(const int32_t* members, const int32_t* pair_start, const int32_t* pair_colstart,
                                   const int32_t* pair_partner, const int64_t* items, int64_t n_items,
                                   const int32_t* elemsE, const int32_t* elemsF, int64_t n_elems, int64_t nE,
                                   int64_t nF, int p, const int64_t* rowptr, int64_t nnz, const uint8_t* pec_flags,
                                   void* records, int32_t* status, void* stream) {
  if (p < 1 || p > 6 || n_items < 1 || nnz < 1 || !members || !pair_start || !pair_colstart || !pair_partner ||
      !items || !elemsE || !elemsF || !rowptr || !records || !status) {
    pg_set_error("pg_assembly_records: bad argument");
    return PG_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(records) & 15) != 0) {
    pg_set_error("pg_assembly_records: records must be 16-byte aligned");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  const Ent E(nE, nF, n_elems, p);
  const unsigned g = pg_blocks(n_items, 256);
  if (pg_assembly_record_bytes(nnz) == 16)
    k_records<<<g, 256, 0, s>>>(items, n_items, members, pair_start, pair_colstart, pair_partner, elemsE, elemsF, E,
                                rowptr, pec_flags, reinterpret_cast<RecS*>(records), status);
  else
    k_records<<<g, 256, 0, s>>>(items, n_items, members, pair_start, pair_colstart, pair_partner, elemsE, elemsF, E,
                                rowptr, pec_flags, reinterpret_cast<RecL*>(records), status);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_tuple_tables_entry_major(const double* tables, int64_t n_tuples, int p, int arithmetic, void* out,
                                           void* stream) {
  if (p < 1 || p > 6 || n_tuples < 1 || !tables || !out || (arithmetic != 0 && arithmetic != 1)) {
    pg_set_error("pg_tuple_tables_entry_major: bad argument");
    return PG_ERR_ARG;
  }
  const int nd = p * (p + 2) * (p + 3) / 2;
  const int NT = nd * (nd + 1) / 2;
  cudaStream_t s = pg_stream(stream);
  const unsigned g = pg_blocks(n_tuples * NT * 12, 256);
  if (arithmetic == 0)
    k_tables_entry_major<<<g, 256, 0, s>>>(tables, n_tuples, NT, reinterpret_cast<double*>(out));
  else
    k_tables_entry_major<<<g, 256, 0, s>>>(tables, n_tuples, NT, reinterpret_cast<float2*>(out));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_assemble_records(const void* coef, const int32_t* tuple_of_elem, const void* tables_entry_major,
                                   const int32_t* members, const void* records, int64_t n_items, int64_t nnz, int p,
                                   int arithmetic, int apply_pec, double* vals, void* stream) {
  if (p < 1 || p > 6 || n_items < 1 || nnz < 1 || !coef || !tuple_of_elem || !tables_entry_major || !members ||
      !records || !vals || (arithmetic != 0 && arithmetic != 1)) {
    pg_set_error("pg_assemble_records: bad argument");
    return PG_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(coef) | reinterpret_cast<uintptr_t>(tables_entry_major) |
       reinterpret_cast<uintptr_t>(records) | reinterpret_cast<uintptr_t>(vals)) & 15) {
    pg_set_error("pg_assemble_records: coef, tables, records and vals must be 16-byte aligned");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  double2* v = reinterpret_cast<double2*>(vals);
  int64_t blocks = (n_items + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  const unsigned grid = (unsigned)blocks;
  const bool small = pg_assembly_record_bytes(nnz) == 16;
#define PG_REC(P, C, A, R)                                                                                \
  k_values_rec<P, C, A, R><<<grid, 256, 0, s>>>(reinterpret_cast<const C*>(coef), tuple_of_elem,        \
                                                reinterpret_cast<const C*>(tables_entry_major), members, \
                                                reinterpret_cast<const R*>(records), n_items, apply_pec, v)
#define PG_REC_P(C, A, R)              \
  switch (p) {                         \
    case 1: PG_REC(1, C, A, R); break; \
    case 2: PG_REC(2, C, A, R); break; \
    case 3: PG_REC(3, C, A, R); break; \
    case 4: PG_REC(4, C, A, R); break; \
    case 5: PG_REC(5, C, A, R); break; \
    case 6: PG_REC(6, C, A, R); break; \
  }
  if (arithmetic == 0) {
    if (small) { PG_REC_P(double, AccD, RecS) } else { PG_REC_P(double, AccD, RecL) }
  } else {
    if (small) { PG_REC_P(float2, AccDF, RecS) } else { PG_REC_P(float2, AccDF, RecL) }
  }
#undef PG_REC_P
#undef PG_REC
  PG_LAUNCH_CHECK();
  return PG_OK;
}

// ---- per-element bilinear form of the mass term (adjoint contraction) --------
// out[e] = y_e^T (sum_t cM_t R^t) x_e = y_e^T (-omega mu M_e) x_e with x_e, y_e
// the element's DOF values; one warp per element, packed symmetric entries
// over the lanes, fixed-order warp reduction.
namespace {

// inverse of packed_index: row j (the largest with start(j) <= t) and column k
__device__ __forceinline__ void unpack_index(int t, int nd, int& j, int& k) {
  const float b = 2.0f * nd + 1.0f;
  int r = (int)floorf(0.5f * (b - sqrtf(fmaxf(b * b - 8.0f * t, 0.0f))));
  r = max(0, min(r, nd - 1));
  while (r > 0 && r * nd - r * (r - 1) / 2 > t) --r;
  while (r + 1 < nd && (r + 1) * nd - (r + 1) * r / 2 <= t) ++r;
  j = r;
  k = r + (t - (r * nd - r * (r - 1) / 2));
}

template <int P>
__global__ void __launch_bounds__(256) k_mass_bilinear(const double* __restrict__ coef,
                                                       const int32_t* __restrict__ tuple_of_elem,
                                                       const double* __restrict__ tables,
                                                       const int32_t* __restrict__ dofs, const double2* __restrict__ x,
                                                       const double2* __restrict__ y, int64_t T,
                                                       double2* __restrict__ out) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  constexpr int NT = ND * (ND + 1) / 2;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < T; e += warps) {
    const int32_t* de = dofs + e * ND;
    const double* tb = tables + (int64_t)tuple_of_elem[e] * (12 * NT);
    double qr[6] = {0, 0, 0, 0, 0, 0}, qi[6] = {0, 0, 0, 0, 0, 0};
    for (int t = lane; t < NT; t += 32) {
      int j, k;
      unpack_index(t, ND, j, k);
      const double2 yj = y[de[j]], xk = x[de[k]];
      double sr = yj.x * xk.x - yj.y * xk.y, si = yj.x * xk.y + yj.y * xk.x;
      if (j != k) {
        const double2 yk = y[de[k]], xj = x[de[j]];
        sr += yk.x * xj.x - yk.y * xj.y;
        si += yk.x * xj.y + yk.y * xj.x;
      }
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        const double r = tb[a * NT + t];
        qr[a] = fma(r, sr, qr[a]);
        qi[a] = fma(r, si, qi[a]);
      }
    }
#pragma unroll
    for (int a = 0; a < 6; ++a)
      for (int off = 16; off > 0; off >>= 1) {
        qr[a] += __shfl_xor_sync(0xffffffffu, qr[a], off);
        qi[a] += __shfl_xor_sync(0xffffffffu, qi[a], off);
      }
    if (lane == 0) {
      double orr = 0.0, oi = 0.0;
      for (int a = 0; a < 6; ++a) {
        const double c = coef[12 * e + 6 + a];
        orr = fma(c, qr[a], orr);
        oi = fma(c, qi[a], oi);
      }
      out[e] = make_double2(orr, oi);
    }
  }
}

}  // namespace

extern "C" int pg_element_mass_bilinear(const double* coef, const int32_t* tuple_of_elem, const double* tables,
                                        const int32_t* dofs, const double* x, const double* y, int64_t n_elems,
                                        int p, double* out, void* stream) {
  if (p < 1 || p > 6 || n_elems < 1 || !coef || !tuple_of_elem || !tables || !dofs || !x || !y || !out) {
    pg_set_error("pg_element_mass_bilinear: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  int64_t blocks = (n_elems + 7) / 8;
  if (blocks > 152 * 32) blocks = 152 * 32;
  const unsigned grid = (unsigned)blocks;
  const double2* xx = reinterpret_cast<const double2*>(x);
  const double2* yy = reinterpret_cast<const double2*>(y);
  double2* o = reinterpret_cast<double2*>(out);
#define PG_MB(P) k_mass_bilinear<P><<<grid, 256, 0, s>>>(coef, tuple_of_elem, tables, dofs, xx, yy, n_elems, o)
  switch (p) {
    case 1: PG_MB(1); break;
    case 2: PG_MB(2); break;
    case 3: PG_MB(3); break;
    case 4: PG_MB(4); break;
    case 5: PG_MB(5); break;
    case 6: PG_MB(6); break;
  }
#undef PG_MB
  PG_LAUNCH_CHECK();
  return PG_OK;
}
