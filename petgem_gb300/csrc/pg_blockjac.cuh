// Entity block-Jacobi scaling for the COCG solvers.
//
// DOFs are numbered entity by entity (hvfem.py:15-98): p per edge, p(p-1) per
// face, p(p-1)(p-2)/2 per volume, so the diagonal blocks of A are the
// (entity, entity) blocks of its pattern.  Each block is factored as
// A_aa = L D L^T (complex symmetric, no pivoting) and S_a = D^(-1/2) L^(-1);
// the solver then runs on S A S^T, which stays complex symmetric, with
// b~ = S b and x = S^T y.  Rows of one entity share the same column list
// (the pattern is built in entity-pair blocks) and the columns of one entity
// are contiguous in a row, so S_a A_ab S_b^T is formed row by row without
// searching.  Blocks larger than PG_BJ_MAX fall back to diagonal scaling.
#pragma once
#include "pg_common.cuh"

#define PG_BJ_MAX 12

struct BjInfo {
  int64_t nE, nF, nV;
  int p;
  int64_t n;
  int64_t c0 = 0;   // column index of DOF 0 (a system stored inside a larger block-diagonal matrix)
  __host__ __device__ int de() const { return p; }
  __host__ __device__ int df() const { return p * (p - 1); }
  __host__ __device__ int dv() const { return p * (p - 1) * (p - 2) / 2; }
  // block of DOF r: first DOF, size, local index, offset of its S block
  __device__ void block(int64_t r, int64_t& first, int& size, int& local, int64_t& soff) const {
    const int64_t ne = nE * de(), nf = nF * (int64_t)df();
    if (r < ne) {
      const int64_t a = r / de();
      first = a * de();
      size = de();
      soff = a * de() * de();
    } else if (r < ne + nf) {
      const int64_t a = (r - ne) / df();
      first = ne + a * df();
      size = df();
      soff = nE * (int64_t)de() * de() + a * (int64_t)df() * df();
    } else {
      const int64_t a = (r - ne - nf) / dv();
      first = ne + nf + a * dv();
      size = dv();
      soff = nE * (int64_t)de() * de() + nF * (int64_t)df() * df() + a * (int64_t)dv() * dv();
    }
    local = (int)(r - first);
  }
  __host__ __device__ int64_t s_size() const {
    return nE * (int64_t)de() * de() + nF * (int64_t)df() * df() + nV * (int64_t)dv() * dv();
  }
  __host__ __device__ int64_t n_blocks() const { return nE + (df() ? nF : 0) + (dv() ? nV : 0); }
};

// the kernels below are compiled into every solver translation unit
namespace {

__device__ __forceinline__ double2 bj_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 bj_div(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// principal 1/sqrt(z)
__device__ __forceinline__ double2 bj_rsqrt(double2 z) {
  const double m = sqrt(z.x * z.x + z.y * z.y);
  double sr = sqrt(0.5 * (m + z.x));
  double si = sqrt(fmax(0.0, 0.5 * (m - z.x)));
  if (z.y < 0) si = -si;
  return bj_div(make_double2(1.0, 0.0), make_double2(sr, si));
}

// position of column c in row r (binary search; the column is present)
__device__ __forceinline__ int64_t bj_find(const int64_t* rowptr, const int32_t* col, int64_t r, int64_t c) {
  int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// one thread per block: S_a (row-major na x na, lower triangular), wd = |D|
__global__ void k_bj_factor(const int64_t* rowptr, const int32_t* col, const double2* val, BjInfo B, double2* S,
                            double* wd, int* status) {
  for (int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r0 < B.n; r0 += (int64_t)gridDim.x * blockDim.x) {
    int64_t first, soff;
    int na, loc;
    B.block(r0, first, na, loc, soff);
    if (loc != 0) continue;             // the block's first DOF does the work
    double2* Sa = S + soff;
    if (na > PG_BJ_MAX) {
      for (int i = 0; i < na; ++i) {
        for (int j = 0; j < na; ++j) Sa[i * na + j] = make_double2(0.0, 0.0);
        const int64_t k = bj_find(rowptr, col, first + i, B.c0 + first + i);
        const double2 d = val[k];
        if (d.x == 0.0 && d.y == 0.0) *status = PG_ERR_BREAKDOWN;
        Sa[i * na + i] = bj_rsqrt(d);
        wd[first + i] = sqrt(d.x * d.x + d.y * d.y);
      }
      continue;
    }
    double2 W[PG_BJ_MAX][PG_BJ_MAX], L[PG_BJ_MAX][PG_BJ_MAX], D[PG_BJ_MAX];
    for (int i = 0; i < na; ++i) {
      const int64_t k = bj_find(rowptr, col, first + i, B.c0 + first);
      for (int j = 0; j < na; ++j) W[i][j] = val[k + j];
    }
    bool bad = false;
    for (int c = 0; c < na; ++c) {
      D[c] = W[c][c];
      if (D[c].x == 0.0 && D[c].y == 0.0) {
        bad = true;
        D[c] = make_double2(1.0, 0.0);
      }
      for (int i = 0; i < na; ++i) L[i][c] = make_double2(i == c ? 1.0 : 0.0, 0.0);
      for (int i = c + 1; i < na; ++i) L[i][c] = bj_div(W[i][c], D[c]);
      for (int i = c + 1; i < na; ++i)
        for (int j = c + 1; j < na; ++j) {
          const double2 t = bj_mul(bj_mul(L[i][c], D[c]), L[j][c]);
          W[i][j].x -= t.x;
          W[i][j].y -= t.y;
        }
    }
    if (bad) *status = PG_ERR_BREAKDOWN;
    // L^-1 (unit lower triangular) by forward substitution, row by row
    double2 Li[PG_BJ_MAX][PG_BJ_MAX];
    for (int i = 0; i < na; ++i)
      for (int j = 0; j < na; ++j) {
        double2 s = make_double2(i == j ? 1.0 : 0.0, 0.0);
        if (j < i)
          for (int t = j; t < i; ++t) {
            const double2 u = bj_mul(L[i][t], Li[t][j]);
            s.x -= u.x;
            s.y -= u.y;
          }
        Li[i][j] = j <= i ? s : make_double2(0.0, 0.0);
      }
    for (int i = 0; i < na; ++i) {
      const double2 di = bj_rsqrt(D[i]);
      for (int j = 0; j < na; ++j) Sa[i * na + j] = bj_mul(di, Li[i][j]);
      wd[first + i] = sqrt(D[i].x * D[i].x + D[i].y * D[i].y);
    }
  }
}

// out = S A S^T row by row (FP64), then converted to the solver's precision
template <typename CM, typename Conv>
__global__ void k_bj_scale_matrix(const int64_t* rowptr, const int32_t* col, const double2* val, BjInfo B,
                                  const double2* S, CM* out, Conv conv) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < B.n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t fa, sa;
    int na, i;
    B.block(r, fa, na, i, sa);
    const double2* Sa = S + sa;
    const int64_t base = rowptr[r];
    for (int64_t k = base; k < rowptr[r + 1]; ++k) {
      int64_t fb, sb;
      int nb, j;
      B.block(col[k] - B.c0, fb, nb, j, sb);
      const double2* Sb = S + sb;
      double2 acc = make_double2(0.0, 0.0);
      for (int ip = 0; ip <= i; ++ip) {
        const double2 sai = Sa[i * na + ip];
        if (sai.x == 0.0 && sai.y == 0.0) continue;
        const int64_t kr = rowptr[fa + ip] + (k - base) - j;   // entity b's first column in row fa + ip
        double2 inner = make_double2(0.0, 0.0);
        for (int jp = 0; jp <= j; ++jp) {
          const double2 sbj = Sb[j * nb + jp];
          if (sbj.x == 0.0 && sbj.y == 0.0) continue;
          const double2 t = bj_mul(val[kr + jp], sbj);
          inner.x += t.x;
          inner.y += t.y;
        }
        const double2 t = bj_mul(sai, inner);
        acc.x += t.x;
        acc.y += t.y;
      }
      out[k] = conv(acc);
    }
  }
}

// out[:, col] = S in[:, col] (block lower-triangular apply), K columns
template <int K>
__global__ void k_bj_apply(const double2* S, BjInfo B, const double2* in, double2* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < B.n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int c = (int)(e % K);
    int64_t fa, sa;
    int na, i;
    B.block(r, fa, na, i, sa);
    double2 acc = make_double2(0.0, 0.0);
    for (int ip = 0; ip <= i; ++ip) {
      const double2 t = bj_mul(S[sa + i * na + ip], in[(fa + ip) * K + c]);
      acc.x += t.x;
      acc.y += t.y;
    }
    out[e] = acc;
  }
}

// x[:, col] += S^T y[:, col]; Y converts the solver's y element to double2
template <int K, typename YT, typename Y>
__global__ void k_bj_apply_t_add(const double2* S, BjInfo B, const YT* y, double2* x, Y toD) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < B.n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int c = (int)(e % K);
    int64_t fa, sa;
    int na, i;
    B.block(r, fa, na, i, sa);
    double2 acc = x[e];
    for (int ip = i; ip < na; ++ip) {
      const double2 t = bj_mul(S[sa + ip * na + i], toD(y[(fa + ip) * K + c]));
      acc.x += t.x;
      acc.y += t.y;
    }
    x[e] = acc;
  }
}

}  // namespace
