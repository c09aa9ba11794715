// Several independent complex-symmetric systems in one double-float COCG
// (pg_cocg_segments).
#include "pg_cocg.cuh"

namespace {

// ---- several systems in one solve -------------------------------------------
// Independent complex-symmetric systems (meshes of different sizes, or one
// mesh at several frequencies) stored as one block-diagonal CSR matrix: system
// j owns rows [row[j], row[j+1]) and only references its own columns.  Each
// system keeps its own COCG scalars, convergence test and iteration count, so
// the result is the one each would reach alone, while every launch covers all
// of them: small systems no longer leave most of the GPU idle, and one graph
// replay advances every system.  Every launch splits its blocks over the
// systems in proportion to their rows (blk[j] .. blk[j+1] - 1 for system j),
// so a block's partial sums belong to one system and the per-system totals
// are fixed-order sums over that block range.
struct Seg {
  const int64_t* row;   // [S + 1] first row of each system (device)
  const int* blk;       // [S + 1] first block of each system (device)
  int S;
};

struct SegPos {
  int j, lb, nbj;       // system, block index inside it, blocks it owns
  int64_t r0, r1;       // its rows
};

__device__ __forceinline__ SegPos seg_pos(const Seg& g) {
  __shared__ int sj;
  if (threadIdx.x == 0) {
    int lo = 0, hi = g.S - 1;   // largest j with blk[j] <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.blk[mid] <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    sj = lo;
  }
  __syncthreads();
  SegPos p;
  p.j = sj;
  p.lb = (int)blockIdx.x - g.blk[sj];
  p.nbj = g.blk[sj + 1] - g.blk[sj];
  p.r0 = g.row[sj];
  p.r1 = g.row[sj + 1];
  return p;
}

// sum of partial[b * K + rhs] over the blocks of system t / K (one warp; fixed order)
template <int K>
__device__ double2 seg_pair_sum(const double2* partial, const Seg& g, int t) {
  const int lane = threadIdx.x & 31, j = t / K, rhs = t % K;
  double2 acc = make_double2(0.0, 0.0);
  for (int b = g.blk[j] + lane; b < g.blk[j + 1]; b += 32) acc = dadd(acc, __ldcg(partial + (int64_t)b * K + rhs));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc = dadd(acc, shfl_xor(acc, off));
  return acc;
}

// 1 if some right-hand side of system j is iterating
template <int K>
__device__ int seg_live(const CgState* st, int j) {
  __shared__ int live;
  if (threadIdx.x == 0) live = 0;
  __syncthreads();
  if (threadIdx.x < K && st[j * K + threadIdx.x].active) atomicOr(&live, 1);
  __syncthreads();
  return live;
}

// 1 if some right-hand side of system j was updated in this iteration
template <int K>
__device__ int seg_due(const CgState* st, int j) {
  __shared__ int due;
  if (threadIdx.x == 0) due = 0;
  __syncthreads();
  if (threadIdx.x < K && st[j * K + threadIdx.x].beta_iter == 1) atomicOr(&due, 1);
  __syncthreads();
  return due;
}

template <int K>
__device__ void seg_alpha_final(const double2* partial, const Seg& g, CgState* st, CgCtl* ctl) {
  for (int t = threadIdx.x >> 5; t < g.S * K; t += kThreads / 32) {
    const double2 m = seg_pair_sum<K>(partial, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (S.active) {
        if (m.x == 0.0 && m.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.alpha = make_double2(0.0, 0.0);
        } else {
          S.alpha = ddiv(S.rho, m);
        }
      } else {
        S.alpha = make_double2(0.0, 0.0);
      }
    }
  }
  if (threadIdx.x == 0) ctl->counter = 0;
}

// GRAD (gradient correction): rho and beta are left to k_sg_prolong
template <int K, bool GRAD = false>
__device__ void seg_beta_final(const double2* prho, const double2* pw, const Seg& g, CgState* st, CgCtl* ctl,
                               double delta) {
  __shared__ int any, stop;
  if (threadIdx.x == 0) {
    any = 0;
    stop = 0;
  }
  __syncthreads();
  for (int t = threadIdx.x >> 5; t < g.S * K; t += kThreads / 32) {
    double2 rho = make_double2(0.0, 0.0);
    if constexpr (!GRAD) rho = seg_pair_sum<K>(prho, g, t);
    const double2 w = seg_pair_sum<K>(pw, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (S.active) {
        S.beta_iter = 1;
        S.its += 1;
        S.res = sqrt(w.x);
        if (!isfinite(S.res)) ctl->nonfinite = 1;
        if constexpr (!GRAD) {
          if (S.rho.x == 0.0 && S.rho.y == 0.0) {
            S.breakdown = 1;
            S.active = 0;
            S.beta = make_double2(0.0, 0.0);
          } else {
            S.beta = ddiv(rho, S.rho);
          }
          S.rho = rho;
        }
        if (S.res <= S.target || !isfinite(S.res)) S.active = 0;
        else if (S.res <= delta * S.res0 || S.res > 1e3 * S.res0) atomicOr(&stop, 1);
      } else {
        S.beta = make_double2(0.0, 0.0);
        S.beta_iter = 0;
      }
      if (S.active) atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any && !stop;
    ctl->pending = 1;
    ctl->counter = 0;
  }
}

// q = At p for every system (G lanes per (row, rhs) item; G > 1 only for one
// RHS), partial mu = p^T q; last block: alpha of every system
template <int K, int G, int U>
__global__ void __launch_bounds__(kThreads) k_sg_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, Seg g,
                                                      const float4* __restrict__ pv, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  static_assert(K == 1 || G == 1, "several lanes per item only for one right-hand side");
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  if (seg_live<K>(st, sp.j)) {
    const int64_t items = (sp.r1 - sp.r0) * K;
    const int lane = threadIdx.x % G;
    const int64_t groups = ((int64_t)sp.nbj * kThreads) / G;
    const int64_t gid = ((int64_t)sp.lb * kThreads + threadIdx.x) / G;
    const int64_t warp_base = gid - (threadIdx.x & 31) / G;
    for (int64_t iw = warp_base; iw < items; iw += groups) {
      const int64_t it = iw + (gid - warp_base);
      const bool valid = it < items;
      const int64_t r = sp.r0 + it / K;
      const int rhs = (int)(it % K);
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (valid) {
        const int64_t e = rowptr[r + 1];
        int64_t kk = rowptr[r] + lane;
        if (U == 2) {
          // two independent accumulators: two gathers in flight per lane
          float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
          for (; kk + G < e; kk += 2 * G) {
            const int32_t c0 = col[kk], c1 = col[kk + G];
            const float4 v0 = val[kk], v1 = val[kk + G];
            cdf_mac(acc, v0, pv[(int64_t)c0 * K + rhs]);
            cdf_mac(acc1, v1, pv[(int64_t)c1 * K + rhs]);
          }
          if (kk < e) cdf_mac(acc, val[kk], pv[(int64_t)col[kk] * K + rhs]);
          cdf_add(acc, acc1);
        } else {
          for (; kk < e; kk += G) cdf_mac(acc, val[kk], pv[(int64_t)col[kk] * K + rhs]);
        }
      }
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) cdf_add(acc, shfl_xor4(acc, off));
      if (valid && lane == 0) {
        acc = df_norm(acc);
        q[r * K + rhs] = acc;
        cdf_mac(mu, pv[r * K + rhs], acc);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) seg_alpha_final<K>(partial, g, st, ctl);
}

// one RHS, G lanes per group of R rows (the rows of one mesh entity share
// their column list); each lane issues the loads of B column steps before
// using them.  Every system's rows start at a multiple of R.
template <int R, int G, int B>
__global__ void __launch_bounds__(kThreads) k_sg_spmv_grpb(const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ col,
                                                           const float4* __restrict__ val, Seg g,
                                                           const float4* __restrict__ pv, float4* __restrict__ q,
                                                           double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  if (seg_live<1>(st, sp.j)) {
    const int64_t ngroups = (sp.r1 - sp.r0) / R;
    const int lane = threadIdx.x % G;
    const int64_t groups = ((int64_t)sp.nbj * kThreads) / G;
    const int64_t gid = ((int64_t)sp.lb * kThreads + threadIdx.x) / G;
    const int64_t warp_base = gid - (threadIdx.x & 31) / G;
    for (int64_t gw = warp_base; gw < ngroups; gw += groups) {
      const int64_t gi = gw + (gid - warp_base);
      const bool valid = gi < ngroups;
      const int64_t r0 = sp.r0 + gi * R;
      float4 acc[R];
#pragma unroll
      for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (valid) {
        int64_t off[R];
#pragma unroll
        for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
        const int len = (int)(rowptr[r0 + 1] - off[0]);
        for (int k0 = lane; k0 < len; k0 += G * B) {
          int c[B];
          float4 v[B][R], x[B];
#pragma unroll
          for (int j = 0; j < B; ++j) {
            const int k = k0 + j * G;
            c[j] = k < len ? col[off[0] + k] : 0;
#pragma unroll
            for (int i = 0; i < R; ++i) v[j][i] = k < len ? val[off[i] + k] : make_float4(0.f, 0.f, 0.f, 0.f);
          }
#pragma unroll
          for (int j = 0; j < B; ++j) x[j] = k0 + j * G < len ? pv[c[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int j = 0; j < B; ++j)
            if (k0 + j * G < len) {
#pragma unroll
              for (int i = 0; i < R; ++i) cdf_mac(acc[i], v[j][i], x[j]);
            }
        }
      }
#pragma unroll
      for (int i = 0; i < R; ++i)
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) cdf_add(acc[i], shfl_xor4(acc[i], o));
      if (valid && lane == 0) {
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const float4 a = df_norm(acc[i]);
          q[r0 + i] = a;
          cdf_mac(mu, pv[r0 + i], a);
        }
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) seg_alpha_final<1>(partial, g, st, ctl);
}

// K RHS: one thread per (group of R rows, rhs)
template <int K, int R>
__global__ void __launch_bounds__(kThreads) k_sg_spmm_grp(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const float4* __restrict__ val, Seg g,
                                                          const float4* __restrict__ pv, float4* __restrict__ q,
                                                          double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  const int rhs = threadIdx.x % K;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  if (seg_live<K>(st, sp.j)) {
    const int64_t items = ((sp.r1 - sp.r0) / R) * K;
    for (int64_t it = (int64_t)sp.lb * kThreads + threadIdx.x; it < items; it += (int64_t)sp.nbj * kThreads) {
      const int64_t r0 = sp.r0 + (it / K) * R;
      int64_t off[R];
#pragma unroll
      for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
      const int64_t len = rowptr[r0 + 1] - off[0];
      float4 acc[R];
#pragma unroll
      for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int64_t k = 0; k < len; ++k) {
        const float4 x = pv[(int64_t)col[off[0] + k] * K + rhs];
#pragma unroll
        for (int i = 0; i < R; ++i) cdf_mac(acc[i], val[off[i] + k], x);
      }
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 a = df_norm(acc[i]);
        q[(r0 + i) * K + rhs] = a;
        cdf_mac(mu, pv[(r0 + i) * K + rhs], a);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) seg_alpha_final<K>(partial, g, st, ctl);
}

// y += alpha p ; r -= alpha q with each system's alpha; partial rho and w.
// GRAD: also u = S^-1 r (FP32); rho and beta are left to k_sg_prolong.
template <int K, bool GRAD = false>
__global__ void __launch_bounds__(kThreads) k_sg_update(float4* __restrict__ y, float4* __restrict__ r,
                                                        const float4* __restrict__ pv, const float4* __restrict__ q,
                                                        const float* __restrict__ wd, Seg g, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, double delta,
                                                        float2* __restrict__ u = nullptr,
                                                        const float2* __restrict__ Sinv = nullptr) {
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  __shared__ float4 al[kMaxK];
  if (threadIdx.x < K) al[threadIdx.x] = cdf_from(st[sp.j * K + threadIdx.x].alpha);
  const int live = seg_live<K>(st, sp.j);   // synchronises al as well
  const float4 a = al[threadIdx.x % K];
  const float4 na = make_float4(-a.x, -a.y, -a.z, -a.w);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
  float ww = 0.f;
  if (live)
    for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
      float4 ye = y[e], re = r[e];
      cdf_mac(ye, a, pv[e]);
      cdf_mac(re, na, q[e]);
      ye = df_norm(ye);
      re = df_norm(re);
      y[e] = ye;
      r[e] = re;
      if constexpr (GRAD) {
        u[e] = cmul(Sinv[e / K], make_float2(re.x, re.z));
      } else {
        cdf_mac(rho, re, re);
      }
      ww += (re.x * re.x + re.z * re.z) * wd[e / K];
    }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  if constexpr (!GRAD) block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  block_reduce_f<K>(ww, reinterpret_cast<float*>(smf), pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) seg_beta_final<K, GRAD>(prho, pw, g, st, ctl, delta);
}

// Gradient correction, several systems: z = r + S^-1 (G t) over each
// block's own system rows (G is block-diagonal over the systems), partial
// rho = r^T z per block; in an iteration the last block sets every system's
// beta = rho / rho_old and rho for the RHS updated in it (beta_iter == 1).
// At a cycle start (start = 1) p = z when set_p.
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_prolong(const int64_t* __restrict__ gp,
                                                         const int32_t* __restrict__ gc,
                                                         const double* __restrict__ gv,
                                                         const float2* __restrict__ Sinv,
                                                         const float2* __restrict__ t,
                                                         const float4* __restrict__ r, Seg g,
                                                         float4* __restrict__ z, float4* __restrict__ pv, int set_p,
                                                         double2* prho, CgState* st, CgCtl* ctl, int start) {
  if (!start && !ctl->pending) return;
  const SegPos sp = seg_pos(g);
  // systems with no RHS updated in this iteration skip their rows (a
  // converged system keeps one block)
  const int due = start ? 1 : seg_due<K>(st, sp.j);
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = due ? min(base + total, lo + chunk) : lo;
  float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const int64_t row = e / K;
    const float2 acc = grad_row_sum<K>(gc, gv, t, gp[row], gp[row + 1], (int)(e % K));
    const float2 cr = cmul(Sinv[row], acc);
    const float4 re = r[e];
    float4 ze = re;
    df_add(ze.x, ze.y, cr.x, 0.f);
    df_add(ze.z, ze.w, cr.y, 0.f);
    ze = df_norm(ze);
    z[e] = ze;
    if (set_p) pv[e] = ze;
    cdf_mac(rho, re, ze);
  }
  block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  if (!start && arrive_last(&ctl->counter)) {
    for (int tt = threadIdx.x >> 5; tt < g.S * K; tt += kThreads / 32) {
      const double2 rr = seg_pair_sum<K>(prho, g, tt);
      if ((threadIdx.x & 31) == 0) {
        CgState& S = st[tt];
        if (S.beta_iter == 1) {
          if (S.rho.x == 0.0 && S.rho.y == 0.0) {
            S.breakdown = 1;
            S.active = 0;
            S.beta = make_double2(0.0, 0.0);
          } else {
            S.beta = ddiv(rr, S.rho);
          }
          S.rho = rr;
        } else {
          S.beta = make_double2(0.0, 0.0);
        }
      }
    }
    if (threadIdx.x == 0) ctl->counter = 0;
  }
}

template <int K>
__global__ void k_sg_u_start(const double2* __restrict__ r64, int64_t n, float2* __restrict__ u) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    u[e] = make_float2((float)r64[e].x, (float)r64[e].y);
}

// p = r + beta p with each system's beta
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_pupdate(float4* __restrict__ pv, const float4* __restrict__ r, Seg g,
                                                         const CgState* st, const CgCtl* ctl) {
  if (!ctl->pending) return;
  const SegPos sp = seg_pos(g);
  __shared__ float4 bt[kMaxK];
  __shared__ int use[kMaxK];
  __shared__ int anyuse;
  if (threadIdx.x == 0) anyuse = 0;
  __syncthreads();
  if (threadIdx.x < K) {
    const CgState& S = st[sp.j * K + threadIdx.x];
    bt[threadIdx.x] = cdf_from(S.beta);
    use[threadIdx.x] = S.beta_iter == 1;
    if (S.beta_iter == 1) atomicOr(&anyuse, 1);
  }
  __syncthreads();
  if (!anyuse) return;
  const int64_t hi = sp.r1 * K;
  for (int64_t e = sp.r0 * K + (int64_t)sp.lb * kThreads + threadIdx.x; e < hi; e += (int64_t)sp.nbj * kThreads)
    if (use[e % K]) {
      float4 v = r[e];
      cdf_mac(v, bt[e % K], pv[e]);
      pv[e] = df_norm(v);
    }
}

// r = S r64 (double-float), y = 0, first cycle p = r; partial rho (FP64)
template <int K>
__global__ void k_sg_start(const double2* __restrict__ r64, const double2* __restrict__ S, Seg g, float4* r, float4* y,
                           float4* pv, int set_p, double2* prho) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const SegPos sp = seg_pos(g);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 v = cmul(S[e / K], r64[e]);
    const float4 vf = cdf_from(v);
    r[e] = vf;
    y[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (set_p) pv[e] = vf;
    rho = dadd(rho, cmul(v, v));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
}

// per-block sums of |r|^2 per right-hand side
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_norm2(const double2* __restrict__ r, Seg g, double2* partial) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const SegPos sp = seg_pos(g);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  double s = 0.0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) s += dabs2(r[e]);
  block_reduce_rhs<K>(make_double2(s, 0.0), smem, partial + (int64_t)blockIdx.x * K);
}

template <int K>
__global__ void k_sg_norm_final(const double2* partial, Seg g, double* out) {
  for (int t = threadIdx.x >> 5; t < g.S * K; t += blockDim.x / 32) {
    const double2 s = seg_pair_sum<K>(partial, g, t);
    if ((threadIdx.x & 31) == 0) out[t] = sqrt(s.x);
  }
}

template <int K>
__global__ void k_sg_cycle_init(const double2* prho, Seg g, CgState* st, const double* rnorm, const double* target,
                                const int* want, CgCtl* ctl, int first) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int t = threadIdx.x >> 5; t < g.S * K; t += blockDim.x / 32) {
    const double2 rho = seg_pair_sum<K>(prho, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (first) {
        S.its = 0;
        S.breakdown = 0;
        S.beta_iter = 0;
      }
      S.rho = rho;
      S.target = target[t];
      S.res = rnorm[t];
      S.res0 = rnorm[t];
      S.active = want[t] && rnorm[t] > 0.0;
      S.alpha = S.beta = make_double2(0.0, 0.0);
      if (S.active) atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any;
    ctl->nonfinite = 0;
    ctl->counter = 0;
  }
}

__device__ __forceinline__ int seg_of_row(const Seg& g, int64_t r) {
  int lo = 0, hi = g.S - 1;   // largest j with row[j] <= r
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.row[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// v[r, c] *= f[system(r) * K + c] (FP64 vectors)
template <int K>
__global__ void k_sg_scale_d2(double2* v, Seg g, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    v[e] = dscale(f[seg_of_row(g, e / K) * K + e % K], v[e]);
}

// the same for double-float vectors
template <int K>
__global__ void k_sg_scale_df(float4* v, Seg g, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const double fc = f[seg_of_row(g, e / K) * K + e % K];
    const float fh = __double2float_rn(fc);
    const float fl = __double2float_rn(fc - (double)fh);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(acc, v[e], make_float4(fh, fl, 0.f, 0.f));
    v[e] = df_norm(acc);
  }
}

// every stored column of system j lies in its own rows (block-diagonal)
__global__ void k_sg_check(const int64_t* rowptr, const int32_t* col, Seg g, int64_t n, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int j = seg_of_row(g, r);
    const int64_t c0 = g.row[j], c1 = g.row[j + 1];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] < c0 || col[k] >= c1) *status = PG_ERR_ARG;
  }
}

// host block map: blocks of system j in proportion to its rows, at least 1
// and at most one per kThreads (row, rhs) items
std::vector<int> seg_blocks(const int64_t* rows, int S, int k) {
  const int64_t n = rows[S] - rows[0];
  const double target = 152.0 * 16.0;
  std::vector<int> blk(S + 1, 0);
  for (int j = 0; j < S; ++j) {
    const int64_t nj = rows[j + 1] - rows[j];
    int64_t b = n > 0 ? (int64_t)(target * (double)nj / (double)n) : 1;
    const int64_t cap = (nj * k + kThreads - 1) / kThreads;
    b = std::min<int64_t>(b, cap);
    blk[j + 1] = blk[j] + (int)std::max<int64_t>(b, 1);
  }
  return blk;
}

// the same total of blocks re-split over the systems still iterating: a
// converged system keeps one (idle) block, the others share the rest in
// proportion to their rows; blocks no system can use go to the largest
// active system, where they find no rows
void seg_rebalance(const int64_t* rows, int S, int k, const std::vector<char>& active, int total,
                   std::vector<int>& blk) {
  blk.assign(S + 1, 0);
  int64_t n_act = 0;
  int big = -1;
  for (int j = 0; j < S; ++j) {
    const int64_t nj = rows[j + 1] - rows[j];
    if (active[j]) {
      n_act += nj;
      if (big < 0 || nj > rows[big + 1] - rows[big]) big = j;
    }
  }
  // every system holds one block; the total - S others go to the active
  // systems (total >= S: the first map gives each system at least one)
  const int spare = total - S;
  std::vector<int> b(S, 1);
  int used = S;
  for (int j = 0; j < S; ++j) {
    if (!active[j]) continue;
    const int64_t nj = rows[j + 1] - rows[j];
    int64_t v = n_act > 0 ? (int64_t)((double)spare * (double)nj / (double)n_act) : 0;
    v = std::min<int64_t>(v, std::max<int64_t>((nj * k + kThreads - 1) / kThreads - 1, 0));
    b[j] += (int)v;
    used += (int)v;
  }
  if (used < total) b[big >= 0 ? big : S - 1] += total - used;
  for (int j = 0; j < S; ++j) blk[j + 1] = blk[j] + b[j];
}

struct SegPlan {
  int64_t n, nnz;
  int64_t gn = 0;           // gradient correction: columns of the block-diagonal G (0: off)
  int k, S, nb;
  int p;                    // block-Jacobi order (0: diagonal)
  std::vector<BjInfo> bj;   // per system, c0 = its first row
  std::vector<int64_t> soff;  // per system offset of its factors (S + 1 entries)
};

size_t sg_layout(const SegPlan& P, size_t* off /* 24 */) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  const size_t pairs = (size_t)P.S * P.k;
  put(0, P.nnz * sizeof(float4));                // At
  put(1, sizeof(double2) * P.n);                 // S
  put(2, sizeof(double) * P.n);                  // |D|
  put(3, sizeof(float) * P.n);                   // |D| f32
  put(4, sizeof(float4) * P.n * P.k);            // p
  put(5, sizeof(float4) * P.n * P.k);            // q
  put(6, sizeof(float4) * P.n * P.k);            // r
  put(7, sizeof(float4) * P.n * P.k);            // y
  put(8, sizeof(double2) * P.n * P.k);           // r64
  put(9, sizeof(double2) * (size_t)P.nb * P.k * 3);
  put(10, sizeof(CgState) * pairs);
  put(11, sizeof(CgCtl));
  put(12, sizeof(double) * pairs * 6);           // rnorm, target, pair scales, inverses, ratios
  put(13, sizeof(int) * (pairs + 1));            // want, status
  put(14, sizeof(int64_t) * (P.S + 1));          // system rows
  put(15, sizeof(int) * (P.S + 1));              // system blocks
  put(16, P.p ? sizeof(double2) * P.soff[P.S] : 0);      // block-Jacobi factors
  put(17, P.p ? sizeof(double2) * P.n * P.k : 0);        // S r64
  // gradient correction (FP32 products): S^-1, invD, t, z (FP64 scratch at setup), u
  put(18, P.gn ? sizeof(float2) * P.n : 0);
  put(19, P.gn ? sizeof(float2) * P.gn : 0);
  put(20, P.gn ? sizeof(float2) * P.gn * P.k : 0);
  put(21, P.gn ? std::max(sizeof(float4) * P.n * P.k, sizeof(double2) * (size_t)std::max(P.n, P.gn)) : 0);
  put(22, P.gn ? sizeof(float2) * P.n * P.k : 0);
  return o;
}

int seg_plan(int64_t n, int64_t nnz, int k, const int64_t* rows, int S, const int64_t* ents, int bp, SegPlan& P) {
  if (S < 1 || rows == nullptr || rows[0] != 0 || rows[S] != n) return PG_ERR_ARG;
  for (int j = 0; j < S; ++j)
    if (rows[j + 1] < rows[j]) return PG_ERR_ARG;
  P.n = n;
  P.nnz = nnz;
  P.k = k;
  P.S = S;
  const std::vector<int> blk = seg_blocks(rows, S, k);
  P.nb = blk[S];
  P.p = bp >= 1 && bp <= 6 ? bp : 0;
  P.bj.clear();
  P.soff.assign(S + 1, 0);
  if (P.p) {
    if (ents == nullptr) return PG_ERR_ARG;
    for (int j = 0; j < S; ++j) {
      BjInfo B{ents[3 * j], ents[3 * j + 1], ents[3 * j + 2], P.p, rows[j + 1] - rows[j]};
      B.c0 = rows[j];
      if (B.nE < 0 || B.nF < 0 || B.nV < 0 ||
          B.nE * B.de() + B.nF * (int64_t)B.df() + B.nV * (int64_t)B.dv() != B.n)
        return PG_ERR_ARG;
      P.bj.push_back(B);
      P.soff[j + 1] = P.soff[j] + B.s_size();
    }
  }
  return PG_OK;
}

int run_cocg_seg(const SegPlan& P, const int64_t* hrows, const int64_t* rowptr, const int32_t* col, const double2* A,
                 const double2* b, double2* x, const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out,
                 int64_t* its_out, char* ws, cudaStream_t s) {
  size_t off[24];
  sg_layout(P, off);
  float4* At = reinterpret_cast<float4*>(ws + off[0]);
  double2* Sd = reinterpret_cast<double2*>(ws + off[1]);
  double* wd = reinterpret_cast<double*>(ws + off[2]);
  float* wdf = reinterpret_cast<float*>(ws + off[3]);
  float4* pv = reinterpret_cast<float4*>(ws + off[4]);
  float4* q = reinterpret_cast<float4*>(ws + off[5]);
  float4* r = reinterpret_cast<float4*>(ws + off[6]);
  float4* y = reinterpret_cast<float4*>(ws + off[7]);
  double2* r64 = reinterpret_cast<double2*>(ws + off[8]);
  double2* part = reinterpret_cast<double2*>(ws + off[9]);
  double2* part2 = part + (size_t)P.nb * P.k;
  CgState* st = reinterpret_cast<CgState*>(ws + off[10]);
  CgCtl* ctl = reinterpret_cast<CgCtl*>(ws + off[11]);
  const int pairs = P.S * P.k;
  double* rnorm = reinterpret_cast<double*>(ws + off[12]);
  double* target = rnorm + pairs;
  // per-pair scales: every cycle starts from the true residual at unit norm
  // (r^T r stays inside the FP32 exponent range of the double-float pairs)
  double* cscale = rnorm + 2 * pairs;
  double* cinv = rnorm + 3 * pairs;
  double* clam = rnorm + 4 * pairs;
  int* want = reinterpret_cast<int*>(ws + off[13]);
  int* dstatus = want + pairs;
  int64_t* drows = reinterpret_cast<int64_t*>(ws + off[14]);
  int* dblk = reinterpret_cast<int*>(ws + off[15]);
  double2* Sblk = reinterpret_cast<double2*>(ws + off[16]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[17]);
  const int k = P.k, G = P.nb;
  const bool bj = P.p > 0;
  const bool grad = P.gn > 0;   // diagonal scaling only (checked by pg_cocg_segments)
  float2* gSinv = reinterpret_cast<float2*>(ws + off[18]);
  float2* ginvD = reinterpret_cast<float2*>(ws + off[19]);
  float2* gt = reinterpret_cast<float2*>(ws + off[20]);
  float4* gz = reinterpret_cast<float4*>(ws + off[21]);
  float2* gu = reinterpret_cast<float2*>(ws + off[22]);
  const unsigned gblocks = pg_blocks(P.gn * P.k / kGradQ(P.k), kThreads);   // k_grad_restrict32 only
  std::vector<int> hblk = seg_blocks(hrows, P.S, k), cur_blk;
  std::vector<char> sys_active(P.S, 1);
  PG_CUDA_TRY(cudaMemcpyAsync(drows, hrows, sizeof(int64_t) * (P.S + 1), cudaMemcpyHostToDevice, s));
  PG_CUDA_TRY(cudaMemcpyAsync(dblk, hblk.data(), sizeof(int) * (P.S + 1), cudaMemcpyHostToDevice, s));
  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  const Seg g{drows, dblk, P.S};
  int hstatus = 0;
  k_sg_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, g, P.n, dstatus);
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));   // also keeps the host block map alive for the copies
  if (hstatus) {
    pg_set_error("pg_cocg_segments: a row references a column outside its own system");
    return PG_ERR_ARG;
  }
  if (bj) {
    k_fill_one<<<pg_blocks(P.n, 256), 256, 0, s>>>(Sd, P.n);
    for (int j = 0; j < P.S; ++j) {
      const BjInfo& B = P.bj[j];
      if (B.n == 0) continue;
      k_bj_check<<<pg_blocks(B.n, 256), 256, 0, s>>>(rowptr + hrows[j], col, B, dstatus);
    }
    PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstatus) {
      pg_set_error("pg_cocg_segments: block-Jacobi needs the entity-block pattern (rows of one entity share their columns)");
      return PG_ERR_ARG;
    }
    for (int j = 0; j < P.S; ++j) {
      const BjInfo& B = P.bj[j];
      if (B.n == 0) continue;
      k_bj_factor<<<pg_blocks(B.n, 128), 128, 0, s>>>(rowptr + hrows[j], col, A, B, Sblk + P.soff[j], wd + hrows[j],
                                                       dstatus);
      k_bj_scale_matrix<<<pg_blocks(B.n, 128), 128, 0, s>>>(rowptr + hrows[j], col, A, B, Sblk + P.soff[j], At, ToDF());
    }
    k_wd_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(wd, P.n, wdf);
  } else {
    k_cg_scaling<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, Sd, wd, dstatus);
    k_df_scale_matrix<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, Sd, At, wdf, wd);
    if (grad) {
      double2* tmp = reinterpret_cast<double2*>(gz);   // FP64 scratch until the first z
      k_grad_sinv<<<pg_blocks(P.n, 256), 256, 0, s>>>(Sd, P.n, tmp);
      k_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(tmp, P.n, gSinv);
      k_grad_diag<<<pg_blocks(P.gn * 32, 256), 256, 0, s>>>(rowptr, col, A, o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                       P.gn, tmp);
      k_to_f32<<<pg_blocks(P.gn, 256), 256, 0, s>>>(tmp, P.gn, ginvD);
    }
  }
  PG_LAUNCH_CHECK();
  std::vector<double> bnorm(pairs), rn(pairs), tgt(pairs), sc(pairs), sc_prev(pairs, 1.0), scal(4 * (size_t)pairs);
  std::vector<int> wnt(pairs);
  PG_KSWITCH(k, (k_sg_norm2<K><<<G, kThreads, 0, s>>>(b, g, part), k_sg_norm_final<K><<<1, kThreads, 0, s>>>(part, g, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * pairs, cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_cocg_segments: zero diagonal entry (Jacobi scaling undefined)");
    return PG_ERR_BREAKDOWN;
  }
  // rows of one entity share their columns (checked): the group products apply
  int group = 0;
  if (bj && (P.p == 2 || P.p == 3)) {
    int* gflag = reinterpret_cast<int*>(part);
    int hg = 1;
    PG_CUDA_TRY(cudaMemsetAsync(gflag, 0, sizeof(int), s));
    k_group_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, P.n, P.p, gflag);
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(&hg, gflag, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    group = hg == 0 ? P.p : 0;
  }
  // product variants (same numbering as the single-system solver): one RHS
  // 10 G + U for G lanes per row and unroll U, 100 R + 30 + G for the group
  // product with G lanes per group and 4 batched column steps; several RHS
  // U = 1, 2 or 100 R for the group product
  std::vector<int> cands;
  if (k == 1) {
    cands = {42, 41, 22, 82};
    if (group) {
      cands.push_back(100 * group + 32);
      cands.push_back(100 * group + 34);
    }
  } else {
    cands = {2, 1};
    if (group) cands.push_back(100 * group);
  }
  auto launch_prod = [&](int v, cudaStream_t ss) {
    if (k == 1) {
      switch (v) {
        case 41: k_sg_spmm<1, 4, 1><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 22: k_sg_spmm<1, 2, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 82: k_sg_spmm<1, 8, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 232: k_sg_spmv_grpb<2, 2, 4><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 234: k_sg_spmv_grpb<2, 4, 4><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 332: k_sg_spmv_grpb<3, 2, 4><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        case 334: k_sg_spmv_grpb<3, 4, 4><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
        default: k_sg_spmm<1, 4, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl); break;
      }
    } else if (v == 200) {
      PG_KSWITCH(k, (k_sg_spmm_grp<K, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl)));
    } else if (v == 300) {
      PG_KSWITCH(k, (k_sg_spmm_grp<K, 3><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl)));
    } else if (v == 1) {
      PG_KSWITCH(k, (k_sg_spmm<K, 1, 1><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl)));
    } else {
      PG_KSWITCH(k, (k_sg_spmm<K, 1, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl)));
    }
  };
  int variant = cands[0];
  Plan Pf{P.n, P.nnz, k, 1, 0, 1, sizeof(double2), BjInfo{}};
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);
  auto true_residual = [&]() { launch_spmv<double2>(Pf, rowptr, col, A, x, r64, b, nullptr, npr, s); };
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  int64_t its = 0, checks = 0;
  int status = PG_OK;
  const int64_t max_it = o->max_it > 0 ? o->max_it : 100000;
  int chunk = o->check_every > 0 ? o->check_every : 50;
  bool first = true;
  const double delta = 1e-3;
  auto one_iteration = [&](cudaStream_t ss) {
    launch_prod(variant, ss);
    if (grad) {
      PG_KSWITCH(k, (k_sg_update<K, true><<<G, kThreads, 0, ss>>>(y, r, pv, q, wdf, g, st, part, part2, ctl, delta, gu,
                                                                  gSinv),
                     k_grad_restrict32<K><<<gblocks, kThreads, 0, ss>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                        ginvD, gu, P.gn, gt, ctl, 0),
                     k_sg_prolong<K><<<G, kThreads, 0, ss>>>(o->grad_rowptr, o->grad_col, o->grad_val, gSinv, gt, r,
                                                             g, gz, pv, 0, part, st, ctl, 0),
                     k_sg_pupdate<K><<<G, kThreads, 0, ss>>>(pv, gz, g, st, ctl)));
      return;
    }
    PG_KSWITCH(k, (k_sg_update<K><<<G, kThreads, 0, ss>>>(y, r, pv, q, wdf, g, st, part, part2, ctl, delta),
                   k_sg_pupdate<K><<<G, kThreads, 0, ss>>>(pv, r, g, st, ctl)));
  };
  const char* genv = getenv("PG_GRAPHS");
  const bool use_graphs = !(genv && genv[0] == '0');
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_failed = false;
  auto build_graph = [&]() {
    if (graph_failed) return;
    cudaGraph_t graph = nullptr;
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      for (int i = 0; i < kGraphIters; ++i) one_iteration(cs);
      ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph != nullptr;
    }
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      cudaGetLastError();
      gexec = nullptr;
      graph_failed = true;
    }
  };
  struct GraphCleanup {
    cudaStream_t& cs;
    cudaEvent_t& a;
    cudaEvent_t& b;
    cudaGraphExec_t& gx;
    ~GraphCleanup() {
      if (gx) cudaGraphExecDestroy(gx);
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (cs) cudaStreamDestroy(cs);
    }
  } graph_cleanup{cs, ev_in, ev_out, gexec};
  std::vector<CgState> hst(pairs);
  auto residual_norms = [&]() -> int {
    true_residual();
    PG_KSWITCH(k, (k_sg_norm2<K><<<G, kThreads, 0, s>>>(r64, g, part),
                   k_sg_norm_final<K><<<1, kThreads, 0, s>>>(part, g, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * pairs, cudaMemcpyDeviceToHost, s));
    return PG_OK;
  };
  for (;;) {
    const int e0 = residual_norms();
    if (e0) return e0;
    CgCtl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!first && hctl.nonfinite) {
      pg_set_error("pg_cocg_segments: non-finite residual");
      status = PG_ERR_NONFINITE;
      break;
    }
    bool all = true;
    for (int t = 0; t < pairs; ++t) {
      if (monitor)
        fprintf(stderr, "pg_cocg_segments: check %lld its %lld system %d rhs %d true ||r||/||b|| = %.6e\n",
                (long long)checks, (long long)its, t / k, t % k, bnorm[t] > 0 ? rn[t] / bnorm[t] : 0.0);
      if (!isfinite(rn[t])) {
        pg_set_error("pg_cocg_segments: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[t];
      const bool ok = rn[t] <= tb || bnorm[t] == 0.0;
      wnt[t] = ok ? 0 : 1;
      sc[t] = rn[t] > 0.0 && isfinite(rn[t]) ? rn[t] : 1.0;
      tgt[t] = 0.5 * tb / sc[t];
      if (!ok) all = false;
    }
    if (status || all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    for (int t = 0; t < pairs; ++t) {
      scal[t] = rn[t] > 0.0 ? 1.0 : 0.0;
      scal[pairs + t] = sc[t];
      scal[2 * pairs + t] = 1.0 / sc[t];
      scal[3 * pairs + t] = sc_prev[t] / sc[t];
      sc_prev[t] = sc[t];
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(rnorm, scal.data(), sizeof(double) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(cscale, scal.data() + pairs, sizeof(double) * 3 * pairs, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_sg_scale_d2<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, g, P.n, cinv)));
    if (!first) PG_KSWITCH(k, (k_sg_scale_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(pv, g, P.n, clam)));
    // systems already converged keep one idle block; the others take the rest
    for (int j = 0; j < P.S; ++j) {
      sys_active[j] = 0;
      for (int i = 0; i < k; ++i) sys_active[j] |= (char)wnt[j * k + i];
    }
    seg_rebalance(hrows, P.S, k, sys_active, G, cur_blk);
    if (cur_blk != hblk) {
      hblk = cur_blk;
      PG_CUDA_TRY(cudaMemcpyAsync(dblk, hblk.data(), sizeof(int) * (P.S + 1), cudaMemcpyHostToDevice, s));
    }
    if (bj)
      for (int j = 0; j < P.S; ++j) {
        const BjInfo& B = P.bj[j];
        if (B.n == 0) continue;
        PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(B.n * K, 256), 256, 0, s>>>(Sblk + P.soff[j], B, r64 + hrows[j] * K,
                                                                             r64b + hrows[j] * K)));
      }
    if (grad) {
      // r = S r64, then z = r + S^-1 G invD G^T S^-1 r (S^-1 r = r64), rho = r^T z, p = z on the first cycle
      PG_KSWITCH(k, (k_sg_start<K><<<G, kThreads, 0, s>>>(r64, Sd, g, r, y, pv, 0, part),
                     k_sg_u_start<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, P.n, gu),
                     k_grad_restrict32<K><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                       ginvD, gu, P.gn, gt, ctl, 1),
                     k_sg_prolong<K><<<G, kThreads, 0, s>>>(o->grad_rowptr, o->grad_col, o->grad_val, gSinv, gt, r, g,
                                                            gz, pv, first ? 1 : 0, part, st, ctl, 1),
                     k_sg_cycle_init<K><<<1, kThreads, 0, s>>>(part, g, st, rnorm, target, want, ctl,
                                                               first ? 1 : 0)));
    } else {
      PG_KSWITCH(k, (k_sg_start<K><<<G, kThreads, 0, s>>>(bj ? r64b : r64, Sd, g, r, y, pv, first ? 1 : 0, part),
                     k_sg_cycle_init<K><<<1, kThreads, 0, s>>>(part, g, st, rnorm, target, want, ctl,
                                                               first ? 1 : 0)));
    }
    if (first) {
      // PG_SPMV_VARIANT forces a candidate; else the fastest on these operands
      const char* fv = getenv("PG_SPMV_VARIANT");
      int forced = -1;
      if (fv && fv[0])
        for (int c : cands)
          if (c == atoi(fv)) forced = c;
      if (forced >= 0) variant = forced;
      else if (autotune_enabled()) variant = pick_fastest(cands, [&](int v) { launch_prod(v, s); }, s);
      PG_LAUNCH_CHECK();
      if (monitor) fprintf(stderr, "pg_cocg_segments: SpMV variant %d for n=%lld nnz=%lld k=%d\n", variant,
                           (long long)P.n, (long long)P.nnz, k);
    }
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    int done = 0;
    if (use_graphs && steps >= kGraphIters) {
      if (!gexec) build_graph();
      if (gexec) {
        cudaEventRecord(ev_in, s);
        cudaStreamWaitEvent(cs, ev_in, 0);
        for (; done + kGraphIters <= steps; done += kGraphIters) cudaGraphLaunch(gexec, cs);
        cudaEventRecord(ev_out, cs);
        cudaStreamWaitEvent(s, ev_out, 0);
      }
    }
    for (; done < steps; ++done) one_iteration(s);
    PG_LAUNCH_CHECK();
    PG_KSWITCH(k, (k_sg_scale_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(y, g, P.n, cscale)));
    if (bj) {
      for (int j = 0; j < P.S; ++j) {
        const BjInfo& B = P.bj[j];
        if (B.n == 0) continue;
        PG_KSWITCH(k, (k_bj_apply_t_add<K><<<pg_blocks(B.n * K, 256), 256, 0, s>>>(
                           Sblk + P.soff[j], B, y + hrows[j] * K, x + hrows[j] * K, DfToD2())));
      }
    } else {
      PG_KSWITCH(k, (k_df_xupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, Sd, P.n, x)));
    }
    PG_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(CgState) * pairs, cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    bool brk = false;
    for (int t = 0; t < pairs; ++t) {
      used = hst[t].its > used ? hst[t].its : used;
      brk = brk || hst[t].breakdown;
    }
    const int64_t cycle_its = used - its;
    its = used;
    ++checks;
    if (brk) {
      pg_set_error("pg_cocg_segments: breakdown (p^T A p = 0 or r^T r = 0)");
      status = PG_ERR_BREAKDOWN;
      const int e1 = residual_norms();
      if (e1) return e1;
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      break;
    }
    int64_t c2 = cycle_its + cycle_its / 4 + 8;
    chunk = (int)(c2 < 16 ? 16 : (c2 > 4000 ? 4000 : c2));
  }
  if (its_out) {
    PG_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(CgState) * pairs, cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    for (int t = 0; t < pairs; ++t) its_out[t] = first ? 0 : hst[t].its;
  }
  double worst = 0.0;
  for (int t = 0; t < pairs; ++t) {
    const double rr = bnorm[t] > 0 ? rn[t] / bnorm[t] : 0.0;
    if (relres_out) relres_out[t] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = checks;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_cocg_segments: max_it reached before rtol");
  return status;
}

}  // namespace
extern "C" size_t pg_cocg_segments_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const int64_t* seg_rows,
                                                   int n_seg, const int64_t* seg_entities, const pg_cocg_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  SegPlan P;
  if (seg_plan(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts->block_p, P) != PG_OK) return 0;
  P.gn = opts->grad_rowptr && opts->grad_cols > 0 ? opts->grad_cols : 0;
  size_t off[24];
  return sg_layout(P, off) + 256;
}

extern "C" int pg_cocg_segments(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                                const int64_t* seg_rows, int n_seg, const int64_t* seg_entities, const double* b,
                                double* x, int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result,
                                double* relres, int64_t* its, void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || !seg_rows || n < 1 || nnz < n || n_seg < 1 ||
      !valid_k(nrhs) || !(opts->rtol > 0.0) || opts->precision != 2) {
    pg_set_error("pg_cocg_segments: bad argument (n_seg >= 1, nrhs 1..32 power of two, rtol > 0, precision 2)");
    return PG_ERR_ARG;
  }
  SegPlan P;
  if (seg_plan(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts->block_p, P) != PG_OK) {
    pg_set_error("pg_cocg_segments: seg_rows must rise from 0 to n; with block_p, seg_entities must give each "
                 "system's (edges, faces, elements) matching its rows");
    return PG_ERR_ARG;
  }
  if (opts->grad_rowptr && (!opts->grad_col || !opts->grad_val || !opts->gradt_rowptr || !opts->gradt_row ||
                            !opts->gradt_val || opts->grad_cols < 1 || opts->grad_cols >= (int64_t(1) << 31) ||
                            opts->block_p > 0)) {
    pg_set_error("pg_cocg_segments: gradient correction needs all six G arrays (block-diagonal over the systems), "
                 "grad_cols >= 1 and diagonal Jacobi (block_p 0)");
    return PG_ERR_ARG;
  }
  P.gn = opts->grad_rowptr && opts->grad_cols > 0 ? opts->grad_cols : 0;
  const size_t need = pg_cocg_segments_workspace_bytes(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_cocg_segments: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  return run_cocg_seg(P, seg_rows, rowptr, col, reinterpret_cast<const double2*>(vals),
                      reinterpret_cast<const double2*>(b), reinterpret_cast<double2*>(x), opts, result, relres, its,
                      ws, pg_stream(stream));
}

extern "C" int pg_segments_block_map(const int64_t* seg_rows, int n_seg, int nrhs, const unsigned char* active,
                                     int* blk) {
  if (!seg_rows || !blk || n_seg < 1 || !valid_k(nrhs) || seg_rows[0] != 0) {
    pg_set_error("pg_segments_block_map: bad argument");
    return PG_ERR_ARG;
  }
  for (int j = 0; j < n_seg; ++j)
    if (seg_rows[j + 1] < seg_rows[j]) {
      pg_set_error("pg_segments_block_map: seg_rows must not fall");
      return PG_ERR_ARG;
    }
  std::vector<int> b = seg_blocks(seg_rows, n_seg, nrhs);
  if (active) {
    std::vector<char> act(n_seg);
    for (int j = 0; j < n_seg; ++j) act[j] = active[j] ? 1 : 0;
    std::vector<int> r;
    seg_rebalance(seg_rows, n_seg, nrhs, act, b[n_seg], r);
    b = r;
  }
  for (int j = 0; j <= n_seg; ++j) blk[j] = b[j];
  return PG_OK;
}
