// Double-float COCG: FP64-class accuracy on the FP32 pipes (products,
// vector updates, graph-replayed iterations, product variant autotuner,
// entity-group products) and the several-frequencies form.
#include "pg_cocg.cuh"

namespace {

// q = At p (double-float), partial mu = p^T q; last block: alpha
template <int G, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmv1(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                       const float4* __restrict__ val, int64_t n,
                                                       const float4* __restrict__ pv, float4* __restrict__ q,
                                                       double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t rw = warp_base; rw < n; rw += groups) {
    const int64_t r = rw + (gid - warp_base);
    const bool valid = r < n;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t e = rowptr[r + 1];
      int64_t k = rowptr[r] + lane;
      if (U == 2) {
        // two independent accumulators: two gathers in flight per lane
        float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (; k + G < e; k += 2 * G) {
          const int32_t c0 = col[k], c1 = col[k + G];
          const float4 v0 = val[k], v1 = val[k + G];
          cdf_mac(acc, v0, pv[c0]);
          cdf_mac(acc1, v1, pv[c1]);
        }
        if (k < e) cdf_mac(acc, val[k], pv[col[k]]);
        cdf_add(acc, acc1);
      } else {
        for (; k < e; k += G) cdf_mac(acc, val[k], pv[col[k]]);
      }
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) cdf_add(acc, shfl_xor4(acc, off));
    if (valid && lane == 0) {
      acc = df_norm(acc);
      q[r] = acc;
      cdf_mac(mu, pv[r], acc);
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

template <int K, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, int64_t n,
                                                      const float4* __restrict__ pv, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t e = rowptr[r + 1];
    int64_t k = rowptr[r];
    if (U == 2) {
      float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
      for (; k + 1 < e; k += 2) {
        const int32_t c0 = col[k], c1 = col[k + 1];
        const float4 v0 = val[k], v1 = val[k + 1];
        cdf_mac(acc, v0, pv[(int64_t)c0 * K + rhs]);
        cdf_mac(acc1, v1, pv[(int64_t)c1 * K + rhs]);
      }
      if (k < e) cdf_mac(acc, val[k], pv[(int64_t)col[k] * K + rhs]);
      cdf_add(acc, acc1);
    } else {
      for (; k < e; ++k) cdf_mac(acc, val[k], pv[(int64_t)col[k] * K + rhs]);
    }
    acc = df_norm(acc);
    q[r * K + rhs] = acc;
    cdf_mac(mu, pv[r * K + rhs], acc);
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// y += alpha p ; r -= alpha q ; partials rho = r^T r (df), w = sum |r|^2 |D| (FP32 estimate).
// GRAD: no rho (the gradient prolongation forms z and rho = r^T z).
template <int K, bool PC = false, bool GRAD = false>
__global__ void __launch_bounds__(kThreads) k_df_update(float4* __restrict__ y, float4* __restrict__ r,
                                                        const float4* __restrict__ pv, const float4* __restrict__ q,
                                                        const float* __restrict__ wd, int64_t n, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, int iter,
                                                        double delta, float2* __restrict__ u = nullptr,
                                                        const float2* __restrict__ Sinv = nullptr) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  __shared__ float4 al[kMaxK];
  if (threadIdx.x < K) {
    const double2 a = st[threadIdx.x].alpha;
    al[threadIdx.x] = cdf_from(a);
  }
  __syncthreads();
  const int rhs = threadIdx.x % K;
  const float4 a = al[rhs];
  const float4 na = make_float4(-a.x, -a.y, -a.z, -a.w);
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
  float ww = 0.f;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    float4 ye = y[e], re = r[e];
    cdf_mac(ye, a, pv[e]);
    cdf_mac(re, na, q[e]);
    ye = df_norm(ye);
    re = df_norm(re);
    y[e] = ye;
    r[e] = re;
    if constexpr (GRAD) {
      u[e] = cmul(Sinv[PC ? e : e / K], make_float2(re.x, re.z));
    } else {
      cdf_mac(rho, re, re);
    }
    ww += (re.x * re.x + re.z * re.z) * wd[PC ? e : e / K];
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  if constexpr (!GRAD) block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  block_reduce_f<K>(ww, reinterpret_cast<float*>(smf), pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_beta_final<K, GRAD>(prho, pw, gridDim.x, st, ctl, iter, delta, smem);
}

// Gradient correction on the double-float recurrence (diagonal scaling, PEC
// systems): z = r + S^-1 G invD G^T S^-1 r.  The residual recurrence and rho
// stay double-float; the correction only shapes the search direction, so its
// products run in FP32 (the update writes u = S^-1 r from r's leading
// float, the restriction t = invD G^T u and the prolongation S^-1 G t are
// FP32, and z = r + S^-1 G t is a double-float sum).  Inside an iteration
// both run only when this iteration's update ran (ctl->pending, cleared by
// the next product); start = 1 at a cycle start.
template <int K>
__global__ void k_dfg_u_start(const double2* __restrict__ r64, int64_t n, float2* __restrict__ u) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    u[e] = make_float2((float)r64[e].x, (float)r64[e].y);
}

// z = r + S^-1 (G t), partial rho = r^T z (double-float); in an iteration the
// last block sets beta = rho / rho_old and rho for the RHS updated in it
// (beta_iter == 1); at a cycle start p = z when set_p.  PC (several
// frequencies): S^-1 per element, and ps = S o p is set with p.  K >= 4: a
// thread takes one row and 4 RHS (two 16-byte gathers of t per entry, the
// entry's index and value loaded once for the 4).
template <int K, bool PC = false>
__global__ void __launch_bounds__(kThreads) k_dfg_prolong(const int64_t* __restrict__ gp,
                                                          const int32_t* __restrict__ gc,
                                                          const double* __restrict__ gv,
                                                          const float2* __restrict__ Sinv,
                                                          const float2* __restrict__ t,
                                                          const float4* __restrict__ r, int64_t n,
                                                          float4* __restrict__ z, float4* __restrict__ pv, int set_p,
                                                          double2* prho, CgState* st, CgCtl* ctl, int start,
                                                          float4* __restrict__ ps = nullptr,
                                                          const float4* __restrict__ Sdf = nullptr) {
  if (!start && !ctl->pending) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  auto finish = [&](int64_t e, float2 acc, float4& re, float4& ze) {
    const float2 cr = cmul(Sinv[PC ? e : e / K], acc);
    re = r[e];
    ze = re;
    df_add(ze.x, ze.y, cr.x, 0.f);
    df_add(ze.z, ze.w, cr.y, 0.f);
    ze = df_norm(ze);
  };
  auto item = [&](int64_t e, float4& re, float4& ze) {
    const int64_t row = e / K;
    finish(e, grad_row_sum<K>(gc, gv, t, gp[row], gp[row + 1], (int)(e % K)), re, ze);
  };
  auto store = [&](int64_t e, float4 ze) {
    z[e] = ze;
    if (set_p) {
      pv[e] = ze;
      if (PC) {
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        cdf_mac(w, Sdf[e], ze);
        ps[e] = df_norm(w);
      }
    }
  };
  if constexpr (kGradQ(K) == 4) {
    // (row, quad) items; a block's range starts on a row, so a thread's
    // quad is lane % KQ throughout
    constexpr int KQ = K / 4;
    const int64_t totq = n * KQ;
    const int64_t chq = ((totq + gridDim.x - 1) / gridDim.x + KQ - 1) / KQ * KQ;
    const int64_t lq = (int64_t)blockIdx.x * chq, hq = min(totq, lq + chq);
    float4 rq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) rq[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t f = lq + threadIdx.x; f < hq; f += kThreads) {
      const int64_t row = f / KQ;
      const int r0 = (int)(f % KQ) * 4;
      float2 acc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = make_float2(0.f, 0.f);
      const int64_t j1 = gp[row + 1];
#pragma unroll 2
      for (int64_t j = gp[row]; j < j1; ++j) {
        const float g = __double2float_rn(gv[j]);
        const float4* tp = reinterpret_cast<const float4*>(t + (int64_t)gc[j] * K + r0);
        const float4 a = tp[0], b = tp[1];
        acc[0].x = fmaf(g, a.x, acc[0].x);
        acc[0].y = fmaf(g, a.y, acc[0].y);
        acc[1].x = fmaf(g, a.z, acc[1].x);
        acc[1].y = fmaf(g, a.w, acc[1].y);
        acc[2].x = fmaf(g, b.x, acc[2].x);
        acc[2].y = fmaf(g, b.y, acc[2].y);
        acc[3].x = fmaf(g, b.z, acc[3].x);
        acc[3].y = fmaf(g, b.w, acc[3].y);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t e = row * K + r0 + q;
        float4 re, ze;
        finish(e, acc[q], re, ze);
        store(e, ze);
        cdf_mac(rq[q], re, ze);
      }
    }
    block_reduce_df_q4<K>(rq, smf, prho + (int64_t)blockIdx.x * K);
  } else {
    const int64_t total = n * K;
    const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
    const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
    float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
    // two items per step (e and e + kThreads), so each thread has two
    // independent load chains in flight; the items are summed into rho in
    // increasing e, as a one-item loop would
    int64_t e = lo + threadIdx.x;
    for (; e + kThreads < hi; e += 2 * kThreads) {
      // both rows' entries in one loop (each row summed in entry order); one
      // RHS: four entries of each row per step, eight gathers in flight
      const int64_t eb = e + kThreads, rowa = e / K, rowb = eb / K;
      const int64_t ja0 = gp[rowa], jae = gp[rowa + 1], jb0 = gp[rowb], jbe = gp[rowb + 1];
      const int rha = (int)(e % K), rhb = (int)(eb % K);
      float2 acca = make_float2(0.f, 0.f), accb = make_float2(0.f, 0.f);
      if constexpr (K == 1) {
        const int64_t nmin = min(jae - ja0, jbe - jb0);
        int64_t s = 0;
        for (; s + 4 <= nmin; s += 4) {
          grad_gather4<K>(gc, gv, t, ja0 + s, rha, acca);
          grad_gather4<K>(gc, gv, t, jb0 + s, rhb, accb);
        }
        grad_row_acc<K>(gc, gv, t, ja0 + s, jae, rha, acca);
        grad_row_acc<K>(gc, gv, t, jb0 + s, jbe, rhb, accb);
      } else {
        const int64_t steps = max(jae - ja0, jbe - jb0);
        for (int64_t s = 0; s < steps; ++s) {
          if (ja0 + s < jae) grad_gather1<K>(gc, gv, t, ja0 + s, rha, acca);
          if (jb0 + s < jbe) grad_gather1<K>(gc, gv, t, jb0 + s, rhb, accb);
        }
      }
      float4 ra, za, rb, zb;
      finish(e, acca, ra, za);
      finish(eb, accb, rb, zb);
      store(e, za);
      store(e + kThreads, zb);
      cdf_mac(rho, ra, za);
      cdf_mac(rho, rb, zb);
    }
    if (e < hi) {
      float4 ra, za;
      item(e, ra, za);
      store(e, za);
      cdf_mac(rho, ra, za);
    }
    block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  }
  if (!start && arrive_last(&ctl->counter)) {
    const double2 rr = sum_partials<K>(prho, gridDim.x, threadIdx.x < K ? threadIdx.x : 0, smem);
    if (threadIdx.x < K) {
      CgState& S = st[threadIdx.x];
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
    if (threadIdx.x == 0) ctl->counter = 0;
  }
}

template <int K, bool PC = false>
__global__ void __launch_bounds__(kThreads) k_df_pupdate(float4* __restrict__ pv, const float4* __restrict__ r, int64_t n,
                                                         const CgState* st, const CgCtl* ctl,
                                                         float4* __restrict__ ps = nullptr,
                                                         const float4* __restrict__ Sdf = nullptr) {
  __shared__ float4 bt[kMaxK];
  __shared__ int use[kMaxK];
  if (!ctl->pending) return;
  if (threadIdx.x < K) {
    bt[threadIdx.x] = cdf_from(st[threadIdx.x].beta);
    use[threadIdx.x] = st[threadIdx.x].beta_iter == 1;
  }
  __syncthreads();
  int anyuse = 0;
  for (int i = 0; i < K; ++i) anyuse |= use[i];
  if (!anyuse) return;
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    if (use[e % K]) {
      float4 v = r[e];
      cdf_mac(v, bt[e % K], pv[e]);
      v = df_norm(v);
      pv[e] = v;
      if (PC) {
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        cdf_mac(w, Sdf[e], v);
        ps[e] = df_norm(w);
      }
    }
}

template <int K, bool PC = false>
__global__ void k_df_start(const double2* __restrict__ r64, const double2* __restrict__ S, int64_t n, float4* r,
                           float4* y, float4* pv, int set_p, double2* prho, float4* ps = nullptr) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 sc = S[PC ? e : e / K];
    const double2 v = cmul(sc, r64[e]);
    const float4 vf = cdf_from(v);
    r[e] = vf;
    y[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (set_p) pv[e] = vf;
    if (PC && set_p) ps[e] = cdf_from(cmul(sc, v));
    rho = dadd(rho, cmul(v, v));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
}

// v[:, c] *= f[c] (FP64 vectors)
template <int K>
__global__ void k_scale_cols_d2(double2* v, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    v[e] = dscale(f[e % K], v[e]);
}

// v[:, c] *= f[c] (double-float vectors; f split into hi + lo)
template <int K>
__global__ void k_scale_cols_df(float4* v, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const double fc = f[e % K];
    const float fh = __double2float_rn(fc);
    const float fl = __double2float_rn(fc - (double)fh);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(acc, v[e], make_float4(fh, fl, 0.f, 0.f));
    v[e] = df_norm(acc);
  }
}

// ---- several frequencies in one solve --------------------------------------
// Column j solves (Re A0 + i s_j Im A0) x_j = b_j: A0 assembled at omega_0
// (K - i omega_0 mu M, PEC rows unit), s_j = omega_j / omega_0.  The matrix is
// read once per iteration for all columns; each column has its own Jacobi
// scaling S_j = diag(A_j)^(-1/2), applied to the direction (ps = S_j o p, kept
// by the p update) and to the product's rows.

// S[r * K + j], |D|[r * K + j] for every column
template <int K>
__global__ void k_mf_scaling(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n,
                             const double* scale, double2* S, double* wd, float* wdf, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 d = make_double2(0.0, 0.0);
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] == r) d = val[k];
    for (int j = 0; j < K; ++j) {
      const double2 dj = make_double2(d.x, scale[j] * d.y);
      const double m = hypot(dj.x, dj.y);
      if (!(m > 0.0)) {
        *status = 1;
        S[r * K + j] = make_double2(1.0, 0.0);
        wd[r * K + j] = 1.0;
        wdf[r * K + j] = 1.0f;
        continue;
      }
      // principal square root of 1/d
      const double2 inv = make_double2(dj.x / (m * m), -dj.y / (m * m));
      const double mi = 1.0 / m;
      const double re = sqrt(0.5 * (mi + inv.x));
      const double im = inv.y >= 0.0 ? sqrt(fmax(0.5 * (mi - inv.x), 0.0)) : -sqrt(fmax(0.5 * (mi - inv.x), 0.0));
      S[r * K + j] = make_double2(re, im);
      wd[r * K + j] = m;
      wdf[r * K + j] = (float)m;
    }
  }
}

__global__ void k_mf_df_matrix(const double2* val, int64_t nnz, float4* out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = cdf_from(val[k]);
}

__global__ void k_mf_sdf(const double2* S, int64_t total, float4* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = cdf_from(S[e]);
}

// q = S o (A_j ps), A_j = Re A0 + i s_j Im A0, partial mu = p^T q; last block: alpha
template <int K>
__global__ void __launch_bounds__(kThreads) k_mf_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, int64_t n,
                                                      const float* __restrict__ scale_hl,
                                                      const float4* __restrict__ Sdf, const float4* __restrict__ pv,
                                                      const float4* __restrict__ ps, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const float sh = scale_hl[2 * rhs], sl = scale_hl[2 * rhs + 1];
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t e = rowptr[r + 1];
    for (int64_t k = rowptr[r]; k < e; ++k) {
      const float4 a = val[k];
      // imaginary part times s_j (double-float product)
      const dfv im = df_mul(dfv{a.z, a.w}, dfv{sh, sl});
      cdf_mac(acc, make_float4(a.x, a.y, im.h, im.l), ps[(int64_t)col[k] * K + rhs]);
    }
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(out, Sdf[r * K + rhs], df_norm(acc));
    out = df_norm(out);
    q[r * K + rhs] = out;
    cdf_mac(mu, pv[r * K + rhs], out);
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// r64 = b - A_j x (FP64), one thread per (row, column)
template <int K>
__global__ void k_mf_resid(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double2* __restrict__ val, int64_t n, const double* __restrict__ scale,
                           const double2* __restrict__ x, const double2* __restrict__ b, double2* __restrict__ r64) {
  const int64_t total = n * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int j = (int)(e % K);
    const double sj = scale[j];
    double ar = 0.0, ai = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const double2 a = val[k];
      const double2 xv = x[(int64_t)col[k] * K + j];
      const double im = sj * a.y;
      ar = fma(a.x, xv.x, fma(-im, xv.y, ar));
      ai = fma(a.x, xv.y, fma(im, xv.x, ai));
    }
    r64[e] = make_double2(b[e].x - ar, b[e].y - ai);
  }
}

// ---- entity-group products --------------------------------------------------
// DOFs are numbered entity by entity with p, p(p-1) and p(p-1)(p-2)/2 DOFs per
// edge, face and volume: all multiples of p, and every entity starts at a
// multiple of p.  So rows [R i, R i + R) with R = p belong to one entity and
// share their column list (entity-pair pattern; checked column by column
// before use).  The group product loads each column index and p value once
// and uses them for R rows: fewer loads per stored entry and R independent
// accumulations per lane.

// one RHS: G lanes per group of R rows, U column steps per loop pass
template <int R, int G, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmv_grp(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const float4* __restrict__ val, int64_t n,
                                                          const float4* __restrict__ pv, float4* __restrict__ q,
                                                          double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t ngroups = n / R;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t gw = warp_base; gw < ngroups; gw += groups) {
    const int64_t gi = gw + (gid - warp_base);
    const bool valid = gi < ngroups;
    float4 acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t r0 = gi * R;
      int64_t off[R];
#pragma unroll
      for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
      const int64_t len = rowptr[r0 + 1] - off[0];
      int64_t k = lane;
      if (U == 2) {
        // a second set of accumulators: two column steps in flight per lane
        float4 acc1[R];
#pragma unroll
        for (int i = 0; i < R; ++i) acc1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (; k + G < len; k += 2 * G) {
          const int32_t c0 = col[off[0] + k], c1 = col[off[0] + k + G];
          float4 v0[R], v1[R];
#pragma unroll
          for (int i = 0; i < R; ++i) {
            v0[i] = val[off[i] + k];
            v1[i] = val[off[i] + k + G];
          }
          const float4 x0 = pv[c0], x1 = pv[c1];
#pragma unroll
          for (int i = 0; i < R; ++i) {
            cdf_mac(acc[i], v0[i], x0);
            cdf_mac(acc1[i], v1[i], x1);
          }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) cdf_add(acc[i], acc1[i]);
      }
      for (; k < len; k += G) {
        const float4 x = pv[col[off[0] + k]];
#pragma unroll
        for (int i = 0; i < R; ++i) cdf_mac(acc[i], val[off[i] + k], x);
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) cdf_add(acc[i], shfl_xor4(acc[i], o));
    if (valid && lane == 0) {
      const int64_t r0 = gi * R;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 a = df_norm(acc[i]);
        q[r0 + i] = a;
        cdf_mac(mu, pv[r0 + i], a);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

// one RHS, G lanes per group of R rows; each lane issues the column, value
// and p loads of B column steps back to back before using them, so a warp
// keeps B times more bytes in flight than one step at a time.  MB > 1 asks
// the compiler for MB resident blocks per SM (fewer registers per thread,
// more warps to hide the p gathers).
template <int R, int G, int B, int MB = 1>
__global__ void __launch_bounds__(kThreads, MB) k_df_spmv_grpb(const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ col,
                                                           const float4* __restrict__ val, int64_t n,
                                                           const float4* __restrict__ pv, float4* __restrict__ q,
                                                           double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t ngroups = n / R;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t gw = warp_base; gw < ngroups; gw += groups) {
    const int64_t gi = gw + (gid - warp_base);
    const bool valid = gi < ngroups;
    float4 acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t r0 = gi * R;
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
      const int64_t r0 = gi * R;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 a = df_norm(acc[i]);
        q[r0 + i] = a;
        cdf_mac(mu, pv[r0 + i], a);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

// K RHS: one thread per (group of R rows, rhs)
template <int K, int R>
__global__ void __launch_bounds__(kThreads) k_df_spmm_grp(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const float4* __restrict__ val, int64_t n,
                                                          const float4* __restrict__ pv, float4* __restrict__ q,
                                                          double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const int64_t items = (n / R) * K;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items; it += stride) {
    const int64_t r0 = (it / K) * R;
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
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// K RHS (K >= 2): one thread per (group of R rows, pair of RHS c, c + K/2):
// every column index and matrix value loaded serves two RHS
template <int K, int R>
__global__ void __launch_bounds__(kThreads) k_df_spmm_grp2(const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ col,
                                                           const float4* __restrict__ val, int64_t n,
                                                           const float4* __restrict__ pv, float4* __restrict__ q,
                                                           double2* partial, CgState* st, CgCtl* ctl) {
  static_assert(K >= 2, "two RHS per thread");
  constexpr int H = K / 2;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int ra = threadIdx.x % H, rb = ra + H;
  const int64_t items = (n / R) * H;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float4 mua = make_float4(0.f, 0.f, 0.f, 0.f), mub = mua;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items; it += stride) {
    const int64_t r0 = (it / H) * R;
    int64_t off[R];
#pragma unroll
    for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
    const int64_t len = rowptr[r0 + 1] - off[0];
    float4 acca[R], accb[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acca[i] = accb[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t k = 0; k < len; ++k) {
      const int64_t c = col[off[0] + k];
      const float4 xa = pv[c * K + ra], xb = pv[c * K + rb];
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 v = val[off[i] + k];
        cdf_mac(acca[i], v, xa);
        cdf_mac(accb[i], v, xb);
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const float4 a = df_norm(acca[i]), b = df_norm(accb[i]);
      q[(r0 + i) * K + ra] = a;
      q[(r0 + i) * K + rb] = b;
      cdf_mac(mua, pv[(r0 + i) * K + ra], a);
      cdf_mac(mub, pv[(r0 + i) * K + rb], b);
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<H>(mua, smf, partial + (int64_t)blockIdx.x * K);
  block_reduce_df<H>(mub, smf, partial + (int64_t)blockIdx.x * K + H);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// ---- SpMV variant autotuner ------------------------------------------------
// The double-float product's best lanes-per-row / unrolling depends on the
// matrix (rows, stored entries per row) and the RHS count.  At the first
// cycle of a solve each candidate runs 3 times on the actual operands (the
// product is the first kernel of an iteration and recomputes alpha, so extra
// runs change no solver state) and the fastest is kept per (n, nnz, k).
// PG_AUTOTUNE=0 keeps the default variant.
struct TuneEntry {
  int64_t n, nnz;
  int k, group, variant;
};
std::vector<TuneEntry> g_tune;
std::mutex g_tune_mu;

int tuned_variant(int64_t n, int64_t nnz, int k, int group) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (const TuneEntry& t : g_tune)
    if (t.n == n && t.nnz == nnz && t.k == k && t.group == group) return t.variant;
  return -1;
}

void store_variant(int64_t n, int64_t nnz, int k, int group, int v) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.push_back(TuneEntry{n, nnz, k, group, v});
}

// PG_SPMV_VARIANT=v forces a product variant when it is valid for the solve
// (a group variant only when the rows were checked to group by R); -1 otherwise
int forced_variant(int k, int group) {
  const char* e = getenv("PG_SPMV_VARIANT");
  if (!(e && e[0])) return -1;
  const int v = atoi(e);
  if (k == 1) {
    if (v == 21 || v == 22 || v == 41 || v == 42 || v == 81 || v == 82) return v;
    const int gv = v - 100 * group;
    if (group && (gv == 2 || gv == 4 || gv == 8 || gv == 12 || gv == 14 || gv == 32 || gv == 34 || gv == 44 ||
                  gv == 54))
      return v;
  } else {
    if (v == 1 || v == 2) return v;
    if (group && (v == 100 * group || v == 100 * group + 50)) return v;
  }
  return -1;
}


// single RHS: variant = lanes per row G (1..8) * 10 + unroll U, or
// 100 R + 10 (U - 1) + G for the product over groups of R rows with G lanes
// per group and unroll U, 100 R + 30 + G for the group product with 4 column
// steps batched, 100 R + 44 / 100 R + 54 for that product with 4 / 3 column
// steps and a register budget of 4 resident blocks per SM; several RHS: unroll 1 or 2, 100 R for the group product, or
// 100 R + 50 for the group product with two RHS per thread
void launch_df_spmv1(int variant, int grid, cudaStream_t s, const int64_t* rowptr, const int32_t* col,
                     const float4* At, int64_t n, const float4* pv, float4* q, double2* part, CgState* st,
                     CgCtl* ctl) {
  switch (variant) {
    case 202: k_df_spmv_grp<2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 204: k_df_spmv_grp<2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 208: k_df_spmv_grp<2, 8><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 302: k_df_spmv_grp<3, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 304: k_df_spmv_grp<3, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 308: k_df_spmv_grp<3, 8><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 212: k_df_spmv_grp<2, 2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 232: k_df_spmv_grpb<2, 2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 234: k_df_spmv_grpb<2, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 244: k_df_spmv_grpb<2, 4, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 254: k_df_spmv_grpb<2, 4, 3, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 344: k_df_spmv_grpb<3, 4, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 354: k_df_spmv_grpb<3, 4, 3, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 332: k_df_spmv_grpb<3, 2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 334: k_df_spmv_grpb<3, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 214: k_df_spmv_grp<2, 4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 312: k_df_spmv_grp<3, 2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 314: k_df_spmv_grp<3, 4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 21: k_df_spmv1<2, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 22: k_df_spmv1<2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 42: k_df_spmv1<4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 81: k_df_spmv1<8, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 82: k_df_spmv1<8, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    default: k_df_spmv1<4, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
  }
}

template <int K>
void launch_df_spmm(int variant, int grid, cudaStream_t s, const int64_t* rowptr, const int32_t* col,
                    const float4* At, int64_t n, const float4* pv, float4* q, double2* part, CgState* st, CgCtl* ctl) {
  if (K >= 2 && variant == 250)
    k_df_spmm_grp2<(K >= 2 ? K : 2), 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (K >= 2 && variant == 350)
    k_df_spmm_grp2<(K >= 2 ? K : 2), 3><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (variant == 200)
    k_df_spmm_grp<K, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (variant == 300)
    k_df_spmm_grp<K, 3><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (variant == 2)
    k_df_spmm<K, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else
    k_df_spmm<K, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
}


}  // namespace

namespace pgk {

size_t df_layout(const Plan& P, size_t* off /* 28 */, bool mf) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  const size_t ns = mf ? (size_t)P.n * P.k : (size_t)P.n;   // scaling entries: per column with several frequencies
  put(0, P.nnz * sizeof(float4));               // At (double-float)
  put(1, sizeof(double2) * ns);                 // S
  put(2, sizeof(double) * ns);                  // |D|
  put(3, sizeof(float) * ns);                   // |D| f32
  put(4, sizeof(float4) * P.n * P.k);           // p
  put(5, sizeof(float4) * P.n * P.k);           // q
  put(6, sizeof(float4) * P.n * P.k);           // r
  put(7, sizeof(float4) * P.n * P.k);           // y
  put(8, sizeof(double2) * P.n * P.k);          // r64
  put(9, sizeof(double2) * (size_t)P.nb * P.k * 3);
  put(10, sizeof(CgState) * P.k);
  put(11, sizeof(CgCtl));
  put(12, sizeof(double) * P.k * 6);              // rnorm, target, column scales, inverses, ratios
  put(13, sizeof(int) * (P.k + 1));
  put(14, mf ? sizeof(float4) * P.n * P.k : 0);   // ps = S o p
  put(15, mf ? sizeof(float4) * ns : 0);          // S (double-float)
  put(16, sizeof(double) * P.k);                  // column frequency scales
  put(17, sizeof(float) * 2 * P.k);               // the same as (hi, lo)
  put(18, P.bj.p ? sizeof(double2) * P.bj.s_size() : 0);     // block-Jacobi factors
  put(19, P.bj.p ? sizeof(double2) * P.n * P.k : 0);         // S r64
  // gradient correction (FP32 products): S^-1, diag(G^T A G)^-1, t = invD G^T u,
  // z, u = S^-1 r; z also holds diag(G^T A G)^-1 in FP64 while it is formed
  put(20, P.gn ? sizeof(float2) * ns : 0);
  put(21, P.gn ? sizeof(float2) * P.gn : 0);
  put(22, P.gn ? sizeof(float2) * P.gn * P.k : 0);
  put(23, P.gn ? std::max(sizeof(float4) * P.n * P.k, sizeof(double2) * (size_t)P.gn) : 0);
  put(24, P.gn ? sizeof(float2) * P.n * P.k : 0);
  put(25, P.gn && mf ? sizeof(float) * P.k : 0);   // s_j per column
  return o;
}

int run_cocg_df(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
                const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s,
                const double* col_scale) {
  const bool mf = col_scale != nullptr;
  size_t off[28];
  df_layout(P, off, mf);
  float4* ps = reinterpret_cast<float4*>(ws + off[14]);
  float4* Sdf = reinterpret_cast<float4*>(ws + off[15]);
  double* dscale = reinterpret_cast<double*>(ws + off[16]);
  float* dscale_hl = reinterpret_cast<float*>(ws + off[17]);
  const bool bj = !mf && P.bj.p > 0;
  double2* Sblk = reinterpret_cast<double2*>(ws + off[18]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[19]);
  const bool grad = P.gn > 0;   // diagonal scaling only (checked by pg_cocg / pg_cocg_multifreq)
  float2* Sinv = reinterpret_cast<float2*>(ws + off[20]);
  float2* invD = reinterpret_cast<float2*>(ws + off[21]);
  float2* gt = reinterpret_cast<float2*>(ws + off[22]);
  float4* gz = reinterpret_cast<float4*>(ws + off[23]);
  float2* gu = reinterpret_cast<float2*>(ws + off[24]);
  float* gscale = reinterpret_cast<float*>(ws + off[25]);
  const unsigned gblocks = pg_blocks(P.gn * P.k / kGradQ(P.k), kThreads);   // k_grad_restrict32 only
  float4* At = reinterpret_cast<float4*>(ws + off[0]);
  double2* S = reinterpret_cast<double2*>(ws + off[1]);
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
  double* rnorm = reinterpret_cast<double*>(ws + off[12]);
  double* target = rnorm + P.k;
  // per-column scales of the double-float recurrence: every cycle starts from
  // the true residual scaled to unit norm, so r^T r stays far inside the
  // FP32 exponent range whatever the units of b
  double* cscale = rnorm + 2 * P.k;
  double* cinv = rnorm + 3 * P.k;
  double* clam = rnorm + 4 * P.k;
  int* want = reinterpret_cast<int*>(ws + off[13]);
  int* dstatus = want + P.k;
  const int k = P.k, nb = P.nb;
  // vector-update grid: at least ~4 elements per thread, so the per-block
  // reduction does not dominate on small systems (its last block sums
  // gridDim.x partials)
  const int nbu = (int)std::min<int64_t>(nb, std::max<int64_t>(152 * 2, (P.n * P.k + 4 * kThreads - 1) / (4 * kThreads)));
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);
  const int spmv_grid = 152 * 16;
  if (spmv_grid > nb) return PG_ERR_ARG;

  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  PG_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(CgCtl), s));
  int group = 0;   // rows per entity group for the group product (0: not used)
  if (mf) {
    std::vector<float> hl(2 * (size_t)k);
    for (int i = 0; i < k; ++i) {
      hl[2 * i] = (float)col_scale[i];
      hl[2 * i + 1] = (float)(col_scale[i] - (double)hl[2 * i]);
    }
    PG_CUDA_TRY(cudaMemcpyAsync(dscale, col_scale, sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(dscale_hl, hl.data(), sizeof(float) * 2 * k, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_mf_scaling<K><<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, dscale, S, wd, wdf,
                                                                          dstatus)));
    k_mf_sdf<<<pg_blocks(P.n * k, 256), 256, 0, s>>>(S, P.n * k, Sdf);
    k_mf_df_matrix<<<pg_blocks(P.nnz, 256), 256, 0, s>>>(A, P.nnz, At);
    if (grad) {
      double2* tmp = reinterpret_cast<double2*>(gz);   // FP64 scratch until the first z
      k_grad_sinv<<<pg_blocks(P.n * k, 256), 256, 0, s>>>(S, P.n * k, tmp);
      k_to_f32<<<pg_blocks(P.n * k, 256), 256, 0, s>>>(tmp, P.n * k, Sinv);
      // diag(G^T A_j G) = Re d + i s_j Im d with d = diag(G^T A0 G): exact for
      // every column (the vector P1 columns have Re d != 0); the restriction
      // divides per column
      k_grad_diag<<<pg_blocks(P.gn * 32, 256), 256, 0, s>>>(rowptr, col, A, o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                       P.gn, tmp, 1);
      k_to_f32<<<pg_blocks(P.gn, 256), 256, 0, s>>>(tmp, P.gn, invD);
      std::vector<float> ci(k);
      for (int i = 0; i < k; ++i) ci[i] = (float)col_scale[i];
      PG_CUDA_TRY(cudaMemcpyAsync(gscale, ci.data(), sizeof(float) * k, cudaMemcpyHostToDevice, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));   // ci must outlive the copy
    }
    // the host copy of the scales must outlive the asynchronous copy
    PG_CUDA_TRY(cudaStreamSynchronize(s));
  } else if (bj) {
    const int st0 = bj_setup(P, rowptr, col, A, S, wd, Sblk, At, ToDF(), dstatus, s);
    if (st0) return st0;
    k_wd_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(wd, P.n, wdf);
    if ((P.bj.p == 2 || P.bj.p == 3) && P.n % P.bj.p == 0) {
      // the group product needs every aligned group of p rows on one column list
      int* gflag = reinterpret_cast<int*>(part);
      int hg = 1;
      PG_CUDA_TRY(cudaMemsetAsync(gflag, 0, sizeof(int), s));
      k_group_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, P.n, P.bj.p, gflag);
      PG_LAUNCH_CHECK();
      PG_CUDA_TRY(cudaMemcpyAsync(&hg, gflag, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      group = hg == 0 ? P.bj.p : 0;
    }
  } else {
    k_cg_scaling<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, wd, dstatus);
    k_df_scale_matrix<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, At, wdf, wd);
    if (grad) {
      double2* tmp = reinterpret_cast<double2*>(gz);   // FP64 scratch until the first z
      k_grad_sinv<<<pg_blocks(P.n, 256), 256, 0, s>>>(S, P.n, reinterpret_cast<double2*>(gz));
      k_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(reinterpret_cast<double2*>(gz), P.n, Sinv);
      k_grad_diag<<<pg_blocks(P.gn * 32, 256), 256, 0, s>>>(rowptr, col, A, o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                       P.gn, tmp);
      k_to_f32<<<pg_blocks(P.gn, 256), 256, 0, s>>>(tmp, P.gn, invD);
    }
  }
  PG_LAUNCH_CHECK();
  std::vector<double> bnorm(k), rn(k), tgt(k), sc(k), sc_prev(k, 1.0), scal(4 * (size_t)k);
  std::vector<int> wnt(k);
  PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(b, P.n, part), k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  int hstatus = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_cocg: zero diagonal entry (Jacobi scaling undefined)");
    return PG_ERR_BREAKDOWN;
  }
  auto true_residual = [&]() {
    if (mf) {
      PG_KSWITCH(k, (k_mf_resid<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(rowptr, col, A, P.n, dscale, x, b, r64)));
    } else {
      launch_spmv<double2>(P, rowptr, col, A, x, r64, b, nullptr, npr, s);
    }
  };
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  int64_t its = 0, checks = 0;
  int status = PG_OK;
  const int64_t max_it = o->max_it > 0 ? o->max_it : 100000;
  int chunk = o->check_every > 0 ? o->check_every : 50;
  bool first = true;
  int variant = 41;
  const double delta = 1e-3;   // double-float recurrence: replace after 3 decades
  auto launch_single = [&](int v, cudaStream_t ss) {
    launch_df_spmv1(v, spmv_grid, ss, rowptr, col, At, P.n, pv, q, part, st, ctl);
  };
  // one iteration: product (alpha), vector update (beta), direction update;
  // no per-iteration launch arguments, so a run of them can be captured once
  // in a CUDA graph and replayed
  auto one_iteration = [&](cudaStream_t ss) {
    if (mf && grad) {
      PG_KSWITCH(k, (k_mf_spmm<K><<<spmv_grid, kThreads, 0, ss>>>(rowptr, col, At, P.n, dscale_hl, Sdf, pv, ps, q,
                                                                  part, st, ctl),
                     k_df_update<K, true, true><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2, ctl,
                                                                          0, delta, gu, Sinv),
                     k_grad_restrict32<K, true><<<gblocks, kThreads, 0, ss>>>(o->gradt_rowptr, o->gradt_row,
                                                                           o->gradt_val, invD, gu, P.gn, gt, ctl, 0,
                                                                           gscale),
                     k_dfg_prolong<K, true><<<nbu, kThreads, 0, ss>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv,
                                                                      gt, r, P.n, gz, pv, 0, part, st, ctl, 0),
                     k_df_pupdate<K, true><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, gz, P.n, st, ctl,
                                                                                              ps, Sdf)));
      return;
    }
    if (mf) {
      PG_KSWITCH(k, (k_mf_spmm<K><<<spmv_grid, kThreads, 0, ss>>>(rowptr, col, At, P.n, dscale_hl, Sdf, pv, ps, q,
                                                                  part, st, ctl),
                     k_df_update<K, true><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2, ctl, 0,
                                                                    delta),
                     k_df_pupdate<K, true><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, r, P.n, st, ctl,
                                                                                              ps, Sdf)));
      return;
    }
    if (k == 1)
      launch_single(variant, ss);
    else
      PG_KSWITCH(k, (launch_df_spmm<K>(variant, spmv_grid, ss, rowptr, col, At, P.n, pv, q, part, st, ctl)));
    if (grad) {
      PG_KSWITCH(k, (k_df_update<K, false, true><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2,
                                                                           ctl, 0, delta, gu, Sinv),
                     k_grad_restrict32<K><<<gblocks, kThreads, 0, ss>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                     invD, gu, P.gn, gt, ctl, 0),
                     k_dfg_prolong<K><<<nbu, kThreads, 0, ss>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv, gt,
                                                                r, P.n, gz, pv, 0, part, st, ctl, 0),
                     k_df_pupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, gz, P.n, st, ctl)));
      return;
    }
    PG_KSWITCH(k, (k_df_update<K><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2, ctl, 0, delta),
                   k_df_pupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, r, P.n, st, ctl)));
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
      for (int g = 0; g < kGraphIters; ++g) one_iteration(cs);
      ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph != nullptr;
    }
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      cudaGetLastError();   // capture unavailable: keep launching directly
      gexec = nullptr;
      graph_failed = true;
    }
  };
  struct GraphCleanup {
    cudaStream_t& cs;
    cudaEvent_t& a;
    cudaEvent_t& b;
    cudaGraphExec_t& g;
    ~GraphCleanup() {
      if (g) cudaGraphExecDestroy(g);
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (cs) cudaStreamDestroy(cs);
    }
  } graph_cleanup{cs, ev_in, ev_out, gexec};
  for (;;) {
    true_residual();
    PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                   k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    CgCtl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!first && hctl.nonfinite) {
      pg_set_error("pg_cocg: non-finite residual");
      status = PG_ERR_NONFINITE;
      break;
    }
    bool all = true;
    for (int i = 0; i < k; ++i) {
      if (monitor)
        fprintf(stderr, "pg_cocg(df64): check %lld its %lld rhs %d true ||r||/||b|| = %.6e\n", (long long)checks,
                (long long)its, i, bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0);
      if (!isfinite(rn[i])) {
        pg_set_error("pg_cocg: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[i];
      const bool ok = rn[i] <= tb || bnorm[i] == 0.0;
      wnt[i] = ok ? 0 : 1;
      sc[i] = rn[i] > 0.0 && isfinite(rn[i]) ? rn[i] : 1.0;
      tgt[i] = 0.5 * tb / sc[i];
      if (!ok) all = false;
    }
    if (status || all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    // unit-norm cycle: the residual estimate starts at 1 (0 for an exact
    // column), p is carried over in the new scale
    for (int i = 0; i < k; ++i) {
      scal[i] = rn[i] > 0.0 ? 1.0 : 0.0;
      scal[k + i] = sc[i];
      scal[2 * k + i] = 1.0 / sc[i];
      scal[3 * k + i] = sc_prev[i] / sc[i];
      sc_prev[i] = sc[i];
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(rnorm, scal.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(cscale, scal.data() + k, sizeof(double) * 3 * k, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_scale_cols_d2<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, P.n, cinv)));
    if (!first) {
      PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(pv, P.n, clam)));
      if (mf) PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(ps, P.n, clam)));
    }
    if (mf && grad) {
      PG_KSWITCH(k, (k_df_start<K, true><<<nb, kThreads, 0, s>>>(r64, S, P.n, r, y, pv, 0, part, ps),
                     k_dfg_u_start<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, P.n, gu),
                     k_grad_restrict32<K, true><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row,
                                                                          o->gradt_val, invD, gu, P.gn, gt, ctl, 1,
                                                                          gscale),
                     k_dfg_prolong<K, true><<<nb, kThreads, 0, s>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv,
                                                                     gt, r, P.n, gz, pv, first ? 1 : 0, part, st, ctl,
                                                                     1, ps, Sdf)));
    } else if (mf) {
      PG_KSWITCH(k, (k_df_start<K, true><<<nb, kThreads, 0, s>>>(r64, S, P.n, r, y, pv, first ? 1 : 0, part, ps)));
    } else {
      if (bj) PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, r64, r64b)));
      if (grad) {
        // r = S r64, then z = r + S^-1 G invD G^T S^-1 r and rho = r^T z (p = z on the first cycle)
        PG_KSWITCH(k, (k_df_start<K><<<nb, kThreads, 0, s>>>(r64, S, P.n, r, y, pv, 0, part),
                       k_dfg_u_start<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, P.n, gu),
                       k_grad_restrict32<K><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                      invD, gu, P.gn, gt, ctl, 1),
                       k_dfg_prolong<K><<<nb, kThreads, 0, s>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv, gt,
                                                                r, P.n, gz, pv, first ? 1 : 0, part, st, ctl, 1)));
      } else {
        PG_KSWITCH(k, (k_df_start<K><<<nb, kThreads, 0, s>>>(bj ? r64b : r64, S, P.n, r, y, pv, first ? 1 : 0,
                                                             part)));
      }
    }
    PG_KSWITCH(k, (k_cg_cycle_init<K><<<1, 32 * K, 0, s>>>(part, nb, st, rnorm, target, want, ctl, first ? 1 : 0)));
    if (first && !mf) {
      variant = forced_variant(k, group);
      if (variant < 0) variant = tuned_variant(P.n, P.nnz, k, group);
      if (variant < 0) {
        if (autotune_enabled()) {
          if (k == 1) {
            std::vector<int> cands = {41, 42, 22, 82, 21};
            if (group)
              for (int gv : {2, 4, 8, 12, 14, 32, 34, 44, 54}) cands.push_back(100 * group + gv);
            variant = pick_fastest(cands, [&](int v) { launch_single(v, s); }, s);
          } else {
            std::vector<int> cands = {1, 2};
            if (group) {
              cands.push_back(100 * group);
              cands.push_back(100 * group + 50);
            }
            variant = pick_fastest(cands, [&](int v) {
              PG_KSWITCH(k, (launch_df_spmm<K>(v, spmv_grid, s, rowptr, col, At, P.n, pv, q, part, st, ctl)));
            }, s);
          }
          PG_LAUNCH_CHECK();
        } else {
          variant = k == 1 ? 41 : 1;
        }
        store_variant(P.n, P.nnz, k, group, variant);
      }
      if (monitor) fprintf(stderr, "pg_cocg(df64): SpMV variant %d for n=%lld nnz=%lld k=%d\n", variant,
                           (long long)P.n, (long long)P.nnz, k);
    }
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    int done = 0;
    if (use_graphs && steps >= kGraphIters) {
      if (!gexec) build_graph();
      if (gexec) {
        // replay the captured iterations on the capture stream, joined to s
        cudaEventRecord(ev_in, s);
        cudaStreamWaitEvent(cs, ev_in, 0);
        for (; done + kGraphIters <= steps; done += kGraphIters) cudaGraphLaunch(gexec, cs);
        cudaEventRecord(ev_out, cs);
        cudaStreamWaitEvent(s, ev_out, 0);
      }
    }
    for (; done < steps; ++done) one_iteration(s);
    PG_LAUNCH_CHECK();
    PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(y, P.n, cscale)));
    if (mf) {
      PG_KSWITCH(k, (k_df_xupdate<K, true><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, S, P.n, x)));
    } else if (bj) {
      PG_KSWITCH(k, (k_bj_apply_t_add<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, y, x, DfToD2())));
    } else {
      PG_KSWITCH(k, (k_df_xupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, S, P.n, x)));
    }
    std::vector<int> hits(k), hbrk(k);
    for (int i = 0; i < k; ++i) {
      PG_CUDA_TRY(cudaMemcpyAsync(&hits[i], &st[i].its, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaMemcpyAsync(&hbrk[i], &st[i].breakdown, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    for (int i = 0; i < k; ++i) used = hits[i] > used ? hits[i] : used;
    const int64_t cycle_its = used - its;
    its = used;
    ++checks;
    bool brk = false;
    for (int i = 0; i < k; ++i) brk = brk || hbrk[i];
    if (brk) {
      pg_set_error("pg_cocg: breakdown (p^T A p = 0 or r^T r = 0)");
      status = PG_ERR_BREAKDOWN;
      true_residual();
      PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                     k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
      PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      break;
    }
    int64_t c2 = cycle_its + cycle_its / 4 + 8;
    chunk = (int)(c2 < 16 ? 16 : (c2 > 4000 ? 4000 : c2));
  }
  double worst = 0.0;
  for (int i = 0; i < k; ++i) {
    const double rr = bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0;
    if (relres_out) relres_out[i] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = checks;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_cocg: max_it reached before rtol");
  return status;
}

}  // namespace pgk

using pgk::df_layout;
using pgk::run_cocg_df;
extern "C" size_t pg_cocg_multifreq_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* opts) {
  if (n < 1 || !valid_k(nrhs)) return 0;
  pg_cocg_opts o;
  pg_cocg_default_opts(&o);
  if (opts) o = *opts;
  o.precision = 2;
  o.block_p = 0;
  Plan P = cg_plan(n, nnz, nrhs, &o);
  size_t off[28];
  return df_layout(P, off, true) + 256;
}

extern "C" int pg_cocg_multifreq(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                                 const double* b, double* x, int nrhs, const double* col_scale,
                                 const pg_cocg_opts* opts, pg_gmres_result* result, double* relres_per_rhs,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || !col_scale || n < 1 || nnz < n || !valid_k(nrhs) ||
      !(opts->rtol > 0.0) || opts->precision != 2) {
    pg_set_error("pg_cocg_multifreq: bad argument (nrhs 1..32 power of two, rtol > 0, precision 2)");
    return PG_ERR_ARG;
  }
  for (int i = 0; i < nrhs; ++i)
    if (!(col_scale[i] > 0.0) || !isfinite(col_scale[i])) {
      pg_set_error("pg_cocg_multifreq: column frequency scales must be positive");
      return PG_ERR_ARG;
    }
  if (opts->grad_rowptr && (!opts->grad_col || !opts->grad_val || !opts->gradt_rowptr || !opts->gradt_row ||
                            !opts->gradt_val || opts->grad_cols < 1 || opts->grad_cols >= (int64_t(1) << 31))) {
    pg_set_error("pg_cocg_multifreq: gradient correction needs all six G arrays and grad_cols >= 1");
    return PG_ERR_ARG;
  }
  const size_t need = pg_cocg_multifreq_workspace_bytes(n, nnz, nrhs, opts);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_cocg_multifreq: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  pg_cocg_opts o = *opts;
  o.block_p = 0;   // diagonal scaling per column
  Plan P = cg_plan(n, nnz, nrhs, &o);
  return run_cocg_df(P, rowptr, col, reinterpret_cast<const double2*>(vals), reinterpret_cast<const double2*>(b),
                     reinterpret_cast<double2*>(x), &o, result, relres_per_rhs, ws, pg_stream(stream), col_scale);
}

