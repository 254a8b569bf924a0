// Adjoint sensitivities of a batched linear transient (trapezoidal or backward Euler).
//
// The reference has no sensitivity code; this is the discrete adjoint of the companion-model
// recurrence the transient engine integrates.  In matrix form one step is
//     M x_{n+1} = N x_n + s_{n+1} + s_n,     TR: M = G + (2/h) C,  N = (2/h) C - G
//                                            BE: M = G + C/h,      N = C/h     (s_n -> 0)
// (G: conductances and incidence, C: capacitances and -L on inductor branches).  For a loss
// L = sum_{n=1..N} x_out(t_n)^2 the adjoint recurrence is
//     M^T lambda_n = dl/dx_n + N^T lambda_{n+1},   lambda_{N+1} = 0
// and dL/dtheta = sum_n lambda_n^T (dN/dtheta x_{n-1} - dM/dtheta x_n).  Per element:
//     R (TR): (1/R^2) (l_p - l_m)(v_{n-1} + v_n)      R (BE): (1/R^2) (l_p - l_m) v_n
//     C:      (2/h | 1/h) (l_p - l_m)(v_{n-1} - v_n)
//     L:      (2/h | 1/h) l_b (i_n - i_{n-1})
// With TR, N^T lambda_{n+1} = 2 (2/h) C^T lambda_{n+1} - M^T lambda_{n+1}, and
// M^T lambda_{n+1} is the right-hand side of the previous backward step, so a backward step
// costs one transposed solve plus O(elements) work, like a forward step.
//
// Memory: the forward pass stores a checkpoint (state and TR capacitor currents) every K
// steps and keeps the states of the last segment; the backward sweep walks the segments from
// the last, recomputing each segment's states from its checkpoint into a segment buffer.
// Transposed solves use the same LU values (double-float) through the transposed program
// built by the host symbolic pass.  The operating point at t = 0 must be zero (the
// sensitivity of a non-zero operating point is not propagated; the call reports it).
#pragma once

#include "warp_kernels.cuh"

namespace krets {

#define KS_OP_NONZERO 64

struct AdjLay {
  int lu, x, cdyn, cb, icap, lam, cba, slot, coef64;
  int bytes;
  int sprog_bytes, tprog_bytes;
};

// One row of a transposed solve (entries sub, sub + spl, ... of it), without the diagonal.
__device__ __forceinline__ df df_trow(const int4 d, const int2 *ent, const df *__restrict__ lu, const df *z, int sub,
                                      int spl) {
  const int r = d.x & 0xffff, cnt = (int)((unsigned)d.x >> 16);
  df s = sub == 0 ? z[r] : df{0.f, 0.f};
  for (int e = d.y + sub; e < d.y + cnt; e += spl) {
    const int2 en = ent[e];
    s = df_fma_acc(df_neg(lu[en.x]), z[en.y], s);
  }
  return df_norm(s);
}

// One level of a transposed solve: rows split over `spl` lanes as in df_level_split, or,
// unsplit, two rows in flight per thread.
template <bool UPPER>
__device__ __forceinline__ void df_tlevel(const int *ptr, const int4 *desc, const int2 *ent, int l,
                                          const df *__restrict__ lu, df *z, int gl, int nthreads, int spl) {
  const int r0 = ptr[l], r1 = ptr[l + 1];
  if (spl == 1) {
    for (int t = r0 + gl; t < r1; t += 2 * nthreads) {
      const int4 d0 = desc[t];
      const bool two = t + nthreads < r1;
      const int4 d1 = two ? desc[t + nthreads] : d0;
      df v0 = df_trow(d0, ent, lu, z, 0, 1);
      df v1 = two ? df_trow(d1, ent, lu, z, 0, 1) : v0;
      if (UPPER) {
        v0 = df_mul(v0, lu[d0.z]);
        v1 = df_mul(v1, lu[d1.z]);
      }
      z[d0.x & 0xffff] = v0;
      if (two) z[d1.x & 0xffff] = v1;
    }
    return;
  }
  const int sub = gl & (spl - 1);
  const unsigned mask = lane_mask(spl);
  for (int t = r0 + gl / spl; t < r1; t += nthreads / spl) {
    const int4 d = desc[t];
    df s = df_lane_sum(df_trow(d, ent, lu, z, sub, spl), spl, mask);
    if (sub == 0) z[d.x & 0xffff] = UPPER ? df_mul(s, lu[d.z]) : s;
  }
}

// Transposed solve A^T y = c, in place on z: on entry z[j] = c at column position j, on exit
// z[k] = y at row position k.  lu holds the LU with reciprocal diagonals (df).
template <int G>
__device__ __forceinline__ void df_tsolve(const int *T, const int *toff, int nut, int nlt, const df *__restrict__ lu,
                                          df *z, int gl, int gid) {
  const int *ut_ptr = T + toff[0];
  const int4 *ut_desc = reinterpret_cast<const int4 *>(T + toff[1]);
  const int *lt_ptr = T + toff[2];
  const int4 *lt_desc = reinterpret_cast<const int4 *>(T + toff[3]);
  const int2 *ent = reinterpret_cast<const int2 *>(T + toff[4]);
  const int *ut_max = T + toff[6], *lt_max = T + toff[7];
  for (int l = 0; l < nut; ++l) {
    df_tlevel<true>(ut_ptr, ut_desc, ent, l, lu, z, gl, G, split_lanes<G>(ut_max[l]));
    gsync<G>(gid);
  }
  for (int l = 0; l < nlt; ++l) {
    df_tlevel<false>(lt_ptr, lt_desc, ent, l, lu, z, gl, G, split_lanes<G>(lt_max[l]));
    gsync<G>(gid);
  }
}

// One forward step of the double-float engine on x (in place), as k_tran_dfd; row splits
// chosen for a group of SG threads (the forward pass splits rows for the whole CTA, the
// recomputation for its half, so recomputed states match the forward pass's to rounding).
// CBREC (trapezoidal rule): the capacitor history is carried as the companion current in
// cb itself (cb <- 2 (2C/h) v - cb, as dfd_steps), so no pass after the solve forms the
// currents and the step ends at the solve's last barrier (the next step's first barrier
// orders every read of x before the gather overwrites it).
template <int G, int SG, bool CBREC = false>
__device__ __forceinline__ void adj_forward_step(const DevProg &P, const SProg &S, const df *lu, df *x, const df *cdyn,
                                                 df *cb, df *icap, const double *vals, int method, int step, double h,
                                                 const WaveTab &wt, int gl, int gid) {
  for (int d = gl; d < P.ndyn; d += G) {
    const int4 dd = S.dyn[d];
    const int kind = (int)((unsigned)dd.x >> 24);
    df v{0.f, 0.f};
    if (kind == KRETS_ELEM_C) {
      const df vprev = df_sub(df_at(x, dd.y), df_at(x, dd.z));
      if (CBREC) {
        const df c2{2.f * cdyn[d].hi, 2.f * cdyn[d].lo};  // exact doubling
        v = df_fma(c2, vprev, df_neg(cb[d]));
      } else {
        v = method == KRETS_METHOD_TR ? df_fma(cdyn[d], vprev, icap[d]) : df_mul(cdyn[d], vprev);
      }
    } else if (kind == KRETS_ELEM_L) {
      const df li = df_neg(df_mul(cdyn[d], x[dd.w]));
      v = method == KRETS_METHOD_TR ? df_sub(li, df_sub(df_at(x, dd.y), df_at(x, dd.z))) : li;
    } else if (kind == KRETS_ELEM_V) {
      const int e = dd.x & 0xffffff;
      const krets_element &E = P.el[e];
      const int wr = wt.tab ? wt.row[d] : -1;
      if (wr >= 0) v = df_from_double(wt.tab[(size_t)wr * wt.stride + step]);
      else if (E.wave == KRETS_WAVE_NONE) v = cdyn[d];
      else v = df_from_double(wave_value(E, vals ? vals[e] : E.value, (double)step * h));
    } else if (kind == KRETS_ELEM_I) {
      v = cdyn[d];
    }
    cb[d] = v;
  }
  gsync<G>(gid);
  for (int k = gl; k < P.n; k += G) {
    df acc{0.f, 0.f};
    for (int u = S.bd_ptr[k]; u < S.bd_ptr[k + 1]; ++u) {
      const int code = S.bd_op[u];
      acc = df_add(acc, (code & 1) ? df_neg(cb[code >> 1]) : cb[code >> 1]);
    }
    x[k] = acc;
  }
  gsync<G>(gid);
  df_solve<G, false, SG>(S, lu, x, gl, gid, -1);
  df_solve<G, true, SG>(S, lu, x, gl, gid, -1);
  if (CBREC) return;
  if (method == KRETS_METHOD_TR) {
    for (int d = gl; d < P.ncap; d += G) {
      const int4 dd = S.dyn[d];
      const df vn = df_sub(df_at(x, dd.y), df_at(x, dd.z));
      icap[d] = df_sub(df_mul(cdyn[d], vn), cb[d]);
    }
  }
  gsync<G>(gid);
}

// One instance per CTA of 512 threads.  Set-up and the forward pass run on all of them;
// the reverse sweep is pipelined over the two halves.  In iteration j (segments from the
// last), threads 0-255 walk segment j backwards: the scaled C^T lambda, the right-hand side
// and the transposed solves, writing every lambda_n to a history buffer.  Meanwhile threads
// 256-511 recompute segment j-1 from its checkpoint and then form the gradient terms of
// segment j+1 from its stored states and lambda history, with no barrier (a thread per
// element, summing over the segment's steps).  The backward steps are the only latency-
// bound chain left; the recomputation and the gradient fill the idle issue slots.
// Buffers per CTA (global memory): checkpoints J x (n + ncap), three segment buffers of
// (K+1) x n states (segment j in buffer j % 3) and two lambda histories of K x n (j & 1).
//
// mode 0: forward pass only (loss), mode 1: loss and gradient, mode 2: gradient only, the
// forward pass having run on the double-float engine (k_tran_dfd with AdjFwd: per-instance
// checkpoints and the loss); the last segment is then recomputed from its checkpoint.
// ck_cb (mode 2, trapezoidal rule): the checkpoints hold the capacitors' companion values
// (the forward pass ran the direct right-hand-side step) instead of their currents.
// adj: per element {kind, row position of p, row position of m, row position of branch}
// cc_ptr/cc_op: per column position, the rhs contributions of C^T lambda: range
//       [cc_ptr[j], cc_ptr[j+1]) of (dyn index << 1 | neg) entries.
// Register caches (one warp thread owns rows / dynamic elements / elements t + 256 i):
// backward half: RK rows (previous rhs, up to two C^T lambda terms), RD dynamic elements
// (row positions); recompute half: RE elements (positions, gradient sums).  The host
// launches this only for n <= 256 RK, ndyn <= 256 RD and ne <= 256 RE.
// Named barriers: 1 = whole CTA as one group, 2 = backward half, 3 = recompute half.
constexpr int kAdjThreads = 512, kAdjHalf = 256;
constexpr int kNone = 0xffff;  // absent position in a packed pair

__device__ __forceinline__ df df_pick(const df *v, int i) { return i != kNone ? v[i] : df{0.f, 0.f}; }
__device__ __forceinline__ int pack2(int a, int b) { return (a < 0 ? kNone : a) | ((b < 0 ? kNone : b) << 16); }

template <int RK, int RD, int RE>
__global__ void __launch_bounds__(kAdjThreads, 1)
    k_adjoint_dfd(DevProg P, AdjLay L, const double *values, int n_inst, double h, int n_steps, int method, int K,
                  int out_pos, const int4 *adj, const int *cc_ptr, const int *cc_op, df *ckpt, df *seg, df *hist,
                  double *loss_out, double *grad_out, int *inst_status, int *queue, int mode, WaveTab wt,
                  int ck_cb) {
  constexpr int GF = kAdjThreads, GH = kAdjHalf;
  extern __shared__ __align__(16) char smem[];
  const int tid = threadIdx.x;
  {
    // step program without its residual operators; tp_off[5] ends the transposed program
    const int sw = P.sp_off[5], tw = P.tp_off[5];
    const int4 *src = reinterpret_cast<const int4 *>(P.sprog);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int i = tid; i < sw / 4; i += GF) dst[i] = src[i];
    const int4 *tsrc = reinterpret_cast<const int4 *>(P.tprog);
    int4 *tdst = reinterpret_cast<int4 *>(smem + L.sprog_bytes);
    for (int i = tid; i < tw / 4; i += GF) tdst[i] = tsrc[i];
    __syncthreads();
  }
  const SProg S = sprog_view(P, reinterpret_cast<const int *>(smem));
  const int *T = reinterpret_cast<const int *>(smem + L.sprog_bytes);
  char *base = smem + L.sprog_bytes + L.tprog_bytes;
  df *lu = reinterpret_cast<df *>(base + L.lu);
  double *lu64 = reinterpret_cast<double *>(base + L.lu);
  df *x = reinterpret_cast<df *>(base + L.x);
  df *cdyn = reinterpret_cast<df *>(base + L.cdyn);
  df *cb = reinterpret_cast<df *>(base + L.cb);
  df *icap = reinterpret_cast<df *>(base + L.icap);
  df *lam = reinterpret_cast<df *>(base + L.lam);
  df *cba = reinterpret_cast<df *>(base + L.cba);
  int *slot = reinterpret_cast<int *>(base + L.slot);
  double *coef64 = reinterpret_cast<double *>(base + L.coef64);
  const bool back_half = tid < GH;
  const int hl = tid & (GH - 1);
  const int n = P.n;
  const bool tr = method == KRETS_METHOD_TR;
  // ---- register caches of the index data the reverse sweep reads every step (filled
  // before each reverse sweep, so they are not live during the forward pass)
  int crow[RD];              // backward half: dynamic element's row positions (C: p | m << 16, L: branch)
  int cc0[RK], cc1[RK];      // backward half: up to two C^T terms per row, -1 none, cc1 = -2: use the list
  int erow[RE], ecol[RE];    // recompute half: element's row / column positions (p | m << 16, L: branch)
  int ekind = 0;             // owned elements: 3 bits each: 0 none, 1 R, 2 C, 3 L, 4 source
  // the backward half, faster per segment, forms the gradient terms of about 3/8 of the
  // elements (slots i < RB), the recompute half the rest
  constexpr int RB = (RE * 3 + 4) / 8;
  const int J = (n_steps + K - 1) / K;          // segments
  const size_t ck_words = (size_t)n + P.ncap;  // per checkpoint, in df
  const size_t seg_words = (size_t)(K + 1) * n, hist_words = (size_t)K * n;
  df *cta_ck = ckpt + (size_t)blockIdx.x * J * ck_words;  // modes 0/1: the CTA's checkpoints
  df *my_seg = seg + (size_t)blockIdx.x * 3 * seg_words;
  df *my_hist = hist + (size_t)blockIdx.x * 2 * hist_words;
  while (true) {
    if (tid == 0) slot[0] = atomicAdd(queue, 1);
    __syncthreads();
    const int inst = slot[0];
    __syncthreads();
    if (inst >= n_inst) break;
    const double *vals = values ? values + (size_t)inst * P.ne : nullptr;
    // mode 2: the forward pass ran on the double-float engine, checkpoints per instance
    df *my_ck = mode == 2 ? ckpt + (size_t)inst * J * ck_words : cta_ck;
    // ---- set-up (as the double-float transient engine)
    int st = g_coef_pass<GF>(P, vals, h, method, coef64, tid);
    gsync<GF>(0);
    for (int sl = tid; sl < P.nnz_lu; sl += GF) {
      const int t = P.lu_src[sl];
      lu64[sl] = t < 0 ? 0.0 : sum_entry<double>(P, t, coef64, nullptr);
    }
    gsync<GF>(0);
    st |= g_factor64<GF>(P, lu64, tid, 0);
    for (int sl = tid; sl < P.nnz_lu; sl += GF) lu[sl] = df_from_double(lu64[sl]);
    for (int d = tid; d < P.ndyn; d += GF) {
      const int e = S.dyn[d].x & 0xffffff;
      const krets_element &E = P.el[e];
      const double val = vals ? vals[e] : E.value;
      double c = val;
      if (E.kind == KRETS_ELEM_C || E.kind == KRETS_ELEM_L) c = tr ? 2.0 * val / h : val / h;
      cdyn[d] = df_from_double(c);
    }
    // zero operating point (the recurrence starts from x_0 = 0, icap = 0)
    for (int k = tid; k < n; k += GF) x[k] = df{0.f, 0.f};
    for (int d = tid; d < P.ncap; d += GF) icap[d] = df{0.f, 0.f};
    df wr[RK], gr[RE];
#pragma unroll
    for (int i = 0; i < RK; ++i) wr[i] = df{0.f, 0.f};
#pragma unroll
    for (int i = 0; i < RE; ++i) gr[i] = df{0.f, 0.f};
    gsync<GF>(0);
    df loss{0.f, 0.f};  // thread 0 accumulates
    const bool fatal = gany<GF>((st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) != 0, 0);
    // ---- forward pass with checkpoints; the last segment's states go to its buffer
    const int last0 = (J - 1) * K;
    df *last_seg = my_seg + (size_t)((J - 1) % 3) * seg_words;
    for (int s = 1; s <= n_steps && !fatal && mode != 2; ++s) {
      if ((s - 1) % K == 0) {
        df *ck = my_ck + (size_t)((s - 1) / K) * ck_words;
        for (int k = tid; k < n; k += GF) ck[k] = x[k];
        for (int d = tid; d < P.ncap; d += GF) ck[n + d] = icap[d];
      }
      if (mode == 1 && s - 1 == last0)
        for (int k = tid; k < n; k += GF) last_seg[k] = x[k];
      adj_forward_step<GF, GF>(P, S, lu, x, cdyn, cb, icap, vals, method, s, h, wt, tid, 0);
      if (tid == 0) loss = df_fma(x[out_pos], x[out_pos], loss);
      if (mode == 1 && s > last0)
        for (int k = tid; k < n; k += GF) last_seg[(size_t)(s - last0) * n + k] = x[k];
    }
    // gradient terms of segment jj (recompute half): states from buffer jj % 3, lambda
    // history from buffer jj & 1; thread per element, steps in order
    auto segment_gradient = [&](int jj) {
      const int s0 = jj * K, s1 = min(s0 + K, n_steps);
      const df *sg = my_seg + (size_t)(jj % 3) * seg_words;
      const df *hs = my_hist + (size_t)(jj & 1) * hist_words;
      for (int nn = s0 + 1; nn <= s1; ++nn) {
        const df *ln = hs + (size_t)(nn - s0 - 1) * n;
        const df *xn = sg + (size_t)(nn - s0) * n, *xp = xn - n;
#pragma unroll
        for (int i = 0; i < RE; ++i) {
          const int kind = (ekind >> (3 * i)) & 7;
          if (!kind) continue;
          const int rp = erow[i] & 0xffff, rm = (int)((unsigned)erow[i] >> 16);
          const int cp = ecol[i] & 0xffff, cm = (int)((unsigned)ecol[i] >> 16);
          df term;
          if (kind == 4) {
            // source: rhs of step nn at its row is w_nn (BE) or w_nn + w_{nn-1} (TR form)
            const int d = ecol[i], e = hl + i * GH;
            const int wr = wt.tab ? wt.row[d] : -1;
            const double dc = vals ? vals[e] : P.el[e].value;
            const double w1 = wr >= 0 ? wt.tab[(size_t)wr * wt.stride + nn] : dc;
            const double w0 = wr >= 0 ? wt.tab[(size_t)wr * wt.stride + nn - 1] : dc;
            term = df_mul(ln[rp], df_from_double(tr ? w1 + w0 : w1));
          } else if (kind == 3) {
            term = df_mul(ln[rp], df_sub(xn[cp], xp[cp]));
          } else {
            const df dl = df_sub(df_pick(ln, rp), df_pick(ln, rm));
            const df vn = df_sub(df_pick(xn, cp), df_pick(xn, cm));
            const df vp = df_sub(df_pick(xp, cp), df_pick(xp, cm));
            term = df_mul(dl, kind == 1 ? (tr ? df_add(vp, vn) : vn) : df_sub(vp, vn));
          }
          gr[i] = df_add(gr[i], term);
        }
      }
    };
    if (mode == 2 && !fatal) {
      // the last segment's states, from its checkpoint (the forward pass kept none)
      const df *ck = my_ck + (size_t)(J - 1) * ck_words;
      for (int k = tid; k < n; k += GF) {
        x[k] = ck[k];
        last_seg[k] = ck[k];
      }
      if (tr && ck_cb) {
        for (int d = tid; d < P.ncap; d += GF) cb[d] = ck[n + d];
        gsync<GF>(0);
        for (int s = last0 + 1; s <= n_steps; ++s) {
          adj_forward_step<GF, GF, true>(P, S, lu, x, cdyn, cb, icap, vals, method, s, h, wt, tid, 0);
          for (int k = tid; k < n; k += GF) last_seg[(size_t)(s - last0) * n + k] = x[k];
        }
      } else {
        for (int d = tid; d < P.ncap; d += GF) icap[d] = ck[n + d];
        gsync<GF>(0);
        for (int s = last0 + 1; s <= n_steps; ++s) {
          adj_forward_step<GF, GF>(P, S, lu, x, cdyn, cb, icap, vals, method, s, h, wt, tid, 0);
          for (int k = tid; k < n; k += GF) last_seg[(size_t)(s - last0) * n + k] = x[k];
        }
      }
      gsync<GF>(0);
    }
    if ((mode == 1 || mode == 2) && !fatal) {
      for (int k = tid; k < n; k += GF) lam[k] = df{0.f, 0.f};
      ekind = 0;
      if (back_half) {
#pragma unroll
        for (int i = 0; i < RD; ++i) {
          const int d = hl + i * GH;
          crow[i] = kNone | (kNone << 16);
          if (d < P.ndyn) {
            const int4 a = adj[S.dyn[d].x & 0xffffff];
            crow[i] = (a.x & 0xff) == KRETS_ELEM_L ? pack2(a.w, -1) : pack2(a.y, a.z);
          }
        }
#pragma unroll
        for (int i = 0; i < RK; ++i) {
          const int k = hl + i * GH;
          cc0[i] = cc1[i] = -1;
          if (k < n) {
            const int c0 = cc_ptr[k], cnt = cc_ptr[k + 1] - c0;
            if (cnt > 2) cc1[i] = -2;
            else {
              if (cnt > 0) cc0[i] = cc_op[c0];
              if (cnt > 1) cc1[i] = cc_op[c0 + 1];
            }
          }
        }
      }
      // element caches: the backward half owns slots i < RB of its lane's elements, the
      // recompute half the others (their gradient terms are formed by the owner)
#pragma unroll
      for (int i = 0; i < RE; ++i) {
        const int e = hl + i * GH;
        erow[i] = ecol[i] = kNone | (kNone << 16);
        if (e < P.ne && (back_half ? i < RB : i >= RB)) {
          {
            const int4 a = adj[e];
            const int4 pos = P.el_pos[e];
            const int kind = a.x & 0xff;
            int code = 0;
            if (kind == KRETS_ELEM_R || kind == KRETS_ELEM_C) {
              code = kind == KRETS_ELEM_R ? 1 : 2;
              erow[i] = pack2(a.y, a.z);
              ecol[i] = pack2(pos.x, pos.y);
            } else if (kind == KRETS_ELEM_L) {
              code = 3;
              erow[i] = pack2(a.w, -1);
              ecol[i] = pack2(pos.z, -1);
            } else if ((kind == KRETS_ELEM_V || kind == KRETS_ELEM_I) && a.w >= 0 && (a.x >> 8) > 0) {
              code = 4;
              erow[i] = pack2(a.w, -1);
              ecol[i] = (a.x >> 8) - 1;  // rhs-element index
            }
            ekind |= code << (3 * i);
          }
        }
      }
      __syncthreads();
      for (int j = J - 1; j >= 0; --j) {
        if (back_half) {
          // ---- backward over segment j; states x_{s0..s1} in buffer j % 3
          const int s0 = j * K, s1 = min(s0 + K, n_steps);
          const df *sg = my_seg + (size_t)(j % 3) * seg_words;
          df *hs = my_hist + (size_t)(j & 1) * hist_words;
          // x_out of the step, loaded one step ahead by the thread that owns row out_pos
          const bool own_out = (out_pos & (GH - 1)) == hl;
          df xo_next = own_out ? sg[(size_t)(s1 - s0) * n + out_pos] : df{0.f, 0.f};
          for (int nn = s1; nn > s0; --nn) {
            const df xo = xo_next;
            if (own_out && nn - 1 > s0) xo_next = sg[(size_t)(nn - 1 - s0) * n + out_pos];
            // scaled C^T lambda_{nn+1} per dynamic element
#pragma unroll
            for (int i = 0; i < RD; ++i) {
              const int d = hl + i * GH;
              if (d < P.ndyn) {
                const int kind = (int)((unsigned)S.dyn[d].x >> 24);
                const int r0 = crow[i] & 0xffff, r1 = (int)((unsigned)crow[i] >> 16);
                df u{0.f, 0.f};
                if (kind == KRETS_ELEM_C) u = df_mul(cdyn[d], df_sub(df_pick(lam, r0), df_pick(lam, r1)));
                else if (kind == KRETS_ELEM_L) u = df_neg(df_mul(cdyn[d], lam[r0]));
                if (tr) u = df{2.f * u.hi, 2.f * u.lo};  // exact doubling
                cba[d] = u;
              }
            }
            gsync<GH>(1);
            // rhs (column positions) = dl/dx + N^T lambda_{nn+1}; it is also M^T lambda_nn
#pragma unroll
            for (int i = 0; i < RK; ++i) {
              const int k = hl + i * GH;
              if (k < n) {
                df acc{0.f, 0.f};
                if (cc1[i] == -2) {
                  for (int u = cc_ptr[k]; u < cc_ptr[k + 1]; ++u) {
                    const int code = cc_op[u];
                    acc = df_add(acc, (code & 1) ? df_neg(cba[code >> 1]) : cba[code >> 1]);
                  }
                } else {
                  if (cc0[i] >= 0) acc = (cc0[i] & 1) ? df_neg(cba[cc0[i] >> 1]) : cba[cc0[i] >> 1];
                  if (cc1[i] >= 0) acc = df_add(acc, (cc1[i] & 1) ? df_neg(cba[cc1[i] >> 1]) : cba[cc1[i] >> 1]);
                }
                if (tr) acc = df_sub(acc, wr[i]);
                if (k == out_pos) acc = df_add(acc, df{2.f * xo.hi, 2.f * xo.lo});
                wr[i] = acc;
                lam[k] = acc;
              }
            }
            gsync<GH>(1);
            df_tsolve<GH>(T, P.tp_off, P.n_utlev, P.n_ltlev, lu, lam, hl, 1);  // lam <- lambda_nn (row positions)
            df *hn = hs + (size_t)(nn - s0 - 1) * n;
            for (int k = hl; k < n; k += GH) hn[k] = lam[k];
          }
          if (RB > 0) {  // the segment's lambda history complete: its owned gradient terms
            gsync<GH>(1);
            segment_gradient(j);
          }
        } else {
          if (j > 0) {
            // ---- recompute segment j-1 from its checkpoint into buffer (j-1) % 3
            const int s0 = (j - 1) * K, s1 = s0 + K;
            df *sg = my_seg + (size_t)((j - 1) % 3) * seg_words;
            const df *ck = my_ck + (size_t)(j - 1) * ck_words;
            for (int k = hl; k < n; k += GH) {
              x[k] = ck[k];
              sg[k] = ck[k];
            }
            for (int d = hl; d < P.ncap; d += GH) icap[d] = ck[n + d];
            gsync<GH>(2);
            if (tr) {  // companion currents of step s0 (the checkpoint's, or from its currents)
              for (int d = hl; d < P.ncap; d += GH) {
                const int4 dd = S.dyn[d];
                cb[d] = ck_cb ? icap[d] : df_sub(df_mul(cdyn[d], df_sub(df_at(x, dd.y), df_at(x, dd.z))), icap[d]);
              }
              for (int s = s0 + 1; s <= s1; ++s) {
                adj_forward_step<GH, GH, true>(P, S, lu, x, cdyn, cb, icap, vals, method, s, h, wt, hl, 2);
                for (int k = hl; k < n; k += GH) sg[(size_t)(s - s0) * n + k] = x[k];
              }
            } else {
              for (int s = s0 + 1; s <= s1; ++s) {
                adj_forward_step<GH, GH>(P, S, lu, x, cdyn, cb, icap, vals, method, s, h, wt, hl, 2);
                for (int k = hl; k < n; k += GH) sg[(size_t)(s - s0) * n + k] = x[k];
              }
            }
          }
          if (j + 1 < J) segment_gradient(j + 1);
        }
        __syncthreads();
      }
      if (!back_half) segment_gradient(0);
      {
        // scale and write the gradient, each half its own elements
#pragma unroll
        for (int i = 0; i < RE; ++i) {
          const int e = hl + i * GH;
          if (e >= P.ne || !(back_half ? i < RB : i >= RB)) continue;
          const int kind = (ekind >> (3 * i)) & 7;
          const double val = vals ? vals[e] : P.el[e].value;
          const double gsum = df_to_double(gr[i]);
          double r = 0.0;
          if (kind == 1) r = gsum / (val * val);
          else if (kind == 2 || kind == 3) r = gsum * (tr ? 2.0 / h : 1.0 / h);
          else if (kind == 4) r = gsum;
          grad_out[(size_t)inst * P.ne + e] = r;
        }
      }
    }
    if (tid == 0) {
      if (mode != 2) loss_out[inst] = df_to_double(loss);
      slot[1] = 0;
    }
    __syncthreads();
    if (st) atomicOr(&slot[1], st);
    __syncthreads();
    if (tid == 0 && inst_status) inst_status[inst] = slot[1];
  }
}

}  // namespace krets
