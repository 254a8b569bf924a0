// sm_103a kernels of the MNA solve path.
//
//   k_op           Newton operating point, FP64, one CTA per instance
//                  (op.rs:15-86; a single instance is the plain OP form)
//   k_dc_sweep     warm-started DC sweep, FP64, one CTA per sweep (dc.rs:14-124)
//   k_tran_step    plain transient: ONE time step of ONE instance per launch, FP64,
//                  Newton loop inside, state in global memory (transient.rs:43-112)
//   k_tran_batch   batched transient: persistent CTAs draw instances from a device work
//                  queue and run the whole step loop with factors and state in shared
//                  memory; FP64 or FP32-factor + FP64-refinement
//   k_tran_adaptive batched transient with truncation-error step control (extension),
//                  FP64, one CTA per instance
//   k_ac_batch     batched AC: one (instance, frequency) complex system per work item;
//                  complex128 or complex64-factor + complex128 refinement (ac.rs:39-107)
#pragma once
#include <cuda_runtime.h>

#include "engine.cuh"

namespace krets {

struct KCfg {
  double reltol, iabstol, vabstol;
  int maxiter;
};

// Byte offsets of the per-CTA arrays of one kernel (shared memory, or a slice of a
// global workspace when the instance does not fit in shared memory).
struct Lay {
  int off[16];
  size_t bytes;
};

struct TranState {
  double *x, *prev, *guess, *b, *ca, *cb, *icap, *lu;
  int *status, *step, *factored;
};

#define ARR(T, name, idx) T *name = reinterpret_cast<T *>(base + L.off[idx])

// One contribution of an A entry (packed slot << 2 | unit << 1 | neg), signed.
template <typename T>
__device__ __forceinline__ T contrib_value(int code, const double *ca_re, const double *ca_im);
template <>
__device__ __forceinline__ double contrib_value<double>(int code, const double *ca_re, const double *) {
  const double v = (code & 2) ? 1.0 : ca_re[code >> 2];
  return (code & 1) ? -v : v;
}
template <>
__device__ __forceinline__ cx<double> contrib_value<cx<double>>(int code, const double *ca_re, const double *ca_im) {
  double vr = (code & 2) ? 1.0 : ca_re[code >> 2];
  double vi = (code & 2) ? 0.0 : ca_im[code >> 2];
  if (code & 1) { vr = -vr; vi = -vi; }
  return cx<double>(vr, vi);
}

// Stamp every LU slot (A entries summed in emission order, fill slots zero) and return.
// Four slots per thread at a time, so their chains of dependent loads (slot -> A entry ->
// contribution range -> contributions) are in flight together; each slot's sum keeps the
// emission order of sum_entry, so the values are the same bits.
template <typename T>
__device__ __forceinline__ void stamp_lu(const DevProg &P, T *lu, const double *ca_re, const double *ca_im) {
  const int nb = blockDim.x;
  for (int s0 = threadIdx.x; s0 < P.nnz_lu; s0 += 4 * nb) {
    int t[4], u[4], ue[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) t[q] = s0 + q * nb < P.nnz_lu ? P.lu_src[s0 + q * nb] : -1;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      u[q] = t[q] >= 0 ? P.a_cptr[t[q]] : 0;
      ue[q] = t[q] >= 0 ? P.a_cptr[t[q] + 1] : 0;
    }
    T acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = T(0);
    bool more = true;
    while (more) {
      more = false;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (u[q] < ue[q]) {
          acc[q] = acc[q] + contrib_value<T>(P.a_contrib[u[q]], ca_re, ca_im);
          ++u[q];
          more = more || u[q] < ue[q];
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (s0 + q * nb < P.nnz_lu) lu[s0 + q * nb] = acc[q];
  }
}

__device__ __forceinline__ void coef_pass(const DevProg &P, const double *vals, const PassCtx &c, double *ca_re,
                                          double *ca_im, double *cb, int *status) {
  int err = 0;
  for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
    const krets_element &E = P.el[e];
    double val = vals ? vals[e] : E.value;
    double ar, ai, b, x0, x1;
    elem_coefs(E, e, P.el_pos[e], val, c, ar, ai, b, x0, x1, err);
    ca_re[e] = ar;
    if (ca_im) ca_im[e] = ai;
    cb[e] = b;
    const int xs = P.xslot[e];
    if (xs >= 0) {
      ca_re[xs] = x0;
      ca_re[xs + 1] = x1;
      if (ca_im) ca_im[xs] = ca_im[xs + 1] = 0.0;
    }
  }
  if (err) atomicOr(status, err);
}

// Newton convergence test (solver.rs:76-104) over all unknowns plus the extra key
// ("time" / "step"), which uses the voltage tolerance.
__device__ __forceinline__ bool converged(const DevProg &P, const KCfg &cfg, const double *prev, const double *x,
                                          bool has_extra, double extra_prev, double extra_new) {
  int ok = 1;
  for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
    double v = x[k], p = prev[k];
    double diff = fabs(v - p), scale = fmax(fabs(v), fabs(p));
    double atol = P.is_cur[k] ? cfg.iabstol : cfg.vabstol;
    if (!(diff <= cfg.reltol * scale + atol)) ok = 0;
  }
  if (has_extra && threadIdx.x == 0) {
    double diff = fabs(extra_new - extra_prev), scale = fmax(fabs(extra_new), fabs(extra_prev));
    if (!(diff <= cfg.reltol * scale + cfg.vabstol)) ok = 0;
  }
  return __syncthreads_and(ok);
}

__global__ void k_gather(double *dst, const double *src, const int *q, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = src[q[k]];
}

// ============================================================== L1 warm-up
// A single-CTA solve (plain OP, DC sweep, few batched instances) is bound by dependent
// loads of its program arrays (pivot entry -> update pairs -> LU slots; slot -> stamp
// contributions) at L2 latency.  The host lists those arrays (factorisation, solves,
// stamps) and the CTA first issues one L1 prefetch per 128-byte line of each, so the
// chains then hit L1.  Only addresses inside the listed arrays are touched.
struct OpWarm {
  int count;
  const char *ptr[16];
  int bytes[16];
};

__device__ __forceinline__ void warm_l1(const OpWarm &w) {
  for (int a = 0; a < w.count; ++a)
    for (int off = threadIdx.x * 128; off < w.bytes[a]; off += blockDim.x * 128)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(w.ptr[a] + off));
}

// ============================================================== program staging
// A single-CTA solve whose workspace leaves room copies the factorisation and solve arrays
// into shared memory behind the workspace (byte `off` of the dynamic shared memory) before
// its first factorisation.  Array a goes to off + at[a] (16-byte aligned) as n16[a]
// 16-byte words: the program image keeps every array at a 16-byte aligned offset, so the
// words a copy rounds up to stay inside the image.  Order: lev_ptr, lev_rows, piv_ptr,
// lu_diag, lu_rowptr, lu_col, ulev_ptr, ulev_rows, piv, upd.
struct OpStage {
  int on, off;
  int at[10], n16[10];
};

__device__ __forceinline__ void stage_fac(const OpStage &S, char *smem, FacView &F) {
  if (!S.on) return;
  const void *src[10] = {F.lev_ptr,   F.lev_rows, F.piv_ptr,  F.lu_diag,   F.lu_rowptr,
                         F.lu_col,    F.ulev_ptr, F.ulev_rows, F.piv,      F.upd};
  char *dst = smem + S.off;
#pragma unroll
  for (int a = 0; a < 10; ++a) {
    const int4 *s4 = reinterpret_cast<const int4 *>(src[a]);
    int4 *d4 = reinterpret_cast<int4 *>(dst + S.at[a]);
    for (int i = threadIdx.x; i < S.n16[a]; i += blockDim.x) d4[i] = s4[i];
  }
  __syncthreads();
  F.lev_ptr = reinterpret_cast<const int *>(dst + S.at[0]);
  F.lev_rows = reinterpret_cast<const int *>(dst + S.at[1]);
  F.piv_ptr = reinterpret_cast<const int *>(dst + S.at[2]);
  F.lu_diag = reinterpret_cast<const int *>(dst + S.at[3]);
  F.lu_rowptr = reinterpret_cast<const int *>(dst + S.at[4]);
  F.lu_col = reinterpret_cast<const int *>(dst + S.at[5]);
  F.ulev_ptr = reinterpret_cast<const int *>(dst + S.at[6]);
  F.ulev_rows = reinterpret_cast<const int *>(dst + S.at[7]);
  F.piv = reinterpret_cast<const int4 *>(dst + S.at[8]);
  F.upd = reinterpret_cast<const int2 *>(dst + S.at[9]);
}

// ============================================================== k_op
// Newton OP in FP64.  guess0 (optional, original numbering) warm-starts the iteration
// as the DC sweep does; step_key >= 0 adds the "step" key to the convergence test.
__device__ int newton_dc(const DevProg &P, const FacView &F, const KCfg &cfg, const double *vals, double *lu,
                         double *b, double *x, double *guess, double *ca, double *cb, int *status, bool guess_empty,
                         double step_key, int *iters_out) {
  PassCtx c{};
  c.mode = 0;
  c.guess = guess;
  c.guess_empty = guess_empty;
  double prev_step = step_key - 1.0;
  int it;
  for (it = 0; it < cfg.maxiter; ++it) {
    coef_pass(P, vals, c, ca, nullptr, cb, status);
    __syncthreads();
    stamp_lu<double>(P, lu, ca, nullptr);
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) b[k] = sum_rhs(P, k, cb);
    __syncthreads();
    factor_v<double>(F, lu, status);
    if (*status & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) break;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = b[k];
    __syncthreads();
    lsolve_v<double, double>(F, lu, x);
    usolve_v<double, double>(F, lu, x);
    if (!P.nonlinear) break;
    bool conv = !c.guess_empty && converged(P, cfg, guess, x, step_key >= 0.0, prev_step, step_key);
    if (conv) break;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = x[k];
    __syncthreads();
    c.guess_empty = false;
    prev_step = step_key;
    if (it == cfg.maxiter - 1) {
      if (threadIdx.x == 0) atomicOr(status, KS_MAXITER);
      __syncthreads();
    }
  }
  if (iters_out && threadIdx.x == 0) *iters_out = it + 1;
  return it + 1;
}

__global__ void k_op(DevProg P, KCfg cfg, Lay L, char *gws, const double *values, double *x_out,
                     size_t out_stride, int *inst_status, int *iters, int n_inst, OpWarm warm, OpStage stage) {
  extern __shared__ __align__(16) char smem[];
  char *base = gws ? gws + (size_t)blockIdx.x * L.bytes : smem;
  warm_l1(warm);
  FacView F = fac_view(P);
  stage_fac(stage, smem, F);
  ARR(double, lu, 0);
  ARR(double, b, 1);
  ARR(double, x, 2);
  ARR(double, guess, 3);
  ARR(double, ca, 4);
  ARR(double, cb, 5);
  ARR(int, status, 6);
  for (int inst = blockIdx.x; inst < n_inst; inst += gridDim.x) {
    if (threadIdx.x == 0) *status = 0;
    __syncthreads();
    const double *vals = values ? values + (size_t)inst * P.ne : nullptr;
    newton_dc(P, F, cfg, vals, lu, b, x, guess, ca, cb, status, true, -1.0, iters ? iters + inst : nullptr);
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) x_out[(size_t)inst * out_stride + P.q[k]] = x[k];
    if (threadIdx.x == 0 && inst_status) inst_status[inst] = *status;
    __syncthreads();
  }
}

// ============================================================== k_dc_sweep
// Warm-started source sweep (dc.rs:14-124).  One CTA per instance (values NULL: the
// nominal values, one instance); instance i writes its points at x_out + i * inst_stride
// and stops at its first failing point, as dc::solve returns on the first error.
__global__ void k_dc_sweep(DevProg P, KCfg cfg, Lay L, char *gws, int sweep_elem, double start, double step,
                           int n_points, const double *values, int n_inst, size_t inst_stride, double *x_out,
                           int *out_status, OpWarm warm, OpStage stage) {
  extern __shared__ __align__(16) char smem[];
  char *base = gws ? gws + (size_t)blockIdx.x * L.bytes : smem;
  warm_l1(warm);
  FacView F = fac_view(P);
  stage_fac(stage, smem, F);
  ARR(double, lu, 0);
  ARR(double, b, 1);
  ARR(double, x, 2);
  ARR(double, guess, 3);
  ARR(double, ca, 4);
  ARR(double, cb, 5);
  ARR(int, status, 6);
  ARR(double, vals, 7);
  for (int inst = blockIdx.x; inst < n_inst; inst += gridDim.x) {
    const double *src = values ? values + (size_t)inst * P.ne : nullptr;
    for (int e = threadIdx.x; e < P.ne; e += blockDim.x) vals[e] = src ? src[e] : P.el[e].value;
    if (threadIdx.x == 0) *status = 0;
    __syncthreads();
    double *out = x_out + (size_t)inst * inst_stride;
    for (int i = 0; i < n_points; ++i) {
      if (threadIdx.x == 0) vals[sweep_elem] = start + ((double)i * step);  // dc.rs:157-164
      // warm start from the previous point's solution (dc.rs:167)
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = x[k];
      __syncthreads();
      newton_dc(P, F, cfg, vals, lu, b, x, guess, ca, cb, status, i == 0, (double)i, nullptr);
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) out[(size_t)i * P.n + P.q[k]] = x[k];
      __syncthreads();
      if (*status) break;
    }
    if (threadIdx.x == 0) out_status[inst] = *status;
    __syncthreads();
  }
}

// ============================================================== k_tran_adaptive
// Transient with local-truncation-error step control (an extension: krets steps at a
// fixed h).  One CTA per instance, FP64 throughout: each attempt stamps and refactors when
// h changed (or every Newton iteration for nonlinear circuits), solves, and estimates the
// LTE by divided differences over the attempt and the last accepted points
//   BE: LTE = h^2 DD2,  TR: LTE = h^3/2 DD3,
// r = max_k |LTE_k| / (lte_tol max(|x_k|, |x_n,k|) + abstol_k); r <= 1 accepts.  The step
// factor is the largest of a fixed set with r f^(p+1) <= 1/2 (adapt_factor), so the time
// grid is exact binary arithmetic.  Accepted points go to t_out / x_out (row 0 = the
// operating point, written before the launch); the history for the divided differences is
// read back from those rows.
#define KS_TSTEP 128  // the step fell below h_min
#define KS_FULL 256   // more accepted points than max_points

__device__ __forceinline__ double adapt_factor(double r, int order, bool accepted) {
  if (accepted) {
    const double fa[5] = {2.0, 1.5, 1.0, 0.75, 0.5};
    const double p2[5] = {4.0, 2.25, 1.0, 0.5625, 0.25}, p3[5] = {8.0, 3.375, 1.0, 0.421875, 0.125};
    for (int i = 0; i < 5; ++i)
      if (r * (order == 1 ? p2[i] : p3[i]) <= 0.5) return fa[i];
    return 0.5;
  }
  const double fr[3] = {0.5, 0.25, 0.125};
  const double p2[3] = {0.25, 0.0625, 0.015625}, p3[3] = {0.125, 0.015625, 0.001953125};
  for (int i = 0; i < 3; ++i)
    if (r * (order == 1 ? p2[i] : p3[i]) <= 0.5) return fr[i];
  return 0.125;
}

__global__ void k_tran_adaptive(DevProg P, KCfg cfg, Lay L, char *gws, const double *values, int n_inst, double h0,
                                double t_stop, int method, double lte_tol, double h_min, double h_max,
                                int max_points, double *t_out, double *x_out, int *n_points, int *inst_status) {
  extern __shared__ __align__(16) char smem[];
  char *base = gws ? gws + (size_t)blockIdx.x * L.bytes : smem;
  ARR(double, vals, 0);
  ARR(double, lu, 1);
  ARR(double, x, 2);
  ARR(double, guess, 3);
  ARR(double, b, 4);
  ARR(double, ca, 5);
  ARR(double, cb, 6);
  ARR(double, icap, 7);
  ARR(double, red, 8);
  ARR(int, status, 9);
  ARR(double, xn, 10);
  const bool trap = method == KRETS_METHOD_TR;
  const int order = trap ? 2 : 1;
  for (int inst = blockIdx.x; inst < n_inst; inst += gridDim.x) {
    double *xo = x_out + (size_t)inst * max_points * P.n;
    double *to = t_out + (size_t)inst * max_points;
    for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
      vals[e] = values ? values[(size_t)inst * P.ne + e] : P.el[e].value;
      icap[e] = 0.0;
    }
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) xn[k] = xo[P.q[k]];
    if (threadIdx.x == 0) {
      *status = 0;
      to[0] = 0.0;
    }
    __syncthreads();
    double t = 0.0, h = fmin(h0, h_max), h_fact = -1.0;
    int n_acc = 1;
    bool fatal = false;
    while (t < t_stop) {
      if (t + h >= t_stop || t_stop - (t + h) < h_min) h = t_stop - t;
      const double t_new = (t + h >= t_stop) ? t_stop : t + h;
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = xn[k];
      __syncthreads();
      PassCtx c{};
      c.mode = 2;
      c.method = method;
      c.h = h;
      c.prev = xn;
      c.guess = guess;
      c.guess_empty = false;
      c.icap = icap;
      c.t_src = t_new;
      double guess_time = t;
      bool newton_ok = false;
      for (int it = 0; it < cfg.maxiter; ++it) {
        coef_pass(P, vals, c, ca, nullptr, cb, status);
        __syncthreads();
        if (P.nonlinear || h != h_fact) {
          stamp_lu<double>(P, lu, ca, nullptr);
          __syncthreads();
          factor<double>(P, lu, status);
          h_fact = h;
        }
        if (*status & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) {
          fatal = true;
          break;
        }
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = sum_rhs(P, k, cb);
        __syncthreads();
        lsolve<double, double>(P, lu, x);
        usolve<double, double>(P, lu, x);
        if (!P.nonlinear) {
          newton_ok = true;
          break;
        }
        if (converged(P, cfg, guess, x, true, guess_time, t_new)) {
          newton_ok = true;
          break;
        }
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = x[k];
        __syncthreads();
        guess_time = t_new;
      }
      if (fatal) break;
      int bad = 0;
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) bad |= !isfinite(x[k]);
      if (__syncthreads_or(bad)) {
        if (threadIdx.x == 0) atomicOr(status, KS_NONFINITE);
        break;
      }
      // truncation error of the attempt over the accepted history (rows of x_out)
      double r = 0.0;
      const bool checked = newton_ok && n_acc >= order + 1;
      if (checked) {
        const double *x1 = xo + (size_t)(n_acc - 2) * P.n;
        const double *x2 = trap ? xo + (size_t)(n_acc - 3) * P.n : x1;
        const double t1 = to[n_acc - 2], t2 = trap ? to[n_acc - 3] : 0.0;
        double rl = 0.0;
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
          const int o = P.q[k];
          double lte;
          if (!trap) {
            const double d1 = (x[k] - xn[k]) / h, d0 = (xn[k] - x1[o]) / (t - t1);
            const double dd2 = (d1 - d0) / (t_new - t1);
            lte = (h * h) * dd2;
          } else {
            const double d2 = (x[k] - xn[k]) / h, d1 = (xn[k] - x1[o]) / (t - t1), d0 = (x1[o] - x2[o]) / (t1 - t2);
            const double e1 = (d2 - d1) / (t_new - t1), e0 = (d1 - d0) / (t - t2);
            const double dd3 = (e1 - e0) / (t_new - t2);
            lte = (0.5 * (h * h * h)) * dd3;
          }
          const double tol = __dadd_rn(__dmul_rn(lte_tol, fmax(fabs(x[k]), fabs(xn[k]))),
                                       P.is_cur[k] ? cfg.iabstol : cfg.vabstol);
          rl = fmax(rl, fabs(lte) / tol);
        }
        r = block_max(rl, red);
      }
      if (newton_ok && !(r > 1.0)) {
        if (n_acc >= max_points) {
          if (threadIdx.x == 0) atomicOr(status, KS_FULL);
          break;
        }
        double *row = xo + (size_t)n_acc * P.n;
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) row[P.q[k]] = x[k];
        if (threadIdx.x == 0) to[n_acc] = t_new;
        if (trap) {
          for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
            if (P.el[e].kind != KRETS_ELEM_C) continue;
            const int4 ps = P.el_pos[e];
            const double vn = (ps.x >= 0 ? x[ps.x] : 0.0) - (ps.y >= 0 ? x[ps.y] : 0.0);
            icap[e] = ca[e] * vn - cb[e];
          }
        }
        __syncthreads();  // the row, the history reads and icap before xn moves on
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) xn[k] = x[k];
        __syncthreads();
        ++n_acc;
        t = t_new;
        const double f = checked ? adapt_factor(r, order, true) : 1.0;
        h = fmin(h * f, h_max);
        if (h < h_min) h = h_min;
      } else {
        h = h * (newton_ok ? adapt_factor(r, order, false) : 0.125);
        if (h < h_min) {
          if (threadIdx.x == 0) atomicOr(status, KS_TSTEP);
          break;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      n_points[inst] = n_acc;
      if (inst_status) inst_status[inst] = *status;
    }
    __syncthreads();
  }
}

// ============================================================== k_tran_step (plain form)
// One time step of one instance.  Global state (position space of the TRAN program):
//   st.x (solution at t_{n-1} on entry, t_n on exit), st.icap (TR capacitor currents),
//   st.lu (factors; reused when !refactor and the circuit is linear).
// The step index comes from st.step (device counter) so a captured CUDA graph of K
// launches advances K steps per replay.
__global__ void k_tran_step(DevProg P, KCfg cfg, TranState st, double h, int method, int lag, int refactor,
                            int n_steps, double *x_out) {
  int s = *st.step + 1;  // step being computed
  if (s > n_steps) return;
  __syncthreads();
  const double *vals = nullptr;
  double *x = st.x, *prev = st.prev, *guess = st.guess;
  for (int k = threadIdx.x; k < P.n; k += blockDim.x) { prev[k] = x[k]; guess[k] = x[k]; }
  __syncthreads();
  PassCtx c{};
  c.mode = 2;
  c.method = method;
  c.h = h;
  c.prev = prev;
  c.guess = guess;
  c.guess_empty = false;
  c.icap = st.icap;
  double t = (double)s * h;
  double guess_time = (double)(s - 1) * h;
  int it;
  for (it = 0; it < cfg.maxiter; ++it) {
    c.t_src = lag ? guess_time : t;
    coef_pass(P, vals, c, st.ca, nullptr, st.cb, st.status);
    __syncthreads();
    bool need_factor = refactor || P.nonlinear || !*st.factored;
    if (need_factor) {
      stamp_lu<double>(P, st.lu, st.ca, nullptr);
      __syncthreads();
      factor<double>(P, st.lu, st.status);
      if (threadIdx.x == 0) *st.factored = 1;
    }
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = sum_rhs(P, k, st.cb);
    __syncthreads();
    if (*st.status & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) break;
    lsolve<double, double>(P, st.lu, x);
    usolve<double, double>(P, st.lu, x);
    if (!P.nonlinear) break;
    if (converged(P, cfg, guess, x, true, guess_time, t)) break;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = x[k];
    __syncthreads();
    guess_time = t;
    if (it == cfg.maxiter - 1 && threadIdx.x == 0) atomicOr(st.status, KS_MAXITER);
  }
  __syncthreads();
  if (method == KRETS_METHOD_TR) {
    for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
      if (P.el[e].kind != KRETS_ELEM_C) continue;
      int4 ps = P.el_pos[e];
      double vn = (ps.x >= 0 ? x[ps.x] : 0.0) - (ps.y >= 0 ? x[ps.y] : 0.0);
      st.icap[e] = st.ca[e] * vn - st.cb[e];
    }
  }
  int nonfinite = 0;
  for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
    nonfinite |= !isfinite(x[k]);
    x_out[(size_t)s * P.n + P.q[k]] = x[k];
  }
  if (__syncthreads_or(nonfinite) && threadIdx.x == 0) atomicOr(st.status, KS_NONFINITE);
  __syncthreads();
  if (threadIdx.x == 0) *st.step = s;
}

// ============================================================== k_tran_batch
// Persistent batched transient.  Work item = one instance; row 0 of its output (the OP)
// must already be written.  Per instance, in shared memory for the whole run:
//   vals[ne], a64[nnz_a] (mixed), lu[nnz_lu] (FP32 or FP64), x[n], prev[n], guess[n]
//   (nonlinear), b[n], w32[n] (mixed), ca[ne], cb[ne], icap[ne].
template <typename F>
__device__ __forceinline__ void stamp_a64(const DevProg &P, double *a64, const double *ca) {
  for (int t = threadIdx.x; t < P.nnz_a; t += blockDim.x) a64[t] = sum_entry<double>(P, t, ca, nullptr);
}

template <typename F>
__device__ __forceinline__ void load_lu_from_a(const DevProg &P, const double *a64, F *lu) {
  for (int s = threadIdx.x; s < P.nnz_lu; s += blockDim.x) {
    int t = P.lu_src[s];
    lu[s] = t < 0 ? F(0) : F(a64[t]);
  }
}

// Mixed-precision solve of A x = b: FP32 LU, FP64 residual, refinement until the
// correction is below tol*|x|.  x holds the initial guess.  Returns iterations, or -1
// on stall / non-convergence.
__device__ int refine_solve(const DevProg &P, const double *a64, const float *lu32, const double *b, double *x,
                            float *w, double *red, double tol, int max_it) {
  double dprev = 0.0;
  for (int it = 0; it < max_it; ++it) {
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
      double r = b[k];
      for (int t = P.a_rowptr[k]; t < P.a_rowptr[k + 1]; ++t) r -= a64[t] * x[P.a_col[t]];
      w[k] = (float)r;
    }
    __syncthreads();
    lsolve<float, float>(P, lu32, w);
    usolve<float, float>(P, lu32, w);
    double dmax = 0.0, xmax = 0.0;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
      double d = (double)w[k];
      double xn = x[k] + d;
      x[k] = xn;
      dmax = fmax(dmax, fabs(d));
      xmax = fmax(xmax, fabs(xn));
    }
    dmax = block_max(dmax, red);
    xmax = block_max(xmax, red);
    if (!(dmax == dmax) || !(xmax == xmax)) return -1;
    if (dmax <= tol * xmax) return it + 1;
    if (it > 0 && dmax > 0.5 * dprev) return -1;  // stalled
    dprev = dmax;
  }
  return -1;
}

template <int MIXED>
__global__ void k_tran_batch(DevProg P, KCfg cfg, Lay L, char *gws, const double *values, int n_inst, double h,
                             int n_steps, int method, int lag, double *x_out, int *inst_status, int *queue,
                             unsigned long long *hist, int *fallbacks, double *lu64_scratch) {
  extern __shared__ __align__(16) char smem[];
  char *base = gws ? gws + (size_t)blockIdx.x * L.bytes : smem;
  ARR(double, vals, 0);
  ARR(double, a64, 1);
  ARR(double, x, 3);
  ARR(double, prev, 4);
  ARR(double, guess, 5);
  ARR(double, b, 6);
  ARR(float, w32, 7);
  ARR(double, ca, 8);
  ARR(double, cb, 9);
  ARR(double, icap, 10);
  ARR(double, red, 11);
  ARR(int, status, 12);
  ARR(int, item, 13);
  float *lu32 = reinterpret_cast<float *>(base + L.off[2]);
  double *lu64 = reinterpret_cast<double *>(base + L.off[2]);
  const size_t stride = (size_t)(n_steps + 1) * P.n;
  const double tol = 1e-12;
  const int max_ref = 6;
  while (true) {
    if (threadIdx.x == 0) *item = atomicAdd(queue, 1);
    __syncthreads();
    int inst = *item;
    if (inst >= n_inst) break;
    if (threadIdx.x == 0) *status = 0;
    unsigned long long local_hist[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    bool use64 = !MIXED;
    double *lu_fb = lu64_scratch ? lu64_scratch + (size_t)blockIdx.x * P.nnz_lu : nullptr;
    for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
      vals[e] = values ? values[(size_t)inst * P.ne + e] : P.el[e].value;
      icap[e] = 0.0;
    }
    double *out = x_out + (size_t)inst * stride;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = out[P.q[k]];
    __syncthreads();
    PassCtx c{};
    c.mode = 2;
    c.method = method;
    c.h = h;
    c.icap = icap;
    c.guess_empty = false;
    bool linear = !P.nonlinear;
    if (linear) {
      // constant matrix: stamp and factor once (a refactor would give identical factors)
      c.prev = x;
      c.guess = x;
      c.t_src = 0.0;
      coef_pass(P, vals, c, ca, nullptr, cb, status);
      __syncthreads();
      if (MIXED) {
        stamp_a64<float>(P, a64, ca);
        __syncthreads();
        load_lu_from_a<float>(P, a64, lu32);
        __syncthreads();
        factor<float>(P, lu32, status);
      } else {
        stamp_lu<double>(P, lu64, ca, nullptr);
        __syncthreads();
        factor<double>(P, lu64, status);
      }
    }
    for (int s = 1; s <= n_steps && !(*status & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)); ++s) {
      double t = (double)s * h;
      double guess_time = (double)(s - 1) * h;
      double *xp = linear ? x : prev;
      if (!linear) {
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) { prev[k] = x[k]; guess[k] = x[k]; }
        __syncthreads();
      }
      c.prev = xp;
      c.guess = linear ? x : guess;
      int it;
      for (it = 0; it < cfg.maxiter; ++it) {
        c.t_src = lag ? guess_time : t;
        coef_pass(P, vals, c, ca, nullptr, cb, status);
        __syncthreads();
        if (!linear) {
          if (MIXED && !use64) {
            stamp_a64<float>(P, a64, ca);
            __syncthreads();
            load_lu_from_a<float>(P, a64, lu32);
            __syncthreads();
            factor<float>(P, lu32, status);
          } else {
            double *luw = MIXED ? lu_fb : lu64;
            if (MIXED) { stamp_a64<float>(P, a64, ca); __syncthreads(); }
            stamp_lu<double>(P, luw, ca, nullptr);
            __syncthreads();
            factor<double>(P, luw, status);
          }
          if (*status & (KS_SINGULAR | KS_NONFINITE)) break;
        }
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) b[k] = sum_rhs(P, k, cb);
        __syncthreads();
        if (MIXED && !use64) {
          // initial guess: the Newton guess (previous step for the first iteration)
          if (!linear) {
            for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = guess[k];
            __syncthreads();
          }
          int r = refine_solve(P, a64, lu32, b, x, w32, red, tol, max_ref);
          if (r > 0) {
            local_hist[r < 8 ? r : 7]++;
          } else if (lu_fb) {
            // refinement stalled: FP64 refactor on the device and direct FP64 solve
            use64 = true;
            if (threadIdx.x == 0) atomicAdd(fallbacks, 1);
            load_lu_from_a<double>(P, a64, lu_fb);
            __syncthreads();
            factor<double>(P, lu_fb, status);
            for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = b[k];
            __syncthreads();
            lsolve<double, double>(P, lu_fb, x);
            usolve<double, double>(P, lu_fb, x);
          } else {
            if (threadIdx.x == 0) atomicOr(status, KS_STALL);
          }
        } else {
          double *luw = MIXED ? lu_fb : lu64;
          for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = b[k];
          __syncthreads();
          lsolve<double, double>(P, luw, x);
          usolve<double, double>(P, luw, x);
        }
        if (linear) break;
        if (converged(P, cfg, guess, x, true, guess_time, t)) break;
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) guess[k] = x[k];
        __syncthreads();
        guess_time = t;
        if (it == cfg.maxiter - 1 && threadIdx.x == 0) atomicOr(status, KS_MAXITER);
      }
      __syncthreads();
      if (method == KRETS_METHOD_TR) {
        for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
          if (P.el[e].kind != KRETS_ELEM_C) continue;
          int4 ps = P.el_pos[e];
          double vn = (ps.x >= 0 ? x[ps.x] : 0.0) - (ps.y >= 0 ? x[ps.y] : 0.0);
          icap[e] = ca[e] * vn - cb[e];
        }
      }
      double *row = out + (size_t)s * P.n;
      int nonfinite = 0;
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
        double v = x[k];
        nonfinite |= !isfinite(v);
        __stcs(row + P.q[k], v);
      }
      if (__syncthreads_or(nonfinite) && threadIdx.x == 0) atomicOr(status, KS_NONFINITE);
      __syncthreads();
    }
    if (threadIdx.x == 0 && inst_status) inst_status[inst] = *status;
    if (MIXED && hist) {
      // every thread holds identical counts (block-uniform control flow); thread 0 adds
      if (threadIdx.x == 0)
        for (int k = 0; k < 8; ++k)
          if (local_hist[k]) atomicAdd(hist + k, local_hist[k]);
    }
    __syncthreads();
  }
}


// ============================================================== k_ac_batch
// Work item = (instance, frequency).  op_x: operating point per instance, original
// numbering (used by the diode's small-signal conductance).
// ccache (MIXED): per CTA 2 n_coef + ne doubles.  A CTA keeps there the coefficients of
// its current instance that do not depend on the frequency — the real parts (1/R, diode
// conductances), the C and L values, the rhs coefficients — and forms only
// ca_im = 2 pi f value per point, with the operations of elem_coefs (the same bits).
template <int MIXED>
__global__ void k_ac_batch(DevProg P, Lay L, char *gws, const double *values, const double *op_x, int n_inst,
                           const double *freqs, int n_freq, double *x_out, int *item_status, int *queue,
                           double *ccache) {
  extern __shared__ __align__(16) char smem[];
  char *base = gws ? gws + (size_t)blockIdx.x * L.bytes : smem;
  using C64 = cx<double>;
  using C32 = cx<float>;
  double *vals = MIXED ? nullptr : reinterpret_cast<double *>(base + L.off[0]);  // MIXED: caller's values
  ARR(C64, a128, 1);
  ARR(C64, x, 3);
  ARR(C64, b, 4);
  ARR(C32, w, 5);
  ARR(double, ca_re, 6);
  ARR(double, ca_im, 7);
  ARR(double, cb, 8);
  ARR(double, opx, 9);
  ARR(double, red, 10);
  ARR(int, status, 11);
  ARR(int, item, 12);
  C32 *lu32 = reinterpret_cast<C32 *>(base + L.off[2]);
  C64 *lu64 = reinterpret_cast<C64 *>(base + L.off[2]);
  const int total = n_inst * n_freq;
  const bool cached = MIXED && ccache;
  double *cre = cached ? ccache + (size_t)blockIdx.x * (2 * (size_t)P.n_coef + P.ne) : nullptr;
  double *ccl = cre + P.n_coef, *ccb = ccl + P.n_coef;
  if (threadIdx.x == 0) item[1] = -1;  // instance whose coefficients the cache holds
  while (true) {
    if (threadIdx.x == 0) *item = atomicAdd(queue, 1);
    __syncthreads();
    int it_idx = *item;
    if (it_idx >= total) break;
    int inst = it_idx / n_freq, fi = it_idx % n_freq;
    if (threadIdx.x == 0) *status = 0;
    const double *ca_src = ca_re, *cb_src = cb;
    if (cached) {
      if (inst != item[1]) {
        for (int k = threadIdx.x; k < P.n; k += blockDim.x) opx[k] = op_x[(size_t)inst * P.n + P.q[k]];
        if (threadIdx.x == 0) item[2] = 0;
        __syncthreads();
        PassCtx c0{};
        c0.mode = 1;
        c0.guess = opx;
        c0.guess_empty = false;
        const double *iv = values ? values + (size_t)inst * P.ne : nullptr;
        int err = 0;
        for (int e = threadIdx.x; e < P.ne; e += blockDim.x) {
          const krets_element &E = P.el[e];
          const double val = iv ? iv[e] : E.value;
          double ar, ai, bb, x0, x1;
          elem_coefs(E, e, P.el_pos[e], val, c0, ar, ai, bb, x0, x1, err);
          cre[e] = ar;
          ccl[e] = (E.kind == KRETS_ELEM_C || E.kind == KRETS_ELEM_L) ? val : 0.0;
          ccb[e] = bb;
          const int xs = P.xslot[e];
          if (xs >= 0) {
            cre[xs] = x0;
            cre[xs + 1] = x1;
            ccl[xs] = ccl[xs + 1] = 0.0;
          }
        }
        if (err) atomicOr(&item[2], err);
        __syncthreads();
        if (threadIdx.x == 0) item[1] = inst;  // read again only after the next item's barrier
      }
      if (threadIdx.x == 0) *status |= item[2];
      const double w2f = 2.0 * kPiD * freqs[fi];
      for (int e = threadIdx.x; e < P.n_coef; e += blockDim.x) ca_im[e] = w2f * ccl[e];
      ca_src = cre;
      cb_src = ccb;
    } else {
      if (!MIXED)
        for (int e = threadIdx.x; e < P.ne; e += blockDim.x)
          vals[e] = values ? values[(size_t)inst * P.ne + e] : P.el[e].value;
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) opx[k] = op_x[(size_t)inst * P.n + P.q[k]];
      __syncthreads();
      PassCtx c{};
      c.mode = 1;
      c.freq = freqs[fi];
      c.guess = opx;
      c.guess_empty = false;
      coef_pass(P, MIXED ? (values ? values + (size_t)inst * P.ne : nullptr) : vals, c, ca_re, ca_im, cb, status);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) b[k] = C64(sum_rhs(P, k, cb_src), 0.0);
    if (MIXED) {
      for (int t = threadIdx.x; t < P.nnz_a; t += blockDim.x) a128[t] = sum_entry<C64>(P, t, ca_src, ca_im);
      __syncthreads();
      for (int s = threadIdx.x; s < P.nnz_lu; s += blockDim.x) {
        int t = P.lu_src[s];
        lu32[s] = t < 0 ? C32(0.0f, 0.0f) : C32(a128[t]);
      }
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = C64(0.0, 0.0);
      __syncthreads();
      factor<C32>(P, lu32, status);
      if (!(*status & (KS_SINGULAR | KS_NONFINITE))) {
        // Corrections until the largest is at most 1e-13 of the solution's largest part
        // (measured on the first solve, x_0).  The magnitudes come from the complex64
        // corrections themselves, so the test and its reduction stay off the FP64 pipe;
        // the first residual is b itself (x = 0).
        float dprev = 0.f, xref = 0.f;
        for (int r = 0; r < 8; ++r) {
          for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
            C64 acc = b[k];
            if (r > 0)
              for (int t = P.a_rowptr[k]; t < P.a_rowptr[k + 1]; ++t) acc = acc - a128[t] * x[P.a_col[t]];
            w[k] = C32(acc);
          }
          __syncthreads();
          lsolve<C32, C32>(P, lu32, w);
          usolve<C32, C32>(P, lu32, w);
          float dmax = 0.f;
          for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
            const C32 d = w[k];
            x[k] = x[k] + C64(d);
            dmax = fmaxf(dmax, fmaxf(fabsf(d.re), fabsf(d.im)));
          }
          dmax = block_maxf(dmax, red);
          if (r == 0) xref = dmax;
          if (dmax <= 1e-13f * xref) break;
          if ((r > 0 && dmax > 0.5f * dprev) || r == 7 || !(dmax == dmax)) {
            if (threadIdx.x == 0) atomicOr(status, KS_STALL);
            break;
          }
          dprev = dmax;
        }
      }
    } else {
      stamp_lu<C64>(P, lu64, ca_re, ca_im);
      __syncthreads();
      factor<C64>(P, lu64, status);
      for (int k = threadIdx.x; k < P.n; k += blockDim.x) x[k] = b[k];
      __syncthreads();
      lsolve<C64, C64>(P, lu64, x);
      usolve<C64, C64>(P, lu64, x);
    }
    __syncthreads();
    double *o = x_out + (size_t)it_idx * P.n * 2;
    for (int k = threadIdx.x; k < P.n; k += blockDim.x) {
      int j = P.q[k];
      o[2 * j] = x[k].re;
      o[2 * j + 1] = x[k].im;
    }
    if (threadIdx.x == 0 && item_status) item_status[it_idx] = *status;
    __syncthreads();
  }
}


__global__ void k_fill(double *p, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace krets
