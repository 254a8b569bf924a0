// Warp-per-instance batched transient engine (persistent, work queue).
//
// Each warp of a CTA pulls instances from a device work queue (one atomicAdd per instance)
// and runs that instance's whole transient with its factors and state in the warp's own
// slice of shared memory.  All synchronisation inside an instance is __syncwarp() (level
// barriers of the triangular solves) and warp shuffles (convergence tests), so warps of a
// CTA never wait for each other.  The static program (level descriptors, residual and rhs
// contribution lists) is read from global memory through L1: the carve-out leaves room
// for it, and every warp on the SM walks the same arrays.
//
// Per step (linear circuit, constant matrix, factored once per instance):
//   dyn pass      companion / source rhs coefficients of C, L, V, I (and D) elements (FP64)
//   rhs gather    b = segmented sums of those coefficients, emission order (FP64)
//   refinement    r = b - A x (FP64, element form), w = LU32^-1 r (FP32), x += w,
//                 until max|w| <= tol * max|x|; a stall switches the instance to an FP64
//                 refactor on the device
//   state update  TR capacitor currents (FP64), then the whole solution row is streamed out.
// Nonlinear circuits (diodes) run the same Newton loop as the reference, refactoring in
// each iteration.
#pragma once

#include "kernels.cuh"
#include "df.cuh"

namespace krets {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Shared-memory view of the compact step program (layout: pack_step_program()).
struct SProg {
  const int *lev_ptr, *ulev_ptr;
  const int4 *ldesc, *udesc;
  const unsigned short *lu_col;
  const int2 *res_row;
  const int *res_op;
  const int4 *dyn;
  const int *bd_ptr, *bd_op, *qinv;
  const int *lmax, *umax;  // split code of each L / U level (lanes per row, longest row)
  int nlev, nulev;
  int tail0, tail_m;  // dense trailing block (tail_m = 0: none)
  df *dense_stage;    // 32 x 33 shared-memory tile for diagonal blocks read from global memory (or null)
  const int *dense_rows;  // slot of column tail0 of each dense-block row, in shared memory (or null)
  // border of the dense block (U entries of rows before it in its columns): chunks of
  // <= 16 entries {first slot, count}, rows {row, first chunk, chunks, 0}, and scratch
  // for the chunks' partial sums (set by the kernel)
  const int2 *bchunk;
  const int4 *brow;
  int n_bchunk, n_brow;
  df *bpart;
};

__device__ __forceinline__ SProg sprog_view(const DevProg &P, const int *sp) {
  SProg S;
  S.lev_ptr = sp + P.sp_off[0];
  S.ulev_ptr = sp + P.sp_off[1];
  S.ldesc = reinterpret_cast<const int4 *>(sp + P.sp_off[2]);
  S.udesc = reinterpret_cast<const int4 *>(sp + P.sp_off[3]);
  S.lu_col = reinterpret_cast<const unsigned short *>(sp + P.sp_off[4]);
  S.res_row = reinterpret_cast<const int2 *>(sp + P.sp_off[5]);
  S.res_op = sp + P.sp_off[6];
  S.dyn = reinterpret_cast<const int4 *>(sp + P.sp_off[7]);
  S.bd_ptr = sp + P.sp_off[8];
  S.bd_op = sp + P.sp_off[9];
  S.qinv = sp + P.sp_off[10];
  S.lmax = sp + P.sp_off[12];
  S.umax = sp + P.sp_off[13];
  S.nlev = P.nlev;
  S.nulev = P.nulev;
  S.tail0 = P.tail0;
  S.tail_m = P.tail_m;
  S.dense_stage = nullptr;
  S.dense_rows = nullptr;
  S.bchunk = reinterpret_cast<const int2 *>(sp + P.sp_off[14]);
  S.brow = reinterpret_cast<const int4 *>(sp + P.sp_off[15]);
  S.n_bchunk = P.n_bchunk;
  S.n_brow = P.n_brow;
  S.bpart = nullptr;
  return S;
}

// One row of a triangular solve: y[k] - sum(l * y[col]) (times the reciprocal diagonal
// for U).  The first two entries come from the descriptor, so their loads issue together.
template <typename T, typename V, bool UPPER>
__device__ __forceinline__ V s_row(const SProg &S, const T *__restrict__ lu, const V *y, const int4 d, int &k) {
  k = d.x & 0xffff;
  const int rest = (int)((unsigned)d.x >> 16);
  const int first = UPPER ? d.y + 1 : d.y;
  const int c0 = d.z & 0xffff, c1 = (int)((unsigned)d.z >> 16);
  const V a0 = d.w > 0 ? V(lu[first]) : V(0);
  const V a1 = d.w > 1 ? V(lu[first + 1]) : V(0);
  V s = y[k];
  s -= a0 * y[c0];
  s -= a1 * y[c1];
  for (int j = 2; j < 2 + rest; ++j) s -= V(lu[first + j]) * y[S.lu_col[first + j]];
  if (UPPER) s *= V(lu[d.y]);
  return s;
}

// Level-scheduled solve, two rows per lane in flight.
template <typename T, typename V, bool UPPER>
__device__ __forceinline__ void s_solve(const SProg &S, const T *__restrict__ lu, V *y, int lane) {
  const int nl = UPPER ? S.nulev : S.nlev;
  const int *ptr = UPPER ? S.ulev_ptr : S.lev_ptr;
  const int4 *desc = UPPER ? S.udesc : S.ldesc;
  for (int l = UPPER ? 0 : 1; l < nl; ++l) {  // L level 0 rows have no L entries
    const int r0 = ptr[l], r1 = ptr[l + 1];
    for (int t = r0 + lane; t < r1; t += 64) {
      int k0, k1 = -1;
      const V v0 = s_row<T, V, UPPER>(S, lu, y, desc[t], k0);
      V v1 = V(0);
      if (t + 32 < r1) v1 = s_row<T, V, UPPER>(S, lu, y, desc[t + 32], k1);
      y[k0] = v0;
      if (k1 >= 0) y[k1] = v1;
    }
    __syncwarp();
  }
}

template <typename T, typename V>
__device__ __forceinline__ void s_lsolve(const SProg &S, const T *lu, V *y, int lane) {
  s_solve<T, V, false>(S, lu, y, lane);
}

// Upper solve; the diagonal slots hold reciprocals (see w_factor).
template <typename T, typename V>
__device__ __forceinline__ void s_usolve(const SProg &S, const T *lu, V *y, int lane) {
  s_solve<T, V, true>(S, lu, y, lane);
}

// Static-pivot up-looking LU, rows of a level spread over the lanes; afterwards every
// diagonal slot is replaced by its reciprocal.  Returns status bits (warp-uniform).
template <typename T>
__device__ int w_factor(const DevProg &P, T *lu, int lane) {
  int bad = 0;
  for (int l = 0; l < P.nlev; ++l) {
    const int r0 = P.lev_ptr[l], r1 = P.lev_ptr[l + 1];
    for (int t = r0 + lane; t < r1; t += 32) {
      const int k = P.ldesc[t].x;
      for (int pi = P.piv_ptr[k]; pi < P.piv_ptr[k + 1]; ++pi) {
        const int4 pv = P.piv[pi];
        const T l_kj = lu[pv.x] / lu[P.lu_diag[pv.y]];
        lu[pv.x] = l_kj;
        for (int u = pv.z; u < pv.w; ++u) {
          const int2 d = P.upd[u];
          lu[d.x] -= l_kj * lu[d.y];
        }
      }
      const T dk = lu[P.lu_diag[k]];
      if (!(scal<T>::mag(dk) > 0)) bad |= KS_SINGULAR;
      else if (!scal<T>::finite(dk)) bad |= KS_NONFINITE;
    }
    __syncwarp();
  }
  for (int k = lane; k < P.n; k += 32) {
    const int s = P.lu_diag[k];
    lu[s] = recip(lu[s]);
  }
  __syncwarp();
  return (int)__reduce_or_sync(kFull, (unsigned)bad);
}

// Matrix coefficient of every element for this pass (R: 1/R, C: C/h or 2C/h, L: L/h or
// 2L/h, D: linearised conductance at the guess; V and I keep their value, which their
// rhs coefficient needs).
__device__ __forceinline__ int w_coef_pass(const DevProg &P, const double *values, double h, int method,
                                           const double *guess, double *coef, int lane) {
  int err = 0;
  for (int e = lane; e < P.ne; e += 32) {
    const krets_element &E = P.el[e];
    const double val = values ? values[e] : E.value;
    double c = 0.0;
    switch (E.kind) {
      case KRETS_ELEM_R: c = (E.flags & KRETS_FLAG_G2) ? val : recip(val); break;
      case KRETS_ELEM_C: c = method == KRETS_METHOD_TR ? 2.0 * val / h : val / h; break;
      case KRETS_ELEM_L: c = method == KRETS_METHOD_TR ? 2.0 * val / h : val / h; break;
      case KRETS_ELEM_V:
      case KRETS_ELEM_I: c = val; break;
      case KRETS_ELEM_D: {
        double g, ieq;
        diode_lin(E, val, P.el_pos[e], guess, false, g, ieq);
        c = g;
        break;
      }
      case KRETS_ELEM_M: break;
      default: err |= KS_NOTIMPL;
    }
    coef[e] = c;
  }
  __syncwarp();
  return (int)__reduce_or_sync(kFull, (unsigned)err);
}

// Load the LU slots from the element coefficients (A entries summed in emission order,
// fill slots zero).  When a64 is given, the FP64 A entries are kept there as well.
template <typename T>
__device__ __forceinline__ void w_stamp_lu(const DevProg &P, const double *coef, T *lu, int lane) {
  for (int s = lane; s < P.nnz_lu; s += 32) {
    const int t = P.lu_src[s];
    lu[s] = t < 0 ? T(0) : T(sum_entry<double>(P, t, coef, nullptr));
  }
  __syncwarp();
}

// rhs coefficients of the dynamic elements (capacitors first), then the row gather.
__device__ __forceinline__ void s_rhs(const DevProg &P, const SProg &S, const double *values, const double *coef,
                                      const double *xp, const double *guess, const double *icap, int method,
                                      double t_src, double *cb, double *b, int lane) {
  for (int d = lane; d < P.ndyn; d += 32) {
    const int4 dd = S.dyn[d];
    const int e = dd.x & 0xffffff, kind = (int)((unsigned)dd.x >> 24);
    double v = 0.0;
    switch (kind) {
      case KRETS_ELEM_C: {
        const double vprev = (dd.y >= 0 ? xp[dd.y] : 0.0) - (dd.z >= 0 ? xp[dd.z] : 0.0);
        if (method == KRETS_METHOD_TR) {
          v = coef[e] * vprev + icap[d];
        } else {
          const double ieq = -(coef[e]) * vprev;  // -(C/h) v_prev  (stampable.rs:493)
          v = -ieq;
        }
        break;
      }
      case KRETS_ELEM_L: {
        const double iprev = xp[dd.w];
        if (method == KRETS_METHOD_TR) {
          const double vl = (dd.y >= 0 ? xp[dd.y] : 0.0) - (dd.z >= 0 ? xp[dd.z] : 0.0);
          v = -coef[e] * iprev - vl;
        } else {
          v = -(coef[e]) * iprev;  // -(L/h) i_prev  (stampable.rs:812)
        }
        break;
      }
      case KRETS_ELEM_V: v = wave_value(P.el[e], coef[e], t_src); break;
      case KRETS_ELEM_I: v = coef[e]; break;
      case KRETS_ELEM_D: {
        double g, ieq;
        diode_lin(P.el[e], values ? values[e] : P.el[e].value, make_int4(dd.y, dd.z, dd.w, -1), guess, false, g,
                  ieq);
        v = ieq;
        break;
      }
      default: break;
    }
    cb[d] = v;
  }
  __syncwarp();
  for (int k = lane; k < P.n; k += 32) {
    double s = 0.0;
    for (int u = S.bd_ptr[k]; u < S.bd_ptr[k + 1]; ++u) {
      const int code = S.bd_op[u];
      const double v = cb[code >> 1];
      s += (code & 1) ? -v : v;
    }
    b[k] = s;
  }
  __syncwarp();
}

// Mixed-precision solve: FP64 residual in element form, FP32 LU correction.  x holds the
// initial guess on entry.  Returns the iteration count, or -1 on stall / non-convergence.
__device__ int s_refine(const DevProg &P, const SProg &S, const double *coef, const float *lu32, const double *b,
                        double *x, float *w, double tol, int max_it, int lane) {
  double dprev = 0.0;
  for (int it = 0; it < max_it; ++it) {
    for (int k = lane; k < P.n; k += 32) {
      double r = b[k];
      const int2 rr = S.res_row[k];
      const int nu = rr.y & 0xffff, nt = (int)((unsigned)rr.y >> 16);
      for (int u = 0; u < nu; ++u) {
        const int op = S.res_op[rr.x + u];
        const double xj = x[op & 0x7fff];
        r = (op & 0x8000) ? r + xj : r - xj;
      }
      for (int u = nu; u < nt; ++u) {
        const int op = S.res_op[rr.x + u];
        const double a = coef[((unsigned)op >> 16) - 1];
        r = fma((op & 0x8000) ? a : -a, x[op & 0x7fff], r);
      }
      w[k] = (float)r;
    }
    __syncwarp();
    s_lsolve<float, float>(S, lu32, w, lane);
    s_usolve<float, float>(S, lu32, w, lane);
    double dmax = 0.0, xmax = 0.0;
    for (int k = lane; k < P.n; k += 32) {
      const double d = (double)w[k];
      const double xn = x[k] + d;
      x[k] = xn;
      dmax = fmax(dmax, fabs(d));
      xmax = fmax(xmax, fabs(xn));
    }
    __syncwarp();
    dmax = warp_max(dmax);
    xmax = warp_max(xmax);
    if (!(dmax == dmax) || !(xmax == xmax)) return -1;
    if (dmax <= tol * xmax) return it + 1;
    if (it > 0 && dmax > 0.5 * dprev) return -1;
    dprev = dmax;
  }
  return -1;
}

// Newton convergence test at warp level (solver.rs:76-104, "time" key included).
__device__ __forceinline__ bool w_converged(const DevProg &P, const KCfg &cfg, const double *prev,
                                            const double *x, double tprev, double tnew, int lane) {
  int ok = 1;
  for (int k = lane; k < P.n; k += 32) {
    const double v = x[k], p = prev[k];
    const double diff = fabs(v - p), scale = fmax(fabs(v), fabs(p));
    const double atol = P.is_cur[k] ? cfg.iabstol : cfg.vabstol;
    if (!(diff <= cfg.reltol * scale + atol)) ok = 0;
  }
  const double diff = fabs(tnew - tprev), scale = fmax(fabs(tnew), fabs(tprev));
  if (!(diff <= cfg.reltol * scale + cfg.vabstol)) ok = 0;
  return __all_sync(kFull, ok);
}

struct WarpLay {
  int lu, coef, x, b, w, cb, icap, prev, guess;
  int bytes;        // per warp
  int sprog_bytes;  // staged step program at the start of shared memory
};

template <int MIXED>
__global__ void __launch_bounds__(256, 1) k_tran_warp(DevProg P, KCfg cfg, WarpLay L, const double *values, int n_inst,
                                                   double h, int n_steps, int method, int lag, double *x_out,
                                                   int *inst_status, int *queue, unsigned long long *hist,
                                                   int *fallbacks, double *lu64_scratch, double tol) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // stage the compact step program in shared memory once per CTA
  {
    const int words = P.sp_off[11];
    const int4 *src = reinterpret_cast<const int4 *>(P.sprog);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int i = threadIdx.x; i < words / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
  }
  const SProg S = sprog_view(P, reinterpret_cast<const int *>(smem));
  char *base = smem + L.sprog_bytes + (size_t)wid * L.bytes;
  double *coef = reinterpret_cast<double *>(base + L.coef);
  double *x = reinterpret_cast<double *>(base + L.x);
  double *b = reinterpret_cast<double *>(base + L.b);
  float *w32 = reinterpret_cast<float *>(base + L.w);
  double *cb = reinterpret_cast<double *>(base + L.cb);
  double *icap = reinterpret_cast<double *>(base + L.icap);
  double *prev = reinterpret_cast<double *>(base + L.prev);
  double *guess = reinterpret_cast<double *>(base + L.guess);
  float *lu32 = reinterpret_cast<float *>(base + L.lu);
  double *lu64 = reinterpret_cast<double *>(base + L.lu);
  double *lu_fb = lu64_scratch ? lu64_scratch + (size_t)(blockIdx.x * (blockDim.x >> 5) + wid) * P.nnz_lu : nullptr;
  const size_t stride = (size_t)(n_steps + 1) * P.n;
  const int max_ref = 6;
  const bool linear = !P.nonlinear;
  while (true) {
    int inst = 0;
    if (lane == 0) inst = atomicAdd(queue, 1);
    inst = __shfl_sync(kFull, inst, 0);
    if (inst >= n_inst) break;
    int st = 0;
    bool use64 = !MIXED;
    unsigned long long lh[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double *vals = values ? values + (size_t)inst * P.ne : nullptr;
    double *out = x_out + (size_t)inst * stride;
    for (int k = lane; k < P.n; k += 32) x[k] = out[P.q[k]];
    for (int d = lane; d < P.ncap; d += 32) icap[d] = 0.0;
    __syncwarp();
    if (linear) {
      st |= w_coef_pass(P, vals, h, method, x, coef, lane);
      if (MIXED) {
        w_stamp_lu<float>(P, coef, lu32, lane);
        st |= w_factor<float>(P, lu32, lane);
      } else {
        w_stamp_lu<double>(P, coef, lu64, lane);
        st |= w_factor<double>(P, lu64, lane);
      }
    }
    for (int s = 1; s <= n_steps && !(st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)); ++s) {
      const double t = (double)s * h;
      double guess_time = (double)(s - 1) * h;
      const double *xp = x;
      if (!linear) {
        for (int k = lane; k < P.n; k += 32) {
          prev[k] = x[k];
          guess[k] = x[k];
        }
        __syncwarp();
        xp = prev;
      }
      int it;
      for (it = 0; it < cfg.maxiter; ++it) {
        const double t_src = lag ? guess_time : t;
        if (!linear) {
          st |= w_coef_pass(P, vals, h, method, guess, coef, lane);
          if (MIXED && !use64) {
            w_stamp_lu<float>(P, coef, lu32, lane);
            st |= w_factor<float>(P, lu32, lane);
          } else {
            double *luw = MIXED ? lu_fb : lu64;
            w_stamp_lu<double>(P, coef, luw, lane);
            st |= w_factor<double>(P, luw, lane);
          }
          if (st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) break;
        }
        s_rhs(P, S, vals, coef, xp, linear ? x : guess, icap, method, t_src, cb, b, lane);
        if (MIXED && !use64) {
          if (!linear) {
            for (int k = lane; k < P.n; k += 32) x[k] = guess[k];
            __syncwarp();
          }
          const int r = s_refine(P, S, coef, lu32, b, x, w32, tol, max_ref, lane);
          if (r > 0) {
            lh[r < 8 ? r : 7]++;
          } else if (lu_fb) {
            // refinement stalled: refactor in FP64 on the device, solve directly
            use64 = true;
            if (lane == 0) atomicAdd(fallbacks, 1);
            w_stamp_lu<double>(P, coef, lu_fb, lane);
            st |= w_factor<double>(P, lu_fb, lane);
            for (int k = lane; k < P.n; k += 32) x[k] = b[k];
            __syncwarp();
            s_lsolve<double, double>(S, lu_fb, x, lane);
            s_usolve<double, double>(S, lu_fb, x, lane);
          } else {
            st |= KS_STALL;
          }
        } else {
          const double *luw = MIXED ? lu_fb : lu64;
          for (int k = lane; k < P.n; k += 32) x[k] = b[k];
          __syncwarp();
          s_lsolve<double, double>(S, luw, x, lane);
          s_usolve<double, double>(S, luw, x, lane);
        }
        if (linear) break;
        if (w_converged(P, cfg, guess, x, guess_time, t, lane)) break;
        for (int k = lane; k < P.n; k += 32) guess[k] = x[k];
        __syncwarp();
        guess_time = t;
        if (it == cfg.maxiter - 1) st |= KS_MAXITER;
      }
      if (method == KRETS_METHOD_TR) {
        for (int d = lane; d < P.ncap; d += 32) {
          const int4 dd = S.dyn[d];
          const double vn = (dd.y >= 0 ? x[dd.y] : 0.0) - (dd.z >= 0 ? x[dd.z] : 0.0);
          icap[d] = coef[dd.x & 0xffffff] * vn - cb[d];
        }
      }
      // stream the solution row out in unknown order (contiguous, coalesced)
      double *row = out + (size_t)s * P.n;
      int nonfinite = 0;
      for (int k = lane; k < P.n; k += 32) {
        const double v = x[S.qinv[k]];
        nonfinite |= !isfinite(v);
        __stcs(row + k, v);
      }
      if (__any_sync(kFull, nonfinite)) st |= KS_NONFINITE;
      __syncwarp();
    }
    if (lane == 0 && inst_status) inst_status[inst] = st;
    if (MIXED && hist && lane == 0)
      for (int k = 0; k < 8; ++k)
        if (lh[k]) atomicAdd(hist + k, lh[k]);
    __syncwarp();
  }
}

}  // namespace krets

// ===================================================================== double-float path
// Linear circuits, FP32 factors: the same step as k_tran_warp<1>, with the residual,
// right-hand side, companion state and solution held in double-float (df.cuh) so the inner
// loop runs on FP32 pipes.  FP64 is used at set-up (coefficients, LU values before rounding
// to FP32), for source waveforms, and to write each solution row as FP64.
namespace krets {

__device__ __forceinline__ float warp_maxf(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ df df_at(const df *x, int i) { return i >= 0 ? x[i] : df{0.f, 0.f}; }

__device__ int df_refine(const DevProg &P, const SProg &S, const df *__restrict__ coef, const float *__restrict__ lu32,
                         const df *__restrict__ b, df *__restrict__ x, float *__restrict__ w, float tol, int max_it,
                         int lane) {
  float dprev = 0.f;
  for (int it = 0; it < max_it; ++it) {
    for (int k = lane; k < P.n; k += 32) {
      df r = b[k];
      const int2 rr = S.res_row[k];
      const int nu = rr.y & 0xffff, nt = (int)((unsigned)rr.y >> 16);
      for (int u = 0; u < nu; ++u) {
        const int op = S.res_op[rr.x + u];
        const df xj = x[op & 0x7fff];
        r = df_add(r, (op & 0x8000) ? xj : df_neg(xj));
      }
      for (int u = nu; u < nt; ++u) {
        const int op = S.res_op[rr.x + u];
        const df a = coef[((unsigned)op >> 16) - 1];
        r = df_fma((op & 0x8000) ? a : df_neg(a), x[op & 0x7fff], r);
      }
      w[k] = df_approx(r);
    }
    __syncwarp();
    s_lsolve<float, float>(S, lu32, w, lane);
    s_usolve<float, float>(S, lu32, w, lane);
    float dmax = 0.f, xmax = 0.f;
    for (int k = lane; k < P.n; k += 32) {
      const float d = w[k];
      const df xn = df_add_f(x[k], d);
      x[k] = xn;
      dmax = fmaxf(dmax, fabsf(d));
      xmax = fmaxf(xmax, fabsf(xn.hi));
    }
    __syncwarp();
    dmax = warp_maxf(dmax);
    xmax = warp_maxf(xmax);
    if (!(dmax == dmax) || !(xmax == xmax)) return -1;
    if (dmax <= tol * xmax) return it + 1;
    if (it > 0 && dmax > 0.5f * dprev) return -1;
    dprev = dmax;
  }
  return -1;
}

__global__ void __launch_bounds__(256, 1) k_tran_warp_df(DevProg P, KCfg cfg, WarpLay L, const double *values, int n_inst,
                                                      double h, int n_steps, int method, int lag, double *x_out,
                                                      int *inst_status, int *queue, unsigned long long *hist,
                                                      float tol) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  {
    const int words = P.sp_off[11];
    const int4 *src = reinterpret_cast<const int4 *>(P.sprog);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int i = threadIdx.x; i < words / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
  }
  const SProg S = sprog_view(P, reinterpret_cast<const int *>(smem));
  char *base = smem + L.sprog_bytes + (size_t)wid * L.bytes;
  float *lu32 = reinterpret_cast<float *>(base + L.lu);
  df *coef = reinterpret_cast<df *>(base + L.coef);
  double *coef64 = reinterpret_cast<double *>(base + L.coef);  // same bytes, set-up only
  df *x = reinterpret_cast<df *>(base + L.x);
  df *b = reinterpret_cast<df *>(base + L.b);
  float *w32 = reinterpret_cast<float *>(base + L.w);
  df *cb = reinterpret_cast<df *>(base + L.cb);
  df *icap = reinterpret_cast<df *>(base + L.icap);
  const size_t stride = (size_t)(n_steps + 1) * P.n;
  const int max_ref = 6;
  while (true) {
    int inst = 0;
    if (lane == 0) inst = atomicAdd(queue, 1);
    inst = __shfl_sync(kFull, inst, 0);
    if (inst >= n_inst) break;
    int st = 0;
    unsigned long long lh[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double *vals = values ? values + (size_t)inst * P.ne : nullptr;
    double *out = x_out + (size_t)inst * stride;
    // set-up: FP64 coefficients -> FP32 LU -> factor; then the coefficients become df
    st |= w_coef_pass(P, vals, h, method, nullptr, coef64, lane);
    w_stamp_lu<float>(P, coef64, lu32, lane);
    st |= w_factor<float>(P, lu32, lane);
    for (int e = lane; e < P.ne; e += 32) coef[e] = df_from_double(coef64[e]);
    for (int k = lane; k < P.n; k += 32) x[k] = df_from_double(out[P.q[k]]);
    for (int d = lane; d < P.ncap; d += 32) icap[d] = df{0.f, 0.f};
    __syncwarp();
    for (int s = 1; s <= n_steps && !(st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL | KS_STALL)); ++s) {
      const double t = (double)s * h;
      const double t_src = lag ? (double)(s - 1) * h : t;
      // companion / source coefficients from the previous solution
      for (int d = lane; d < P.ndyn; d += 32) {
        const int4 dd = S.dyn[d];
        const int e = dd.x & 0xffffff, kind = (int)((unsigned)dd.x >> 24);
        df v{0.f, 0.f};
        if (kind == KRETS_ELEM_C) {
          const df vprev = df_sub(df_at(x, dd.y), df_at(x, dd.z));
          v = method == KRETS_METHOD_TR ? df_fma(coef[e], vprev, icap[d]) : df_mul(coef[e], vprev);
        } else if (kind == KRETS_ELEM_L) {
          const df li = df_neg(df_mul(coef[e], x[dd.w]));
          v = method == KRETS_METHOD_TR ? df_sub(li, df_sub(df_at(x, dd.y), df_at(x, dd.z))) : li;
        } else if (kind == KRETS_ELEM_V) {
          const krets_element &E = P.el[e];
          v = df_from_double(wave_value(E, vals ? vals[e] : E.value, t_src));
        } else if (kind == KRETS_ELEM_I) {
          v = coef[e];
        }
        cb[d] = v;
      }
      __syncwarp();
      for (int k = lane; k < P.n; k += 32) {
        df acc{0.f, 0.f};
        for (int u = S.bd_ptr[k]; u < S.bd_ptr[k + 1]; ++u) {
          const int code = S.bd_op[u];
          acc = (code & 1) ? df_sub(acc, cb[code >> 1]) : df_add(acc, cb[code >> 1]);
        }
        b[k] = acc;
      }
      __syncwarp();
      const int r = df_refine(P, S, coef, lu32, b, x, w32, tol, max_ref, lane);
      if (r > 0) lh[r < 8 ? r : 7]++;
      else st |= KS_STALL;
      if (method == KRETS_METHOD_TR) {
        for (int d = lane; d < P.ncap; d += 32) {
          const int4 dd = S.dyn[d];
          const df vn = df_sub(df_at(x, dd.y), df_at(x, dd.z));
          icap[d] = df_sub(df_mul(coef[dd.x & 0xffffff], vn), cb[d]);
        }
      }
      double *row = out + (size_t)s * P.n;
      int nonfinite = 0;
      for (int k = lane; k < P.n; k += 32) {
        const double v = df_to_double(x[S.qinv[k]]);
        nonfinite |= !isfinite(v);
        __stcs(row + k, v);
      }
      if (__any_sync(kFull, nonfinite)) st |= KS_NONFINITE;
      __syncwarp();
    }
    if (lane == 0 && inst_status) inst_status[inst] = st;
    if (hist && lane == 0)
      for (int k = 0; k < 8; ++k)
        if (lh[k]) atomicAdd(hist + k, lh[k]);
    __syncwarp();
  }
}

}  // namespace krets

// ===================================================================== double-float direct
// Linear circuits: the LU is computed once in FP64 and each entry split into hi + lo FP32
// (reciprocal diagonals included); every step then does one forward and one backward solve
// in double-float arithmetic on the FP32 pipes.  No refinement loop: the factors carry
// 48 significand bits.
//
// One instance is handled by a group of G threads (G = 32, 64 or 128): a warp, or several
// warps joined by a named barrier.  More threads per instance shorten the wide levels of
// the solves and give each SM scheduler several warps to switch between, without more
// shared memory per instance.
namespace krets {

template <int G>
__device__ __forceinline__ void gsync(int gid) {
  if (G == 32) __syncwarp();
  else asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "n"(G) : "memory");
}

// group-wide "any": every thread of the group gets the same answer
template <int G>
__device__ __forceinline__ bool gany(bool v, int gid) {
  if (G == 32) return __any_sync(kFull, v);
  int r;
  asm volatile(
      "{ .reg .pred p, q;\n\t"
      "setp.ne.s32 p, %1, 0;\n\t"
      "barrier.red.or.pred q, %2, %3, p;\n\t"
      "selp.s32 %0, 1, 0, q; }"
      : "=r"(r)
      : "r"((int)v), "r"(gid + 1), "n"(G)
      : "memory");
  return r != 0;
}

template <int G>
__device__ int g_coef_pass(const DevProg &P, const double *values, double h, int method, double *coef, int gl) {
  int err = 0;
  for (int e = gl; e < P.ne; e += G) {
    const krets_element &E = P.el[e];
    const double val = values ? values[e] : E.value;
    double c = 0.0;
    switch (E.kind) {
      case KRETS_ELEM_R: c = (E.flags & KRETS_FLAG_G2) ? val : recip(val); break;
      case KRETS_ELEM_C: c = method == KRETS_METHOD_TR ? 2.0 * val / h : val / h; break;
      case KRETS_ELEM_L: c = method == KRETS_METHOD_TR ? 2.0 * val / h : val / h; break;
      case KRETS_ELEM_V:
      case KRETS_ELEM_I: c = val; break;
      case KRETS_ELEM_M: break;
      default: err |= KS_NOTIMPL;  // diodes never reach the linear engine
    }
    coef[e] = c;
  }
  return err;
}

// As g_factor64_merge with a warp per row and the dense LU by rows over lanes: for LU
// values in global memory, where the thread-per-row merge is a chain of dependent loads.
// Row k eliminates its L entries in order; the lanes share each U row j, finding their
// column in row k by binary search (or directly in the dense block).
__device__ __forceinline__ int row_find(const int *__restrict__ col, int lo, int hi, int c) {
  while (lo < hi) {  // first position in [lo, hi) with col >= c
    const int mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// smem (scratch, may be null): room for a per-warp map from the dense block's columns to
// the slots of the row being factored (rows before the block keep their entries in those
// columns, the border, at the end of the row); without room the border is searched too.
template <int G>
__device__ int g_factor64_warp(const DevProg &P, double *lu, int gl, int gid, double *tile, int tw, int *smem_map,
                               long long smem_bytes) {
  int bad = 0;
  const int m = P.tail_m, t0 = P.tail0;
  const int lane = gl & 31, warp = gl >> 5;
  constexpr int NW = G / 32;
  int *wmap = (m && smem_map && (long long)NW * m * 4 <= smem_bytes) ? smem_map + warp * m : nullptr;
  if (wmap) {
    for (int i = lane; i < m; i += 32) wmap[i] = -1;
    __syncwarp();
  }
  // dense-block rows (last level): each warp stages its row in shared memory — the dense
  // part (m values) and the sparse part (values and columns, at most cap entries) — so the
  // eliminations of the sparse columns (the Schur update of the block) update shared
  // memory instead of chaining global read-modify-writes
  const int cap = m ? (P.sprog[P.sp_off[12] + P.nlev - 1] >> 18) : 0;
  const long long st_words = ((long long)m * 2 + cap * 3 + 3) & ~3ll;  // 4-byte words; 16-byte aligned per warp
  double *wst = (m && smem_map && (long long)NW * st_words * 4 <= smem_bytes)
                    ? reinterpret_cast<double *>(smem_map + warp * st_words) : nullptr;
  for (int l = 0; l < P.nlev; ++l) {
    const int r0 = P.lev_ptr[l], r1 = P.lev_ptr[l + 1];
    const bool tail_level = m && l == P.nlev - 1;  // rows of the dense block: sparse columns only
    for (int t = r0 + warp; t < r1; t += NW) {
      const int k = P.ldesc[t].x;
      const int re = P.lu_rowptr[k + 1];
      const int dense0 = tail_level ? re - m : re;  // first slot of the dense part (tail rows)
      const int dk = tail_level ? dense0 : P.lu_diag[k];
      if (tail_level && wst && dense0 - P.lu_rowptr[k] <= cap) {
        const int s0 = P.lu_rowptr[k], ns = dense0 - s0;
        double *D = wst, *Sv = wst + m;
        int *Sc = reinterpret_cast<int *>(Sv + cap);
        for (int i = lane; i < m; i += 32) D[i] = lu[dense0 + i];
        for (int i = lane; i < ns; i += 32) {
          Sv[i] = lu[s0 + i];
          Sc[i] = P.lu_col[s0 + i];
        }
        __syncwarp();
        int dj = ns > 0 ? P.lu_diag[Sc[0]] : 0;  // diagonal slot of the next column, loaded ahead
        for (int q = 0; q < ns; ++q) {
          const int j = Sc[q];
          const int ub = dj + 1, ue = P.lu_rowptr[j + 1];
          const double rpiv = lu[dj];  // rows before the block hold reciprocal pivots
          if (q + 1 < ns) dj = P.lu_diag[Sc[q + 1]];
          const double l_kj = Sv[q] * rpiv;
          __syncwarp();
          if (lane == 0) Sv[q] = l_kj;
          for (int u0 = ub + lane; u0 < ue; u0 += 128) {  // four entries of U row j in flight per lane
            int cs[4];
            double vs[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              const int u = u0 + 32 * r;
              cs[r] = u < ue ? P.lu_col[u] : -1;
              vs[r] = u < ue ? lu[u] : 0.0;
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              const int c = cs[r];
              if (c < 0) continue;
              const double v = l_kj * vs[r];
              if (c >= t0) {
                D[c - t0] -= v;
              } else {
                int lo = q + 1, hi = ns;  // c > j: among this row's later sparse columns
                while (lo < hi) {
                  const int mid = (lo + hi) >> 1;
                  if (Sc[mid] < c) lo = mid + 1;
                  else hi = mid;
                }
                if (lo < ns && Sc[lo] == c) Sv[lo] -= v;
                else bad |= KS_SINGULAR;  // not in the pattern: an inconsistent program
              }
            }
          }
          __syncwarp();
        }
        for (int i = lane; i < m; i += 32) lu[dense0 + i] = D[i];
        for (int i = lane; i < ns; i += 32) lu[s0 + i] = Sv[i];
        __syncwarp();
        continue;
      }
      // row before the block: map its border columns to their slots
      int b0 = dense0;
      if (!tail_level && wmap) {
        b0 = row_find(P.lu_col, dk + 1, re, t0);
        for (int q = b0 + lane; q < re; q += 32) wmap[P.lu_col[q] - t0] = q;
        __syncwarp();
      }
      for (int s = P.lu_rowptr[k]; s < dk; ++s) {
        const int j = P.lu_col[s];
        const double l_kj = lu[s] * lu[P.lu_diag[j]];  // reciprocal pivot of the finished row j
        __syncwarp();
        if (lane == 0) lu[s] = l_kj;
        const int ue = P.lu_rowptr[j + 1];
        for (int u = P.lu_diag[j] + 1 + lane; u < ue; u += 32) {
          const int c = P.lu_col[u];
          int p;
          if (tail_level && c >= t0) {
            p = dense0 + (c - t0);
          } else if (wmap && c >= t0) {
            p = wmap[c - t0];
            if (p < 0) {
              bad |= KS_SINGULAR;  // not in the pattern: an inconsistent program
              continue;
            }
          } else {
            p = row_find(P.lu_col, s + 1, b0, c);
            if (p >= b0 || P.lu_col[p] != c) {
              bad |= KS_SINGULAR;
              continue;
            }
          }
          lu[p] -= l_kj * lu[u];
        }
        __syncwarp();
      }
      if (!tail_level && wmap) {
        for (int q = b0 + lane; q < re; q += 32) wmap[P.lu_col[q] - t0] = -1;
        __syncwarp();
      }
      if (!tail_level && lane == 0) {
        // the row is final: check its pivot and keep its reciprocal, so later rows
        // multiply instead of dividing (FP64 division is a long chain on this GPU)
        const double d = lu[dk];
        if (!(fabs(d) > 0)) bad |= KS_SINGULAR;
        else if (!isfinite(d)) bad |= KS_NONFINITE;
        lu[dk] = recip(d);
      }
    }
    gsync<G>(gid);
  }
  if (m) {
    // blocked right-looking LU of the dense block (rows in global memory), panels of 32
    // columns: (1) the panel by columns (a warp per row, lanes over the panel's columns);
    // (2) per tile of tw columns right of it: the tile staged in shared memory, the unit
    // lower 32 x 32 solve on it (a thread per column), the tile written back as U12, and
    // (3) the rows below updated from it, A22 -= L21 U12 (a warp per row, lanes over the
    // tile's columns, L21 broadcast by shuffles).  Each trailing element is read and
    // written once per panel instead of once per column.
    auto row = [&](int i) { return lu + (P.lu_rowptr[t0 + i + 1] - m); };
    for (int kb = 0; kb < m; kb += 32) {
      const int nb = min(32, m - kb);
      for (int kk = kb; kk < kb + nb; ++kk) {
        const double *pr = row(kk);
        const double piv = pr[kk];
        if (gl == 0) {
          if (!(fabs(piv) > 0)) bad |= KS_SINGULAR;
          else if (!isfinite(piv)) bad |= KS_NONFINITE;
        }
        for (int i = kk + 1 + warp; i < m; i += NW) {
          double *ri = row(i);
          const double l_ik = ri[kk] / piv;
          __syncwarp();
          if (lane == 0) ri[kk] = l_ik;
          for (int c = kk + 1 + lane; c < kb + nb; c += 32) ri[c] -= l_ik * row(kk)[c];
        }
        gsync<G>(gid);
      }
      for (int c0 = kb + nb; c0 < m; c0 += tw) {
        const int w = min(tw, m - c0);
        for (int q = gl; q < nb * w; q += G) tile[(q / w) * tw + q % w] = row(kb + q / w)[c0 + q % w];
        gsync<G>(gid);
        for (int c = gl; c < w; c += G)
          for (int r = 1; r < nb; ++r) {
            const double *lr = row(kb + r) + kb;
            double acc = tile[r * tw + c];
            for (int q = 0; q < r; ++q) acc -= lr[q] * tile[q * tw + c];
            tile[r * tw + c] = acc;
          }
        gsync<G>(gid);
        for (int q = gl; q < nb * w; q += G) row(kb + q / w)[c0 + q % w] = tile[(q / w) * tw + q % w];
        for (int i = kb + nb + warp; i < m; i += NW) {
          double *ri = row(i);
          const double lq = lane < nb ? ri[kb + lane] : 0.0;
          for (int cb = 0; cb < w; cb += 32) {  // every lane takes part in the shuffles
            const int c = cb + lane;
            double acc = 0.0;
            for (int q = 0; q < nb; ++q) acc += __shfl_sync(kFull, lq, q) * (c < w ? tile[q * tw + c] : 0.0);
            if (c < w) ri[c0 + c] -= acc;
          }
        }
        gsync<G>(gid);
      }
    }
  }
  for (int k = (m ? t0 : P.n) + gl; k < P.n; k += G) {  // pivots of the dense block
    const int sl = P.lu_diag[k];
    lu[sl] = recip(lu[sl]);
  }
  gsync<G>(gid);
  return bad;
}

// As g_factor64, without an update list: row k merges each U row j (columns ascending)
// into its own sorted pattern.  The host checked that every update lands in the pattern;
// an entry not found (an inconsistent program) stops the row and reports it singular.
template <int G>
__device__ int g_factor64_merge(const DevProg &P, double *lu, int gl, int gid) {
  int bad = 0;
  const int m = P.tail_m;
  for (int l = 0; l < P.nlev; ++l) {
    const int r0 = P.lev_ptr[l], r1 = P.lev_ptr[l + 1];
    const bool tail_level = m && l == P.nlev - 1;  // rows of the dense block: sparse columns only
    for (int t = r0 + gl; t < r1; t += G) {
      const int k = P.ldesc[t].x;
      const int dk = tail_level ? P.lu_rowptr[k + 1] - m : P.lu_diag[k], re = P.lu_rowptr[k + 1];
      for (int s = P.lu_rowptr[k]; s < dk; ++s) {
        const int j = P.lu_col[s];
        const double l_kj = lu[s] / lu[P.lu_diag[j]];
        lu[s] = l_kj;
        int p = s + 1;
        const int ue = P.lu_rowptr[j + 1];
        for (int u = P.lu_diag[j] + 1; u < ue; ++u) {
          const int c = P.lu_col[u];
          while (p < re && P.lu_col[p] < c) ++p;
          if (p >= re || P.lu_col[p] != c) {
            bad |= KS_SINGULAR;
            break;
          }
          lu[p] -= l_kj * lu[u];
        }
      }
      if (!tail_level) {
        const double d = lu[dk];
        if (!(fabs(d) > 0)) bad |= KS_SINGULAR;
        else if (!isfinite(d)) bad |= KS_NONFINITE;
      }
    }
    gsync<G>(gid);
  }
  if (m) {
    // dense right-looking LU of the trailing block, row i of the block at slots
    // lu_rowptr[tail0 + i + 1] - m .. (column j of the block at offset j)
    const int t0 = P.tail0;
    for (int kk = 0; kk < m; ++kk) {
      const double *pr = lu + (P.lu_rowptr[t0 + kk + 1] - m);
      const double piv = pr[kk];
      if (!(fabs(piv) > 0)) bad |= KS_SINGULAR;
      else if (!isfinite(piv)) bad |= KS_NONFINITE;
      for (int i = kk + 1 + gl; i < m; i += G) {
        double *ri = lu + (P.lu_rowptr[t0 + i + 1] - m);
        ri[kk] = ri[kk] / piv;
      }
      gsync<G>(gid);
      const int w = m - kk - 1;  // rows and columns below / right of the pivot
      for (long long q = gl; q < (long long)w * w; q += G) {
        const int i = kk + 1 + (int)(q / w), c = kk + 1 + (int)(q % w);
        double *ri = lu + (P.lu_rowptr[t0 + i + 1] - m);
        ri[c] -= ri[kk] * pr[c];
      }
      gsync<G>(gid);
    }
  }
  for (int k = gl; k < P.n; k += G) {
    const int sl = P.lu_diag[k];
    lu[sl] = recip(lu[sl]);
  }
  gsync<G>(gid);
  return bad;
}

template <int G>
__device__ int g_factor64(const DevProg &P, double *lu, int gl, int gid) {
  int bad = 0;
  for (int l = 0; l < P.nlev; ++l) {
    const int r0 = P.lev_ptr[l], r1 = P.lev_ptr[l + 1];
    for (int t = r0 + gl; t < r1; t += G) {
      const int k = P.ldesc[t].x;
      for (int pi = P.piv_ptr[k]; pi < P.piv_ptr[k + 1]; ++pi) {
        const int4 pv = P.piv[pi];
        const double l_kj = lu[pv.x] / lu[P.lu_diag[pv.y]];
        lu[pv.x] = l_kj;
        for (int u = pv.z; u < pv.w; ++u) {
          const int2 d = P.upd[u];
          lu[d.x] -= l_kj * lu[d.y];
        }
      }
      const double dk = lu[P.lu_diag[k]];
      if (!(fabs(dk) > 0)) bad |= KS_SINGULAR;
      else if (!isfinite(dk)) bad |= KS_NONFINITE;
    }
    gsync<G>(gid);
  }
  for (int k = gl; k < P.n; k += G) {
    const int sl = P.lu_diag[k];
    lu[sl] = recip(lu[sl]);
  }
  gsync<G>(gid);
  return bad;
}

template <bool UPPER>
__device__ __forceinline__ df df_row(const SProg &S, const df *__restrict__ lu, const df *y, const int4 d, int &k) {
  k = d.x & 0xffff;
  const int rest = (int)((unsigned)d.x >> 16);
  const int first = UPPER ? d.y + 1 : d.y;
  const int c0 = d.z & 0xffff, c1 = (int)((unsigned)d.z >> 16);
  const df zero{0.f, 0.f};
  const df a0 = d.w > 0 ? lu[first] : zero;
  const df a1 = d.w > 1 ? lu[first + 1] : zero;
  df s = y[k];
  s = df_fma_acc(df_neg(a0), y[c0], s);
  s = df_fma_acc(df_neg(a1), y[c1], s);
  for (int j = 2; j < 2 + rest; ++j) s = df_fma_acc(df_neg(lu[first + j]), y[S.lu_col[first + j]], s);
  s = df_norm(s);
  if (UPPER) s = df_mul(s, lu[d.y]);
  return s;
}

// Level-scheduled double-float solve by a group of G threads.  Levels with at most 64 rows
// (the top of the elimination tree: its last levels for L, its first for U) run on the
// group's first warp alone with warp barriers; `nar` is the first narrow level of L (rows
// of every later level <= 64) or the number of leading narrow levels of U.
template <int G, bool UPPER>
__device__ __forceinline__ void df_level(const SProg &S, const df *__restrict__ lu, df *y, const int *ptr,
                                         const int4 *desc, int l, int tid, int stride) {
  const int r0 = ptr[l], r1 = ptr[l + 1];
  for (int t = r0 + tid; t < r1; t += 2 * stride) {
    int k0, k1 = -1;
    const df v0 = df_row<UPPER>(S, lu, y, desc[t], k0);
    df v1{0.f, 0.f};
    if (t + stride < r1) v1 = df_row<UPPER>(S, lu, y, desc[t + stride], k1);
    y[k0] = v0;
    if (k1 >= 0) y[k1] = v1;
  }
}

// Lanes per row of a level for a group of G threads, from the level's split code (host
// symbolic pass: split_code()).
// G = 0: the wide 256-thread split (a warp per row allowed)
template <int G>
__device__ __forceinline__ int split_lanes(int code) {
  constexpr int g = G == 0 ? 5 : G >= 512 ? 4 : G >= 256 ? 3 : G >= 128 ? 2 : G >= 64 ? 1 : 0;
  return 1 << ((code >> (3 * g)) & 7);
}

// lanes of this thread's aligned group of spl lanes (spl a power of two <= 32)
__device__ __forceinline__ unsigned lane_mask(int spl) {
  return spl >= 32 ? 0xffffffffu : ((1u << spl) - 1u) << ((threadIdx.x & 31) & ~(spl - 1));
}

// Sum a double-float over the `spl` aligned lanes of a row (xor butterfly: every lane ends
// with the same sum, formed in the same order on every run).
__device__ __forceinline__ df df_lane_sum(df s, int spl, unsigned mask) {
  for (int o = spl >> 1; o > 0; o >>= 1) {
    df r;
    r.hi = __shfl_xor_sync(mask, s.hi, o);
    r.lo = __shfl_xor_sync(mask, s.lo, o);
    s = df_add(s, r);
  }
  return s;
}

// One level with each row split over `spl` lanes (a power of two <= 8): lane j of a row
// takes entries j, j + spl, ...; the first lane adds the right-hand side and writes.
template <bool UPPER>
__device__ __forceinline__ void df_level_split(const SProg &S, const df *__restrict__ lu, df *y, const int *ptr,
                                               const int4 *desc, int l, int tid, int nthreads, int spl) {
  const int r0 = ptr[l], r1 = ptr[l + 1];
  const int sub = tid & (spl - 1);
  const unsigned mask = lane_mask(spl);
  for (int t = r0 + tid / spl; t < r1; t += nthreads / spl) {
    const int4 d = desc[t];
    const int k = d.x & 0xffff;
    const int cnt = d.w + (int)((unsigned)d.x >> 16);
    const int first = UPPER ? d.y + 1 : d.y;
    df s = sub == 0 ? y[k] : df{0.f, 0.f};
    int j = sub;
    for (; j + 3 * spl < cnt; j += 4 * spl) {  // four entries' loads in flight
      df a[4], v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = lu[first + j + q * spl];
        v[q] = y[S.lu_col[first + j + q * spl]];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) s = df_fma_acc(df_neg(a[q]), v[q], s);
    }
    for (; j < cnt; j += spl) s = df_fma_acc(df_neg(lu[first + j]), y[S.lu_col[first + j]], s);
    s = df_lane_sum(df_norm(s), spl, mask);
    if (sub == 0) y[k] = UPPER ? df_mul(s, lu[d.y]) : s;
  }
}

// SG: group size the row splits are chosen for (a caller that must reproduce another
// group size's arithmetic bit for bit passes that size)
// Blocked dense triangular solves of the trailing block (positions tail0 ..).  Row i of the
// block keeps its dense part (columns tail0 ..) at slot `base` from the descriptor of the
// last L level: first entry + entries before the block.  Blocks of 32 rows: the diagonal
// block on the group's first warp (a lane per row, values broadcast by shuffles), then
// the rows after (lower) or before (upper) it updated in parallel, 8 lanes per row.
__device__ __forceinline__ int dense_base(const int4 d) { return d.y + d.w + (int)((unsigned)d.x >> 16); }

// Two rows per 8-lane group per pass, so their loads are in flight together.
template <int G, bool UPPER>
__device__ __forceinline__ void df_dense_update(const SProg &S, const int4 *td, const df *__restrict__ lu, df *y,
                                                int t0, int kb, int nb, int r_begin, int r_end, int gl) {
  const int sub = gl & 7;
  const unsigned mask = 0xffu << ((threadIdx.x & 31) & ~7);
  df yv[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) yv[q] = sub + 8 * q < nb ? y[t0 + kb + sub + 8 * q] : df{0.f, 0.f};
  constexpr int R = G / 8;  // rows per pass of the group
  for (int r = r_begin + (gl >> 3); r < r_end; r += 2 * R) {
    const bool two = r + R < r_end;
    const int b0 = S.dense_rows ? S.dense_rows[r] : dense_base(td[r]);
    const int b1 = two ? (S.dense_rows ? S.dense_rows[r + R] : dense_base(td[r + R])) : b0;
    df a0[4], a1[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool in = sub + 8 * q < nb;
      a0[q] = in ? lu[b0 + kb + sub + 8 * q] : df{0.f, 0.f};
      a1[q] = in && two ? lu[b1 + kb + sub + 8 * q] : df{0.f, 0.f};
    }
    df s0{0.f, 0.f}, s1{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      s0 = df_fma_acc(a0[q], yv[q], s0);
      s1 = df_fma_acc(a1[q], yv[q], s1);
    }
    s0 = df_lane_sum(df_norm(s0), 8, mask);
    s1 = df_lane_sum(df_norm(s1), 8, mask);
    if (sub == 0) {
      y[t0 + r] = df_sub(y[t0 + r], s0);
      if (two) y[t0 + r + R] = df_sub(y[t0 + r + R], s1);
    }
  }
}

// Diagonal block rows of the first warp: lane i holds row kb + i; with a staging tile the
// block is loaded once (all loads in flight) and read from shared memory.
__device__ __forceinline__ const df *dense_diag_rows(const SProg &S, const df *__restrict__ lu, int base, int kb,
                                                     int nb, int i) {
  if (!S.dense_stage) return lu + base + kb;
  df *t = S.dense_stage + i * 33;
  if (i < nb) {
    df v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = j < nb ? lu[base + kb + j] : df{0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 32; ++j) t[j] = v[j];
  }
  __syncwarp();
  return t;
}

template <int G>
__device__ __forceinline__ void df_dense_lower(const SProg &S, const df *__restrict__ lu, df *y, int gl, int gid) {
  const int m = S.tail_m, t0 = S.tail0;
  const int4 *td = S.ldesc + S.lev_ptr[S.nlev - 1];
  for (int kb = 0; kb < m; kb += 32) {
    const int nb = min(32, m - kb);
    if (gl < 32) {
      const int i = gl;
      df yi{0.f, 0.f};
      int base = 0;
      if (i < nb) {
        base = S.dense_rows ? S.dense_rows[kb + i] : dense_base(td[kb + i]);
        yi = y[t0 + kb + i];
      }
      const df *row = dense_diag_rows(S, lu, base, kb, nb, i);
      for (int j = 0; j < nb - 1; ++j) {
        df yj;
        yj.hi = __shfl_sync(kFull, yi.hi, j);
        yj.lo = __shfl_sync(kFull, yi.lo, j);
        if (i > j && i < nb) yi = df_fma(df_neg(row[j]), yj, yi);
      }
      if (i < nb) y[t0 + kb + i] = yi;
      __syncwarp();  // staging tile free for the next block
    }
    gsync<G>(gid);
    if (kb + nb < m) {
      df_dense_update<G, false>(S, td, lu, y, t0, kb, nb, kb + nb, m, gl);
      gsync<G>(gid);
    }
  }
}

template <int G>
__device__ __forceinline__ void df_dense_upper(const SProg &S, const df *__restrict__ lu, df *y, int gl, int gid) {
  const int m = S.tail_m, t0 = S.tail0;
  const int4 *td = S.ldesc + S.lev_ptr[S.nlev - 1];
  for (int kb = ((m - 1) / 32) * 32; kb >= 0; kb -= 32) {
    const int nb = min(32, m - kb);
    if (gl < 32) {
      const int i = gl;
      df yi{0.f, 0.f};
      int base = 0;
      if (i < nb) {
        base = S.dense_rows ? S.dense_rows[kb + i] : dense_base(td[kb + i]);
        yi = y[t0 + kb + i];
      }
      const df *row = dense_diag_rows(S, lu, base, kb, nb, i);
      for (int j = nb - 1; j >= 0; --j) {
        if (i == j) yi = df_mul(yi, row[j]);  // reciprocal diagonal
        df xj;
        xj.hi = __shfl_sync(kFull, yi.hi, j);
        xj.lo = __shfl_sync(kFull, yi.lo, j);
        if (i < j) yi = df_fma(df_neg(row[j]), xj, yi);
      }
      if (i < nb) y[t0 + kb + i] = yi;
      __syncwarp();  // staging tile free for the next block
    }
    gsync<G>(gid);
    if (kb > 0) {
      df_dense_update<G, true>(S, td, lu, y, t0, kb, nb, 0, kb, gl);
      gsync<G>(gid);
    }
  }
}

// Border of the dense block, after its backward solve: every row before the block
// subtracts its U entries in the block's columns (x there is final), all rows at once.
// Pass 1: chunks of <= 16 entries over all threads (four loads in flight); pass 2: each
// row sums its chunks' partial sums in order.
template <int G>
__device__ __forceinline__ void df_border(const SProg &S, const df *__restrict__ lu, df *y, int gl, int gid) {
  for (int c = gl; c < S.n_bchunk; c += G) {
    const int2 ch = S.bchunk[c];
    df s{0.f, 0.f};
    for (int e = 0; e < ch.y; e += 4) {
      df a[4], v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool in = e + q < ch.y;
        a[q] = in ? lu[ch.x + e + q] : df{0.f, 0.f};
        v[q] = in ? y[S.lu_col[ch.x + e + q]] : df{0.f, 0.f};
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) s = df_fma_acc(a[q], v[q], s);
    }
    S.bpart[c] = df_norm(s);
  }
  gsync<G>(gid);
  for (int r = gl; r < S.n_brow; r += G) {
    const int4 br = S.brow[r];
    df s = S.bpart[br.y];
    for (int c = br.y + 1; c < br.y + br.z; ++c) s = df_add(s, S.bpart[c]);
    y[br.x] = df_sub(y[br.x], s);
  }
  gsync<G>(gid);
}

// TAIL: the program may have a dense trailing block (multi-circuit programs); the
// single-topology engines compile without that code.
template <int G, bool UPPER, int SG = G, bool TAIL = true>
__device__ __forceinline__ void df_solve(const SProg &S, const df *__restrict__ lu, df *y, int gl, int gid, int nar) {
  const int nl = UPPER ? S.nulev : S.nlev;
  const int *ptr = UPPER ? S.ulev_ptr : S.lev_ptr;
  const int4 *desc = UPPER ? S.udesc : S.ldesc;
  const int *mx = UPPER ? S.umax : S.lmax;
  const bool w0 = gl < 32;
  if (nar < 0) {  // no narrow-level split: every level on the whole group
    if (TAIL && UPPER && S.tail_m) df_dense_upper<G>(S, lu, y, gl, gid);
    if (TAIL && UPPER && S.n_brow) df_border<G>(S, lu, y, gl, gid);
    for (int l = UPPER ? 0 : 1; l < nl; ++l) {
      const int spl = split_lanes<SG>(mx[l]);
      if (spl > 1) df_level_split<UPPER>(S, lu, y, ptr, desc, l, gl, G, spl);
      else df_level<G, UPPER>(S, lu, y, ptr, desc, l, gl, G);
      gsync<G>(gid);
    }
    if (TAIL && !UPPER && S.tail_m) df_dense_lower<G>(S, lu, y, gl, gid);
    return;
  }
  if (!UPPER) {
    for (int l = 1; l < nar; ++l) {
      df_level<G, UPPER>(S, lu, y, ptr, desc, l, gl, G);
      gsync<G>(gid);
    }
    if (w0) {
      for (int l = nar > 1 ? nar : 1; l < nl; ++l) {
        df_level<G, UPPER>(S, lu, y, ptr, desc, l, gl, 32);
        __syncwarp();
      }
    }
    gsync<G>(gid);
  } else {
    if (w0) {
      for (int l = 0; l < nar; ++l) {
        df_level<G, UPPER>(S, lu, y, ptr, desc, l, gl, 32);
        __syncwarp();
      }
    }
    gsync<G>(gid);
    for (int l = nar; l < nl; ++l) {
      df_level<G, UPPER>(S, lu, y, ptr, desc, l, gl, G);
      gsync<G>(gid);
    }
  }
}

// Shared-memory layout of one instance of the double-float direct engine.
struct DfdLay {
  int lu;     // df[nnz_lu] (shared memory; unused when the factors are in global memory)
  int x;      // df[n]  (solution; the rhs is assembled and solved in place)
  int cdyn;   // df[ndyn] coefficients of the rhs elements (C/h or 2C/h, L/h or 2L/h, source values)
  int cb;     // df[ndyn] rhs coefficients of the step
  int icap;   // df[ncap] trapezoidal capacitor currents
  int slot;   // int[4]   group's work item and status words
  int coef64; // double[ne] set-up scratch (aliases x / cdyn / cb / icap and padding)
  int bytes;  // per instance
  int sprog_bytes;
  // 1: the interleaved step with a direct right-hand side (dfd_steps_lean; factors in
  // global memory): x holds n + 2 values (a zero for ground at n, a write-only slot at
  // n + 1), cb is the second state buffer (n + 2 values), icap the capacitor companion
  // values; the staged program is the direct right-hand side, qinv and the interleaved
  // solves
  int lean;
};

// Set-up of one instance for the double-float direct engine: FP64 coefficients, LU
// stamped and factored in FP64 (in lu64), then split to double-float pairs in place (lu);
// coefficients of the rhs elements (C/h or 2C/h, L/h or 2L/h, source values) to cdyn.
// coef64 may alias x / cdyn / cb / icap: it is dead once the LU is formed, and the
// rhs-element coefficients are recomputed with the same expressions as g_coef_pass.
// MERGE: 0 = update list, 1 = thread-per-row merge, 2 = warp-per-row (global memory)
template <int G, int MERGE = 0>
__device__ __forceinline__ int dfd_setup(const DevProg &P, const SProg &S, const double *vals, double h, int method,
                                         df *lu, double *lu64, double *coef64, df *cdyn, int gl, int gid,
                                         double *tile = nullptr, int tw = 0, long long tile_bytes = 0) {
  int st = g_coef_pass<G>(P, vals, h, method, coef64, gl);
  gsync<G>(gid);
  for (int sl = gl; sl < P.nnz_lu; sl += G) {
    const int t = P.lu_src[sl];
    lu64[sl] = t < 0 ? 0.0 : sum_entry<double>(P, t, coef64, nullptr);
  }
  gsync<G>(gid);
  st |= MERGE == 2   ? g_factor64_warp<G>(P, lu64, gl, gid, tile, tw, reinterpret_cast<int *>(tile), tile_bytes)
        : MERGE == 1 ? g_factor64_merge<G>(P, lu64, gl, gid)
                     : g_factor64<G>(P, lu64, gl, gid);
  for (int sl = gl; sl < P.nnz_lu; sl += G) lu[sl] = df_from_double(lu64[sl]);
  for (int d = gl; d < P.ndyn; d += G) {
    const int e = P.dyn_e[d];
    const krets_element &E = P.el[e];
    const double val = vals ? vals[e] : E.value;
    double c = val;
    if (E.kind == KRETS_ELEM_C || E.kind == KRETS_ELEM_L) c = method == KRETS_METHOD_TR ? 2.0 * val / h : val / h;
    cdyn[d] = df_from_double(c);
  }
  return st;
}

// Transient steps 1..n_steps of one instance from the state in x (position space), rows
// of `out` (original unknown order, n per row) written with streaming stores.
// Source waveforms tabulated per step (k_wave_table): row wrow[d] of wtab holds the
// value of rhs element d's PULSE/SIN source at the source time of every step, so the
// step loop reads one value instead of evaluating fmod and divisions on the FP64 pipe
// (a latency on every step's critical path).  Without a table the waveform is evaluated.
struct WaveTab {
  const double *tab;  // [rows][n_steps + 1]
  const int *row;     // [ndyn]: row of a tabulated source, -1 otherwise
  int stride;         // n_steps + 1
};

// value of every PULSE / SIN source at each step's source time (transient.rs:49 timing
// when lag is set), same expression as the step loop's wave_value call
__global__ void k_wave_table(const krets_element *el, const int *src_elem, int n_src, double h, int n_steps, int lag,
                             double *tab) {
  const long long total = (long long)n_src * (n_steps + 1);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / (n_steps + 1)), s = (int)(i % (n_steps + 1));
    const double t_src = lag ? (double)(s - 1) * h : (double)s * h;
    const krets_element &E = el[src_elem[r]];
    tab[i] = wave_value(E, E.value, t_src);
  }
}

// Output selection of the double-float transient: n = 0 writes every unknown each step;
// otherwise only the unknowns idx[0..n) (original numbering), in that order, and the
// instance's operating point is read from x0 ([n_inst][P.n]) instead of its output row 0.
struct Probe {
  const int *idx;
  int n;
  const double *x0;
};

// Forward pass of the adjoint on this engine: from x_0 = 0 (zero operating point), no
// waveform output; before step s with (s-1) % K == 0 the state (x in position space, the
// TR capacitor currents) goes to checkpoint (s-1)/K at ck + that * ck_words, and
// sum_n x_n[out_pos]^2 is accumulated in double-float and written to *loss.  ck and loss
// point at the instance's own slots (ck == nullptr: not an adjoint forward pass).
struct AdjFwd {
  df *ck;
  int K, ck_words, out_pos;
  double *loss;
};

// Interleaved solves (factors in global memory; layout: pack_interleaved in the host
// symbolic pass).  A level record is two int4: {W, log2 lanes per row, entry slots per
// lane, first entry slot} and {row base, diagonal slot base, flags, 0}; lane lam of the
// level handles row lam >> lsh with its entries j = lam % spl + i spl (slot first + i W +
// lam), visited in the same order as df_level / df_level_split and padded with exact
// zeros, so the results are identical.  Flag bit 0: the level has at most 32 lanes and
// runs on the group's first warp alone; bit 1: so does the next level, and a warp barrier
// separates the two instead of a group barrier.
struct IlProg {
  const int4 *rec;                 // level records (L levels from level 1, then U levels)
  const int *rows;                 // positions of the levels' rows
  const unsigned short *cols;      // column of every entry slot
  const df *lui;                   // interleaved factors (this instance's region)
  int nl, nu;                      // L levels (from level 1), U levels
};

// One level on GG threads (gl < GG).  Lane lam = base + gl (and base + GG + gl when the
// level is wider than GG); a lane past the level's width repeats the loads of its last
// lane (in range) and drops the result, so loop trip counts and shuffles are uniform over
// each warp and the rows of a lane group are never split (W is a multiple of spl).
template <int GG, bool UPPER>
__device__ __forceinline__ void il_level(const int4 A, const int4 B, const IlProg &I, df *y, int gl) {
  const int W = A.x, lsh = A.y, mc = A.z, spl = 1 << lsh;
  for (int base = 0; base < W; base += 2 * GG) {
    const int lam0 = min(base + gl, W - 1);
    const int r0 = lam0 >> lsh;
    const int k0 = I.rows[B.x + r0];
    const bool f0 = (lam0 & (spl - 1)) == 0, w0 = base + gl < W && f0;
    const df t0 = y[k0];  // in range for every lane; kept only by a row's first lane
    df s0{f0 ? t0.hi : 0.f, f0 ? t0.lo : 0.f};
    df d0{0.f, 0.f};
    if (UPPER) d0 = I.lui[B.y + r0];
    int o0 = A.w + lam0;
    if (base + GG < W) {  // a second lane per thread (uniform over the group)
      const int lam1 = min(base + GG + gl, W - 1);
      const int r1 = lam1 >> lsh;
      const int k1 = I.rows[B.x + r1];
      const bool f1 = (lam1 & (spl - 1)) == 0, w1 = base + GG + gl < W && f1;
      const df t1 = y[k1];
      df s1{f1 ? t1.hi : 0.f, f1 ? t1.lo : 0.f};
      df d1{0.f, 0.f};
      if (UPPER) d1 = I.lui[B.y + r1];
      int o1 = A.w + lam1;
      int i = 0;
      for (; i + 1 < mc; i += 2) {  // two entries of each lane in flight
        const df a0 = I.lui[o0], a1 = I.lui[o1], b0 = I.lui[o0 + W], b1 = I.lui[o1 + W];
        const df y0 = y[I.cols[o0]], y1 = y[I.cols[o1]], z0 = y[I.cols[o0 + W]], z1 = y[I.cols[o1 + W]];
        s0 = df_fma_acc(df_neg(a0), y0, s0);
        s1 = df_fma_acc(df_neg(a1), y1, s1);
        s0 = df_fma_acc(df_neg(b0), z0, s0);
        s1 = df_fma_acc(df_neg(b1), z1, s1);
        o0 += 2 * W;
        o1 += 2 * W;
      }
      if (i < mc) {
        const df a0 = I.lui[o0], a1 = I.lui[o1];
        const df y0 = y[I.cols[o0]], y1 = y[I.cols[o1]];
        s0 = df_fma_acc(df_neg(a0), y0, s0);
        s1 = df_fma_acc(df_neg(a1), y1, s1);
      }
      s0 = df_norm(s0);
      s1 = df_norm(s1);
      for (int o = spl >> 1; o > 0; o >>= 1) {
        df t0, t1;
        t0.hi = __shfl_xor_sync(kFull, s0.hi, o);
        t0.lo = __shfl_xor_sync(kFull, s0.lo, o);
        t1.hi = __shfl_xor_sync(kFull, s1.hi, o);
        t1.lo = __shfl_xor_sync(kFull, s1.lo, o);
        s0 = df_add(s0, t0);
        s1 = df_add(s1, t1);
      }
      // the values on every lane, the stores predicated (no branch around the product)
      const df v0 = UPPER ? df_mul(s0, d0) : s0, v1 = UPPER ? df_mul(s1, d1) : s1;
      if (w0) y[k0] = v0;
      if (w1) y[k1] = v1;
    } else {
      int i = 0;
      for (; i + 1 < mc; i += 2) {  // two entries in flight
        const df a0 = I.lui[o0], b0 = I.lui[o0 + W];
        const df y0 = y[I.cols[o0]], z0 = y[I.cols[o0 + W]];
        s0 = df_fma_acc(df_neg(a0), y0, s0);
        s0 = df_fma_acc(df_neg(b0), z0, s0);
        o0 += 2 * W;
      }
      if (i < mc) s0 = df_fma_acc(df_neg(I.lui[o0]), y[I.cols[o0]], s0);
      s0 = df_norm(s0);
      for (int o = spl >> 1; o > 0; o >>= 1) {
        df t0;
        t0.hi = __shfl_xor_sync(kFull, s0.hi, o);
        t0.lo = __shfl_xor_sync(kFull, s0.lo, o);
        s0 = df_add(s0, t0);
      }
      const df v0 = UPPER ? df_mul(s0, d0) : s0;
      if (w0) y[k0] = v0;
    }
  }
}

// Levels l0 .. l1 - 1 of one triangle, each followed by the barrier its flags ask for.
template <int G, bool UPPER>
__device__ __forceinline__ void il_levels(const IlProg &I, df *y, int l0, int l1, int gl, int gid) {
  for (int l = l0; l < l1; ++l) {
    const int4 A = I.rec[2 * l], B = I.rec[2 * l + 1];
    if (!(B.z & 1)) il_level<G, UPPER>(A, B, I, y, gl);
    else if (gl < 32) il_level<32, UPPER>(A, B, I, y, gl);
    if (B.z & 2) __syncwarp();
    else gsync<G>(gid);
  }
}

// L then U solve in place on y; every thread of the group calls it, and it returns after
// a group barrier (y final).
template <int G>
__device__ __forceinline__ void il_solve(const IlProg &I, df *y, int gl, int gid) {
  il_levels<G, false>(I, y, 0, I.nl, gl, gid);
  il_levels<G, true>(I, y, I.nl, I.nl + I.nu, gl, gid);
}

// FP64 value of a double-float (df_to_double_fast), flagging a non-finite result in st;
// the fast path's parts are finite normal numbers, so only the general path can give one.
__device__ __forceinline__ double df_out(df a, int &st) {
  const unsigned hb = __float_as_uint(a.hi), lb = __float_as_uint(a.lo);
  const unsigned he = (hb >> 23) & 0xff, le = (lb >> 23) & 0xff;
  const bool lo_zero = (lb & 0x7fffffff) == 0;
  if (he != 0 && he != 0xff && (lo_zero || (le != 0 && le != 0xff)))
    return f32_widened(hb) + (lo_zero ? 0.0 : f32_widened(lb));
  const double v = df_to_double(a);
  if (!isfinite(v)) st |= KS_NONFINITE;
  return v;
}

// Steps s_begin .. n_steps; the row of step s is out + (s - row_base) * n_out.
// CBREC (trapezoidal rule, not with an adjoint forward pass): a capacitor's rhs value is
// carried from step to step as its companion current source itself, cb_n = 2 (2C/h) v_{n-1}
// - cb_{n-1} (the same recurrence as cb_n = (2C/h) v_{n-1} + i_{n-1} with
// i_{n-1} = (2C/h) v_{n-1} - cb_{n-1}), so the per-step pass that forms the capacitor
// currents after the solve is not needed.  On entry icap holds the capacitor currents
// (s_begin = 1) or, resuming (s_begin > 1), the companion values a previous call left; on
// return it holds the companion values, so a run split into spans is bit-identical to one
// run.
template <int G, int SG = G, bool CBREC = false, bool TAIL = true>
__device__ __forceinline__ int dfd_steps(const DevProg &P, const SProg &S, const df *lu, df *x, const df *cdyn, df *cb,
                                         df *icap, const double *vals, double h, int n_steps, int method, int lag,
                                         double *out, int lnar, int unar, bool int_cvt, int gl, int gid,
                                         WaveTab wt = WaveTab{nullptr, nullptr, 0},
                                         Probe pr = Probe{nullptr, 0, nullptr},
                                         AdjFwd af = AdjFwd{nullptr, 1, 0, 0, nullptr}, int s_begin = 1,
                                         int row_base = 0,
                                         IlProg il = IlProg{nullptr, nullptr, nullptr, nullptr, 0, 0}) {
  const int n_out = pr.n ? pr.n : P.n;
  df loss{0.f, 0.f};  // adjoint forward pass: lane 0 of the group accumulates
  int st = 0;
  // The first tabulated source among this thread's rhs elements has its next value loaded
  // one step ahead, off the step's critical path (others read the table in the step).
  int pf_d = -1;
  size_t pf_base = 0;
  double pf_val = 0.0;
  if (wt.tab && s_begin <= n_steps)
    for (int d = gl; d < P.ndyn; d += G)
      if ((int)((unsigned)S.dyn[d].x >> 24) == KRETS_ELEM_V && wt.row[d] >= 0) {
        pf_d = d;
        pf_base = (size_t)wt.row[d] * wt.stride;
        pf_val = wt.tab[pf_base + s_begin];
        break;
      }
  if (CBREC)  // companion values of the step before s_begin (x and icap are final: the caller synced)
    for (int d = gl; d < P.ncap; d += G) {
      const int4 dd = S.dyn[d];
      cb[d] = s_begin > 1 ? icap[d] : df_sub(df_mul(cdyn[d], df_sub(df_at(x, dd.y), df_at(x, dd.z))), icap[d]);
    }
  for (int s = s_begin; s <= n_steps; ++s) {
    const double t = (double)s * h;
    const double t_src = lag ? (double)(s - 1) * h : t;
    if (af.ck && (s - 1) % af.K == 0) {  // x and icap are final: the previous step's last level synced
      df *ck = af.ck + (size_t)((s - 1) / af.K) * af.ck_words;
      for (int k = gl; k < P.n; k += G) ck[k] = x[k];
      for (int d = gl; d < P.ncap; d += G) ck[P.n + d] = icap[d];
    }
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
        if (d == pf_d) {
          v = df_from_double(pf_val);
          if (s < n_steps) pf_val = wt.tab[pf_base + s + 1];
        } else {
          const int e = dd.x & 0xffffff;
          const krets_element &E = P.el[e];
          const int wr = wt.tab ? wt.row[d] : -1;
          if (wr >= 0) v = df_from_double(wt.tab[(size_t)wr * wt.stride + s]);
          else if (E.wave == KRETS_WAVE_NONE) v = cdyn[d];  // the DC value, split at set-up
          else v = df_from_double(wave_value(E, vals ? vals[e] : E.value, t_src));
        }
      } else if (kind == KRETS_ELEM_I) {
        v = cdyn[d];
      }
      cb[d] = v;
    }
    gsync<G>(gid);  // x (previous solution) fully read: the rhs overwrites it
    for (int k = gl; k < P.n; k += G) {
      df acc{0.f, 0.f};
      for (int u = S.bd_ptr[k]; u < S.bd_ptr[k + 1]; ++u) {
        const int code = S.bd_op[u];
        acc = df_add(acc, (code & 1) ? df_neg(cb[code >> 1]) : cb[code >> 1]);
      }
      x[k] = acc;
    }
    gsync<G>(gid);
    if (il.lui) {
      il_solve<G>(il, x, gl, gid);
    } else {
      df_solve<G, false, SG, TAIL>(S, lu, x, gl, gid, lnar);
      df_solve<G, true, SG, TAIL>(S, lu, x, gl, gid, unar);
    }
    if (!CBREC && method == KRETS_METHOD_TR) {
      for (int d = gl; d < P.ncap; d += G) {
        const int4 dd = S.dyn[d];
        const df vn = df_sub(df_at(x, dd.y), df_at(x, dd.z));
        icap[d] = df_sub(df_mul(cdyn[d], vn), cb[d]);
      }
    }
    if (af.ck) {
      if (gl == 0) loss = df_fma(x[af.out_pos], x[af.out_pos], loss);
      continue;  // no waveform output in the adjoint forward pass
    }
    double *row = out + (size_t)(s - row_base) * n_out;
    for (int j = gl; j < n_out; j += G) {
      const df xv = x[S.qinv[pr.n ? pr.idx[j] : j]];
      const double v = int_cvt ? df_to_double_int(xv) : df_to_double_fast(xv);
      if (!isfinite(v)) st |= KS_NONFINITE;
      __stcs(row + j, v);
    }
    // no barrier: the next step's first phase reads x (final since the last solve level)
    // and writes only this thread's cb / reads this thread's icap entries; its barrier
    // orders every read of x before the gather overwrites it.  Callers synchronise the
    // group after the last step.
  }
  if (CBREC)  // the companion values of the last step, for a caller that keeps the state
    for (int d = gl; d < P.ncap; d += G) icap[d] = cb[d];
  if (af.loss && gl == 0) *af.loss = df_to_double(loss);
  return st;
}

// The interleaved step with a direct right-hand side (pack_lean), for the trapezoidal
// rule with companion currents (as dfd_steps with CBREC) or backward Euler.  Each step
// reads the previous solution in x, writes the right-hand side into b (every element
// writes the rows it feeds, the rows no element feeds are zeroed: no gather pass and one
// barrier less than dfd_steps), solves in place on b and writes the output row from b;
// then x and b swap, so on return x holds the last solution.  lrec / zrow / qinv are the
// staged direct right-hand-side records, unfed rows and output order.  cb holds the
// capacitor companion values (on entry at s_begin = 1 the capacitor currents, resuming
// the companion values a previous call left; on return the companion values).  Every
// value is formed with the same operations in the same order as dfd_steps with the
// gather (a row fed by one element takes 0 + v = v exactly), so the results are
// bit-identical to it.  As an adjoint forward pass (ADJ, af.ck set) it writes no
// waveforms: every K steps the state goes to a checkpoint (x, then the capacitor companion
// values) and sum_n x_n[out_pos]^2 accumulates in double-float into *af.loss.  (A separate
// instantiation, so the waveform step keeps its registers.)
template <int G, bool TR, bool ADJ = false>
__device__ __forceinline__ int dfd_steps_lean(const DevProg &P, const int4 *lrec, const int *zrow, const int *qinv,
                                              const IlProg &I, df *&x, df *&b, const df *cdyn, df *cb,
                                              const double *vals, double h, int n_steps, int lag, double *out, int gl,
                                              int gid, WaveTab wt, Probe pr, int s_begin, int row_base,
                                              bool cvt64, AdjFwd af = AdjFwd{nullptr, 1, 0, 0, nullptr}) {
  const int n_out = pr.n ? pr.n : P.n;
  const int ncap = P.ncap, nlc = P.ncap + P.n_ind, nd = P.ndyn, nz = P.n_zrow;
  int st = 0;
  df loss{0.f, 0.f};  // adjoint forward pass: lane 0 of the group accumulates
  int pf_d = -1;  // first tabulated source of this thread: next value loaded a step ahead
  size_t pf_base = 0;
  double pf_val = 0.0;
  if (wt.tab && s_begin <= n_steps)
    for (int d = nlc + gl; d < nd; d += G)
      if ((int)((unsigned)lrec[d].x >> 24) == KRETS_ELEM_V && wt.row[d] >= 0) {
        pf_d = d;
        pf_base = (size_t)wt.row[d] * wt.stride;
        pf_val = wt.tab[pf_base + s_begin];
        break;
      }
  if (TR && s_begin == 1)  // capacitor currents -> companion values of step 0
    for (int d = gl; d < ncap; d += G) {
      const int4 r = lrec[d];
      cb[d] = df_sub(df_mul(cdyn[d], df_sub(x[r.x], x[r.y])), cb[d]);
    }
  for (int s = s_begin; s <= n_steps; ++s) {
    if (ADJ && (s - 1) % af.K == 0) {  // x final (the last solve level synced); cb: this thread's
      df *ck = af.ck + (size_t)((s - 1) / af.K) * af.ck_words;
      for (int k = gl; k < P.n; k += G) ck[k] = x[k];
      for (int d = gl; d < ncap; d += G) ck[P.n + d] = cb[d];
    }
    for (int d = gl; d < ncap; d += G) {
      const int4 r = lrec[d];
      const df vprev = df_sub(x[r.x], x[r.y]);
      df v;
      if (TR) {
        const df c2{2.f * cdyn[d].hi, 2.f * cdyn[d].lo};  // exact doubling
        v = df_fma(c2, vprev, df_neg(cb[d]));
        cb[d] = v;
      } else {
        v = df_mul(cdyn[d], vprev);
      }
      b[r.z] = v;
      b[r.w] = df_neg(v);
    }
    for (int d = ncap + gl; d < nlc; d += G) {
      const int4 r = lrec[d];
      const df li = df_neg(df_mul(cdyn[d], x[r.z]));
      const df v = TR ? df_sub(li, df_sub(x[r.x], x[r.y])) : li;
      b[r.w >> 1] = (r.w & 1) ? df_neg(v) : v;
    }
    for (int d = nlc + gl; d < nd; d += G) {
      const int4 r = lrec[d];
      df v;
      if ((int)((unsigned)r.x >> 24) == KRETS_ELEM_V) {
        if (d == pf_d) {
          v = df_from_double(pf_val);
          if (s < n_steps) pf_val = wt.tab[pf_base + s + 1];
        } else {
          const int e = r.x & 0xffffff;
          const krets_element &E = P.el[e];
          const int wr = wt.tab ? wt.row[d] : -1;
          if (wr >= 0) v = df_from_double(wt.tab[(size_t)wr * wt.stride + s]);
          else if (E.wave == KRETS_WAVE_NONE) v = cdyn[d];  // the DC value, split at set-up
          else v = df_from_double(wave_value(E, vals ? vals[e] : E.value, lag ? (double)(s - 1) * h : (double)s * h));
        }
      } else {  // current source
        v = cdyn[d];
      }
      b[r.z] = v;
      b[r.w] = df_neg(v);
    }
    for (int i = gl; i < nz; i += G) b[zrow[i]] = df{0.f, 0.f};
    gsync<G>(gid);  // b assembled (and every read of x done)
    il_solve<G>(I, b, gl, gid);
    if (ADJ) {
      if (gl == 0) loss = df_fma(b[af.out_pos], b[af.out_pos], loss);
    } else if (cvt64) {
      double *row = out + (size_t)(s - row_base) * n_out;  // conversions and the add on the FP64 pipe (same value as df_out)
      for (int j = gl; j < n_out; j += G) {
        const double v = df_to_double(b[qinv[pr.n ? pr.idx[j] : j]]);
        if ((__double2hiint(v) & 0x7ff00000) == 0x7ff00000) st |= KS_NONFINITE;
        __stcs(row + j, v);
      }
    } else {
      double *row = out + (size_t)(s - row_base) * n_out;
      for (int j = gl; j < n_out; j += G) __stcs(row + j, df_out(b[qinv[pr.n ? pr.idx[j] : j]], st));
    }
    // no barrier: the next step reads b (final since the last solve level) and writes the
    // other buffer, whose last readers finished before this step's first barrier
    df *t = x;
    x = b;
    b = t;
  }
  if (ADJ && gl == 0) *af.loss = df_to_double(loss);
  return st;
}

// A span of the time steps for one launch, so that a long transient can run as several
// launches (each writing its rows to a staging buffer that is copied out while the next
// launch runs).  Steps s_begin .. n_steps are computed; step s goes to output row
// s - row_base of the instance, whose rows are `stride` values apart (0: (n_steps + 1)
// rows of the output width).  With `state` ([n_inst][n + ncap] double-float: x in
// position space, then the TR capacitor state: currents, or companion values when the
// spans run with CBREC) a span with s_begin > 1 resumes from the state the previous span
// saved, and every span saves its final state there.
struct Span {
  int s_begin, row_base;
  long long stride;
  df *state;
};

// opts bit 0: run narrow levels on one warp; bit 1: integer-only FP64 output conversion;
// bit 2: trapezoidal capacitor history as companion currents (dfd_steps CBREC); bit 3: no
// direct right-hand side (host side); bit 4: the direct-rhs step converts its output on
// the FP64 pipe instead of widening the parts with integer instructions.
// LUG: the factors live in global memory (an L2-resident region per group, lu_glob), the
// rest of the instance in shared memory: about a third of the shared memory per instance,
// so up to 14 instances share an SM (each step's critical path is a chain of level
// barriers; more instances per SM hide it, and fewer waves of instances are needed).
template <int G, bool LUG = false>
__global__ void __launch_bounds__(896) __maxnreg__(LUG ? 64 : 72) k_tran_dfd(DevProg P, KCfg cfg, DfdLay L, const double *values, int n_inst,
                                                     double h, int n_steps, int method, int lag, double *x_out,
                                                     int *inst_status, int *queue, int opts, WaveTab wt, Probe pr,
                                                     AdjFwd af, Span sp, df *lu_glob) {
  extern __shared__ __align__(16) char smem[];
  const int gl = threadIdx.x % G, gid = threadIdx.x / G;
  // With the factors in global memory the solves run from the interleaved program, and only the step-program sections the step reads besides the
  // solves are staged: the row descriptors and columns of the row-descriptor solves stay
  // in global memory.
  constexpr int gi = G == 64 ? 0 : G == 128 ? 1 : 2;
  const bool il = LUG && P.il_ok;
  // the host sized the layout for the direct right-hand-side step (L.lean); a program
  // without one (never launched so) stages nothing and fails its instances
  const bool bad_lean = L.lean && !(il && P.lean_ok);
  const bool lean = L.lean && !bad_lean;
  SProg S = SProg{};
  IlProg I{nullptr, nullptr, nullptr, nullptr, 0, 0};
  const int4 *lrec = nullptr;
  const int *zrow = nullptr, *qinv = nullptr;
  if (il && !bad_lean) {
    // staged: the rhs sections (direct right-hand side, unfed rows and output order; or
    // rhs elements, gather and output order), then the interleaved program
    const int iw0 = P.ip_off[gi][0], iw1 = P.ip_off[gi][3];
    int head;  // words before the interleaved program, 16-byte aligned
    if (lean) {
      const int lw = (4 * P.ndyn + P.n_zrow + 3) & ~3, qw = (P.n + 3) & ~3;
      const int4 *src = reinterpret_cast<const int4 *>(P.iprog + P.lean_off);
      int4 *dst = reinterpret_cast<int4 *>(smem);
      for (int i = threadIdx.x; i < lw / 4; i += blockDim.x) dst[i] = src[i];
      const int4 *qsrc = reinterpret_cast<const int4 *>(P.sprog + P.sp_off[10]);
      for (int i = threadIdx.x; i < qw / 4; i += blockDim.x) dst[lw / 4 + i] = qsrc[i];
      head = lw + qw;
      const int *sm = reinterpret_cast<const int *>(smem);
      lrec = reinterpret_cast<const int4 *>(sm);
      zrow = sm + 4 * P.ndyn;
      qinv = sm + lw;
    } else {
      const int w0 = P.sp_off[7], w1 = P.sp_off[5];
      head = ((w1 - w0) + 3) & ~3;
      const int4 *src = reinterpret_cast<const int4 *>(P.sprog + w0);
      int4 *dst = reinterpret_cast<int4 *>(smem);
      for (int i = threadIdx.x; i < (w1 - w0) / 4; i += blockDim.x) dst[i] = src[i];
      const int *sm = reinterpret_cast<const int *>(smem);
      S.dyn = reinterpret_cast<const int4 *>(sm + (P.sp_off[7] - w0));
      S.bd_ptr = sm + (P.sp_off[8] - w0);
      S.bd_op = sm + (P.sp_off[9] - w0);
      S.qinv = sm + (P.sp_off[10] - w0);
    }
    const int4 *isrc = reinterpret_cast<const int4 *>(P.iprog + iw0);
    int4 *idst = reinterpret_cast<int4 *>(smem + 4 * head);
    for (int i = threadIdx.x; i < (iw1 - iw0) / 4; i += blockDim.x) idst[i] = isrc[i];
    __syncthreads();
    const int *ip = reinterpret_cast<const int *>(smem) + head;
    I.rec = reinterpret_cast<const int4 *>(ip);
    I.rows = ip + (P.ip_off[gi][1] - iw0);
    I.cols = reinterpret_cast<const unsigned short *>(ip + (P.ip_off[gi][2] - iw0));
    I.nl = P.n_il_lrec;
    I.nu = P.n_il_urec;
  } else if (!bad_lean) {
    const int words = P.sp_off[5];  // everything before the residual operators
    const int4 *src = reinterpret_cast<const int4 *>(P.sprog);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int i = threadIdx.x; i < words / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    S = sprog_view(P, reinterpret_cast<const int *>(smem));
  }
  int lnar = -1, unar = -1;  // narrow-level split points (see df_solve)
  if ((opts & 1) && !il) {
    lnar = S.nlev;
    unar = 0;
    while (lnar > 1 && S.lev_ptr[lnar] - S.lev_ptr[lnar - 1] <= 64) --lnar;
    while (unar < S.nulev && S.ulev_ptr[unar + 1] - S.ulev_ptr[unar] <= 64) ++unar;
  }
  const bool int_cvt = (opts & 2) != 0;
  // bit 2: trapezoidal capacitor history carried as the companion current (the gather
  // step keeps currents in an adjoint forward pass: its checkpoints hold currents)
  const bool cbrec = (opts & 4) != 0 && method == KRETS_METHOD_TR && !af.ck;
  // the direct right-hand-side step runs TR with companion currents (its adjoint
  // checkpoints hold companion values), or BE
  const bool tr_lean = (opts & 4) != 0 && method == KRETS_METHOD_TR;
  const bool lean_ok = lean && (tr_lean || method == KRETS_METHOD_BE);
  char *base = smem + L.sprog_bytes + (size_t)gid * L.bytes;
  // global-memory factors: per group the CSR factors, then (interleaved solves) their
  // interleaved copy
  const size_t greg = (size_t)P.nnz_lu + (il ? (size_t)P.il_slots[gi] : 0);
  df *lu = LUG ? lu_glob + (size_t)(blockIdx.x * (blockDim.x / G) + gid) * greg
               : reinterpret_cast<df *>(base + L.lu);
  if (il) I.lui = lu + P.nnz_lu;
  double *lu64 = reinterpret_cast<double *>(lu);  // same bytes, set-up only
  df *x = reinterpret_cast<df *>(base + L.x);
  df *cdyn = reinterpret_cast<df *>(base + L.cdyn);
  df *cb = reinterpret_cast<df *>(base + L.cb);
  df *icap = reinterpret_cast<df *>(base + L.icap);
  int *slot = reinterpret_cast<int *>(base + L.slot);
  double *coef64 = reinterpret_cast<double *>(base + L.coef64);  // set-up only
  const size_t stride = sp.stride ? (size_t)sp.stride : (size_t)(n_steps + 1) * (pr.n ? pr.n : P.n);
  const int ns = P.n + P.ncap;  // state words of an instance
  while (true) {
    if (gl == 0) slot[0] = atomicAdd(queue, 1);
    gsync<G>(gid);
    const int inst = slot[0];
    gsync<G>(gid);
    if (inst >= n_inst) break;
    const double *vals = values ? values + (size_t)inst * P.ne : nullptr;
    double *out = x_out ? x_out + (size_t)inst * stride : nullptr;
    const double *op = pr.x0 ? pr.x0 + (size_t)inst * P.n : out;  // operating point (none: x_0 = 0)
    int st = dfd_setup<G>(P, S, vals, h, method, lu, lu64, coef64, cdyn, gl, gid);
    if (il) {  // the factors in the interleaved order of the solves (zero pads)
      gsync<G>(gid);
      df *lui = lu + P.nnz_lu;
      const int *map = P.imap + P.imap_off[gi];
      for (int q = gl; q < P.il_slots[gi]; q += G) {
        const int m = map[q];
        lui[q] = m >= 0 ? lu[m] : df{0.f, 0.f};
      }
    }
    df *state = sp.state ? sp.state + (size_t)inst * ns : nullptr;
    if (state && sp.s_begin > 1) {  // resume: x and the TR currents where the previous span stopped
      for (int k = gl; k < P.n; k += G) x[k] = state[k];
      for (int d = gl; d < P.ncap; d += G) icap[d] = state[P.n + d];
    } else {
      for (int k = gl; k < P.n; k += G) x[k] = op ? df_from_double(op[P.q[k]]) : df{0.f, 0.f};
      for (int j = gl; j < pr.n; j += G) out[j] = op[pr.idx[j]];  // probe row 0
      for (int d = gl; d < P.ncap; d += G) icap[d] = df{0.f, 0.f};
    }
    if (lean && gl == 0) {  // ground reads zero in both state buffers
      x[P.n] = df{0.f, 0.f};
      cb[P.n] = df{0.f, 0.f};
    }
    if (bad_lean || (lean && !lean_ok)) st |= KS_NOTIMPL;
    AdjFwd a = af;
    if (af.ck) {
      a.ck = af.ck + (size_t)inst * ((n_steps + af.K - 1) / af.K) * af.ck_words;
      a.loss = af.loss + inst;
    }
    const bool fatal = gany<G>((st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) != 0, gid);
    df *xfin = x;  // where the last solution is
    if (!fatal && lean) {
      df *xs = x, *bs = cb;
      const bool c64 = (opts & 16) != 0;
      if (a.ck) {
        if (tr_lean)
          st |= dfd_steps_lean<G, true, true>(P, lrec, zrow, qinv, I, xs, bs, cdyn, icap, vals, h, n_steps, lag, out,
                                              gl, gid, wt, pr, sp.s_begin, sp.row_base, c64, a);
        else
          st |= dfd_steps_lean<G, false, true>(P, lrec, zrow, qinv, I, xs, bs, cdyn, icap, vals, h, n_steps, lag,
                                               out, gl, gid, wt, pr, sp.s_begin, sp.row_base, c64, a);
      } else if (tr_lean) {
        st |= dfd_steps_lean<G, true>(P, lrec, zrow, qinv, I, xs, bs, cdyn, icap, vals, h, n_steps, lag, out, gl,
                                      gid, wt, pr, sp.s_begin, sp.row_base, c64);
      } else {
        st |= dfd_steps_lean<G, false>(P, lrec, zrow, qinv, I, xs, bs, cdyn, icap, vals, h, n_steps, lag, out, gl,
                                       gid, wt, pr, sp.s_begin, sp.row_base, c64);
      }
      xfin = xs;
    } else if (!fatal) {
      if (cbrec)
        st |= dfd_steps<G, G, true, false>(P, S, lu, x, cdyn, cb, icap, vals, h, n_steps, method, lag, out, lnar, unar,
                                    int_cvt, gl, gid, wt, pr, a, sp.s_begin, sp.row_base, I);
      else
        st |= dfd_steps<G, G, false, false>(P, S, lu, x, cdyn, cb, icap, vals, h, n_steps, method, lag, out, lnar,
                                            unar, int_cvt, gl, gid, wt, pr, a, sp.s_begin, sp.row_base, I);
    }
    if (state) {  // the last step's solution level and TR currents are final once the group syncs
      gsync<G>(gid);
      for (int k = gl; k < P.n; k += G) state[k] = xfin[k];
      for (int d = gl; d < P.ncap; d += G) state[P.n + d] = icap[d];
    }
    if (gl == 0) slot[1] = 0;
    gsync<G>(gid);
    if (st) atomicOr(&slot[1], st);
    gsync<G>(gid);
    // statuses accumulate over the spans of one transient (the caller zeroes them first)
    if (gl == 0 && inst_status) inst_status[inst] |= slot[1];
  }
}

}  // namespace krets
