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

namespace krets {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Shared-memory view of the compact step program (layout: pack_step_program()).
struct SProg {
  const int *lev_ptr, *ulev_ptr;
  const int2 *ldesc, *udesc;
  const unsigned short *lu_col;
  const int *res_ptr, *res_op;
  const int4 *dyn;
  const int *bd_ptr, *bd_op, *qinv;
  int nlev, nulev;
};

__device__ __forceinline__ SProg sprog_view(const DevProg &P, const int *sp) {
  SProg S;
  S.lev_ptr = sp + P.sp_off[0];
  S.ulev_ptr = sp + P.sp_off[1];
  S.ldesc = reinterpret_cast<const int2 *>(sp + P.sp_off[2]);
  S.udesc = reinterpret_cast<const int2 *>(sp + P.sp_off[3]);
  S.lu_col = reinterpret_cast<const unsigned short *>(sp + P.sp_off[4]);
  S.res_ptr = sp + P.sp_off[5];
  S.res_op = sp + P.sp_off[6];
  S.dyn = reinterpret_cast<const int4 *>(sp + P.sp_off[7]);
  S.bd_ptr = sp + P.sp_off[8];
  S.bd_op = sp + P.sp_off[9];
  S.qinv = sp + P.sp_off[10];
  S.nlev = P.nlev;
  S.nulev = P.nulev;
  return S;
}

// Unit-lower solve, level by level (level 0 rows have no L entries).
template <typename T, typename V>
__device__ __forceinline__ void s_lsolve(const SProg &S, const T *lu, V *y, int lane) {
  for (int l = 1; l < S.nlev; ++l) {
    const int r0 = S.lev_ptr[l], r1 = S.lev_ptr[l + 1];
    for (int t = r0 + lane; t < r1; t += 32) {
      const int2 d = S.ldesc[t];
      const int k = d.x & 0xffff, cnt = (int)((unsigned)d.x >> 16);
      V s = y[k];
      for (int j = 0; j < cnt; ++j) s -= V(lu[d.y + j]) * y[S.lu_col[d.y + j]];
      y[k] = s;
    }
    __syncwarp();
  }
}

// Upper solve; the diagonal slots hold reciprocals (see w_factor).
template <typename T, typename V>
__device__ __forceinline__ void s_usolve(const SProg &S, const T *lu, V *y, int lane) {
  for (int l = 0; l < S.nulev; ++l) {
    const int r0 = S.ulev_ptr[l], r1 = S.ulev_ptr[l + 1];
    for (int t = r0 + lane; t < r1; t += 32) {
      const int2 d = S.udesc[t];
      const int k = d.x & 0xffff, cnt = (int)((unsigned)d.x >> 16);
      V s = y[k];
      for (int j = 1; j <= cnt; ++j) s -= V(lu[d.y + j]) * y[S.lu_col[d.y + j]];
      y[k] = s * V(lu[d.y]);
    }
    __syncwarp();
  }
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
    lu[s] = T(1) / lu[s];
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
      case KRETS_ELEM_R: c = (E.flags & KRETS_FLAG_G2) ? val : 1.0 / val; break;
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
      for (int u = S.res_ptr[k]; u < S.res_ptr[k + 1]; ++u) {
        const int op = S.res_op[u];
        const int slot = (int)((unsigned)op >> 16);
        const double a = slot ? coef[slot - 1] : 1.0;
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
__global__ void __launch_bounds__(256) k_tran_warp(DevProg P, KCfg cfg, WarpLay L, const double *values, int n_inst,
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
