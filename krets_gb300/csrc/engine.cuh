// Device engine: the per-instance MNA operations, written once and used by every kernel
// (plain single-instance form and batched persistent forms).
//
// One CTA processes one instance.  All operations walk the static program built by the
// host symbolic pass (symbolic.cpp):
//   stamp   - deterministic segmented sums of element contributions into each matrix /
//             rhs entry, in the reference's emission order (solver.rs:59-70 semantics,
//             no atomics)
//   factor  - up-looking (IKJ) LU, rows of one level in parallel, static pivots
//   lsolve  - unit-lower solve, level by level
//   usolve  - upper solve, level by level (reverse dependency levels)
// Arrays passed in may live in shared or global memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "krets_gpu.h"

namespace krets {

// ------------------------------------------------------------------ complex scalar
template <typename R>
struct cx {
  R re, im;
  __host__ __device__ cx() : re(0), im(0) {}
  __host__ __device__ cx(R r) : re(r), im(0) {}
  __host__ __device__ cx(R r, R i) : re(r), im(i) {}
  template <typename S>
  __host__ __device__ explicit cx(const cx<S> &o) : re((R)o.re), im((R)o.im) {}
};
template <typename R> __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> __device__ __forceinline__ cx<R> operator-(cx<R> a) { return {-a.re, -a.im}; }
template <typename R> __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R> __device__ __forceinline__ cx<R> operator/(cx<R> a, cx<R> b) {
  // Smith's algorithm (robust to large |b| components)
  if (fabs(b.re) >= fabs(b.im)) {
    R r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  R r = b.re / b.im, d = b.re * r + b.im;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

// 1 / x, correctly rounded: the reciprocal instructions (rcp.rn) round to nearest as the
// division 1.0 / x does, so the value is the same bits with fewer FP64 instructions (the
// FP64 pipe issues at 1/64 of the FP32 rate on this GPU).  Complex values divide.
__device__ __forceinline__ double recip(double x) { return __drcp_rn(x); }
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
template <typename R>
__device__ __forceinline__ cx<R> recip(cx<R> x) { return cx<R>(R(1)) / x; }

template <typename T> struct scal;
template <> struct scal<double> {
  using real = double;
  __device__ static double mag(double x) { return fabs(x); }
  __device__ static bool finite(double x) { return isfinite(x); }
  __device__ static double neg(double x) { return -x; }
};
template <> struct scal<float> {
  using real = float;
  __device__ static float mag(float x) { return fabsf(x); }
  __device__ static bool finite(float x) { return isfinite(x); }
};
template <> struct scal<cx<double>> {
  using real = double;
  __device__ static double mag(cx<double> x) { return hypot(x.re, x.im); }
  __device__ static bool finite(cx<double> x) { return isfinite(x.re) && isfinite(x.im); }
};
template <> struct scal<cx<float>> {
  using real = float;
  __device__ static float mag(cx<float> x) { return hypotf(x.re, x.im); }
  __device__ static bool finite(cx<float> x) { return isfinite(x.re) && isfinite(x.im); }
};

// ------------------------------------------------------------------ program view
struct DevProg {
  int n, ne, nnz_a, nnz_lu, nlev, nulev, mode, method;
  const int *q;          // [n]  position -> unknown
  const int *lu_rowptr;  // [n+1]
  const int *lu_col;     // [nnz_lu]
  const int *lu_diag;    // [n]
  const int *lu_src;     // [nnz_lu] A entry feeding this slot, or -1 (fill)
  const int *a_rowptr;   // [n+1]
  const int *a_col;      // [nnz_a]
  const int *a_cptr;     // [nnz_a+1]
  const int *a_contrib;  // packed slot<<2 | unit<<1 | neg (slot = coefficient slot)
  const int *b_cptr;     // [n+1]
  const int *b_contrib;  // packed elem<<1 | neg
  const int *piv_ptr;    // [n+1]
  const int4 *piv;       // {slot, j, upd_begin, upd_end}
  const int2 *upd;       // {dst, src}
  const int *lev_ptr, *lev_rows, *ulev_ptr, *ulev_rows;
  const int4 *el_pos;    // p, m, b, g in position space
  const int *is_cur;     // [n] 1 when the unknown at this position is a branch current
  const krets_element *el;
  const int *xslot;      // [ne] first extra coefficient slot of the element, or -1
  int n_coef;            // coefficient slots (ne + extra slots)
  int nonlinear;         // any diode / MOSFET / BJT among the stamped elements
  // step program (warp engine)
  const int *qinv;       // [n] unknown -> position
  const int4 *ldesc;     // [n] L-level-ordered {row, first, diag, end}
  const int4 *udesc;     // [n] U-level-ordered {row, first, diag, end}
  const int *res_ptr;    // [n+1]
  const int2 *res_op;    // {col position, packed contribution}
  const int *dyn_e;      // [ndyn] capacitors first
  const int *bd_ptr;     // [n+1]
  const int *bd_op;      // dyn << 1 | neg
  int ndyn, ncap, n_resop;
  // compact step program (global copy; the warp engine stages it in shared memory)
  const int *sprog;
  int sp_off[16];
  int n_bchunk, n_brow;  // border of the dense trailing block: chunks, rows
  int sprog_ok;
  // transposed-solve program (adjoint)
  const int *tprog;
  int tp_off[8];
  int n_utlev, n_ltlev;
  const int *prow;  // [n] position -> pivot row (unknown index of the row)
  int tail0, tail_m;  // dense trailing block of the LU (tail_m = 0: none)
  // interleaved solves (Program::iprog; layouts for 64 and 128-thread groups)
  const int *iprog, *imap;
  int ip_off[3][4], il_slots[3], imap_off[3], n_il_lrec, n_il_urec, il_ok;  // layouts: G = 64, 128, 32
  int lean_off, n_zrow, n_ind, lean_ok;  // direct right-hand side (in iprog)
};

// status bits written by the engine
#define KS_SINGULAR 1
#define KS_MAXITER 2
#define KS_NONFINITE 4
#define KS_NOTIMPL 8
#define KS_STALL 16
#define KS_GROWTH 32

static constexpr double kPiD = 3.14159265358979323846;
static constexpr double kVtD = 1.380649e-23 * 300.0 / 1.602176634e-19;
static constexpr double kDblMax = 1.7976931348623157e308;

// ------------------------------------------------------------------ waveforms
// Pulse and sine sources, voltage_source.rs:52-93 (same operation order; fmod and the
// divisions are IEEE-exact, so the pulse value is bit-identical to the reference's).
__device__ __forceinline__ double wave_value(const krets_element &E, double value, double t) {
  if (E.wave == KRETS_WAVE_PULSE) {
    const double *w = E.wp;
    double v1 = w[0], v2 = w[1], td = w[2], tr = w[3], tf = w[4], pw = w[5], per = w[6];
    if (t < td) return v1;
    double tt = fmod(t - td, per);
    if (tt < tr) return v1 + (v2 - v1) * (tt / tr);
    if (tt < tr + pw) return v2;
    if (tt < tr + pw + tf) return v2 + (v1 - v2) * ((tt - tr - pw) / tf);
    return v1;
  }
  if (E.wave == KRETS_WAVE_SIN) {
    const double *w = E.wp;
    if (t < w[3]) return w[0];
    double omega = 2.0 * kPiD * w[2];
    double ph = w[5] * (kPiD / 180.0);
    double tt = t - w[3];
    return w[0] + w[1] * exp(-w[4] * tt) * sin(omega * tt + ph);
  }
  return value;
}

// Diode linearisation (diode.rs:26-70): V(+) defaults to 0.5 V and V(-) to 0 when the
// solution map lacks them (empty map on the first OP iteration, or a ground terminal).
__device__ __forceinline__ void diode_lin(const krets_element &E, double is, int4 pos, const double *guess,
                                          bool empty, double &g, double &ieq) {
  double vp = (!empty && pos.x >= 0) ? guess[pos.x] : 0.5;
  double vm = (!empty && pos.y >= 0) ? guess[pos.y] : 0.0;
  double vd = vp - vm;
  double n = E.wp[0];
  double vc = n * kVtD * log(kDblMax * n * kVtD / is);
  double vl = vd;  // f64::clamp(-vc, vc); NaN stays NaN
  if (vd < -vc) vl = -vc;
  if (vd > vc) vl = vc;
  double nvt = n * kVtD;
  g = (is / nvt) * exp(vl / nvt);
  double cur = is * (exp(vl / nvt) - 1.0);
  ieq = cur - g * vd;
}

// NMOS level 1 (nmosfet.rs:51-103) at the Newton guess: V(gate), V(source), V(drain)
// default to 0 when the solution map lacks them (stampable.rs:825-833); wp = {vto, kp,
// lambda, w, l}.  Region tests and products in the reference's order.
__device__ __forceinline__ void nmos_lin(const krets_element &E, int4 pos, const double *guess, bool empty,
                                         double &gm, double &gds, double &ieq) {
  const double vg = (!empty && pos.w >= 0) ? guess[pos.w] : 0.0;
  const double vs = (!empty && pos.y >= 0) ? guess[pos.y] : 0.0;
  const double vd = (!empty && pos.x >= 0) ? guess[pos.x] : 0.0;
  const double vgs = vg - vs, vds = vd - vs;
  const double vth = E.wp[0], beta = E.wp[1] * (E.wp[3] / E.wp[4]), lambda = E.wp[2];
  double id;
  if (vgs <= vth) {
    gm = 0.0; gds = 0.0; id = 0.0;
  } else if (vds >= 0.0 && vds <= (vgs - vth)) {  // linear region
    gm = beta * vds;
    gds = beta * (vgs - vth - vds);
    id = beta * ((vgs - vth) * vds - (vds * vds / 2.0));
  } else if (vds >= (vgs - vth) && vds >= 0.0) {  // saturation
    const double ov = vgs - vth;
    gm = beta * ov * (1.0 + lambda * vds);
    gds = (beta / 2.0) * lambda * (ov * ov);
    id = (beta / 2.0) * (ov * ov) * (1.0 + lambda * vds);
  } else {
    gm = 0.0; gds = 0.0; id = 0.0;
  }
  ieq = id - gds * vds - gm * vgs;  // stampable.rs:891
}

struct PassCtx {
  int mode, method;
  double h, freq;
  double t_src;          // time at which transient sources are evaluated
  const double *guess;   // Newton guess (position space)
  bool guess_empty;      // the reference's map is empty (first OP iteration)
  const double *prev;    // previous time step (position space)
  const double *icap;    // TR capacitor currents at t_n, per element
};

// Per-element coefficients of one stamping pass: ca = matrix coefficient (real part in
// ca_re, imaginary in ca_im), cb = rhs coefficient.  Expressions and operation order follow
// stampable.rs so the summed entries match the reference's bit for bit (up to exp/sin).
// x0 / x1: the values of the element's extra slots (resolved NMOS: g_ds, g_m).
__device__ __forceinline__ void elem_coefs(const krets_element &E, int e, int4 pos, double val,
                                           const PassCtx &c, double &ca_re, double &ca_im, double &cb,
                                           double &x0, double &x1, int &err) {
  ca_re = 0.0;
  ca_im = 0.0;
  cb = 0.0;
  x0 = 0.0;
  x1 = 0.0;
  switch (E.kind) {
    case KRETS_ELEM_R:
      ca_re = (E.flags & KRETS_FLAG_G2) ? val : recip(val);
      break;
    case KRETS_ELEM_C:
      if (c.mode == 1) {
        ca_im = 2.0 * kPiD * c.freq * val;
      } else if (c.mode == 2) {
        double vp = pos.x >= 0 ? c.prev[pos.x] : 0.0, vm = pos.y >= 0 ? c.prev[pos.y] : 0.0;
        double vprev = vp - vm;
        if (c.method == KRETS_METHOD_TR) {
          ca_re = 2.0 * val / c.h;
          cb = ca_re * vprev + c.icap[e];
        } else {
          ca_re = val / c.h;
          double ieq = -(val / c.h) * vprev;
          cb = -ieq;
        }
      }
      break;
    case KRETS_ELEM_L:
      if (c.mode == 1) {
        ca_im = 2.0 * kPiD * c.freq * val;
      } else if (c.mode == 2) {
        double iprev = pos.z >= 0 ? c.prev[pos.z] : 0.0;
        if (c.method == KRETS_METHOD_TR) {
          double lh = 2.0 * val / c.h;
          double vl = (pos.x >= 0 ? c.prev[pos.x] : 0.0) - (pos.y >= 0 ? c.prev[pos.y] : 0.0);
          ca_re = lh;
          cb = -lh * iprev - vl;
        } else {
          ca_re = val / c.h;
          cb = -(val / c.h) * iprev;
        }
      }
      break;
    case KRETS_ELEM_V:
      cb = c.mode == 0 ? val : (c.mode == 1 ? E.ac : wave_value(E, val, c.t_src));
      break;
    case KRETS_ELEM_I:
      cb = val;
      break;
    case KRETS_ELEM_D: {
      double g, ieq;
      diode_lin(E, val, pos, c.guess, c.guess_empty, g, ieq);
      ca_re = g;
      cb = ieq;
      break;
    }
    case KRETS_ELEM_M:
      if (c.mode == 1) {
        err |= KS_NOTIMPL;
      } else if (E.flags & KRETS_FLAG_NMOS_RESOLVED) {
        double gm, gds, ieq;
        nmos_lin(E, pos, c.guess, c.guess_empty, gm, gds, ieq);
        ca_re = gds + gm;
        x0 = gds;
        x1 = gm;
        cb = ieq;
      }
      break;
    default:
      err |= KS_NOTIMPL;
  }
}

// ------------------------------------------------------------------ block helpers
__device__ __forceinline__ double block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// The same over floats (red: the same 32-double scratch).
__device__ __forceinline__ float block_maxf(float v, double *red) {
  float *rf = reinterpret_cast<float *>(red);
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) rf[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = threadIdx.x < (blockDim.x >> 5) ? rf[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (threadIdx.x == 0) rf[32] = t;
  }
  __syncthreads();
  const float r = rf[32];
  __syncthreads();
  return r;
}

// ------------------------------------------------------------------ stamping
// Sum of one A entry's contributions (emission order).
template <typename T>
__device__ __forceinline__ T sum_entry(const DevProg &P, int t, const double *ca_re, const double *ca_im);

template <>
__device__ __forceinline__ double sum_entry<double>(const DevProg &P, int t, const double *ca_re, const double *) {
  double s = 0.0;
  for (int u = P.a_cptr[t]; u < P.a_cptr[t + 1]; ++u) {
    int code = P.a_contrib[u];
    double v = (code & 2) ? 1.0 : ca_re[code >> 2];
    s += (code & 1) ? -v : v;
  }
  return s;
}

template <>
__device__ __forceinline__ cx<double> sum_entry<cx<double>>(const DevProg &P, int t, const double *ca_re,
                                                            const double *ca_im) {
  double sr = 0.0, si = 0.0;
  for (int u = P.a_cptr[t]; u < P.a_cptr[t + 1]; ++u) {
    int code = P.a_contrib[u];
    double vr = (code & 2) ? 1.0 : ca_re[code >> 2];
    double vi = (code & 2) ? 0.0 : ca_im[code >> 2];
    if (code & 1) { vr = -vr; vi = -vi; }
    sr += vr;
    si += vi;
  }
  return cx<double>(sr, si);
}

// rhs row k (position space)
__device__ __forceinline__ double sum_rhs(const DevProg &P, int k, const double *cb) {
  double s = 0.0;
  for (int u = P.b_cptr[k]; u < P.b_cptr[k + 1]; ++u) {
    int code = P.b_contrib[u];
    double v = cb[code >> 1];
    s += (code & 1) ? -v : v;
  }
  return s;
}

// ------------------------------------------------------------------ factor / solves
// The arrays the factorisation and the two solves read.  They come from the program in
// global memory (fac_view), or from copies in shared memory that a single-CTA solve makes
// first (k_op, k_dc_sweep): the factorisation's deepest rows then wait on shared-memory
// rather than L2 latency at every pivot.
struct FacView {
  int nlev, nulev;
  const int *lev_ptr, *lev_rows, *piv_ptr, *lu_diag, *lu_rowptr, *lu_col, *ulev_ptr, *ulev_rows;
  const int4 *piv;
  const int2 *upd;
};

__device__ __forceinline__ FacView fac_view(const DevProg &P) {
  return FacView{P.nlev,      P.nulev,     P.lev_ptr, P.lev_rows, P.piv_ptr, P.lu_diag,
                 P.lu_rowptr, P.lu_col,    P.ulev_ptr, P.ulev_rows, P.piv,     P.upd};
}

// In-place static-pivot LU of lu[] (values in position space).  Returns status bits.
// Status bits are OR-ed into *status (shared or global) by the threads that see them.
// The diagonal slots hold the reciprocal pivots 1/u_kk on exit (usolve multiplies by
// them): a row's pivots then cost one multiply each instead of a division, which in FP64
// is a chain of about ten instructions on a pipe that issues at 1/64 of the FP32 rate,
// and a factorisation's deepest rows run one pivot after another.  Rows of one level read
// only the diagonals of earlier levels, so a row inverts its own pivot when it finishes.
// Levels with at most one row per warp (the deepest ones) take a warp per row: the
// pivots still run one after another, but a pivot's updates are spread over the lanes
// (one warp instruction for all of them instead of one each on a single thread).  The
// operations are the same (FP64: the same bits; the compiler may contract a complex
// product differently, a last-bit difference).
template <typename T>
__device__ __forceinline__ void factor_v(const FacView &F, T *lu, int *status) {
  int bad = 0;
  const int nwarp = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l = 0; l < F.nlev; ++l) {
    int r0 = F.lev_ptr[l], r1 = F.lev_ptr[l + 1];
    if (r1 - r0 <= nwarp) {
      if (warp < r1 - r0) {
        const int k = F.lev_rows[r0 + warp];
        for (int pi = F.piv_ptr[k]; pi < F.piv_ptr[k + 1]; ++pi) {
          const int4 pv = F.piv[pi];
          const T l_kj = lu[pv.x] * lu[F.lu_diag[pv.y]];
          __syncwarp();  // every lane has read the entry before it is overwritten
          for (int u = pv.z + lane; u < pv.w; u += 32) {
            const int2 d = F.upd[u];
            lu[d.x] = lu[d.x] - l_kj * lu[d.y];
          }
          if (lane == 0) lu[pv.x] = l_kj;
          __syncwarp();  // the row's new values before the next pivot reads them
        }
        if (lane == 0) {
          const int dg = F.lu_diag[k];
          T dk = lu[dg];
          if (!(scal<T>::mag(dk) > 0)) bad |= KS_SINGULAR;
          else if (!scal<T>::finite(dk)) bad |= KS_NONFINITE;
          lu[dg] = recip(dk);
        }
      }
      __syncthreads();
      continue;
    }
    for (int t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
      int k = F.lev_rows[t];
      // A row's pivots run one after another.  What a pivot needs besides its own entry —
      // its record, the reciprocal pivot of row j (final: an earlier level) and its first
      // update pair — is loaded one pivot ahead, before the stores that the compiler must
      // otherwise assume they alias, so each step of the chain waits only on its entry.
      const int p0 = F.piv_ptr[k], p1 = F.piv_ptr[k + 1];
      int4 pv = p0 < p1 ? F.piv[p0] : make_int4(0, 0, 0, 0);
      T rd = p0 < p1 ? lu[F.lu_diag[pv.y]] : T(0);
      int2 d = p0 < p1 && pv.z < pv.w ? F.upd[pv.z] : make_int2(0, 0);
      for (int pi = p0; pi < p1; ++pi) {
        int4 pn = pv;
        T rn = rd;
        int2 dn0 = d;
        if (pi + 1 < p1) {
          pn = F.piv[pi + 1];
          rn = lu[F.lu_diag[pn.y]];
          if (pn.z < pn.w) dn0 = F.upd[pn.z];
        }
        const T l_kj = lu[pv.x] * rd;
        lu[pv.x] = l_kj;
        for (int u = pv.z; u < pv.w; ++u) {
          const int2 dn = u + 1 < pv.w ? F.upd[u + 1] : d;
          lu[d.x] = lu[d.x] - l_kj * lu[d.y];
          d = dn;
        }
        pv = pn;
        rd = rn;
        d = dn0;
      }
      const int dg = F.lu_diag[k];
      T dk = lu[dg];
      if (!(scal<T>::mag(dk) > 0)) bad |= KS_SINGULAR;
      else if (!scal<T>::finite(dk)) bad |= KS_NONFINITE;
      lu[dg] = recip(dk);
    }
    __syncthreads();
  }
  if (bad) atomicOr(status, bad);
  __syncthreads();
}

template <typename T, typename V>
__device__ __forceinline__ void lsolve_v(const FacView &F, const T *lu, V *y) {
  for (int l = 1; l < F.nlev; ++l) {  // level 0 rows have no L entries
    int r0 = F.lev_ptr[l], r1 = F.lev_ptr[l + 1];
    for (int t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
      int k = F.lev_rows[t];
      V s = y[k];
      for (int u = F.lu_rowptr[k]; u < F.lu_diag[k]; ++u) s = s - V(lu[u]) * y[F.lu_col[u]];
      y[k] = s;
    }
    __syncthreads();
  }
}

template <typename T, typename V>
__device__ __forceinline__ void usolve_v(const FacView &F, const T *lu, V *y) {
  for (int l = 0; l < F.nulev; ++l) {
    int r0 = F.ulev_ptr[l], r1 = F.ulev_ptr[l + 1];
    for (int t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
      int k = F.ulev_rows[t];
      V s = y[k];
      int dg = F.lu_diag[k];
      for (int u = dg + 1; u < F.lu_rowptr[k + 1]; ++u) s = s - V(lu[u]) * y[F.lu_col[u]];
      y[k] = s * V(lu[dg]);  // reciprocal pivot
    }
    __syncthreads();
  }
}

template <typename T>
__device__ void factor(const DevProg &P, T *lu, int *status) {
  factor_v<T>(fac_view(P), lu, status);
}

template <typename T, typename V>
__device__ void lsolve(const DevProg &P, const T *lu, V *y) {
  lsolve_v<T, V>(fac_view(P), lu, y);
}

template <typename T, typename V>
__device__ void usolve(const DevProg &P, const T *lu, V *y) {
  usolve_v<T, V>(fac_view(P), lu, y);
}

}  // namespace krets
