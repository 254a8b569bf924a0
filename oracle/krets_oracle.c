/*
 * krets CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, f64 restatement of the reference MNA solve path (prokie/krets,
 * crates/krets-solver), used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg as the checker.  The product (krets_gb300/, libkrets_gpu.so) never
 * links or calls it.
 *
 * What it restates, with the reference file:line each part follows:
 *   - element stamps, emission order and values:   src/stampable.rs:202-1050
 *       resistor 202-317, capacitor 360-506, current source 508-585, diode 587-674,
 *       inductor 676-817, NMOS 819-922 (bare-name index lookups: stamps nothing),
 *       voltage source 960-1050; default transient stamps = DC stamps 106-136
 *   - duplicate summation in emission order:        src/solver.rs:59-70
 *   - Newton convergence test (I-prefixed keys use the current tolerance,
 *     everything else incl. "time"/"step" the voltage tolerance):  src/solver.rs:76-104
 *   - OP (capacitors filtered out, one pass when linear):   src/solver/op.rs:15-86
 *   - DC sweep (warm start, "step" key, restore value):     src/solver/dc.rs:14-124
 *   - AC (OP first, skip f <= 0, complex stamps):           src/solver/ac.rs:17-109
 *   - transient BE with the Newton guess cloned from the previous step, so
 *     sources are evaluated at t_{n-1} in the first Newton iteration:
 *                                                           src/solver/transient.rs:14-114
 *   - PULSE / SIN waveforms:        crates/krets-parser/src/elements/voltage_source.rs:52-93,244-252
 *   - diode linearisation (0.5 V guess when V(+) is absent, clamp): elements/diode.rs:26-70
 * The sparse LU stands in for faer 0.23.2 (see ko_lu_impl.h).
 *
 * Extensions the reference does not have (its own oracle here): trapezoidal companion
 * models (C: G=2C/h, I_hist=G v_n + i_C,n; L: branch diagonal -2L/h, rhs
 * -(2L/h) i_n - v_L,n) and a no-lag source switch.
 */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define KO_OK 0
#define KO_SINGULAR 1
#define KO_MAXITER 2
#define KO_NOTFOUND 3
#define KO_BADELEM 4
#define KO_NOTIMPL 5
#define KO_NOMEM 6
#define KO_NONFINITE 7

enum { K_R = 1, K_C = 2, K_L = 3, K_V = 4, K_I = 5, K_D = 6, K_M = 7, K_Q = 8 };
enum { W_NONE = 0, W_PULSE = 1, W_SIN = 2 };
#define F_G2 1
#define F_NMOS_RESOLVED 2 /* NMOS nodes looked up as V(<node>) (the reference: bare names) */

/* Same 104-byte layout as the element record of the product's C ABI. */
typedef struct ko_elem {
  int32_t kind, p, m, b, g, flags, wave, pad;
  double value, ac, wp[7];
} ko_elem;

typedef struct ko_cfg {
  double reltol, iabstol, vabstol;
  int32_t maxiter;
  int32_t faithful; /* 1: re-stamp + refactor every Newton iteration and step (reference cost) */
} ko_cfg;

static const double KO_PI = 3.14159265358979323846;
static const double KO_VT = 1.380649e-23 * 300.0 / 1.602176634e-19;

/* ---------------------------------------------------------------- sparse LU */
#define KO_T double
#define KO_ABS(x) fabs(x)
#define KO_SFX d
#include "ko_lu_impl.h"
#undef KO_T
#undef KO_ABS
#undef KO_SFX
#define KO_T double complex
#define KO_ABS(x) cabs(x)
#define KO_SFX z
#include "ko_lu_impl.h"
#undef KO_T
#undef KO_ABS
#undef KO_SFX

/* ----------------------------------------------------------- waveforms */
double ko_pulse(const double *w, double t) {
  /* voltage_source.rs:70-93 */
  double v1 = w[0], v2 = w[1], td = w[2], tr = w[3], tf = w[4], pw = w[5], per = w[6];
  if (t < td) return v1;
  double tt = fmod(t - td, per);
  if (tt < tr) return v1 + (v2 - v1) * (tt / tr);
  else if (tt < tr + pw) return v2;
  else if (tt < tr + pw + tf) return v2 + (v1 - v2) * ((tt - tr - pw) / tf);
  return v1;
}

double ko_sin(const double *w, double t) {
  /* voltage_source.rs:52-65 */
  double off = w[0], amp = w[1], freq = w[2], td = w[3], damp = w[4], ph = w[5];
  if (t < td) return off;
  double omega = 2.0 * KO_PI * freq;
  double phr = ph * (KO_PI / 180.0);
  double tt = t - td;
  return off + amp * exp(-damp * tt) * sin(omega * tt + phr);
}

static double ko_source_at(const ko_elem *e, double t) {
  if (e->wave == W_PULSE) return ko_pulse(e->wp, t);
  if (e->wave == W_SIN) return ko_sin(e->wp, t);
  return e->value;
}

/* ------------------------------------------------------------- diode */
static double ko_diode_vcrit(const ko_elem *e) {
  double n = e->wp[0], is = e->value;
  return n * KO_VT * log(DBL_MAX * n * KO_VT / is);
}
/* guess: solution vector or NULL when the reference's map is empty */
static double ko_diode_vd(const ko_elem *e, const double *guess) {
  double vp = (guess && e->p >= 0) ? guess[e->p] : 0.5;
  double vm = (guess && e->m >= 0) ? guess[e->m] : 0.0;
  return vp - vm;
}
static double ko_clamp(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }
static double ko_diode_g(const ko_elem *e, const double *guess) {
  double vc = ko_diode_vcrit(e);
  double vd = ko_clamp(ko_diode_vd(e, guess), -vc, vc);
  double n = e->wp[0], is = e->value;
  return (is / (n * KO_VT)) * exp(vd / (n * KO_VT));
}
static double ko_diode_ieq(const ko_elem *e, const double *guess) {
  double vc = ko_diode_vcrit(e);
  double vdl = ko_clamp(ko_diode_vd(e, guess), -vc, vc);
  double n = e->wp[0], is = e->value;
  double cur = is * (exp(vdl / (n * KO_VT)) - 1.0);
  return cur - ko_diode_g(e, guess) * ko_diode_vd(e, guess);
}

/* NMOS level 1, nmosfet.rs:51-103 (g_m :51-66, g_ds :68-84, i_d :86-102) with
 * beta = kp * (w / l) (models/nmosfet.rs:41-43); wp = {vto, kp, lambda, w, l}.  Terminal
 * voltages come from the solution map with unwrap_or(0.0) (stampable.rs:825-833). */
static void ko_nmos(const ko_elem *e, const double *guess, double *gm, double *gds, double *id, double *vgs_out,
                    double *vds_out) {
  double vg = (guess && e->g >= 0) ? guess[e->g] : 0.0;
  double vs = (guess && e->m >= 0) ? guess[e->m] : 0.0;
  double vd = (guess && e->p >= 0) ? guess[e->p] : 0.0;
  double vgs = vg - vs, vds = vd - vs;
  double vth = e->wp[0], beta = e->wp[1] * (e->wp[3] / e->wp[4]), lambda = e->wp[2];
  *gm = *gds = *id = 0.0;
  if (vgs <= vth) {
  } else if (vds >= 0.0 && vds <= (vgs - vth)) {
    *gm = beta * vds;
    *gds = beta * (vgs - vth - vds);
    *id = beta * ((vgs - vth) * vds - (vds * vds / 2.0));
  } else if (vds >= (vgs - vth) && vds >= 0.0) {
    double ov = vgs - vth;
    *gm = beta * ov * (1.0 + lambda * vds);
    *gds = (beta / 2.0) * lambda * (ov * ov);
    *id = (beta / 2.0) * (ov * ov) * (1.0 + lambda * vds);
  }
  *vgs_out = vgs;
  *vds_out = vds;
}

/* ------------------------------------------------------------ triplets */
typedef struct { int r, c; double complex v; long seq; } ko_trip;
typedef struct { ko_trip *t; long n, cap; } ko_tlist;

static int ko_push(ko_tlist *L, int r, int c, double complex v) {
  if (L->n == L->cap) {
    long nc = L->cap ? L->cap * 2 : 256;
    ko_trip *nt = (ko_trip *)realloc(L->t, sizeof(ko_trip) * nc);
    if (!nt) return -1;
    L->t = nt;
    L->cap = nc;
  }
  L->t[L->n].r = r;
  L->t[L->n].c = c;
  L->t[L->n].v = v;
  L->t[L->n].seq = L->n;
  L->n++;
  return 0;
}

enum { MODE_DC = 0, MODE_AC = 1, MODE_TRAN = 2 };

typedef struct {
  int mode;
  const double *guess;  /* Newton guess map (NULL = empty map) */
  double guess_time;    /* "time" entry of the guess map (transient) */
  const double *prev;   /* previous time step solution (transient) */
  double h;
  int trap;             /* 1 = trapezoidal extension */
  const double *ic_prev;/* TR capacitor currents at t_n, per element */
  double freq;
  const double *dc_sol; /* AC: operating point */
  int lag;              /* transient source time: 1 = guess "time", 0 = t_now */
  double t_now;
} ko_ctx;

#define PUSH(L, r, c, v) do { if (ko_push((L), (r), (c), (v))) return KO_NOMEM; } while (0)

static int ko_stamp(const ko_elem *e, int ei, const ko_ctx *x, ko_tlist *G, ko_tlist *E) {
  int ip = e->p, im = e->m, ic = e->b;
  switch (e->kind) {
    case K_R: {
      if (e->flags & F_G2) {
        if (ip >= 0 && ic >= 0) { PUSH(G, ip, ic, 1.0); PUSH(G, ic, ip, 1.0); }
        if (im >= 0 && ic >= 0) { PUSH(G, im, ic, -1.0); PUSH(G, ic, im, -1.0); }
        if (ic >= 0) PUSH(G, ic, ic, -e->value);
      } else {
        double g = 1.0 / e->value;
        if (ip >= 0) PUSH(G, ip, ip, g);
        if (im >= 0) PUSH(G, im, im, g);
        if (ip >= 0 && im >= 0) { PUSH(G, ip, im, -g); PUSH(G, im, ip, -g); }
      }
      return 0;
    }
    case K_C: {
      if (x->mode == MODE_DC) return 0;
      if (x->mode == MODE_AC) {
        double complex adm = CMPLX(0.0, 2.0 * KO_PI * x->freq * e->value);
        if (!(e->flags & F_G2)) {
          if (ip >= 0) PUSH(G, ip, ip, adm);
          if (im >= 0) PUSH(G, im, im, adm);
          if (ip >= 0 && im >= 0) { PUSH(G, ip, im, -adm); PUSH(G, im, ip, -adm); }
        } else {
          if (ip >= 0 && ic >= 0) PUSH(G, ic, ip, -adm);
          if (im >= 0 && ic >= 0) PUSH(G, ic, im, adm);
          if (ic >= 0) PUSH(G, ic, ic, 1.0);
        }
        return 0;
      }
      double g = x->trap ? 2.0 * e->value / x->h : e->value / x->h;
      if (ip >= 0) PUSH(G, ip, ip, g);
      if (im >= 0) PUSH(G, im, im, g);
      if (ip >= 0 && im >= 0) { PUSH(G, ip, im, -g); PUSH(G, im, ip, -g); }
      double vp = ip >= 0 ? x->prev[ip] : 0.0, vm = im >= 0 ? x->prev[im] : 0.0;
      double vprev = vp - vm;
      if (x->trap) {
        double ihist = g * vprev + x->ic_prev[ei];
        if (ip >= 0) PUSH(E, ip, 0, ihist);
        if (im >= 0) PUSH(E, im, 0, -ihist);
      } else {
        double ieq = -(e->value / x->h) * vprev;
        if (ip >= 0) PUSH(E, ip, 0, -ieq);
        if (im >= 0) PUSH(E, im, 0, ieq);
      }
      return 0;
    }
    case K_I: {
      if (x->mode == MODE_AC) {
        if (ip >= 0 && ic >= 0) PUSH(G, ip, ic, 1.0);
        if (im >= 0 && ic >= 0) PUSH(G, im, ic, -1.0);
      } else {
        if (ic >= 0) PUSH(G, ic, ic, 1.0);
        if (ip >= 0 && ic >= 0) PUSH(G, ip, ic, 1.0);
        if (im >= 0 && ic >= 0) PUSH(G, im, ic, -1.0);
      }
      if (ic >= 0) PUSH(E, ic, 0, e->value);
      return 0;
    }
    case K_D: {
      const double *sol = x->mode == MODE_AC ? x->dc_sol : x->guess;
      double g = ko_diode_g(e, sol);
      if (ip >= 0) PUSH(G, ip, ip, g);
      if (im >= 0) PUSH(G, im, im, g);
      if (ip >= 0 && im >= 0) { PUSH(G, ip, im, -g); PUSH(G, im, ip, -g); }
      if (x->mode != MODE_AC) {
        double ieq = ko_diode_ieq(e, sol);
        if (ip >= 0) PUSH(E, ip, 0, -ieq);
        if (im >= 0) PUSH(E, im, 0, ieq);
      }
      return 0;
    }
    case K_L: {
      if (x->mode == MODE_TRAN) {
        double lh = x->trap ? 2.0 * e->value / x->h : e->value / x->h;
        if (ic >= 0) PUSH(G, ic, ic, -lh);
        if (ip >= 0 && ic >= 0) { PUSH(G, ip, ic, 1.0); PUSH(G, ic, ip, 1.0); }
        if (im >= 0 && ic >= 0) { PUSH(G, im, ic, -1.0); PUSH(G, ic, im, -1.0); }
        double iprev = x->prev[ic];
        if (ic >= 0) {
          if (x->trap) {
            double vl = (ip >= 0 ? x->prev[ip] : 0.0) - (im >= 0 ? x->prev[im] : 0.0);
            PUSH(E, ic, 0, -lh * iprev - vl);
          } else {
            PUSH(E, ic, 0, -(e->value / x->h) * iprev);
          }
        }
        return 0;
      }
      if (ip >= 0 && ic >= 0) PUSH(G, ip, ic, 1.0);
      if (im >= 0 && ic >= 0) PUSH(G, im, ic, -1.0);
      if (ip >= 0 && ic >= 0) PUSH(G, ic, ip, 1.0);
      if (im >= 0 && ic >= 0) PUSH(G, ic, im, -1.0);
      if (x->mode == MODE_AC && ic >= 0)
        PUSH(G, ic, ic, -CMPLX(0.0, 2.0 * KO_PI * x->freq * e->value));
      return 0;
    }
    case K_V: {
      if (ip >= 0 && ic >= 0) { PUSH(G, ip, ic, 1.0); PUSH(G, ic, ip, 1.0); }
      if (im >= 0 && ic >= 0) { PUSH(G, im, ic, -1.0); PUSH(G, ic, im, -1.0); }
      if (ic >= 0) {
        if (x->mode == MODE_DC) PUSH(E, ic, 0, e->value);
        else if (x->mode == MODE_AC) PUSH(E, ic, 0, e->ac);
        else PUSH(E, ic, 0, ko_source_at(e, x->lag ? x->guess_time : x->t_now));
      }
      return 0;
    }
    case K_M: {
      if (x->mode == MODE_AC) return KO_NOTIMPL; /* stampable.rs:914-921 todo!() */
      if (!(e->flags & F_NMOS_RESOLVED)) return 0; /* bare-name lookups never match (:842-844) */
      /* stampable.rs:846-866 and :870-899 with the lookups resolved */
      double gm, gds, id, vgs, vds;
      ko_nmos(e, x->guess, &gm, &gds, &id, &vgs, &vds);
      int d = e->p, src = e->m, g = e->g;
      if (d >= 0) PUSH(G, d, d, gds);
      if (src >= 0) PUSH(G, src, src, gds + gm);
      if (d >= 0 && src >= 0) { PUSH(G, d, src, -(gds + gm)); PUSH(G, src, d, gds + gm); }
      if (src >= 0 && g >= 0) PUSH(G, src, g, gm);
      if (d >= 0 && g >= 0) PUSH(G, d, g, gm);
      double ieq = id - gds * vds - gm * vgs;
      if (src >= 0) PUSH(E, src, 0, ieq);
      if (d >= 0) PUSH(E, d, 0, -ieq);
      return 0;
    }
    case K_Q:
      return KO_NOTIMPL; /* stampable.rs:321-357 todo!() */
  }
  return KO_BADELEM;
}

/* ------------------------------------------- duplicate sum (solver.rs:59-70) */
static int ko_trip_cmp(const void *a, const void *b) {
  const ko_trip *x = (const ko_trip *)a, *y = (const ko_trip *)b;
  if (x->c != y->c) return x->c < y->c ? -1 : 1;
  if (x->r != y->r) return x->r < y->r ? -1 : 1;
  return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

/* Sort by (col,row) keeping emission order inside a key, then sum in that order:
 * the same per-entry summation order as the reference's HashMap `+=`. */
static int ko_to_csc(ko_tlist *G, int n, int **ap, int **ai, double complex **ax) {
  qsort(G->t, G->n, sizeof(ko_trip), ko_trip_cmp);
  int *p = (int *)calloc(n + 1, sizeof(int));
  int *i = (int *)malloc(sizeof(int) * (G->n + 1));
  double complex *x = (double complex *)malloc(sizeof(double complex) * (G->n + 1));
  if (!p || !i || !x) { free(p); free(i); free(x); return KO_NOMEM; }
  long nz = 0;
  for (long k = 0; k < G->n;) {
    long k2 = k;
    double complex s = 0.0;
    while (k2 < G->n && G->t[k2].r == G->t[k].r && G->t[k2].c == G->t[k].c) { s += G->t[k2].v; ++k2; }
    i[nz] = G->t[k].r;
    x[nz] = s;
    p[G->t[k].c + 1]++;
    nz++;
    k = k2;
  }
  for (int c = 0; c < n; ++c) p[c + 1] += p[c];
  *ap = p; *ai = i; *ax = x;
  return 0;
}

/* RHS: dense vector; duplicate rows summed in emission order */
static void ko_rhs(ko_tlist *E, int n, double complex *b) {
  for (int k = 0; k < n; ++k) b[k] = 0.0;
  /* stable order: emission order per row == plain accumulation in emission order */
  for (long k = 0; k < E->n; ++k) b[E->t[k].r] += E->t[k].v;
}

/* --------------------------------------- minimum degree (bitset, n <= 8192) */
static int *ko_mindeg(int n, const int *ap, const int *ai) {
  int *q = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  if (!q) return NULL;
  if (n > 8192) { for (int k = 0; k < n; ++k) q[k] = k; return q; }
  int W = (n + 63) / 64;
  uint64_t *adj = (uint64_t *)calloc((size_t)n * W, sizeof(uint64_t));
  char *elim = (char *)calloc(n > 0 ? n : 1, 1);
  if (!adj || !elim) { free(adj); free(elim); for (int k = 0; k < n; ++k) q[k] = k; return q; }
  for (int c = 0; c < n; ++c)
    for (int p = ap[c]; p < ap[c + 1]; ++p) {
      int r = ai[p];
      if (r == c) continue;
      adj[(size_t)r * W + c / 64] |= 1ull << (c % 64);
      adj[(size_t)c * W + r / 64] |= 1ull << (r % 64);
    }
  int *deg = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  for (int v = 0; v < n; ++v) {
    int d = 0;
    for (int w = 0; w < W; ++w) d += __builtin_popcountll(adj[(size_t)v * W + w]);
    deg[v] = d;
  }
  for (int k = 0; k < n; ++k) {
    int best = -1;
    for (int v = 0; v < n; ++v)
      if (!elim[v] && (best < 0 || deg[v] < deg[best])) best = v;
    q[k] = best;
    elim[best] = 1;
    uint64_t *av = adj + (size_t)best * W;
    for (int w = 0; w < W; ++w) {
      uint64_t bits = av[w];
      while (bits) {
        int u = w * 64 + __builtin_ctzll(bits);
        bits &= bits - 1;
        uint64_t *au = adj + (size_t)u * W;
        int d = 0;
        for (int z = 0; z < W; ++z) { au[z] |= av[z]; }
        au[u / 64] &= ~(1ull << (u % 64));
        au[best / 64] &= ~(1ull << (best % 64));
        for (int z = 0; z < W; ++z) d += __builtin_popcountll(au[z]);
        deg[u] = d;
      }
    }
    /* remove best from the graph: clear its row (neighbours already cleared it) */
    for (int w = 0; w < W; ++w) av[w] = 0;
  }
  free(adj); free(elim); free(deg);
  return q;
}

/* ------------------------------------------------ one linear solve */
typedef struct {
  int n, cplx;
  int *q;                 /* cached column order (pattern is fixed per analysis) */
  ko_lu_d Fd; ko_lu_z Fz; int have;
  double *wd; double complex *wz;
} ko_solver;

static void ko_solver_free(ko_solver *S) {
  free(S->q);
  if (S->have) { if (S->cplx) ko_lu_free_z(&S->Fz); else ko_lu_free_d(&S->Fd); }
  free(S->wd); free(S->wz);
  memset(S, 0, sizeof(*S));
}

/* Factor the summed triplets (fresh, as faer's sp_lu is called every time). */
static int ko_factor(ko_solver *S, ko_tlist *G) {
  int *ap, *ai; double complex *ax;
  int st = ko_to_csc(G, S->n, &ap, &ai, &ax);
  if (st) return st;
  if (!S->q) S->q = ko_mindeg(S->n, ap, ai);
  if (S->have) { if (S->cplx) ko_lu_free_z(&S->Fz); else ko_lu_free_d(&S->Fd); S->have = 0; }
  if (S->cplx) {
    st = ko_lu_factor_z(S->n, ap, ai, ax, S->q, &S->Fz);
    if (!S->wz) S->wz = (double complex *)malloc(sizeof(double complex) * (S->n + 1));
  } else {
    double *axr = (double *)malloc(sizeof(double) * (ap[S->n] + 1));
    for (int k = 0; k < ap[S->n]; ++k) axr[k] = creal(ax[k]);
    st = ko_lu_factor_d(S->n, ap, ai, axr, S->q, &S->Fd);
    free(axr);
    if (!S->wd) S->wd = (double *)malloc(sizeof(double) * (S->n + 1));
  }
  S->have = (st == 0);
  if (st) { if (S->cplx) ko_lu_free_z(&S->Fz); else ko_lu_free_d(&S->Fd); }
  free(ap); free(ai); free(ax);
  return st;
}

static void ko_solve_real(ko_solver *S, const double complex *b, double *x) {
  for (int k = 0; k < S->n; ++k) x[k] = creal(b[k]);
  ko_lu_solve_d(&S->Fd, x, x, S->wd);
}

/* ------------------------------------------------ convergence (solver.rs:76-104) */
static int ko_converged(const ko_cfg *c, const ko_elem *el, int ne, int n, const double *prev,
                        int prev_empty, const double *x, int has_extra, double extra_prev, double extra_new,
                        const char *is_cur) {
  (void)el; (void)ne;
  if (prev_empty) return 0;
  for (int k = 0; k < n; ++k) {
    double v = x[k], p = prev[k];
    double diff = fabs(v - p), scale = fmax(fabs(v), fabs(p));
    double atol = is_cur[k] ? c->iabstol : c->vabstol;
    if (!(diff <= c->reltol * scale + atol)) return 0;
  }
  if (has_extra) {
    double diff = fabs(extra_new - extra_prev), scale = fmax(fabs(extra_new), fabs(extra_prev));
    if (!(diff <= c->reltol * scale + c->vabstol)) return 0;
  }
  return 1;
}

static char *ko_is_current(const ko_elem *el, int ne, int n) {
  char *f = (char *)calloc(n > 0 ? n : 1, 1);
  for (int k = 0; k < ne; ++k)
    if (el[k].b >= 0 && el[k].b < n) f[el[k].b] = 1;
  return f;
}

static int ko_nonlinear(const ko_elem *el, int ne, int skip_caps) {
  for (int k = 0; k < ne; ++k) {
    if (skip_caps && el[k].kind == K_C) continue;
    if (el[k].kind == K_D || el[k].kind == K_M || el[k].kind == K_Q) return 1;
  }
  return 0;
}

/* Newton loop with DC stamps (op.rs:33-82 / dc.rs:67-110).  guess_in: warm start
 * (NULL = empty map).  extra: "step" key handling for DC sweeps (-1 = none). */
static int ko_newton_dc(const ko_elem *el, int ne, int n, const ko_cfg *cfg, const double *guess_in,
                        double step_key, double *x, int *iters_out, ko_solver *S, int reuse) {
  int nonlin = ko_nonlinear(el, ne, 1);
  char *is_cur = ko_is_current(el, ne, n);
  double *prev = (double *)malloc(sizeof(double) * (n + 1));
  double complex *b = (double complex *)malloc(sizeof(double complex) * (n + 1));
  int prev_empty = guess_in == NULL;
  double prev_step = step_key - 1.0;
  if (guess_in) memcpy(prev, guess_in, sizeof(double) * n);
  ko_tlist G = {0}, E = {0};
  int st = KO_OK, it;
  for (it = 0; it < cfg->maxiter; ++it) {
    G.n = E.n = 0;
    ko_ctx cx = {0};
    cx.mode = MODE_DC;
    cx.guess = prev_empty ? NULL : prev;
    for (int k = 0; k < ne; ++k) {
      if (el[k].kind == K_C) continue; /* op.rs:20-24 */
      st = ko_stamp(&el[k], k, &cx, &G, &E);
      if (st) goto done;
    }
    if (!(reuse && S->have && !nonlin)) {
      st = ko_factor(S, &G);
      if (st) goto done;
    }
    ko_rhs(&E, n, b);
    ko_solve_real(S, b, x);
    if (!nonlin) break;
    int has_extra = step_key >= 0.0;
    if (ko_converged(cfg, el, ne, n, prev, prev_empty, x, has_extra, prev_step, step_key, is_cur)) break;
    memcpy(prev, x, sizeof(double) * n);
    prev_empty = 0;
    prev_step = step_key;
    if (it == cfg->maxiter - 1) { st = KO_MAXITER; goto done; }
  }
done:
  if (iters_out) *iters_out = it + 1;
  free(G.t); free(E.t); free(prev); free(b); free(is_cur);
  return st;
}

/* ================================================================== API */
int ko_op(const ko_elem *el, int ne, int n, const ko_cfg *cfg, double *x, int *iters) {
  ko_solver S = {0};
  S.n = n;
  int st = ko_newton_dc(el, ne, n, cfg, NULL, -1.0, x, iters, &S, 0);
  ko_solver_free(&S);
  return st;
}

/* DC sweep of element `sweep` (dc.rs:14-124).  x_out: [n_points][n]. */
int ko_dc(const ko_elem *el_in, int ne, int n, const ko_cfg *cfg, int sweep, double start, double stop,
          double step, double *x_out, int max_points, int *n_points) {
  if (sweep < 0 || sweep >= ne) return KO_NOTFOUND;
  if (el_in[sweep].kind != K_V && el_in[sweep].kind != K_I) return KO_BADELEM;
  long np = (long)fabs((stop - start) / step) + 1;
  if (np > max_points) return KO_NOMEM;
  ko_elem *el = (ko_elem *)malloc(sizeof(ko_elem) * ne);
  memcpy(el, el_in, sizeof(ko_elem) * ne);
  ko_solver S = {0};
  S.n = n;
  int st = 0;
  for (long i = 0; i < np; ++i) {
    el[sweep].value = start + ((double)i * step);
    st = ko_newton_dc(el, ne, n, cfg, i == 0 ? NULL : x_out + (i - 1) * n, (double)i, x_out + i * n, NULL,
                      &S, 0);
    if (st) break;
  }
  *n_points = (int)np;
  ko_solver_free(&S);
  free(el);
  return st;
}

/* AC sweep (ac.rs:17-109).  Frequencies <= 0 are skipped; x_out: [n_kept][n] complex
 * (interleaved re, im); *n_kept returns the number of points solved. */
int ko_ac(const ko_elem *el, int ne, int n, const ko_cfg *cfg, const double *freqs, int nf, double *x_out,
          int *n_kept) {
  double *op = (double *)malloc(sizeof(double) * (n + 1));
  int st = ko_op(el, ne, n, cfg, op, NULL);
  *n_kept = 0;
  if (st) { free(op); return st; }
  ko_solver S = {0};
  S.n = n;
  S.cplx = 1;
  ko_tlist G = {0}, E = {0};
  double complex *b = (double complex *)malloc(sizeof(double complex) * (n + 1));
  double complex *xz = (double complex *)malloc(sizeof(double complex) * (n + 1));
  int kept = 0;
  for (int f = 0; f < nf; ++f) {
    if (freqs[f] <= 0.0) continue;
    G.n = E.n = 0;
    ko_ctx cx = {0};
    cx.mode = MODE_AC;
    cx.freq = freqs[f];
    cx.dc_sol = op;
    for (int k = 0; k < ne; ++k) {
      st = ko_stamp(&el[k], k, &cx, &G, &E);
      if (st) goto done;
    }
    st = ko_factor(&S, &G);
    if (st) goto done;
    ko_rhs(&E, n, b);
    ko_lu_solve_z(&S.Fz, b, xz, S.wz);
    for (int k = 0; k < n; ++k) {
      x_out[((size_t)kept * n + k) * 2] = creal(xz[k]);
      x_out[((size_t)kept * n + k) * 2 + 1] = cimag(xz[k]);
    }
    kept++;
  }
done:
  *n_kept = kept;
  free(G.t); free(E.t); free(b); free(xz); free(op);
  ko_solver_free(&S);
  return st;
}

/* Transient (transient.rs:14-114).  method 0 = BE (reference), 1 = TR (extension).
 * lag 1 = reference source timing (Newton guess "time"), 0 = source at t_n.
 * x_out: [n_steps+1][n]; row 0 is the operating point.  newton_iters (optional):
 * Newton iterations per step. */
int ko_tran(const ko_elem *el, int ne, int n, const ko_cfg *cfg, double h, int n_steps, int method, int lag,
            double *x_out, int *newton_iters) {
  int st = ko_op(el, ne, n, cfg, x_out, NULL);
  if (st) return st;
  int nonlin = ko_nonlinear(el, ne, 0);
  char *is_cur = ko_is_current(el, ne, n);
  double *guess = (double *)malloc(sizeof(double) * (n + 1));
  double *icap = (double *)calloc(ne > 0 ? ne : 1, sizeof(double));
  double complex *b = (double complex *)malloc(sizeof(double complex) * (n + 1));
  ko_solver S = {0};
  S.n = n;
  ko_tlist G = {0}, E = {0};
  for (int s = 1; s <= n_steps; ++s) {
    double t = (double)s * h;
    const double *prev = x_out + (size_t)(s - 1) * n;
    double *x = x_out + (size_t)s * n;
    memcpy(guess, prev, sizeof(double) * n);
    double guess_time = (double)(s - 1) * h;
    int it;
    for (it = 0; it < cfg->maxiter; ++it) {
      G.n = E.n = 0;
      ko_ctx cx = {0};
      cx.mode = MODE_TRAN;
      cx.guess = guess;
      cx.guess_time = guess_time;
      cx.prev = prev;
      cx.h = h;
      cx.trap = method == 1;
      cx.ic_prev = icap;
      cx.lag = lag;
      cx.t_now = t;
      for (int k = 0; k < ne; ++k) {
        st = ko_stamp(&el[k], k, &cx, &G, &E);
        if (st) goto done;
      }
      /* a linear circuit's matrix is identical every step: refactoring it gives the
       * same factors, so the optimised form factors once (faithful form refactors) */
      if (cfg->faithful || nonlin || !S.have) {
        st = ko_factor(&S, &G);
        if (st) goto done;
      }
      ko_rhs(&E, n, b);
      ko_solve_real(&S, b, x);
      if (!nonlin) break;
      if (ko_converged(cfg, el, ne, n, guess, 0, x, 1, guess_time, t, is_cur)) break;
      memcpy(guess, x, sizeof(double) * n);
      guess_time = t;
      if (it == cfg->maxiter - 1) { st = KO_MAXITER; goto done; }
    }
    if (newton_iters) newton_iters[s - 1] = it + 1;
    if (method == 1) {
      for (int k = 0; k < ne; ++k) {
        if (el[k].kind != K_C) continue;
        double g = 2.0 * el[k].value / h;
        double vp = el[k].p >= 0 ? prev[el[k].p] : 0.0, vm = el[k].m >= 0 ? prev[el[k].m] : 0.0;
        double ihist = g * (vp - vm) + icap[k];
        double np_ = el[k].p >= 0 ? x[el[k].p] : 0.0, nm_ = el[k].m >= 0 ? x[el[k].m] : 0.0;
        icap[k] = g * (np_ - nm_) - ihist;
      }
    }
  }
done:
  free(G.t); free(E.t); free(guess); free(icap); free(b); free(is_cur);
  ko_solver_free(&S);
  return st;
}

/* ------------------------------------------------ adaptive steps (extension)
 * Transient with local-truncation-error step control; krets has fixed steps only, so
 * this is an extension with its own oracle (this function), restating the standard
 * divided-difference estimate (SPICE2 timestep control, Nagel 1975):
 *   BE (order 1): LTE ~ h^2/2 x^(2) ~ h^2 DD2     (x^(2) ~ 2! DD2)
 *   TR (order 2): LTE ~ h^3/12 x^(3) ~ h^3/2 DD3  (x^(3) ~ 3! DD3)
 * with divided differences over the attempt and the last accepted points.  Error ratio
 * r = max_k |LTE_k| / (lte_tol * max(|x_k|, |x_n,k|) + abstol_k) (abstol: current or voltage
 * tolerance of the config).  r <= 1 accepts.  The step factor is the largest of a fixed
 * set whose predicted ratio r * f^(p+1) stays <= 1/2 ({2, 1.5, 1, 0.75, 0.5} after an
 * accept, {0.5, 0.25, 0.125} after a reject; 0.125 when Newton does not converge), so the
 * time grid is exact binary arithmetic shared with the device.  The first p steps (not
 * enough history) are accepted at h0.  Sources are evaluated at the new time (no lag).
 * Returns the accepted points (t_out, x_out rows; row 0 = operating point at t = 0). */
#define KO_TSTEP 8 /* step below h_min */
#define KO_FULL 9  /* more accepted points than max_points */

static double ko_step_factor(double r, int order, int accepted) {
  static const double fa[5] = {2.0, 1.5, 1.0, 0.75, 0.5};
  static const double fa2[5] = {4.0, 2.25, 1.0, 0.5625, 0.25}, fa3[5] = {8.0, 3.375, 1.0, 0.421875, 0.125};
  static const double fr[3] = {0.5, 0.25, 0.125};
  static const double fr2[3] = {0.25, 0.0625, 0.015625}, fr3[3] = {0.125, 0.015625, 0.001953125};
  if (accepted) {
    const double *pw = order == 1 ? fa2 : fa3;
    for (int i = 0; i < 5; ++i)
      if (r * pw[i] <= 0.5) return fa[i];
    return 0.5;
  }
  const double *pw = order == 1 ? fr2 : fr3;
  for (int i = 0; i < 3; ++i)
    if (r * pw[i] <= 0.5) return fr[i];
  return 0.125;
}

/* LTE ratio of the attempt x (time t_new = tn + h) given the accepted points xn (tn),
 * x1 (t1), x2 (t2; TR only), in the device's expression order. */
static double ko_lte_ratio(int n, int trap, const double *x, const double *xn, const double *x1, const double *x2,
                           double t_new, double tn, double t1, double t2, double h, double lte_tol,
                           const ko_cfg *cfg, const char *is_cur) {
  double r = 0.0;
  for (int k = 0; k < n; ++k) {
    double lte;
    if (!trap) {
      double d1 = (x[k] - xn[k]) / h, d0 = (xn[k] - x1[k]) / (tn - t1);
      double dd2 = (d1 - d0) / (t_new - t1);
      lte = (h * h) * dd2;
    } else {
      double d2 = (x[k] - xn[k]) / h, d1 = (xn[k] - x1[k]) / (tn - t1), d0 = (x1[k] - x2[k]) / (t1 - t2);
      double e1 = (d2 - d1) / (t_new - t1), e0 = (d1 - d0) / (tn - t2);
      double dd3 = (e1 - e0) / (t_new - t2);
      lte = (0.5 * (h * h * h)) * dd3;
    }
    double tol = lte_tol * fmax(fabs(x[k]), fabs(xn[k]));
    tol = tol + (is_cur[k] ? cfg->iabstol : cfg->vabstol);
    double q = fabs(lte) / tol;
    if (!(q <= r)) r = q; /* NaN propagates */
  }
  return r;
}

int ko_tran_adaptive(const ko_elem *el, int ne, int n, const ko_cfg *cfg, double h0, double t_stop, int method,
                     double lte_tol, double h_min, double h_max, int max_points, double *t_out, double *x_out,
                     int *n_points) {
  *n_points = 0;
  if (max_points < 1) return KO_FULL;
  int st = ko_op(el, ne, n, cfg, x_out, NULL);
  if (st) return st;
  t_out[0] = 0.0;
  int n_acc = 1;
  const int trap = method == 1, order = trap ? 2 : 1;
  int nonlin = ko_nonlinear(el, ne, 0);
  char *is_cur = ko_is_current(el, ne, n);
  double *x = (double *)malloc(sizeof(double) * (n + 1));
  double *guess = (double *)malloc(sizeof(double) * (n + 1));
  double *icap = (double *)calloc(ne > 0 ? ne : 1, sizeof(double));
  double complex *b = (double complex *)malloc(sizeof(double complex) * (n + 1));
  ko_solver S = {0};
  S.n = n;
  ko_tlist G = {0}, E = {0};
  double t = 0.0, h = fmin(h0, h_max), h_fact = -1.0;
  while (t < t_stop) {
    if (t + h >= t_stop || t_stop - (t + h) < h_min) h = t_stop - t;
    const double t_new = (t + h >= t_stop) ? t_stop : t + h;
    const double *xn = x_out + (size_t)(n_acc - 1) * n;
    memcpy(guess, xn, sizeof(double) * n);
    double guess_time = t;
    int it, newton_ok = 0;
    for (it = 0; it < cfg->maxiter; ++it) {
      G.n = E.n = 0;
      ko_ctx cx = {0};
      cx.mode = MODE_TRAN;
      cx.guess = guess;
      cx.guess_time = guess_time;
      cx.prev = xn;
      cx.h = h;
      cx.trap = trap;
      cx.ic_prev = icap;
      cx.lag = 0;
      cx.t_now = t_new;
      for (int k = 0; k < ne; ++k) {
        st = ko_stamp(&el[k], k, &cx, &G, &E);
        if (st) goto done;
      }
      if (nonlin || !S.have || h != h_fact) {
        st = ko_factor(&S, &G);
        if (st) goto done;
        h_fact = h;
      }
      ko_rhs(&E, n, b);
      ko_solve_real(&S, b, x);
      if (!nonlin) { newton_ok = 1; break; }
      if (ko_converged(cfg, el, ne, n, guess, 0, x, 1, guess_time, t_new, is_cur)) { newton_ok = 1; break; }
      memcpy(guess, x, sizeof(double) * n);
      guess_time = t_new;
    }
    for (int k = 0; k < n; ++k)
      if (!isfinite(x[k])) { st = KO_NONFINITE; goto done; }
    double r = 0.0;
    int checked = 0;
    if (newton_ok && n_acc >= order + 1) {
      const double *x1 = x_out + (size_t)(n_acc - 2) * n;
      const double *x2 = trap ? x_out + (size_t)(n_acc - 3) * n : x1;
      r = ko_lte_ratio(n, trap, x, xn, x1, x2, t_new, t, t_out[n_acc - 2], trap ? t_out[n_acc - 3] : 0.0, h,
                       lte_tol, cfg, is_cur);
      checked = 1;
    }
    if (newton_ok && !(r > 1.0)) {
      if (n_acc >= max_points) { st = KO_FULL; goto done; }
      double *row = x_out + (size_t)n_acc * n;
      memcpy(row, x, sizeof(double) * n);
      t_out[n_acc] = t_new;
      if (trap)
        for (int k = 0; k < ne; ++k) {
          if (el[k].kind != K_C) continue;
          double g = 2.0 * el[k].value / h;
          double vp = el[k].p >= 0 ? xn[el[k].p] : 0.0, vm = el[k].m >= 0 ? xn[el[k].m] : 0.0;
          double ihist = g * (vp - vm) + icap[k];
          double np_ = el[k].p >= 0 ? row[el[k].p] : 0.0, nm_ = el[k].m >= 0 ? row[el[k].m] : 0.0;
          icap[k] = g * (np_ - nm_) - ihist;
        }
      n_acc++;
      t = t_new;
      double f = checked ? ko_step_factor(r, order, 1) : 1.0;
      h = fmin(h * f, h_max);
      if (h < h_min) h = h_min;
    } else {
      double f = newton_ok ? ko_step_factor(r, order, 0) : 0.125;
      h = h * f;
      if (h < h_min) { st = KO_TSTEP; goto done; }
    }
  }
done:
  *n_points = n_acc;
  free(G.t); free(E.t); free(x); free(guess); free(icap); free(b); free(is_cur);
  ko_solver_free(&S);
  return st;
}

/* Assemble the summed MNA matrix of one mode as dense row-major (tests compare the
 * device's stamped values against this).  mode 0 = DC (caps filtered), 2 = TRAN with
 * prev = guess = x_prev (no lag), 1 = AC (complex interleaved). */
int ko_assemble(const ko_elem *el, int ne, int n, int mode, double h, int method, double freq,
                const double *sol, double *A_out, double *b_out) {
  ko_tlist G = {0}, E = {0};
  double *icap = (double *)calloc(ne > 0 ? ne : 1, sizeof(double));
  ko_ctx cx = {0};
  cx.mode = mode;
  cx.guess = sol;
  cx.prev = sol;
  cx.dc_sol = sol;
  cx.h = h;
  cx.trap = method == 1;
  cx.ic_prev = icap;
  cx.freq = freq;
  int st = 0;
  for (int k = 0; k < ne; ++k) {
    if (mode == MODE_DC && el[k].kind == K_C) continue;
    st = ko_stamp(&el[k], k, &cx, &G, &E);
    if (st) break;
  }
  if (!st) {
    int w = mode == MODE_AC ? 2 : 1;
    memset(A_out, 0, sizeof(double) * (size_t)n * n * w);
    memset(b_out, 0, sizeof(double) * (size_t)n * w);
    qsort(G.t, G.n, sizeof(ko_trip), ko_trip_cmp);
    for (long k = 0; k < G.n; ++k) {
      size_t off = ((size_t)G.t[k].r * n + G.t[k].c) * w;
      A_out[off] += creal(G.t[k].v);
      if (w == 2) A_out[off + 1] += cimag(G.t[k].v);
    }
    for (long k = 0; k < E.n; ++k) {
      b_out[(size_t)E.t[k].r * w] += creal(E.t[k].v);
      if (w == 2) b_out[(size_t)E.t[k].r * w + 1] += cimag(E.t[k].v);
    }
  }
  free(G.t); free(E.t); free(icap);
  return st;
}

/* ------------------------------------------------ adjoint sensitivities (extension) */
/* Solve A^T y = c with factors of P A Q = L U: U^T w = Q^T c (forward over positions),
 * L^T v = w (backward), y = P^T v.  c and y may alias; work has n entries. */
static void ko_lu_tsolve_d(const ko_lu_d *F, const double *c, double *y, double *work) {
  int n = F->n;
  for (int k = 0; k < n; ++k) work[k] = c[F->q[k]];
  for (int k = 0; k < n; ++k) {
    int pd = F->up[k + 1] - 1;
    double s = work[k];
    for (int p = F->up[k]; p < pd; ++p) s -= F->ux[p] * work[F->ui[p]];
    work[k] = s / F->ux[pd];
  }
  for (int k = n - 1; k >= 0; --k) {
    double s = work[k];
    for (int p = F->lp[k]; p < F->lp[k + 1]; ++p) s -= F->lx[p] * work[F->pinv[F->li[p]]];
    work[k] = s;
  }
  for (int r = 0; r < n; ++r) y[r] = work[F->pinv[r]];
}

/* Loss sum_{s=1..N} x_s[out]^2 of a linear transient from a zero operating point and its
 * gradient with respect to every R, C and L value (0 for other elements), by the discrete
 * adjoint of the companion recurrence  M x_s = N x_{s-1} + src:
 *   TR: M = G + (2/h) C, N = (2/h) C - G;  BE: M = G + C/h, N = C/h
 *   M^T l_s = 2 x_s[out] e_out + N^T l_{s+1},  l_{N+1} = 0
 *   dloss/dp = sum_s l_s^T (dN/dp x_{s-1} - dM/dp x_s).
 * N^T l is formed as a C^T l - (M^T l from M's triplets): an independent route from the
 * device kernel's recurrence on previous right-hand sides. */
int ko_adjoint_tran(const ko_elem *el, int ne, int n, const ko_cfg *cfg, double h, int n_steps, int method,
                    int out, double *loss, double *grad) {
  if (out < 0 || out >= n || n_steps < 1) return KO_BADELEM;
  if (ko_nonlinear(el, ne, 0)) return KO_NOTIMPL;
  for (int k = 0; k < ne; ++k)
    if ((el[k].kind == K_R || el[k].kind == K_C) && (el[k].flags & F_G2)) return KO_NOTIMPL;
  double *X = (double *)malloc(sizeof(double) * (size_t)(n_steps + 1) * n);
  double *lam = (double *)calloc(n, sizeof(double)), *nxt = (double *)calloc(n, sizeof(double));
  double *rhs = (double *)malloc(sizeof(double) * n), *work = (double *)malloc(sizeof(double) * n);
  double *zero = (double *)calloc(n, sizeof(double)), *icap = (double *)calloc(ne > 0 ? ne : 1, sizeof(double));
  ko_tlist G = {0}, E = {0};
  ko_solver S = {0};
  S.n = n;
  int st = ko_tran(el, ne, n, cfg, h, n_steps, method, 0, X, NULL);
  for (int k = 0; !st && k < n; ++k)
    if (X[k] != 0.0) st = KO_NOTIMPL; /* the recurrence starts from x_0 = 0 */
  if (!st) {
    ko_ctx cx = {0};
    cx.mode = MODE_TRAN;
    cx.guess = zero;
    cx.prev = zero;
    cx.h = h;
    cx.trap = method == 1;
    cx.ic_prev = icap;
    cx.t_now = h;
    for (int k = 0; !st && k < ne; ++k) st = ko_stamp(&el[k], k, &cx, &G, &E);
  }
  if (!st) st = ko_factor(&S, &G);
  if (!st) {
    const double a = method == 1 ? 2.0 / h : 1.0 / h, ca = method == 1 ? 2.0 * a : a;
    double L = 0.0;
    for (int k = 0; k < ne; ++k) grad[k] = 0.0;
    for (int s = n_steps; s >= 1; --s) {
      const double *xs = X + (size_t)s * n, *xp = X + (size_t)(s - 1) * n;
      L += xs[out] * xs[out];
      for (int k = 0; k < n; ++k) rhs[k] = 0.0;
      for (int k = 0; k < ne; ++k) { /* C^T l_{s+1}, scaled */
        const ko_elem *e = &el[k];
        if (e->kind == K_C) {
          double u = e->value * ((e->p >= 0 ? nxt[e->p] : 0.0) - (e->m >= 0 ? nxt[e->m] : 0.0));
          if (e->p >= 0) rhs[e->p] += ca * u;
          if (e->m >= 0) rhs[e->m] -= ca * u;
        } else if (e->kind == K_L && e->b >= 0) {
          rhs[e->b] -= ca * e->value * nxt[e->b];
        }
      }
      if (method == 1)
        for (long t = 0; t < G.n; ++t) rhs[G.t[t].c] -= creal(G.t[t].v) * nxt[G.t[t].r];
      rhs[out] += 2.0 * xs[out];
      ko_lu_tsolve_d(&S.Fd, rhs, lam, work);
      for (int k = 0; k < ne; ++k) {
        const ko_elem *e = &el[k];
        double dl = (e->p >= 0 ? lam[e->p] : 0.0) - (e->m >= 0 ? lam[e->m] : 0.0);
        double vn = (e->p >= 0 ? xs[e->p] : 0.0) - (e->m >= 0 ? xs[e->m] : 0.0);
        double vp = (e->p >= 0 ? xp[e->p] : 0.0) - (e->m >= 0 ? xp[e->m] : 0.0);
        if (e->kind == K_R) grad[k] += dl * (method == 1 ? vp + vn : vn) / (e->value * e->value);
        else if (e->kind == K_C) grad[k] += a * dl * (vp - vn);
        else if (e->kind == K_L && e->b >= 0) grad[k] += a * lam[e->b] * (xs[e->b] - xp[e->b]);
        else if ((e->kind == K_V || e->kind == K_I) && e->b >= 0) {
          /* d loss / d alpha for the source's transient value scaled by alpha: the rhs of
           * step s holds w_s (BE) or w_s + w_{s-1} (TR form of the recurrence) at row b */
          double ws = e->kind == K_V ? ko_source_at(e, (double)s * h) : e->value;
          double w0 = e->kind == K_V ? ko_source_at(e, (double)(s - 1) * h) : e->value;
          grad[k] += lam[e->b] * (method == 1 ? ws + w0 : ws);
        }
      }
      double *tmp = nxt;
      nxt = lam;
      lam = tmp;
    }
    *loss = L;
  }
  free(X); free(lam); free(nxt); free(rhs); free(work); free(zero); free(icap);
  free(G.t); free(E.t);
  ko_solver_free(&S);
  return st;
}

/* Solve a dense/CSC system with the oracle LU (used to cross-check the LU itself). */
int ko_lu_solve_csc(int n, const int *ap, const int *ai, const double *ax, const double *b, double *x) {
  int *q = ko_mindeg(n, ap, ai);
  ko_lu_d F;
  int st = ko_lu_factor_d(n, ap, ai, ax, q, &F);
  if (!st) {
    double *w = (double *)malloc(sizeof(double) * (n + 1));
    ko_lu_solve_d(&F, b, x, w);
    free(w);
    ko_lu_free_d(&F);
  }
  free(q);
  return st;
}

int ko_abi_elem_size(void) { return (int)sizeof(ko_elem); }
