/*
 * Oracle sparse LU with partial pivoting (left-looking, Gilbert-Peierls), included
 * twice by krets_oracle.c: once with KO_T = double, once with KO_T = double complex.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the CPU stand-in for the third-party faer 0.23.2
 * `sp_lu()` + `solve()` that the reference calls at
 *   crates/krets-solver/src/solver/op.rs:48-58, dc.rs:81-90, ac.rs:67-95,
 *   transient.rs:74-83.
 * faer's published algorithm is a fill-reducing column ordering followed by LU with
 * partial (row) pivoting; this restatement does the same with its own minimum-degree
 * ordering and a textbook Gilbert-Peierls factorisation, so results agree with faer up
 * to rounding (a different but equally valid pivot order), not bit for bit.
 *
 * Required macros: KO_T (scalar), KO_ABS(x) (magnitude), KO_SFX (name suffix).
 */
#define KO_CAT2(a, b) a##b
#define KO_CAT(a, b) KO_CAT2(a, b)
#define KO_FN(name) KO_CAT(name, KO_SFX)

typedef struct {
  int n;
  /* L: unit lower, column k holds rows (original numbering) strictly below pivot */
  int *lp, *li; KO_T *lx;
  /* U: column k holds pivot-position indices (0..k) of the pivotal rows, diag last */
  int *up, *ui; KO_T *ux;
  int *pinv;      /* pinv[row] = pivot position */
  int *q;         /* column order: position k factors original column q[k] */
  int lnz, unz, lcap, ucap;
} KO_FN(ko_lu_);

static void KO_FN(ko_lu_free_)(KO_FN(ko_lu_) *F) {
  free(F->lp); free(F->li); free(F->lx); free(F->up); free(F->ui); free(F->ux);
  free(F->pinv); free(F->q);
  memset(F, 0, sizeof(*F));
}

static int KO_FN(ko_grow_)(int **idx, KO_T **val, int *cap, int need) {
  if (need <= *cap) return 0;
  int nc = (*cap) * 2 > need ? (*cap) * 2 : need + 16;
  int *ni = (int *)realloc(*idx, sizeof(int) * nc);
  if (!ni) return -1;
  *idx = ni;
  KO_T *nv = (KO_T *)realloc(*val, sizeof(KO_T) * nc);
  if (!nv) return -1;
  *val = nv;
  *cap = nc;
  return 0;
}

/*
 * Factor the n x n CSC matrix (ap, ai, ax) in column order q (NULL = natural).
 * Returns 0, or KO_SINGULAR when a column has no non-zero pivot candidate, or
 * KO_NONFINITE when a pivot is not finite.
 */
static int KO_FN(ko_lu_factor_)(int n, const int *ap, const int *ai, const KO_T *ax, const int *q,
                                KO_FN(ko_lu_) *F) {
  memset(F, 0, sizeof(*F));
  F->n = n;
  F->lp = (int *)malloc(sizeof(int) * (n + 1));
  F->up = (int *)malloc(sizeof(int) * (n + 1));
  F->pinv = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  F->q = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  int nnz = ap[n];
  F->lcap = F->ucap = 4 * nnz + n + 16;
  F->li = (int *)malloc(sizeof(int) * F->lcap);
  F->lx = (KO_T *)malloc(sizeof(KO_T) * F->lcap);
  F->ui = (int *)malloc(sizeof(int) * F->ucap);
  F->ux = (KO_T *)malloc(sizeof(KO_T) * F->ucap);
  KO_T *x = (KO_T *)calloc(n > 0 ? n : 1, sizeof(KO_T));
  int *xi = (int *)malloc(sizeof(int) * 2 * (n > 0 ? n : 1)); /* reach stack */
  int *mark = (int *)calloc(n > 0 ? n : 1, sizeof(int));
  int *stackp = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  if (!F->lp || !F->up || !F->pinv || !F->q || !F->li || !F->lx || !F->ui || !F->ux || !x || !xi ||
      !mark || !stackp) {
    free(x); free(xi); free(mark); free(stackp);
    return KO_NOMEM;
  }
  for (int i = 0; i < n; ++i) { F->pinv[i] = -1; F->q[i] = q ? q[i] : i; }
  int lnz = 0, unz = 0, status = 0;
  for (int k = 0; k < n; ++k) {
    F->lp[k] = lnz;
    F->up[k] = unz;
    if (KO_FN(ko_grow_)(&F->li, &F->lx, &F->lcap, lnz + n) ||
        KO_FN(ko_grow_)(&F->ui, &F->ux, &F->ucap, unz + n)) { status = KO_NOMEM; break; }
    int col = F->q[k];
    /* symbolic reach of A(:,col) through the graph of L (DFS, topological order) */
    int top = n;
    for (int p = ap[col]; p < ap[col + 1]; ++p) {
      int r = ai[p];
      if (mark[r] == k + 1) continue;
      /* iterative DFS from r */
      int head = 0;
      xi[0] = r;
      while (head >= 0) {
        int j = xi[head];
        int jp = F->pinv[j];
        if (mark[j] != k + 1) {
          mark[j] = k + 1;
          stackp[head] = (jp < 0) ? 0 : F->lp[jp];
        }
        int done = 1;
        if (jp >= 0) {
          int end = F->lp[jp + 1];
          for (int pp = stackp[head]; pp < end; ++pp) {
            int i = F->li[pp];
            if (mark[i] == k + 1) continue;
            stackp[head] = pp + 1;
            xi[++head] = i;
            done = 0;
            break;
          }
        }
        if (done) {
          head--;
          xi[--top + n] = j; /* push onto output (stored in xi[n..2n)) */
        }
      }
    }
    /* xi[n+top .. 2n) is the reach in topological order */
    for (int p = top; p < n; ++p) x[xi[n + p]] = 0;
    for (int p = ap[col]; p < ap[col + 1]; ++p) x[ai[p]] += ax[p];
    for (int p = top; p < n; ++p) {
      int j = xi[n + p];
      int jp = F->pinv[j];
      if (jp < 0) continue;
      KO_T xj = x[j];
      for (int pp = F->lp[jp]; pp < F->lp[jp + 1]; ++pp) x[F->li[pp]] -= F->lx[pp] * xj;
    }
    /* partial pivoting: largest magnitude among non-pivotal rows of the reach */
    int ipiv = -1;
    double amax = -1.0;
    for (int p = top; p < n; ++p) {
      int i = xi[n + p];
      if (F->pinv[i] < 0) {
        double a = KO_ABS(x[i]);
        if (a > amax) { amax = a; ipiv = i; }
      } else {
        F->ui[unz] = F->pinv[i];
        F->ux[unz++] = x[i];
      }
    }
    if (ipiv < 0 || amax <= 0.0) { status = KO_SINGULAR; break; }
    if (!isfinite(amax)) { status = KO_NONFINITE; break; }
    KO_T piv = x[ipiv];
    F->ui[unz] = k;
    F->ux[unz++] = piv;
    F->pinv[ipiv] = k;
    for (int p = top; p < n; ++p) {
      int i = xi[n + p];
      if (F->pinv[i] < 0) {
        F->li[lnz] = i;
        F->lx[lnz++] = x[i] / piv;
      }
      x[i] = 0;
    }
  }
  if (status == 0) {
    F->lp[n] = lnz;
    F->up[n] = unz;
    F->lnz = lnz;
    F->unz = unz;
  }
  free(x); free(xi); free(mark); free(stackp);
  return status;
}

/* Solve A x = b with the factors; b and x may alias. work has n entries. */
static void KO_FN(ko_lu_solve_)(const KO_FN(ko_lu_) *F, const KO_T *b, KO_T *x, KO_T *work) {
  int n = F->n;
  /* forward: L y = P b, processed in pivot order; y indexed by original row */
  for (int i = 0; i < n; ++i) work[i] = b[i];
  /* position-indexed vector: entry pinv[r] holds row r of P b */
  KO_T *y = x;
  for (int r = 0; r < n; ++r) y[F->pinv[r]] = work[r];
  for (int k = 0; k < n; ++k) {
    KO_T yk = y[k];
    for (int p = F->lp[k]; p < F->lp[k + 1]; ++p) y[F->pinv[F->li[p]]] -= F->lx[p] * yk;
  }
  /* backward: U z = y (U columns in position space, diagonal stored last) */
  for (int k = n - 1; k >= 0; --k) {
    int pd = F->up[k + 1] - 1;
    y[k] /= F->ux[pd];
    KO_T zk = y[k];
    for (int p = F->up[k]; p < pd; ++p) y[F->ui[p]] -= F->ux[p] * zk;
  }
  /* un-permute columns: position k solves original column q[k] */
  for (int k = 0; k < n; ++k) work[F->q[k]] = y[k];
  for (int i = 0; i < n; ++i) x[i] = work[i];
}

#undef KO_FN
#undef KO_CAT
#undef KO_CAT2
