// Host symbolic pass (see symbolic.h).
//
// Stamp emission follows crates/krets-solver/src/stampable.rs element by element and
// entry by entry, so that the device's segmented sums add duplicate (row, col) entries in
// the same order as the reference's HashMap `+=` (crates/krets-solver/src/solver.rs:59-70).
#include "symbolic.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <queue>
#include <unordered_map>

namespace krets {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kVt = 1.380649e-23 * 300.0 / 1.602176634e-19;

struct MEntry { int r, c, code; };  // code = packed contribution (pack_a)
struct BEntry { int r, code; };     // code = packed contribution (pack_b)

// Emit the matrix and rhs stamp entries of element e for the mode, in the reference's
// order.  Returns false for stamps the reference leaves as todo!().
// xs: first extra coefficient slot of the element (-1 = none).
bool emit(const krets_element &x, int e, int xs, int mode, std::vector<MEntry> &M, std::vector<BEntry> &B) {
  const int ip = x.p, im = x.m, ic = x.b;
  auto A = [&](int r, int c, bool unit, bool neg) { M.push_back({r, c, pack_a(e, unit, neg)}); };
  auto AS = [&](int r, int c, int slot, bool neg) { M.push_back({r, c, pack_a(slot, false, neg)}); };
  auto R = [&](int r, bool neg) { B.push_back({r, pack_b(e, neg)}); };
  switch (x.kind) {
    case KRETS_ELEM_R:  // stampable.rs:203-246
      if (x.flags & KRETS_FLAG_G2) {
        if (ip >= 0 && ic >= 0) { A(ip, ic, true, false); A(ic, ip, true, false); }
        if (im >= 0 && ic >= 0) { A(im, ic, true, true); A(ic, im, true, true); }
        if (ic >= 0) A(ic, ic, false, true);  // -R
      } else {
        if (ip >= 0) A(ip, ip, false, false);
        if (im >= 0) A(im, im, false, false);
        if (ip >= 0 && im >= 0) { A(ip, im, false, true); A(im, ip, false, true); }
      }
      return true;
    case KRETS_ELEM_C:  // stampable.rs:360-506
      if (mode == MODE_DC) return true;
      if (mode == MODE_AC && (x.flags & KRETS_FLAG_G2)) {
        if (ip >= 0 && ic >= 0) A(ic, ip, false, true);
        if (im >= 0 && ic >= 0) A(ic, im, false, false);
        if (ic >= 0) A(ic, ic, true, false);
        return true;
      }
      if (ip >= 0) A(ip, ip, false, false);
      if (im >= 0) A(im, im, false, false);
      if (ip >= 0 && im >= 0) { A(ip, im, false, true); A(im, ip, false, true); }
      if (mode == MODE_TRAN) {
        // BE: (p, -ieq), (m, ieq) with ieq = -(C/h) v_prev.  TR: (p, ihist), (m, -ihist).
        // The per-pass rhs coefficient is -ieq (BE) or ihist (TR): + at p, - at m.
        if (ip >= 0) R(ip, false);
        if (im >= 0) R(im, true);
      }
      return true;
    case KRETS_ELEM_I:  // stampable.rs:508-585
      if (mode == MODE_AC) {
        if (ip >= 0 && ic >= 0) A(ip, ic, true, false);
        if (im >= 0 && ic >= 0) A(im, ic, true, true);
      } else {
        if (ic >= 0) A(ic, ic, true, false);
        if (ip >= 0 && ic >= 0) A(ip, ic, true, false);
        if (im >= 0 && ic >= 0) A(im, ic, true, true);
      }
      if (ic >= 0) R(ic, false);
      return true;
    case KRETS_ELEM_D:  // stampable.rs:587-674
      if (ip >= 0) A(ip, ip, false, false);
      if (im >= 0) A(im, im, false, false);
      if (ip >= 0 && im >= 0) { A(ip, im, false, true); A(im, ip, false, true); }
      if (mode != MODE_AC) {
        // (p, -ieq), (m, ieq): per-pass rhs coefficient = ieq
        if (ip >= 0) R(ip, true);
        if (im >= 0) R(im, false);
      }
      return true;
    case KRETS_ELEM_L:  // stampable.rs:676-817
      if (mode == MODE_TRAN) {
        if (ic >= 0) A(ic, ic, false, true);
        if (ip >= 0 && ic >= 0) { A(ip, ic, true, false); A(ic, ip, true, false); }
        if (im >= 0 && ic >= 0) { A(im, ic, true, true); A(ic, im, true, true); }
        if (ic >= 0) R(ic, false);
        return true;
      }
      if (ip >= 0 && ic >= 0) A(ip, ic, true, false);
      if (im >= 0 && ic >= 0) A(im, ic, true, true);
      if (ip >= 0 && ic >= 0) A(ic, ip, true, false);
      if (im >= 0 && ic >= 0) A(ic, im, true, true);
      if (mode == MODE_AC && ic >= 0) A(ic, ic, false, true);
      return true;
    case KRETS_ELEM_V:  // stampable.rs:960-1050
      if (ip >= 0 && ic >= 0) { A(ip, ic, true, false); A(ic, ip, true, false); }
      if (im >= 0 && ic >= 0) { A(im, ic, true, true); A(ic, im, true, true); }
      if (ic >= 0) R(ic, false);
      return true;
    case KRETS_ELEM_M: {  // stampable.rs:819-922
      if (mode == MODE_AC) return false;                      // todo!() (:914-921)
      if (!(x.flags & KRETS_FLAG_NMOS_RESOLVED)) return true;  // bare-name lookups never match
      // slot e = g_ds + g_m, xs = g_ds, xs + 1 = g_m; the reference's entries in its order
      const int d = x.p, src = x.m, g = x.g;
      if (d >= 0) AS(d, d, xs, false);
      if (src >= 0) AS(src, src, e, false);
      if (d >= 0 && src >= 0) { AS(d, src, e, true); AS(src, d, e, false); }
      if (src >= 0 && g >= 0) AS(src, g, xs + 1, false);
      if (d >= 0 && g >= 0) AS(d, g, xs + 1, false);
      // rhs: (source, i_eq), (drain, -i_eq): per-pass rhs coefficient = i_eq
      if (src >= 0) R(src, false);
      if (d >= 0) R(d, true);
      return true;
    }
    default:
      return false;
  }
}

// Representative value of an element's matrix coefficient (for pivot selection only).
std::complex<double> rep_coef(const krets_element &x, int mode, int method, double h, double f,
                              bool rep_diode_zero) {
  switch (x.kind) {
    case KRETS_ELEM_R:
      return (x.flags & KRETS_FLAG_G2) ? x.value : 1.0 / x.value;
    case KRETS_ELEM_C:
      if (mode == MODE_AC) return std::complex<double>(0.0, 2.0 * kPi * f * x.value);
      return (method == KRETS_METHOD_TR ? 2.0 : 1.0) * x.value / h;
    case KRETS_ELEM_L:
      if (mode == MODE_AC) return std::complex<double>(0.0, 2.0 * kPi * f * x.value);
      return (method == KRETS_METHOD_TR ? 2.0 : 1.0) * x.value / h;
    case KRETS_ELEM_D:
      // A diode's conductance spans ~150 decades between reverse and forward bias, so
      // pivots must not rely on it: it is taken as 0 (the caller retries with the 0.5 V
      // value only if the matrix is singular without it).
      if (rep_diode_zero) return 0.0;
      {
        double n = x.wp[0] > 0 ? x.wp[0] : 1.0;
        return (x.value / (n * kVt)) * std::exp(std::min(0.5 / (n * kVt), 700.0));
      }
    case KRETS_ELEM_M:
      // NMOS conductances are 0 below threshold, which the first Newton iteration sees
      // (all guesses 0): pivots do not rely on them, as for diodes
      return rep_diode_zero ? 0.0 : 1.0;
    default:
      return 1.0;
  }
}

// ------------------------------------------------------------ Gilbert-Peierls LU
// Left-looking LU with threshold partial pivoting (diagonal preferred), used on the
// representative values to fix the pivot sequence and the static fill pattern.
struct GP {
  int n;
  std::vector<int> lp, li, up, ui, pinv;
  double min_ratio = 1.0;
};

constexpr int kFillCapExceeded = -100;  // gp_factor gave up: more L+U entries than the cap
constexpr int kMinDenseTail = 64;       // smallest dense trailing block solved as a dense block

// dense_from < n: columns dense_from .. n-1 of the ordering form a clique of the
// elimination graph (minimum degree's last vertices), so their Schur complement is
// structurally dense.  They are finished by a dense right-looking LU with the same
// pivoting rule: each such column is first reduced by the sparse pivots only (the
// left-looking steps below, without choosing a pivot), and the remaining c x c block is
// factored in place; its L and U patterns are the full block.  This replaces the
// left-looking steps' O(c^3) graph traversals and scattered updates for that block.
template <typename T>
int gp_factor(int n, const std::vector<int> &ap, const std::vector<int> &ai, const std::vector<T> &ax,
              const std::vector<int> &q, double tau, GP &F, size_t fill_cap = 0, int dense_from = -1) {
  F.n = n;
  F.lp.assign(n + 1, 0);
  F.up.assign(n + 1, 0);
  F.li.clear();
  F.ui.clear();
  F.pinv.assign(n, -1);
  std::vector<T> lx, xv(n, T(0));
  std::vector<int> mark(n, -1), stack(n), pstack(n), reach(n);
  const int kd = (dense_from >= 0 && dense_from < n) ? dense_from : n;
  // reach of column col among the finished pivots (marks with stamp k), in topological
  // order at reach[top..n); returns top
  auto find_reach = [&](int col, int k) {
    int top = n;
    for (int p = ap[col]; p < ap[col + 1]; ++p) {
      int r0 = ai[p];
      if (mark[r0] == k) continue;
      int head = 0;
      stack[0] = r0;
      while (head >= 0) {
        int j = stack[head];
        int jp = F.pinv[j];
        if (mark[j] != k) {
          mark[j] = k;
          pstack[head] = jp < 0 ? 0 : F.lp[jp];
        }
        bool done = true;
        if (jp >= 0) {
          int end = F.lp[jp + 1];
          for (int pp = pstack[head]; pp < end; ++pp) {
            int i = F.li[pp];
            if (mark[i] == k) continue;
            pstack[head] = pp + 1;
            stack[++head] = i;
            done = false;
            break;
          }
        }
        if (done) {
          --head;
          reach[--top] = j;
        }
      }
    }
    return top;
  };
  for (int k = 0; k < kd; ++k) {
    F.lp[k] = (int)F.li.size();
    F.up[k] = (int)F.ui.size();
    int col = q[k];
    int top = n;
    for (int p = ap[col]; p < ap[col + 1]; ++p) {
      int r0 = ai[p];
      if (mark[r0] == k) continue;
      int head = 0;
      stack[0] = r0;
      while (head >= 0) {
        int j = stack[head];
        int jp = F.pinv[j];
        if (mark[j] != k) {
          mark[j] = k;
          pstack[head] = jp < 0 ? 0 : F.lp[jp];
        }
        bool done = true;
        if (jp >= 0) {
          int end = F.lp[jp + 1];
          for (int pp = pstack[head]; pp < end; ++pp) {
            int i = F.li[pp];
            if (mark[i] == k) continue;
            pstack[head] = pp + 1;
            stack[++head] = i;
            done = false;
            break;
          }
        }
        if (done) {
          --head;
          reach[--top] = j;
        }
      }
    }
    for (int p = top; p < n; ++p) xv[reach[p]] = T(0);
    for (int p = ap[col]; p < ap[col + 1]; ++p) xv[ai[p]] += ax[p];
    for (int p = top; p < n; ++p) {
      int j = reach[p];
      int jp = F.pinv[j];
      if (jp < 0) continue;
      T xj = xv[j];
      for (int pp = F.lp[jp]; pp < F.lp[jp + 1]; ++pp) xv[F.li[pp]] -= lx[pp] * xj;
    }
    int ipiv = -1;
    double amax = -1.0;
    for (int p = top; p < n; ++p) {
      int i = reach[p];
      if (F.pinv[i] < 0) {
        double a = std::abs(xv[i]);
        if (a > amax) { amax = a; ipiv = i; }
      } else {
        F.ui.push_back(F.pinv[i]);
      }
    }
    if (fill_cap && F.li.size() + F.ui.size() > fill_cap) return kFillCapExceeded;
    if (ipiv < 0) return KRETS_ERR_DECOMPOSITION_FAILED;  // structurally singular column
    if (!(amax > 0.0) || !std::isfinite(amax)) return KRETS_ERR_DECOMPOSITION_FAILED;
    // diagonal preference: keep the row paired with this column if it is large enough
    if (F.pinv[col] < 0 && mark[col] == k && std::abs(xv[col]) >= tau * amax) ipiv = col;
    F.min_ratio = std::min(F.min_ratio, std::abs(xv[ipiv]) / amax);
    T piv = xv[ipiv];
    F.ui.push_back(k);
    F.pinv[ipiv] = k;
    for (int p = top; p < n; ++p) {
      int i = reach[p];
      if (F.pinv[i] < 0) {
        F.li.push_back(i);
        lx.push_back(xv[i] / piv);
      }
      xv[i] = T(0);
    }
  }
  if (kd < n) {
    const int c = n - kd;
    std::vector<int> R, rpos(n, -1);  // the rows without a pivot, and their block position
    for (int r = 0; r < n; ++r)
      if (F.pinv[r] < 0) {
        rpos[r] = (int)R.size();
        R.push_back(r);
      }
    if ((int)R.size() != c) return KRETS_ERR_DECOMPOSITION_FAILED;
    std::vector<T> S((size_t)c * c, T(0));  // S[j c + i]: block column j, row R[i]
    std::vector<std::vector<int>> usp(c);  // sparse pivots each block column reaches
    for (int j = 0; j < c; ++j) {
      const int k = kd + j, col = q[k];
      const int top = find_reach(col, k);
      for (int p = top; p < n; ++p) xv[reach[p]] = T(0);
      for (int p = ap[col]; p < ap[col + 1]; ++p) xv[ai[p]] += ax[p];
      for (int p = top; p < n; ++p) {
        const int jr = reach[p], jp = F.pinv[jr];
        if (jp < 0) continue;
        const T xj = xv[jr];
        for (int pp = F.lp[jp]; pp < F.lp[jp + 1]; ++pp) xv[F.li[pp]] -= lx[pp] * xj;
      }
      for (int p = top; p < n; ++p) {
        const int i = reach[p];
        if (F.pinv[i] >= 0) usp[j].push_back(F.pinv[i]);
        else S[(size_t)j * c + rpos[i]] = xv[i];
        xv[i] = T(0);
      }
    }
    // Right-looking, by columns (contiguous over the rows).  The pivot row is swapped to
    // position j of the columns still to come, so the rows without a pivot stay
    // contiguous at j+1 .. c and the updates touch only them (c^3/3 multiply-adds instead
    // of c^3/2); orig[] keeps each position's block row, and ties in the pivot search go
    // to the lowest block row, as a scan in block-row order would choose.
    std::vector<int> piv_row(c), orig(c), where(c);
    std::iota(orig.begin(), orig.end(), 0);
    std::iota(where.begin(), where.end(), 0);
    std::vector<T> L4((size_t)4 * c, T(0));  // the multipliers of the current group of four pivots
    for (int j = 0; j < c; ++j) {
      const int k = kd + j, col = q[k];
      T *cj = S.data() + (size_t)j * c;
      int ip = -1;
      double amax = -1.0;
      for (int i = j; i < c; ++i) {
        const double a = std::abs(cj[i]);
        if (a > amax || (a == amax && ip >= 0 && orig[i] < orig[ip])) { amax = a; ip = i; }
      }
      if (ip < 0 || !(amax > 0.0) || !std::isfinite(amax)) return KRETS_ERR_DECOMPOSITION_FAILED;
      const int dr = rpos[col];  // diagonal preference, as in the sparse steps
      if (dr >= 0 && where[dr] >= j && std::abs(cj[where[dr]]) >= tau * amax) ip = where[dr];
      const T piv = cj[ip];
      F.min_ratio = std::min(F.min_ratio, std::abs(piv) / amax);
      piv_row[j] = orig[ip];
      F.pinv[R[orig[ip]]] = k;
      if (ip != j) {
        for (int jj = j; jj < c; ++jj) std::swap(S[(size_t)jj * c + ip], S[(size_t)jj * c + j]);
        for (int t = 0; t < (j & 3); ++t)  // the group's earlier multipliers follow their rows
          std::swap(L4[(size_t)t * c + ip], L4[(size_t)t * c + j]);
        std::swap(orig[ip], orig[j]);
        where[orig[ip]] = ip;
        where[orig[j]] = j;
      }
      T *__restrict__ lc = L4.data() + (size_t)(j & 3) * c;
      for (int i = j + 1; i < c; ++i) lc[i] = cj[i] / piv;
      // Columns inside the current group of four are updated at once (their next pivot
      // is chosen from them); the columns after the group take the group's four updates
      // in one pass when the group is complete (or the block ends), in pivot order with
      // the same operations per element, so the values are those of one update at a time
      // (an update whose multiplier u is zero is skipped, as there).
      const int g0 = j & ~3, g1 = std::min(g0 + 4, c);
      for (int jj = j + 1; jj < g1; ++jj) {
        T *__restrict__ cc = S.data() + (size_t)jj * c;
        const T u = cc[j];
        if (u == T(0)) continue;
        for (int i = j + 1; i < c; ++i) cc[i] -= lc[i] * u;
      }
      if (j + 1 == g1) {  // the group's pivots g0 .. j are known: update the columns after it
        const int np = j + 1 - g0;
        for (int jj = g1; jj < c; ++jj) {
          T *__restrict__ cc = S.data() + (size_t)jj * c;
          T u[4];
          bool all = true;
          for (int t = 0; t < np; ++t) {  // the pivot rows' values after the earlier pivots
            const int pr = g0 + t;
            T v = cc[pr];
            for (int t2 = 0; t2 < t; ++t2)
              if (u[t2] != T(0)) v -= L4[(size_t)t2 * c + pr] * u[t2];
            u[t] = v;
            all = all && v != T(0);
          }
          if (all && np == 4) {
            const T *__restrict__ l0 = L4.data(), *__restrict__ l1 = l0 + c, *__restrict__ l2 = l1 + c,
                                  *__restrict__ l3 = l2 + c;
            for (int t = 1; t < 4; ++t) cc[g0 + t] = u[t];
            for (int i = g1; i < c; ++i) {
              T x = cc[i];
              x -= l0[i] * u[0];
              x -= l1[i] * u[1];
              x -= l2[i] * u[2];
              x -= l3[i] * u[3];
              cc[i] = x;
            }
          } else {
            for (int t = 0; t < np; ++t) {
              if (u[t] == T(0)) continue;
              const T *__restrict__ lt = L4.data() + (size_t)t * c;
              for (int i = g0 + t + 1; i < c; ++i) cc[i] -= lt[i] * u[t];
            }
          }
        }
      }
    }
    // patterns: U column k = the sparse pivots it reaches, every earlier block pivot and
    // its own pivot; L column k = the block rows not pivoted yet
    std::vector<char> done(c, 0);
    for (int j = 0; j < c; ++j) {
      const int k = kd + j;
      F.lp[k] = (int)F.li.size();
      F.up[k] = (int)F.ui.size();
      F.ui.insert(F.ui.end(), usp[j].begin(), usp[j].end());
      for (int t = 0; t < j; ++t) F.ui.push_back(kd + t);
      F.ui.push_back(k);
      done[piv_row[j]] = 1;
      for (int i = 0; i < c; ++i)
        if (!done[i]) F.li.push_back(R[i]);
      if (fill_cap && F.li.size() + F.ui.size() > fill_cap) return kFillCapExceeded;
    }
  }
  F.lp[n] = (int)F.li.size();
  F.up[n] = (int)F.ui.size();
  return KRETS_OK;
}

uint64_t fnv1a(uint64_t h, uint64_t v) {
  for (int k = 0; k < 8; ++k) {
    h ^= (v >> (8 * k)) & 0xff;
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace

// ------------------------------------------------------------------ orderings
std::vector<int> order_min_degree(int n, const std::vector<std::vector<int>> &adj0, int *clique) {
  // Explicit elimination graph; the next vertex is the one of least current degree, the
  // smallest index among equals, found through a min-heap of (degree, vertex) entries
  // whose stale entries (a vertex's degree changed since) are skipped when they surface.
  // Once at most 4096 vertices remain and the eliminated vertex has 24 or more
  // neighbours, the remaining graph moves to bit rows (one bit per remaining vertex):
  // merging a neighbourhood is then a few word ORs instead of a sorted-list union, and
  // degrees (popcounts) are the same, so the order is the same.
  std::vector<std::vector<int>> adj = adj0;
  if (clique) *clique = 0;
  std::vector<char> gone(n, 0);
  std::vector<int> order, deg(n);
  order.reserve(n);
  using Key = std::pair<int, int>;
  std::priority_queue<Key, std::vector<Key>, std::greater<Key>> heap;
  for (int v = 0; v < n; ++v) {
    deg[v] = (int)adj[v].size();
    heap.push({deg[v], v});
  }
  std::vector<int> merged;
  bool bit_rows = false;
  int W = 0;
  std::vector<int> cid(n, -1), orig;  // bit-row phase: compact index of a vertex, and back
  std::vector<uint64_t> bits, nbrow;
  for (int step = 0; step < n; ++step) {
    int best = -1;
    while (!heap.empty()) {
      const Key top = heap.top();
      heap.pop();
      if (!gone[top.second] && deg[top.second] == top.first) {
        best = top.second;
        break;
      }
    }
    const int bd = deg[best];
    if (bd + 1 == n - step) {
      // every remaining vertex is adjacent to all others: a clique, whose vertices the
      // selection would take in increasing index order (equal degrees throughout)
      for (int v = 0; v < n; ++v)
        if (!gone[v]) order.push_back(v);
      if (clique) *clique = n - step;
      break;
    }
    if (!bit_rows && n - step <= 4096 && bd >= 24) {
      for (int v = 0; v < n; ++v)
        if (!gone[v]) {
          cid[v] = (int)orig.size();
          orig.push_back(v);
        }
      W = ((int)orig.size() + 63) / 64;
      bits.assign(orig.size() * (size_t)W, 0);
      for (size_t i = 0; i < orig.size(); ++i) {
        for (int u : adj[orig[i]]) bits[i * W + (cid[u] >> 6)] |= 1ull << (cid[u] & 63);
        std::vector<int>().swap(adj[orig[i]]);
      }
      nbrow.resize(W);
      bit_rows = true;
    }
    gone[best] = 1;
    order.push_back(best);
    if (bit_rows) {
      const int b = cid[best];
      std::copy(bits.begin() + (size_t)b * W, bits.begin() + (size_t)(b + 1) * W, nbrow.begin());
      for (int w = 0; w < W; ++w)
        for (uint64_t x = nbrow[w]; x; x &= x - 1) {
          const int i = w * 64 + __builtin_ctzll(x);
          uint64_t *row = bits.data() + (size_t)i * W;
          int d = 0;
          for (int t = 0; t < W; ++t) {
            row[t] |= nbrow[t];
            if (t == (i >> 6)) row[t] &= ~(1ull << (i & 63));
            if (t == (b >> 6)) row[t] &= ~(1ull << (b & 63));
            d += __builtin_popcountll(row[t]);
          }
          const int u = orig[i];
          if (d != deg[u]) {
            deg[u] = d;
            heap.push({d, u});
          }
        }
      continue;
    }
    const std::vector<int> nb = adj[best];
    for (int u : nb) {
      merged.clear();
      merged.reserve(adj[u].size() + nb.size());
      std::set_union(adj[u].begin(), adj[u].end(), nb.begin(), nb.end(), std::back_inserter(merged));
      merged.erase(std::remove_if(merged.begin(), merged.end(), [&](int w) { return w == u || w == best; }),
                   merged.end());
      const bool changed = merged.size() != adj[u].size();
      adj[u].assign(merged.begin(), merged.end());
      deg[u] = (int)adj[u].size();
      if (changed) heap.push({deg[u], u});
    }
    adj[best].clear();
  }
  return order;
}

std::vector<int> order_nested_dissection(int n, const std::vector<std::vector<int>> &adj, int *top_sep,
                                         int max_top_sep) {
  // max_top_sep > 0: stop as soon as the first separator is larger (the caller then
  // discards the ordering; *top_sep reports the size)
  if (top_sep) *top_sep = 0;
  bool stop = false, first_done = false;
  std::vector<int> order;
  order.reserve(n);
  std::vector<int> in_set(n, -1), level(n, -1);
  int stamp = 0;
  const int kLeaf = 1;
  // explicit stack of vertex sets to avoid deep recursion
  std::function<void(std::vector<int> &)> nd = [&](std::vector<int> &V) {
    if (stop) return;
    if ((int)V.size() <= kLeaf) {
      std::sort(V.begin(), V.end());
      order.insert(order.end(), V.begin(), V.end());
      return;
    }
    int id = ++stamp;
    for (int v : V) in_set[v] = id;
    // connected components of V
    std::vector<std::vector<int>> comps;
    int cid = ++stamp;
    for (int s : V) {
      if (in_set[s] != id) continue;
      std::vector<int> comp{s};
      in_set[s] = cid;
      for (size_t h = 0; h < comp.size(); ++h)
        for (int w : adj[comp[h]])
          if (in_set[w] == id) { in_set[w] = cid; comp.push_back(w); }
      comps.push_back(std::move(comp));
    }
    for (auto &C : comps) {
      if ((int)C.size() <= kLeaf) {
        std::sort(C.begin(), C.end());
        order.insert(order.end(), C.begin(), C.end());
        continue;
      }
      int mid = ++stamp;
      for (int v : C) in_set[v] = mid;
      auto bfs = [&](int root, std::vector<std::vector<int>> &levels) {
        levels.clear();
        int bid = ++stamp;
        std::vector<int> cur{root};
        in_set[root] = bid;
        while (!cur.empty()) {
          levels.push_back(cur);
          std::vector<int> nxt;
          for (int v : cur)
            for (int w : adj[v])
              if (in_set[w] == mid) { in_set[w] = bid; nxt.push_back(w); }
          cur.swap(nxt);
        }
        for (int v : C) in_set[v] = mid;
      };
      std::vector<std::vector<int>> levels;
      int root = *std::min_element(C.begin(), C.end());
      for (int rep = 0; rep < 3; ++rep) {  // pseudo-peripheral root
        bfs(root, levels);
        const auto &last = levels.back();
        int cand = last[0];
        for (int v : last)
          if (adj[v].size() < adj[cand].size()) cand = v;
        if (cand == root) break;
        root = cand;
      }
      bfs(root, levels);
      int L = (int)levels.size();
      if (L < 3) {
        std::sort(C.begin(), C.end());
        order.insert(order.end(), C.begin(), C.end());
        continue;
      }
      // separator: smallest level in the middle third (by vertex count)
      std::vector<int> cum(L + 1, 0);
      for (int l = 0; l < L; ++l) cum[l + 1] = cum[l] + (int)levels[l].size();
      // smallest separator level in the middle half; among equally small ones, the most
      // balanced split (keeps the elimination tree shallow)
      int total = cum[L], best = -1;
      auto imbalance = [&](int l) { return std::abs(cum[l] - (total - cum[l + 1])); };
      for (int l = 1; l < L - 1; ++l) {
        if (cum[l] < total / 4 || cum[l + 1] > total - total / 4) continue;
        if (best < 0 || levels[l].size() < levels[best].size() ||
            (levels[l].size() == levels[best].size() && imbalance(l) < imbalance(best)))
          best = l;
      }
      if (best < 0) {
        best = 1;
        while (best < L - 2 && cum[best + 1] < total / 2) ++best;
      }
      std::vector<int> A, B;
      for (int l = 0; l < best; ++l) A.insert(A.end(), levels[l].begin(), levels[l].end());
      for (int l = best + 1; l < L; ++l) B.insert(B.end(), levels[l].begin(), levels[l].end());
      std::vector<int> S = levels[best];
      if (!first_done) {  // the first separator found
        first_done = true;
        if (top_sep) *top_sep = (int)S.size();
        if (max_top_sep > 0 && (int)S.size() > max_top_sep) {
          stop = true;
          return;
        }
      }
      nd(A);
      nd(B);
      std::sort(S.begin(), S.end());
      order.insert(order.end(), S.begin(), S.end());
    }
  };
  std::vector<int> all(n);
  std::iota(all.begin(), all.end(), 0);
  nd(all);
  return order;
}

// ------------------------------------------------------------------ step program
// Compact, shared-memory resident form of everything the per-step loop reads:
//   [0] lev_ptr[nlev+1]      [1] ulev_ptr[nulev+1]
//   [2] ldesc[n] int4, level order   [3] udesc[n] int4, U-level order
//       {row | rest << 16, base slot, col0 | col1 << 16, nfast}: the first nfast (<= 2)
//       entries of the row's L part (U part) are at base, base+1 (base+1, base+2 after the
//       diagonal at base) with columns col0, col1; the remaining `rest` entries follow
//       contiguously and take their columns from lu_col
//   [4] lu_col[nnz_lu] as uint16 pairs
//   [7] dyn[ndyn] int4 {e | kind << 24, p, m, b} (positions, -1 absent)
//   [8] bd_ptr[n+1]   [9] bd_op (dyn << 1 | neg)   [10] qinv[n]
//   [12] lmax[nlev], [13] umax[nulev]: split code of each L / U level (split_code: lanes per
//        row by group size, longest row)
//   [14] border chunks, [15] border rows (dense trailing block only; see below)
//   [5] res_row[n] int2 {first op, n_unit | n_total << 16}
//   [6] res_op: col | neg << 15 | slot << 16 (slot 0 = incidence +-1 entries, listed first;
//       slot e+1 = coefficient of element e)
//   [11] end
// (in this physical order: sp_off[5] ends the part that the direct engines stage)
// Per-level split code: bits 3g..3g+2 hold log2 of the lanes per row a group of 32 << g
// threads uses (g = 0..4, up to 8 lanes), bits 15..17 the same for a 256-thread group
// allowed a whole warp per row (the multi-circuit engine's global-memory class, whose
// long rows read global memory), bits 18.. the longest row (clamped).  A level's rows
// are split over more lanes while a row has more than two entries per lane and the level
// still fits the group.  The device reads the code; the rule lives here only.
static int split_code(int rows, int mx) {
  int code = std::min(mx, 16383) << 18;
  for (int g = 0; g < 6; ++g) {
    const int G = g == 5 ? 256 : 32 << g, cap = g == 5 ? 32 : 8;
    int s = 1, lg = 0;
    while (s < cap && mx > 2 * s && rows * s * 2 <= G) {
      s *= 2;
      ++lg;
    }
    code |= lg << (3 * g);
  }
  return code;
}

// Interleaved ("ELL per level") form of the L and U solves for the double-float engine
// with its factors in global memory.  Within a level, lane lam of the level's W = rows x
// lanes-per-row lanes handles row lam / spl and its entries j = lam % spl + i * spl; entry
// slot i of every lane of the level is stored contiguously (first slot + i * W + lam), so
// a warp's loads of one slot are consecutive addresses, and so are the columns in shared
// memory (one column per entry slot).  The U rows' reciprocal diagonals follow all entry
// slots.  Lanes with fewer entries than the level's longest are padded with zero entries,
// which leave the double-float sums unchanged bit for bit; the entries of a row are
// visited in the same order as by the row-descriptor solves (df_level, df_level_split),
// so both forms give identical results.  Lanes per row are the split of the
// row-descriptor program for the group size (split_code).  A level of at most 32 lanes
// runs on the group's first warp alone (flag bit 0); when the next level does too, a warp
// barrier separates them instead of a group barrier (bit 1).
static void pack_interleaved(Program &P) {
  P.iprog.clear();
  P.imap.clear();
  P.il_ok = false;
  if (!P.sprog_ok || P.tail_m || P.n > 65535) return;
  const int *lmax = P.sprog.data() + P.sp_off[12], *umax = P.sprog.data() + P.sp_off[13];
  const int nlev = (int)P.lev_ptr.size() - 1, nulev = (int)P.ulev_ptr.size() - 1;
  for (int gi = 0; gi < 3; ++gi) {
    const int g = gi == 0 ? 1 : gi == 1 ? 2 : 0;  // split-code field of 64 / 128 / 32-thread groups
    std::vector<int> rec, rows, emap, dmap;
    std::vector<unsigned short> cols;
    auto level = [&](bool upper, int l) {
      const int *ptr = upper ? P.ulev_ptr.data() : P.lev_ptr.data();
      const int *rw = upper ? P.ulev_rows.data() : P.lev_rows.data();
      const int code = upper ? umax[l] : lmax[l];
      const int lsh = (code >> (3 * g)) & 7, spl = 1 << lsh;
      const int nr = ptr[l + 1] - ptr[l], W = nr * spl;
      auto first = [&](int k) { return upper ? P.lu_diag[k] + 1 : P.lu_rowptr[k]; };
      auto count = [&](int k) { return upper ? P.lu_rowptr[k + 1] - P.lu_diag[k] - 1 : P.lu_diag[k] - P.lu_rowptr[k]; };
      int mc = 0;
      for (int t = ptr[l]; t < ptr[l + 1]; ++t) mc = std::max(mc, (count(rw[t]) + spl - 1) / spl);
      rec.insert(rec.end(), {W, lsh, mc, (int)emap.size(), (int)rows.size(), upper ? (int)dmap.size() : -1, 0, 0});
      for (int i = 0; i < mc; ++i)
        for (int lam = 0; lam < W; ++lam) {
          const int k = rw[ptr[l] + lam / spl], j = lam % spl + i * spl;
          const bool real = j < count(k);
          emap.push_back(real ? first(k) + j : -1);
          cols.push_back((unsigned short)(real ? P.lu_col[first(k) + j] : k));
        }
      for (int t = ptr[l]; t < ptr[l + 1]; ++t) rows.push_back(rw[t]);
      if (upper)  // reciprocal diagonals of the level's rows
        for (int t = ptr[l]; t < ptr[l + 1]; ++t) dmap.push_back(P.lu_diag[rw[t]]);
    };
    for (int l = 1; l < nlev; ++l) level(false, l);  // L level 0 rows have no L entries
    for (int l = 0; l < nulev; ++l) level(true, l);
    const int nrec = (int)rec.size() / 8, eslots = (int)emap.size();
    for (int r = 0; r < nrec; ++r) {
      int *R = rec.data() + 8 * r;
      if (R[5] >= 0) R[5] += eslots;  // diagonals after the entry slots
      const bool narrow = R[0] <= 32, next_narrow = r + 1 < nrec && R[8] <= 32;
      R[6] = (narrow ? 1 : 0) | (narrow && next_narrow ? 2 : 0);
    }
    P.n_il_lrec = std::max(0, nlev - 1);
    P.n_il_urec = nulev;
    P.il_slots[gi] = eslots + (int)dmap.size();
    P.imap_off[gi] = (int)P.imap.size();
    P.imap.insert(P.imap.end(), emap.begin(), emap.end());
    P.imap.insert(P.imap.end(), dmap.begin(), dmap.end());
    while (P.iprog.size() % 4) P.iprog.push_back(0);
    P.ip_off[gi][0] = (int)P.iprog.size();
    P.iprog.insert(P.iprog.end(), rec.begin(), rec.end());
    while (P.iprog.size() % 4) P.iprog.push_back(0);
    P.ip_off[gi][1] = (int)P.iprog.size();
    P.iprog.insert(P.iprog.end(), rows.begin(), rows.end());
    while (P.iprog.size() % 4) P.iprog.push_back(0);
    P.ip_off[gi][2] = (int)P.iprog.size();
    for (size_t i = 0; i < cols.size(); i += 2)
      P.iprog.push_back((int)cols[i] | (i + 1 < cols.size() ? (int)cols[i + 1] << 16 : 0));
    while (P.iprog.size() % 4) P.iprog.push_back(0);
    P.ip_off[gi][3] = (int)P.iprog.size();
  }
  P.il_ok = true;
}

// Direct right-hand side of the double-float engine's interleaved step: when no row of
// the right-hand side takes more than one element's companion source, every element
// writes its value straight into the rows it feeds (no gather pass), and the rows that
// no element feeds are zeroed.  Appended to iprog at lean_off: one int4 per dynamic
// element, in dyn order (capacitors, then inductors, then the other sources),
//   capacitor  {node p, node m, row +, row -}
//   inductor   {node p, node m, branch position, row << 1 | negated}
//   other      {e | kind << 24, 0, row +, row -}
// with position n for a ground node (the state holds a zero there) and n + 1 for a row
// that is not fed (a write-only scratch slot); then the rows no element feeds.
static void pack_lean(const krets_element *el, Program &P) {
  P.lean_ok = false;
  P.lean_off = P.n_zrow = 0;
  if (!P.il_ok) return;
  const int n = P.n, nd = (int)P.dyn_e.size(), sink = n + 1;
  std::vector<std::vector<int>> feeds(nd);  // per element: row << 1 | negated
  std::vector<int> zrow;
  for (int k = 0; k < n; ++k) {
    const int cnt = P.bd_ptr[k + 1] - P.bd_ptr[k];
    if (cnt > 1) return;
    if (cnt == 0) zrow.push_back(k);
    else feeds[P.bd_op[P.bd_ptr[k]] >> 1].push_back(k << 1 | (P.bd_op[P.bd_ptr[k]] & 1));
  }
  std::vector<int> L;
  for (int d = 0; d < nd; ++d) {
    const int e = P.dyn_e[d], kind = el[e].kind;
    const bool cap = d < P.ncap, ind = d >= P.ncap && d < P.ncap + P.n_ind;
    if (cap != (kind == KRETS_ELEM_C) || ind != (kind == KRETS_ELEM_L)) return;
    if (kind != KRETS_ELEM_C && kind != KRETS_ELEM_L && kind != KRETS_ELEM_V && kind != KRETS_ELEM_I) return;
    const std::vector<int> &f = feeds[d];
    int rp = sink, rm = sink;
    if (kind == KRETS_ELEM_L || kind == KRETS_ELEM_V) {
      if (f.size() > 1) return;
    } else if (f.size() > 2 || (f.size() == 2 && (f[0] & 1) == (f[1] & 1))) {
      return;
    }
    for (int v : f) ((v & 1) ? rm : rp) = v >> 1;
    auto node = [&](int pos) { return pos < 0 ? n : pos; };
    const int p = node(P.el_pos[4 * e + 0]), m = node(P.el_pos[4 * e + 1]);
    if (kind == KRETS_ELEM_C) {
      L.insert(L.end(), {p, m, rp, rm});
    } else if (kind == KRETS_ELEM_L) {
      if (P.el_pos[4 * e + 2] < 0) return;
      L.insert(L.end(), {p, m, P.el_pos[4 * e + 2], f.empty() ? sink << 1 : f[0]});
    } else {
      L.insert(L.end(), {e | (kind << 24), 0, rp, rm});
    }
  }
  while (P.iprog.size() % 4) P.iprog.push_back(0);
  P.lean_off = (int)P.iprog.size();
  P.iprog.insert(P.iprog.end(), L.begin(), L.end());
  P.iprog.insert(P.iprog.end(), zrow.begin(), zrow.end());
  while (P.iprog.size() % 4) P.iprog.push_back(0);
  P.n_zrow = (int)zrow.size();
  P.lean_ok = true;
}

static void pack_step_program(const krets_element *el, Program &P) {
  const int n = P.n;
  P.sprog.clear();
  // the step-program engines run linear circuits with one coefficient per element
  P.sprog_ok = n < 32768 && P.ne < 65535 && P.max_row_lu < 32768 && P.n_coef == P.ne;
  if (!P.sprog_ok) return;
  std::vector<int> &S = P.sprog;
  auto mark = [&](int i) {
    while (S.size() % 4) S.push_back(0);  // 16-byte alignment of each section
    P.sp_off[i] = (int)S.size();
  };
  auto desc = [&](int k, int first, int cnt, int base) {
    const int nf = std::min(cnt, 2);
    const int c0 = nf > 0 ? P.lu_col[first] : k, c1 = nf > 1 ? P.lu_col[first + 1] : k;
    S.insert(S.end(), {k | ((cnt - nf) << 16), base, c0 | (c1 << 16), nf});
  };
  mark(0);
  S.insert(S.end(), P.lev_ptr.begin(), P.lev_ptr.end());
  mark(1);
  S.insert(S.end(), P.ulev_ptr.begin(), P.ulev_ptr.end());
  // L entries a row's descriptor covers: the whole L part, or for a row of the dense
  // trailing block only its columns before the block
  auto lcount = [&](int k) {
    return (P.tail_m && k >= P.tail0) ? P.lu_rowptr[k + 1] - P.tail_m - P.lu_rowptr[k] : P.lu_diag[k] - P.lu_rowptr[k];
  };
  mark(2);
  for (size_t t = 0; t < P.lev_rows.size(); ++t) {
    int k = P.lev_rows[t];
    desc(k, P.lu_rowptr[k], lcount(k), P.lu_rowptr[k]);
  }
  // U entries a row's descriptor covers: for rows before a dense trailing block, only the
  // columns before it (the block's columns, the border, are a separate parallel phase)
  auto ucount = [&](int k) {
    int e = P.lu_rowptr[k + 1];
    if (P.tail_m)
      while (e > P.lu_diag[k] + 1 && P.lu_col[e - 1] >= P.tail0) --e;
    return e - P.lu_diag[k] - 1;
  };
  mark(3);
  for (size_t t = 0; t < P.ulev_rows.size(); ++t) {
    int k = P.ulev_rows[t];
    desc(k, P.lu_diag[k] + 1, ucount(k), P.lu_diag[k]);
  }
  mark(4);
  for (size_t u = 0; u < P.lu_col.size(); u += 2) {
    int lo = P.lu_col[u], hi = u + 1 < P.lu_col.size() ? P.lu_col[u + 1] : 0;
    S.push_back(lo | (hi << 16));
  }
  mark(7);
  for (int e : P.dyn_e) {
    S.push_back(e | (el[e].kind << 24));
    S.push_back(P.el_pos[4 * e + 0]);
    S.push_back(P.el_pos[4 * e + 1]);
    S.push_back(P.el_pos[4 * e + 2]);
  }
  mark(8);
  S.insert(S.end(), P.bd_ptr.begin(), P.bd_ptr.end());
  mark(9);
  S.insert(S.end(), P.bd_op.begin(), P.bd_op.end());
  mark(10);
  S.insert(S.end(), P.qinv.begin(), P.qinv.end());
  // longest row (entries besides the diagonal) of each L level and each U level
  mark(12);
  for (size_t l = 0; l + 1 < P.lev_ptr.size(); ++l) {
    int mx = 0;
    for (int t = P.lev_ptr[l]; t < P.lev_ptr[l + 1]; ++t) {
      const int k = P.lev_rows[t];
      mx = std::max(mx, lcount(k));
    }
    S.push_back(split_code(P.lev_ptr[l + 1] - P.lev_ptr[l], mx));
  }
  mark(13);
  for (size_t l = 0; l + 1 < P.ulev_ptr.size(); ++l) {
    int mx = 0;
    for (int t = P.ulev_ptr[l]; t < P.ulev_ptr[l + 1]; ++t) {
      const int k = P.ulev_rows[t];
      mx = std::max(mx, ucount(k));
    }
    S.push_back(split_code(P.ulev_ptr[l + 1] - P.ulev_ptr[l], mx));
  }
  // [14] border chunks {first slot, count <= 16}, [15] border rows {row, first chunk,
  // chunks, 0}, for rows before a dense trailing block with entries in its columns
  P.n_bchunk = P.n_brow = 0;
  std::vector<int> chunks, brows;
  if (P.tail_m) {
    for (int k = 0; k < P.tail0; ++k) {
      const int b0 = P.lu_diag[k] + 1 + ucount(k), b1 = P.lu_rowptr[k + 1];
      if (b0 >= b1) continue;
      brows.insert(brows.end(), {k, (int)chunks.size() / 2, 0, 0});
      for (int c = b0; c < b1; c += 16) chunks.insert(chunks.end(), {c, std::min(16, b1 - c)});
      brows[brows.size() - 2] = (int)chunks.size() / 2 - brows[brows.size() - 3];
    }
    P.n_bchunk = (int)chunks.size() / 2;
    P.n_brow = (int)brows.size() / 4;
  }
  mark(14);
  S.insert(S.end(), chunks.begin(), chunks.end());
  mark(15);
  S.insert(S.end(), brows.begin(), brows.end());
  // the residual operators come last: the direct engines stage only the words before them
  mark(5);
  std::vector<int> ops;
  std::vector<int> rows;
  for (int r = 0; r < n; ++r) {
    std::vector<int> unit, coef;
    for (int u = P.res_ptr[r]; u < P.res_ptr[r + 1]; ++u) {
      int col = P.res_op[2 * u], code = P.res_op[2 * u + 1];
      int slot = (code & 2) ? 0 : (code >> 2) + 1;
      (slot ? coef : unit).push_back(col | ((code & 1) << 15) | (slot << 16));
    }
    rows.push_back((int)ops.size());
    rows.push_back((int)unit.size() | ((int)(unit.size() + coef.size()) << 16));
    ops.insert(ops.end(), unit.begin(), unit.end());
    ops.insert(ops.end(), coef.begin(), coef.end());
  }
  S.insert(S.end(), rows.begin(), rows.end());
  mark(6);
  S.insert(S.end(), ops.begin(), ops.end());
  mark(11);
}

// ------------------------------------------------------------------ transposed program
// Rows of U^T are the columns of U (diagonal included), rows of L^T the columns of L; the
// values are read from the same LU slots.  Levels: U^T row j waits for the rows k < j with
// U(k,j) != 0; L^T row k waits for the rows j > k with L(j,k) != 0.  Sections, in order:
//   [0] ut_ptr[nut+1]  [1] ut_desc[n] int4 {row | cnt << 16, first entry, diagonal slot, 0}
//   [2] lt_ptr[nlt+1]  [3] lt_desc[n] int4 {row | cnt << 16, first entry, -1, 0}
//   [6] utmax[nut], [7] ltmax[nlt]: split code of each level (split_code)
//   [4] entries int2 {LU slot, position}   [5] end
static void pack_transposed_program(Program &P) {
  const int n = P.n;
  std::vector<std::vector<std::pair<int, int>>> ut(n), lt(n);  // (slot, col)
  for (int k = 0; k < n; ++k) {
    for (int s = P.lu_rowptr[k]; s < P.lu_diag[k]; ++s) lt[P.lu_col[s]].push_back({s, k});     // L(k,j) -> L^T row j
    for (int s = P.lu_diag[k] + 1; s < P.lu_rowptr[k + 1]; ++s) ut[P.lu_col[s]].push_back({s, k});  // U(k,j) -> U^T row j
  }
  std::vector<int> ulev(n, 0), llev(n, 0);
  int nu = 0, nl = 0;
  for (int j = 0; j < n; ++j) {
    int l = 0;
    for (auto &e : ut[j]) l = std::max(l, ulev[e.second] + 1);
    ulev[j] = l;
    nu = std::max(nu, l + 1);
  }
  for (int k = n - 1; k >= 0; --k) {
    int l = 0;
    for (auto &e : lt[k]) l = std::max(l, llev[e.second] + 1);
    llev[k] = l;
    nl = std::max(nl, l + 1);
  }
  P.n_utlev = nu;
  P.n_ltlev = nl;
  std::vector<int> &T = P.tprog;
  T.clear();
  auto mark = [&](int i) {
    while (T.size() % 4) T.push_back(0);
    P.tp_off[i] = (int)T.size();
  };
  std::vector<int> ent;
  auto emit = [&](const std::vector<int> &lv, int nlev, const std::vector<std::vector<std::pair<int, int>>> &rows,
                  bool with_diag, int ptr_sec, int desc_sec) {
    std::vector<int> ptr(nlev + 1, 0), order;
    for (int k = 0; k < n; ++k) ptr[lv[k] + 1]++;
    for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    order.assign(n, 0);
    for (int k = 0; k < n; ++k) order[fill[lv[k]]++] = k;
    mark(ptr_sec);
    T.insert(T.end(), ptr.begin(), ptr.end());
    mark(desc_sec);
    for (int k : order) {
      T.insert(T.end(), {k | ((int)rows[k].size() << 16), (int)ent.size() / 2, with_diag ? P.lu_diag[k] : -1, 0});
      for (auto &e : rows[k]) ent.insert(ent.end(), {e.first, e.second});
    }
  };
  emit(ulev, nu, ut, true, 0, 1);
  emit(llev, nl, lt, false, 2, 3);
  // longest row of each U^T / L^T level
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<int> &lv = pass ? llev : ulev;
    const auto &rows = pass ? lt : ut;
    const int nlev = pass ? nl : nu;
    std::vector<int> mx(nlev, 0), cnt(nlev, 0);
    for (int k = 0; k < n; ++k) {
      mx[lv[k]] = std::max(mx[lv[k]], (int)rows[k].size());
      cnt[lv[k]]++;
    }
    mark(6 + pass);
    for (int l = 0; l < nlev; ++l) T.push_back(split_code(cnt[l], mx[l]));
  }
  mark(4);
  T.insert(T.end(), ent.begin(), ent.end());
  mark(5);
}

// ------------------------------------------------------------------ program
static int build_with_order(const krets_element *el, int ne, int n, int mode, int method, double h, double f,
                            const std::vector<MEntry> &M, const std::vector<BEntry> &B,
                            const std::vector<int> &q, Program &P, std::string &msg, bool rep_diode_zero,
                            const std::vector<int> &xslot, int n_coef, size_t fill_cap = 0,
                            bool update_list = true, bool dense_tail = false, int dense_from = -1) {
  P = Program();
  P.mode = mode;
  P.method = method;
  P.n = n;
  P.ne = ne;
  P.xslot = xslot;
  P.n_coef = n_coef;
  // ---- representative numeric matrix (CSC, summed), for pivot selection
  std::vector<std::complex<double>> coef(n_coef);
  for (int e = 0; e < ne; ++e) {
    coef[e] = rep_coef(el[e], mode, method, h, f, rep_diode_zero);
    if (xslot[e] >= 0) coef[xslot[e]] = coef[xslot[e] + 1] = coef[e];
  }
  std::vector<std::pair<long long, std::complex<double>>> ent;
  ent.reserve(M.size());
  for (auto &m : M) {
    int e = m.code >> 2;
    std::complex<double> v = (m.code & 2) ? std::complex<double>(1.0) : coef[e];
    if (m.code & 1) v = -v;
    ent.push_back({(long long)m.c * n + m.r, v});
  }
  std::stable_sort(ent.begin(), ent.end(), [](auto &a, auto &b) { return a.first < b.first; });
  std::vector<int> ap(n + 1, 0), ai;
  std::vector<std::complex<double>> axz;
  for (size_t k = 0; k < ent.size();) {
    size_t k2 = k;
    std::complex<double> s = 0;
    while (k2 < ent.size() && ent[k2].first == ent[k].first) s += ent[k2++].second;
    int c = (int)(ent[k].first / n), r = (int)(ent[k].first % n);
    ai.push_back(r);
    axz.push_back(s);
    ap[c + 1]++;
    k = k2;
  }
  for (int c = 0; c < n; ++c) ap[c + 1] += ap[c];
  GP F;
  int st;
  const double tau = 1e-3;  // threshold partial pivoting (diagonal kept when >= tau * column max)
  if (mode == MODE_AC) {
    st = gp_factor<std::complex<double>>(n, ap, ai, axz, q, tau, F, fill_cap, dense_from);
  } else {
    std::vector<double> axr(axz.size());
    for (size_t k = 0; k < axz.size(); ++k) axr[k] = axz[k].real();
    st = gp_factor<double>(n, ap, ai, axr, q, tau, F, fill_cap, dense_from);
  }
  if (st == kFillCapExceeded) return st;
  if (st != KRETS_OK) {
    msg = "matrix is singular for the representative element values (no usable pivot)";
    return st;
  }
  P.pivot_min_ratio = F.min_ratio;
  P.q = q;
  P.qinv.assign(n, 0);
  for (int k = 0; k < n; ++k) P.qinv[q[k]] = k;
  P.pinv = F.pinv;
  P.prow.assign(n, 0);
  for (int r = 0; r < n; ++r) P.prow[F.pinv[r]] = r;
  // ---- static LU pattern in position space
  std::vector<std::vector<int>> rows(n);
  for (int k = 0; k < n; ++k) {
    for (int p = F.lp[k]; p < F.lp[k + 1]; ++p) rows[F.pinv[F.li[p]]].push_back(k);  // L(i,k)
    for (int p = F.up[k]; p < F.up[k + 1]; ++p) rows[F.ui[p]].push_back(k);           // U(i,k), diag
  }
  P.lu_rowptr.assign(n + 1, 0);
  P.lu_diag.assign(n, -1);
  for (int k = 0; k < n; ++k) {
    std::sort(rows[k].begin(), rows[k].end());
    P.lu_rowptr[k + 1] = P.lu_rowptr[k] + (int)rows[k].size();
    P.max_row_lu = std::max(P.max_row_lu, (int)rows[k].size());
  }
  P.lu_col.resize(P.lu_rowptr[n]);
  // slot of column c in row k (rows sorted by column), -1 if absent
  auto slot_of = [&](int k, int c) {
    const int *b = P.lu_col.data() + P.lu_rowptr[k], *e = P.lu_col.data() + P.lu_rowptr[k + 1];
    const int *it = std::lower_bound(b, e, c);
    return (it != e && *it == c) ? (int)(it - P.lu_col.data()) : -1;
  };
  for (int k = 0; k < n; ++k) {
    for (size_t t = 0; t < rows[k].size(); ++t) {
      int s = P.lu_rowptr[k] + (int)t;
      P.lu_col[s] = rows[k][t];
      if (rows[k][t] == k) P.lu_diag[k] = s;
    }
    if (P.lu_diag[k] < 0) {
      msg = "internal: missing diagonal in static pattern";
      return KRETS_ERR_UNEXPECTED;
    }
  }
  // ---- dense trailing block: the largest m whose trailing m x m block is fully dense
  // (row k holds every column from cstart[k] to n-1; a trailing block is dense when each
  // of its rows starts its run at or before the block start, and density of a block
  // implies density of every smaller trailing block)
  if (dense_tail && n > 0) {
    int t0 = n, runmax = 0;
    for (int k = n - 1; k >= 0; --k) {
      int expect = n - 1, s = P.lu_rowptr[k + 1] - 1;
      while (s >= P.lu_rowptr[k] && P.lu_col[s] == expect) { --s; --expect; }
      runmax = std::max(runmax, expect + 1);
      if (runmax > k) break;
      t0 = k;
    }
    if (n - t0 >= kMinDenseTail) {
      P.tail0 = t0;
      P.tail_m = n - t0;
    }
  }
  // ---- factorisation program (IKJ)
  P.piv_ptr.assign(n + 1, 0);
  if (!update_list) {
    // no explicit update list (the device merges each U row into the pattern of row k;
    // the pattern is the fill of this very factorisation, so every update lands in it,
    // and the device reports a row whose update finds no slot): count the work only
    for (int k = 0; k < n; ++k)
      for (int s = P.lu_rowptr[k]; s < P.lu_diag[k]; ++s) {
        const int j = P.lu_col[s];
        P.factor_flops += 2 * (P.lu_rowptr[j + 1] - P.lu_diag[j] - 1) + 1;
      }
  }
  for (int k = 0; k < n && update_list; ++k) {
    for (int s = P.lu_rowptr[k]; s < P.lu_diag[k]; ++s) {
      int j = P.lu_col[s];
      int ub = (int)P.upd.size() / 2;
      for (int t = P.lu_diag[j] + 1; t < P.lu_rowptr[j + 1]; ++t) {
        int c = P.lu_col[t];
        const int at = slot_of(k, c);
        if (at < 0) {
          msg = "internal: fill entry missing from static pattern";
          return KRETS_ERR_UNEXPECTED;
        }
        P.upd.push_back(at);
        P.upd.push_back(t);
        P.factor_flops += 2;
      }
      P.piv.insert(P.piv.end(), {s, j, ub, (int)P.upd.size() / 2});
      P.factor_flops += 1;
    }
    P.piv_ptr[k + 1] = (int)P.piv.size() / 4;
  }
  const int tail0 = P.tail_m ? P.tail0 : n;
  // ---- level schedules (rows of the dense block: one last L level of their sparse
  // parts; no U level)
  std::vector<int> lev(n, 0), ulev(n, 0);
  int nl = 0, nu = 0;
  for (int k = 0; k < tail0; ++k) {
    int l = 0;
    for (int s = P.lu_rowptr[k]; s < P.lu_diag[k]; ++s) l = std::max(l, lev[P.lu_col[s]] + 1);
    lev[k] = l;
    nl = std::max(nl, l + 1);
  }
  for (int k = tail0; k < n; ++k) lev[k] = nl;
  if (tail0 < n) ++nl;
  for (int k = n - 1; k >= 0; --k) {
    if (k >= tail0) {
      ulev[k] = -1;
      continue;
    }
    int l = 0;
    for (int s = P.lu_diag[k] + 1; s < P.lu_rowptr[k + 1]; ++s) l = std::max(l, ulev[P.lu_col[s]] + 1);
    ulev[k] = l;
    nu = std::max(nu, l + 1);
  }
  auto bucket = [&](const std::vector<int> &lv, int nlev, std::vector<int> &ptr, std::vector<int> &rws) {
    ptr.assign(nlev + 1, 0);
    int cnt = 0;
    for (int k = 0; k < n; ++k)
      if (lv[k] >= 0) { ptr[lv[k] + 1]++; ++cnt; }
    for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
    rws.assign(cnt, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int k = 0; k < n; ++k)
      if (lv[k] >= 0) rws[fill[lv[k]]++] = k;
  };
  if (n == 0) { nl = nu = 0; }
  bucket(lev, nl, P.lev_ptr, P.lev_rows);
  bucket(ulev, nu, P.ulev_ptr, P.ulev_rows);
  // ---- stamp maps: A entries (position space) with contributions in emission order
  std::vector<std::pair<long long, int>> am;  // key (row pos * n + col pos), emission index
  am.reserve(M.size());
  for (size_t t = 0; t < M.size(); ++t)
    am.push_back({(long long)P.pinv[M[t].r] * n + P.qinv[M[t].c], (int)t});
  std::stable_sort(am.begin(), am.end(), [](auto &a, auto &b) { return a.first < b.first; });
  P.a_rowptr.assign(n + 1, 0);
  P.a_cptr.push_back(0);
  for (size_t t = 0; t < am.size();) {
    size_t t2 = t;
    int r = (int)(am[t].first / n), c = (int)(am[t].first % n);
    while (t2 < am.size() && am[t2].first == am[t].first) P.a_contrib.push_back(M[am[t2++].second].code);
    P.a_cptr.push_back((int)P.a_contrib.size());
    P.a_col.push_back(c);
    const int at = slot_of(r, c);
    if (at < 0) {
      msg = "internal: A entry outside the LU pattern";
      return KRETS_ERR_UNEXPECTED;
    }
    P.a_slot.push_back(at);
    P.a_rowptr[r + 1]++;
    t = t2;
  }
  for (int r = 0; r < n; ++r) P.a_rowptr[r + 1] += P.a_rowptr[r];
  std::vector<std::vector<int>> brow(n);
  for (auto &b : B) brow[P.pinv[b.r]].push_back(b.code);  // emission order kept
  P.b_cptr.assign(n + 1, 0);
  for (int r = 0; r < n; ++r) {
    P.b_contrib.insert(P.b_contrib.end(), brow[r].begin(), brow[r].end());
    P.b_cptr[r + 1] = (int)P.b_contrib.size();
  }
  P.el_pos.assign(4 * ne, -1);
  for (int e = 0; e < ne; ++e) {
    const int idx[4] = {el[e].p, el[e].m, el[e].b, el[e].g};
    for (int t = 0; t < 4; ++t) P.el_pos[4 * e + t] = idx[t] >= 0 ? P.qinv[idx[t]] : -1;
  }
  // ---- step program
  for (size_t t = 0; t < P.lev_rows.size(); ++t) {
    int k = P.lev_rows[t];
    P.ldesc.insert(P.ldesc.end(), {k, P.lu_rowptr[k], P.lu_diag[k], P.lu_rowptr[k + 1]});
  }
  for (size_t t = 0; t < P.ulev_rows.size(); ++t) {
    int k = P.ulev_rows[t];
    P.udesc.insert(P.udesc.end(), {k, P.lu_rowptr[k], P.lu_diag[k], P.lu_rowptr[k + 1]});
  }
  P.res_ptr.assign(n + 1, 0);
  for (int r = 0; r < n; ++r) {
    for (int t = P.a_rowptr[r]; t < P.a_rowptr[r + 1]; ++t)
      for (int u = P.a_cptr[t]; u < P.a_cptr[t + 1]; ++u) P.res_op.insert(P.res_op.end(), {P.a_col[t], P.a_contrib[u]});
    P.res_ptr[r + 1] = (int)P.res_op.size() / 2;
  }
  // dynamic elements in the order capacitors, inductors, the rest
  std::vector<int> dyn_of(ne, -1);
  for (int pass = 0; pass < 3; ++pass)
    for (int e = 0; e < ne; ++e) {
      int k = el[e].kind;
      bool cap = k == KRETS_ELEM_C, ind = k == KRETS_ELEM_L;
      bool dyn = cap || ind || k == KRETS_ELEM_V || k == KRETS_ELEM_I || k == KRETS_ELEM_D ||
                 (k == KRETS_ELEM_M && (el[e].flags & KRETS_FLAG_NMOS_RESOLVED));
      if (!dyn || (pass == 0) != cap || (pass == 1) != ind) continue;
      if (mode == MODE_DC && cap) continue;
      dyn_of[e] = (int)P.dyn_e.size();
      P.dyn_e.push_back(e);
      if (cap) P.ncap++;
      if (ind) P.n_ind++;
    }
  P.bd_ptr.assign(n + 1, 0);
  for (int r = 0; r < n; ++r) {
    for (int u = P.b_cptr[r]; u < P.b_cptr[r + 1]; ++u) {
      int code = P.b_contrib[u];
      int d = dyn_of[code >> 1];
      if (d < 0) {
        msg = "internal: rhs contribution from a non-dynamic element";
        return KRETS_ERR_UNEXPECTED;
      }
      P.bd_op.push_back((d << 1) | (code & 1));
    }
    P.bd_ptr[r + 1] = (int)P.bd_op.size();
  }
  pack_step_program(el, P);
  // the transposed program serves the adjoint, which runs single-circuit programs (with
  // an update list); multi-circuit programs never need it, nor the interleaved solves
  if (mode == MODE_TRAN && !P.tail_m && update_list) {
    pack_transposed_program(P);
    pack_interleaved(P);
    pack_lean(el, P);
  }
  uint64_t sig = 1469598103934665603ull;
  sig = fnv1a(sig, (uint64_t)mode);
  sig = fnv1a(sig, (uint64_t)n);
  for (auto &m : M) sig = fnv1a(sig, (uint64_t)m.r * 0x9E3779B1u + (uint64_t)m.c);
  P.signature = sig;
  return KRETS_OK;
}

// Estimated per-instance device cost of a program (arbitrary units): per level, the
// longest row divided over the CTA plus a fixed synchronisation cost, for the L and U
// solves and the factorisation.
static double program_cost(const Program &P) {
  const int T = 128;
  const double sync = 24.0;
  double c = 0;
  auto levels = [&](const std::vector<int> &ptr, const std::vector<int> &rws, bool lower) {
    for (size_t l = 0; l + 1 < ptr.size(); ++l) {
      int cnt = ptr[l + 1] - ptr[l];
      int mx = 0;
      for (int t = ptr[l]; t < ptr[l + 1]; ++t) {
        int k = rws[t];
        int len = lower ? ((P.tail_m && k >= P.tail0) ? P.lu_rowptr[k + 1] - P.tail_m - P.lu_rowptr[k]
                                                      : P.lu_diag[k] - P.lu_rowptr[k])
                        : P.lu_rowptr[k + 1] - P.lu_diag[k];
        mx = std::max(mx, len);
      }
      c += ((cnt + T - 1) / T) * (2.0 * mx + 4.0) + sync;
    }
  };
  levels(P.lev_ptr, P.lev_rows, true);
  levels(P.ulev_ptr, P.ulev_rows, false);
  if (P.tail_m) {  // blocked dense solves of the trailing block (forward and backward)
    const double m = P.tail_m, blocks = std::ceil(m / 32.0);
    c += 2.0 * blocks * (2.0 * sync + 32.0 * 4.0 + (m / 2.0) * 32.0 * 2.0 / T);
  }
  c *= 3.0;  // solves dominate (several per step) relative to one factorisation
  c += (double)P.factor_flops / T;
  return c;
}

int build_program(const krets_element *el, int ne, int n, int mode, int method, double h, double f,
                  int forced_ordering, Program &out, std::string &msg, bool update_list, bool dense_tail) {
  if (n <= 0) {
    msg = "circuit has no unknowns";
    return KRETS_ERR_MATRIX_BUILD;
  }
  std::vector<MEntry> M;
  std::vector<BEntry> B;
  // extra coefficient slots: two per resolved NMOS (g_ds, g_m) after the elements' own
  std::vector<int> xslot(ne, -1);
  int n_coef = ne;
  for (int e = 0; e < ne; ++e)
    if (el[e].kind == KRETS_ELEM_M && (el[e].flags & KRETS_FLAG_NMOS_RESOLVED)) {
      xslot[e] = n_coef;
      n_coef += 2;
    }
  for (int e = 0; e < ne; ++e) {
    const krets_element &x = el[e];
    if (x.p >= n || x.m >= n || x.b >= n || x.g >= n) {
      msg = "element " + std::to_string(e) + " references an unknown index >= n";
      return KRETS_ERR_INVALID_ARGUMENT;
    }
    if (mode == MODE_DC && x.kind == KRETS_ELEM_C) continue;  // op.rs:20-24
    if (!emit(x, e, xslot[e], mode, M, B)) {
      if (x.kind == KRETS_ELEM_Q || x.kind == KRETS_ELEM_M) {
        msg = x.kind == KRETS_ELEM_Q ? "BJT stamps are not implemented in the reference (todo!())"
                                     : "NMOS AC stamp is not implemented in the reference (todo!())";
        return KRETS_ERR_NOT_IMPLEMENTED;
      }
      msg = "unknown element kind " + std::to_string(x.kind);
      return KRETS_ERR_INVALID_ELEMENT;
    }
  }
  // symmetric adjacency of the pattern (without diagonal)
  std::vector<std::vector<int>> adj(n);
  for (auto &m : M)
    if (m.r != m.c) { adj[m.r].push_back(m.c); adj[m.c].push_back(m.r); }
  for (auto &a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  // minimum degree first: its fill caps the others (an ordering with more than twice its
  // L+U entries is abandoned during the factorisation; nested dissection by BFS levels
  // suits ladders and meshes but fills in heavily on random graphs)
  std::vector<int> cands = forced_ordering >= 0 ? std::vector<int>{forced_ordering}
                                                : std::vector<int>{ORDER_MINDEG, ORDER_NESTED, ORDER_NATURAL};
  size_t fill_cap = 0;
  double best_cost = 0;
  int best_st = KRETS_ERR_DECOMPOSITION_FAILED;
  std::string best_msg;
  int md_clique = 0;  // the minimum-degree ordering's final clique
  for (int o : cands) {
    std::vector<int> q;
    int clique = 0;  // minimum degree: size of the final clique of the elimination graph
    if (o == ORDER_NATURAL) {
      // the natural order is a candidate only for small systems (chains, tests): on a
      // general graph its fill grows towards n^2
      if (forced_ordering < 0 && n > 256) continue;
      q.resize(n);
      std::iota(q.begin(), q.end(), 0);
    } else if (o == ORDER_MINDEG) {
      if (n > 20000) continue;
      q = order_min_degree(n, adj, &clique);
      md_clique = clique;
    } else {
      // a program with a dense trailing block whose minimum-degree elimination ends in a
      // large clique comes from an irregular graph (random netlists): bisection by BFS
      // levels fills in more there (measured: it won only on netlists of at most 38
      // unknowns, which end in no such clique), so it is not tried
      if (forced_ordering < 0 && dense_tail && md_clique >= kMinDenseTail) continue;
      int top_sep = 0;
      const int sep_cap = std::max(16, (int)(2.0 * std::sqrt((double)n)));
      q = order_nested_dissection(n, adj, &top_sep, fill_cap ? sep_cap : 0);
      // bisection by BFS levels suits chains, ladders and meshes (separators of a few
      // vertices, or ~sqrt(n)); on irregular graphs its first separator is already large and
      // its fill beyond the minimum-degree one, so it is not factored once that is known
      if (fill_cap && top_sep > sep_cap) continue;
      if ((int)q.size() != n) continue;  // stopped early: no ordering
    }
    Program P;
    std::string m2;
    // programs with a dense trailing block finish a large final clique as a dense block
    const int dense_from = dense_tail && clique >= kMinDenseTail ? n - clique : -1;
    int st = build_with_order(el, ne, n, mode, method, h, f, M, B, q, P, m2, true, xslot, n_coef, fill_cap,
                              update_list, dense_tail, dense_from);
    if (st == KRETS_ERR_DECOMPOSITION_FAILED)  // only singular without diode / NMOS conductances
      st = build_with_order(el, ne, n, mode, method, h, f, M, B, q, P, m2, false, xslot, n_coef, fill_cap,
                            update_list, dense_tail, dense_from);
    if (st == kFillCapExceeded) continue;
    if (st != KRETS_OK) {
      if (best_st != KRETS_OK) { best_st = st; best_msg = m2; }
      continue;
    }
    P.ordering = o;
    if (!fill_cap) fill_cap = 2 * P.lu_col.size() + (size_t)n;
    double c = program_cost(P);
    if (best_st != KRETS_OK || c < best_cost) {
      best_cost = c;
      best_st = KRETS_OK;
      out = std::move(P);
    }
  }
  if (best_st != KRETS_OK) msg = best_msg;
  return best_st;
}

}  // namespace krets

// --------------------------------------------------------------- C ABI: introspection
extern "C" krets_status krets_symbolic_export(const krets_element *elems, int32_t n_elem, int32_t n_unknowns,
                                              int32_t mode, int32_t method, double h, double freq,
                                              int32_t ordering, int32_t which, int64_t *out, int64_t cap,
                                              int64_t *len) {
  using namespace krets;
  if (!elems || n_elem < 0 || n_unknowns <= 0 || !len) return KRETS_ERR_INVALID_ARGUMENT;
  Program P;
  std::string msg;
  const bool multi = ordering >= 0 && (ordering & KRETS_PROG_MULTI);
  if (multi) ordering &= ~KRETS_PROG_MULTI;
  if (ordering == 0xff) ordering = -1;
  int st = build_program(elems, n_elem, n_unknowns, mode, method, h, freq, ordering, P, msg, !multi, multi);
  if (st != KRETS_OK) return st;
  std::vector<long long> meta{P.ordering, P.n, (long long)P.a_col.size(), (long long)P.lu_col.size(),
                              (long long)P.lev_ptr.size() - 1, (long long)P.ulev_ptr.size() - 1, P.factor_flops,
                              P.tail0, P.tail_m};
  const std::vector<int> *arrs[] = {&P.q, &P.prow, &P.lu_rowptr, &P.lu_col, &P.lu_diag, &P.a_rowptr, &P.a_col,
                                    &P.a_slot, &P.a_cptr, &P.a_contrib, &P.b_cptr, &P.b_contrib, &P.piv_ptr,
                                    &P.piv, &P.upd, &P.lev_ptr, &P.lev_rows, &P.ulev_ptr, &P.ulev_rows,
                                    &P.el_pos};
  if (which < 0 || which > KRETS_PROG_IMAP) return KRETS_ERR_INVALID_ARGUMENT;
  if (which == KRETS_PROG_TPROG || which == KRETS_PROG_TPOFF || which == KRETS_PROG_SPROG ||
      which == KRETS_PROG_SPOFF || which >= KRETS_PROG_IPROG) {
    std::vector<long long> v;
    if (which == KRETS_PROG_IPROG) v.assign(P.iprog.begin(), P.iprog.end());
    else if (which == KRETS_PROG_IMAP) v.assign(P.imap.begin(), P.imap.end());
    else if (which == KRETS_PROG_IPOFF) {
      for (int gi = 0; gi < 2; ++gi)
        for (int k = 0; k < 4; ++k) v.push_back(P.ip_off[gi][k]);
      v.insert(v.end(), {P.il_slots[0], P.il_slots[1], P.imap_off[0], P.imap_off[1], P.n_il_lrec, P.n_il_urec,
                         P.il_ok ? 1 : 0, P.lean_off, P.n_zrow, P.n_ind, P.lean_ok ? 1 : 0});
      for (int k = 0; k < 4; ++k) v.push_back(P.ip_off[2][k]);  // the 32-thread layout
      v.insert(v.end(), {P.il_slots[2], P.imap_off[2]});
    } else if (which == KRETS_PROG_TPROG) v.assign(P.tprog.begin(), P.tprog.end());
    else if (which == KRETS_PROG_SPROG) v.assign(P.sprog.begin(), P.sprog.end());
    else if (which == KRETS_PROG_SPOFF) {
      v.assign(P.sp_off, P.sp_off + 16);
      v.push_back(P.n_bchunk);
      v.push_back(P.n_brow);
    } else {
      v.assign(P.tp_off, P.tp_off + 8);
      v.push_back(P.n_utlev);
      v.push_back(P.n_ltlev);
    }
    *len = (int64_t)v.size();
    if (out)
      for (int64_t k = 0; k < std::min<int64_t>(cap, *len); ++k) out[k] = v[k];
    return KRETS_OK;
  }
  if (which == KRETS_PROG_META) {
    *len = (int64_t)meta.size();
    if (out)
      for (int64_t k = 0; k < std::min<int64_t>(cap, *len); ++k) out[k] = meta[k];
    return KRETS_OK;
  }
  const std::vector<int> &v = *arrs[which];
  *len = (int64_t)v.size();
  if (out)
    for (int64_t k = 0; k < std::min<int64_t>(cap, *len); ++k) out[k] = v[k];
  return KRETS_OK;
}
