// Host symbolic pass: turns a flattened netlist into a static "program" that the device
// kernels execute without further decisions (ordering, pivot sequence, fill pattern,
// stamp-to-slot maps, level schedules).
//
// The reference re-derives all of this every Newton iteration (a fresh faer
// SparseColMat + sp_lu per iteration: crates/krets-solver/src/solver/op.rs:48-58,
// transient.rs:74-83, ac.rs:67-70, dc.rs:81-84).  Here it runs once per (topology, mode).
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "krets_gpu.h"

namespace krets {

enum Mode { MODE_DC = 0, MODE_AC = 1, MODE_TRAN = 2 };

// A matrix stamp contribution, packed as  slot << 2 | unit << 1 | neg:
//   unit = 1 -> the value is the constant 1 (KCL/KVL incidence), else the per-pass matrix
//   coefficient in slot `slot`; neg = 1 -> negated.  Slot e is element e's coefficient;
//   elements with more than one distinct matrix value (a resolved NMOS: g_ds + g_m, g_ds,
//   g_m) take their further values from slots ne, ne + 1, ... (Program::xslot).
// A right-hand-side contribution, packed as elem << 1 | neg (value = element's
// per-pass rhs coefficient).
inline int pack_a(int e, bool unit, bool neg) { return (e << 2) | (unit ? 2 : 0) | (neg ? 1 : 0); }
inline int pack_b(int e, bool neg) { return (e << 1) | (neg ? 1 : 0); }

enum Ordering { ORDER_NATURAL = 0, ORDER_MINDEG = 1, ORDER_NESTED = 2 };

struct Program {
  int mode = 0, method = 0, n = 0, ne = 0;
  int ordering = 0;
  // position k factors unknown column q[k] with pivot row prow[k]
  std::vector<int> q, qinv, prow, pinv;
  // LU pattern in position space, row-wise: [L part | diag | U part], columns ascending
  std::vector<int> lu_rowptr, lu_col, lu_diag;
  // A entries in position space (subset of the LU pattern), row-wise
  std::vector<int> a_rowptr, a_col, a_slot;
  std::vector<int> a_cptr, a_contrib;  // contributions of each A entry, emission order
  std::vector<int> b_cptr, b_contrib;  // rhs contributions per position row
  // factorisation program (row-oriented, up-looking):
  //   row k: piv entries [piv_ptr[k], piv_ptr[k+1]), each {slot(k,j), j, upd_begin, upd_end}
  //   upd pairs {dst slot(k,c), src slot(j,c)}:  lu[dst] -= l_kj * lu[src]
  std::vector<int> piv_ptr;
  std::vector<int> piv;  // 4 ints per entry
  std::vector<int> upd;  // 2 ints per entry
  // level schedules: rows of the L solve / factorisation, and of the U solve
  std::vector<int> lev_ptr, lev_rows, ulev_ptr, ulev_rows;
  // per element: p, m, b, g in POSITION space (-1 = absent)
  std::vector<int> el_pos;
  // per element: first of its extra coefficient slots (-1 = none); n_coef = slots in all
  std::vector<int> xslot;
  int n_coef = 0;
  // --- step program (used by the warp-per-instance engine)
  // level-ordered row descriptors {row, first entry, diag slot, end}: L solve / U solve
  std::vector<int> ldesc, udesc;
  // residual ops per position row: {column position, packed contribution (pack_a)}
  std::vector<int> res_ptr, res_op;
  // elements with a right-hand-side coefficient (C, L, V, I, D), capacitors first
  std::vector<int> dyn_e;
  int ncap = 0, n_ind = 0;  // dyn_e: capacitors first, then inductors
  // rhs contributions per position row, packed dyn_index << 1 | neg
  std::vector<int> bd_ptr, bd_op;
  // compact step program, copied into shared memory by the warp engine (sprog_ok = the
  // sizes fit its 16-bit packing).  Layout and packing: see pack_step_program().
  std::vector<int> sprog;
  int sp_off[16] = {0};
  int n_bchunk = 0, n_brow = 0;  // border of the dense block (see pack_step_program)
  bool sprog_ok = false;
  // transposed-solve program (adjoint): A^T y = c  <=>  U^T z = c[q], then L^T y' = z, y = y'[pinv]
  //   tprog sections: [0] ut_ptr (levels of U^T, forward)  [1] ut_desc int4 {row | cnt << 16,
  //   first entry, diag slot, 0}  [2] lt_ptr (levels of L^T, backward)  [3] lt_desc
  //   {row | cnt << 16, first entry, -1, 0}  [4] entries int2 {lu slot, column}  [5] end
  std::vector<int> tprog;
  int tp_off[8] = {0};
  int n_utlev = 0, n_ltlev = 0;
  // dense trailing block (multi-circuit programs only): positions tail0 .. n-1 form a
  // fully dense m x m block of the LU (m = tail_m, 0 = none).  Its rows sit in the last L
  // level with descriptors covering only their columns < tail0; the U levels hold rows
  // < tail0 only.  Row k of the block keeps its dense part at slots
  // lu_rowptr[k+1] - m .. lu_rowptr[k+1] - 1 (columns tail0 .. n-1).
  int tail0 = 0, tail_m = 0;
  // Interleaved solve programs of the double-float engine with its factors in global
  // memory, one per group size (layout 0: 64 threads, 1: 128, 2: 32; see pack_interleaved).
  // Per level of the L solve (levels 1..) and of the U solve: a record
  //   {W lanes, log2 lanes per row, entry slots per lane, first entry slot, row base,
  //    diagonal slot base (U; -1 for L), flags, 0}
  // then the rows' positions and the columns (uint16 pairs, one per entry slot); entry i
  // of lane lam of a level sits at slot first + i * W + lam, the U rows' reciprocal
  // diagonals after all entry slots.  imap: interleaved slot -> CSR slot (-1: a zero pad).
  // Then (pack_lean) the direct right-hand-side records at lean_off.
  std::vector<int> iprog, imap;
  int ip_off[3][4] = {{0}};  // records, rows, columns, end (ints into iprog)
  int il_slots[3] = {0, 0, 0};
  int imap_off[3] = {0, 0, 0};
  int n_il_lrec = 0, n_il_urec = 0;
  bool il_ok = false;
  int lean_off = 0, n_zrow = 0;  // direct right-hand side (pack_lean)
  bool lean_ok = false;
  long long factor_flops = 0;
  int max_row_lu = 0;
  uint64_t signature = 0;
  double pivot_min_ratio = 1.0;  // smallest |pivot| / column max seen while pivoting
};

// Build the program for one mode.  h / freq: representative step and frequency used to
// evaluate values for pivot selection.  Returns KRETS_OK or an error code (msg filled).
int build_program(const krets_element *el, int ne, int n, int mode, int method, double h, double freq,
                  int forced_ordering, Program &out, std::string &msg,
                  bool update_list = true, bool dense_tail = false);

// Exposed for tests of the symbolic pass itself.
std::vector<int> order_min_degree(int n, const std::vector<std::vector<int>> &adj, int *clique = nullptr);
std::vector<int> order_nested_dissection(int n, const std::vector<std::vector<int>> &adj, int *top_sep = nullptr,
                                         int max_top_sep = 0);

}  // namespace krets
