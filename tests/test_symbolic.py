"""Host symbolic pass, checked on the CPU: the exported static program (ordering,
pivots, fill, stamp maps, level schedules) is executed by a numpy emulator and must
reproduce the oracle.  Also checks that libkrets_gpu.so exports every declared symbol."""
import re
from pathlib import Path

import numpy as np
import pytest

import program_emulator as PE
from conftest import circuit_from_case
from krets_gb300 import parse_circuit_description
from krets_gb300.generators import config1_circuit, monte_carlo_values, rc_ladder_ac, rlc_ladder
from krets_gb300.table import element_table

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    hdr = (ROOT / "include" / "krets_gpu.h").read_text()
    names = set(re.findall(r"^(?:krets_status|const char \*|int64_t|int32_t)\s*(krets_[a-z0-9_]+)\s*\(", hdr,
                           re.M))
    assert len(names) > 15
    lib = ctypes.CDLL(str(built_lib.LIB_PATH))
    for nm in sorted(names):
        assert hasattr(lib, nm), nm


def test_circuit_create_checks_arguments_before_the_device(built_lib):
    """krets_circuit_create validates the element records before it touches CUDA, and
    without a usable GPU it fails with KRETS_ERR_CUDA (there is no CPU fallback)."""
    import ctypes
    from krets_gb300 import _lib
    L = _lib.lib()
    c = parse_circuit_description("V1 a 0 1\nR1 a b 1000\nR2 b 0 1000\n")
    t = element_table(c)
    h = ctypes.c_void_p()
    bad = t.copy()
    bad["kind"][1] = 42
    assert L.krets_circuit_create(_lib.ptr(bad), len(bad), c.size, None, ctypes.byref(h)) == 3
    assert b"unknown element kind" in L.krets_last_error_message()
    bad = t.copy()
    bad["m"][2] = c.size
    assert L.krets_circuit_create(_lib.ptr(bad), len(bad), c.size, None, ctypes.byref(h)) == 11
    assert L.krets_circuit_create(_lib.ptr(t), len(t), 0, None, ctypes.byref(h)) == 11
    st = L.krets_circuit_create(_lib.ptr(t), len(t), c.size, None, ctypes.byref(h))
    if st == 0:                       # a GPU is present
        assert L.krets_circuit_destroy(h) == 0
    else:
        assert st == 10 and b"no CPU fallback" in L.krets_last_error_message()


@pytest.mark.parametrize("ordering", [-1, 0, 1, 2])
def test_op_programs_match_oracle(built_lib, oracle_lib, golden, ordering):
    for case in golden["op"]:
        c = circuit_from_case(case)
        t = element_table(c)
        prog = PE.export(t, c.size, 0, ordering=ordering)
        ca, cb = PE.element_coefs(t, 0)
        if any(el.is_nonlinear for el in c.elements):
            continue
        x = PE.emulate(prog, t, c.size, ca, cb)
        xo = oracle_lib.op(t, c.size)
        np.testing.assert_allclose(x, xo, rtol=1e-9, atol=1e-12 * max(1.0, np.abs(xo).max()))


@pytest.mark.parametrize("method,h", [("be", 1e-12), ("tr", 1e-12), ("tr", 1e-9), ("be", 1e-6)])
def test_tran_programs_match_dense(built_lib, oracle_lib, method, h):
    c = rlc_ladder(60)
    t = element_table(c)
    n = c.size
    prev = np.cos(np.arange(n) * 0.37)
    prog = PE.export(t, n, 2, method=method, h=h)
    ca, cb = PE.element_coefs(t, 2, method, h, prev=prev, t_src=0.0, icap=np.zeros(len(t)))
    x = PE.emulate(prog, t, n, ca, cb)
    A, b = oracle_lib.assemble(t, n, "tran", h, method, sol=prev)
    xd = np.linalg.solve(A, b)
    # norm-wise: both solutions carry rounding of order cond(A) * eps
    np.testing.assert_allclose(x, xd, rtol=0, atol=1e-9 * np.abs(xd).max())


@pytest.mark.parametrize("sections", [12, 1000])
def test_transposed_program_solves_adjoint_systems(built_lib, oracle_lib, sections):
    """The transposed program (used by the adjoint sweep) solves A^T y = c with the forward
    LU values; its indices stay inside the LU value array and the position vectors."""
    from krets_gb300.generators import rc_ladder_step
    c = rc_ladder_step(sections)
    t = element_table(c)
    n = c.size
    h = 1e-9
    prog = PE.export(t, n, 2, method="tr", h=h)
    T, off = prog["tprog"], prog["tpoff"]
    nnz = len(prog["lu_col"])
    nut, nlt = int(off[8]), int(off[9])
    for dsec, psec, msec, nlev, upper in ((1, 0, 6, nut, True), (3, 2, 7, nlt, False)):
        ptr = T[off[psec]:off[psec] + nlev + 1]
        assert ptr[0] == 0 and ptr[-1] == n and np.all(np.diff(ptr) >= 0)
        desc = T[off[dsec]:off[dsec] + 4 * n].reshape(n, 4)
        rows = desc[:, 0] & 0xffff
        assert sorted(rows) == list(range(n))
        cnt, first = desc[:, 0] >> 16, desc[:, 1]
        mx = T[off[msec]:off[msec] + nlev]        # split codes: longest row in bits 18..
        assert all(mx[l] >> 18 == cnt[ptr[l]:ptr[l + 1]].max() for l in range(nlev))
        assert np.all(first + cnt <= (off[5] - off[4]) // 2)
        if upper:
            assert np.all((desc[:, 2] >= 0) & (desc[:, 2] < nnz))
    ent = T[off[4]:off[5]].reshape(-1, 2)
    assert np.all((ent[:, 0] >= 0) & (ent[:, 0] < nnz) & (ent[:, 1] >= 0) & (ent[:, 1] < n))
    ca, _ = PE.element_coefs(t, 2, "tr", h, prev=np.zeros(n), icap=np.zeros(len(t)))
    lu = PE.factor_only(prog, n, ca)
    A, _ = oracle_lib.assemble(t, n, "tran", h, "tr", sol=np.zeros(n))
    rhs = np.sin(np.arange(n) * 0.7)
    y = PE.transposed_solve(prog, n, lu, rhs)
    yd = np.linalg.solve(A.T, rhs)
    np.testing.assert_allclose(y, yd, rtol=0, atol=1e-10 * np.abs(yd).max())


def test_ac_program_static_pivots_hold_over_nine_decades(built_lib, oracle_lib):
    c = rc_ladder_ac(120)
    t = element_table(c)
    prog = PE.export(t, c.size, 1, freq=3.16e4)
    for f in (1.0, 1e3, 1e6, 1e9):
        ca, cb = PE.element_coefs(t, 1, freq=f)
        x = PE.emulate(prog, t, c.size, ca, cb, complex_=True)
        z = oracle_lib.ac(t, c.size, [f])[0]
        np.testing.assert_allclose(x, z, rtol=1e-9, atol=1e-13 * np.abs(z).max())


def test_nested_dissection_gives_log_depth_on_ladders(built_lib):
    c = config1_circuit()
    prog = PE.export(element_table(c), c.size, 0, ordering=2)
    assert prog["meta"][4] <= 24 and prog["meta"][5] <= 24      # ~2 log2(1001) levels
    nat = PE.export(element_table(c), c.size, 0, ordering=0)
    assert nat["meta"][4] >= 900                                 # natural order: a chain
    auto = PE.export(element_table(c), c.size, 0)
    assert auto["meta"][0] == 2                                  # the cost model picks ND


def test_stamp_contributions_keep_emission_order(built_lib):
    # a node with three resistors: the diagonal entry sums 1/R in element order
    c = parse_circuit_description("V1 a 0 1\nR1 a 0 3\nR2 a 0 7\nR3 a 0 11\n")
    t = element_table(c)
    prog = PE.export(t, c.size, 0)
    a = c.index_map["V(a)"]
    qinv = np.argsort(prog["q"])
    pinv = np.argsort(prog["prow"])
    row = pinv[a]
    found = False
    for tt in range(prog["a_rowptr"][row], prog["a_rowptr"][row + 1]):
        if prog["a_col"][tt] == qinv[a]:
            codes = prog["a_contrib"][prog["a_cptr"][tt]:prog["a_cptr"][tt + 1]]
            assert [int(x) >> 2 for x in codes] == [1, 2, 3]
            found = True
    assert found


def test_singular_topology_is_reported(built_lib):
    from krets_gb300 import _lib
    from krets_gb300.errors import DecompositionFailed
    # node b floats in DC (only a capacitor attaches it)
    c = parse_circuit_description("V1 a 0 1\nR1 a 0 1\nC1 a b 1e-6\n")
    with pytest.raises(DecompositionFailed):
        PE.export(element_table(c), c.size, 0)


def test_monte_carlo_values_deterministic():
    c = rlc_ladder(10)
    v1 = monte_carlo_values(c, 4, seed=9)
    v2 = monte_carlo_values(c, 4, seed=9)
    np.testing.assert_array_equal(v1, v2)
    assert v1.shape == (4, len(c.elements))
    assert np.all(v1[:, 0] == 0.0)            # the source value is not perturbed


def test_multi_circuit_program_dense_tail_solves(built_lib, oracle_lib):
    """Multi-circuit programs of a random netlist: the fully dense trailing block is found,
    its rows leave the U schedule, and factor + solve in the device's order (levels, dense
    block) reproduce a dense solve."""
    from krets_gb300.generators import uneven_table
    t, n = uneven_table(4)
    p = PE.export_multi(t, n, 2)
    t0, m = int(p["meta"][7]), int(p["meta"][8])
    assert m >= 64 and t0 + m == n
    rp, col = p["lu_rowptr"], p["lu_col"]
    for k in range(t0, n):                      # every block row holds columns t0 .. n-1
        assert np.array_equal(col[rp[k + 1] - m:rp[k + 1]], np.arange(t0, n))
    lv = p["lev_ptr"]
    assert np.array_equal(p["lev_rows"][lv[-2]:lv[-1]], np.arange(t0, n))
    assert len(p["ulev_rows"]) == t0
    # the border (U entries of earlier rows in the block's columns) is listed once, whole
    sp, off = p["sprog"], p["spoff"]
    chunks = sp[off[14]:off[14] + 2 * int(off[16])].reshape(-1, 2)
    dg = p["lu_diag"]
    border = sum(int((col[dg[k] + 1:rp[k + 1]] >= t0).sum()) for k in range(t0))
    assert int(chunks[:, 1].sum()) == border > 0
    ca, _ = PE.element_coefs(t, 2, "be", 1e-9, prev=np.zeros(n), icap=np.zeros(len(t)))
    lu = PE.factor_multi(p, n, ca)
    A, _ = oracle_lib.assemble(t, n, "tran", 1e-9, "be", sol=np.zeros(n))
    rhs = np.sin(np.arange(n) * 0.37)
    x = PE.solve_multi(p, n, lu, rhs[p["prow"]])
    xd = np.linalg.solve(A.reshape(n, n), rhs)
    np.testing.assert_allclose(x, xd, rtol=0, atol=1e-10 * np.abs(xd).max())


def _il_solve(P, vals, b, gi):
    """Emulate the interleaved L and U solves of layout gi (64 / 128 / 32-thread groups) in FP64."""
    off = P["ipoff"]
    # layouts 0 and 1 first, the 32-thread layout's offsets, slots and map base at the end
    base4, slot_at, map_at = (4 * gi, 8 + gi, 10 + gi) if gi < 2 else (19, 23, 24)
    rec0, rows0, cols0, end = off[base4:base4 + 4]
    nl, nu = int(off[12]), int(off[13])
    ip = P["iprog"]
    rec = ip[rec0:rows0].reshape(-1, 8)[:nl + nu]
    rows = ip[rows0:cols0]
    packed = ip[cols0:end].astype(np.int64)
    cols = np.stack([packed & 0xffff, (packed >> 16) & 0xffff], axis=1).reshape(-1)
    slots = int(off[slot_at])
    imap = P["imap"][int(off[map_at]):int(off[map_at]) + slots]
    lui = np.where(imap >= 0, vals[np.maximum(imap, 0)], 0.0)
    y = b.copy()
    n_entry = 0
    for li, (W, lsh, mc, first, rbase, dbase, flags, _) in enumerate(rec):
        upper = li >= nl
        spl = 1 << lsh
        assert W % spl == 0 and (dbase >= 0) == upper
        # bit 0: a level of at most 32 lanes (first warp alone); bit 1: so is the next one
        narrow_next = li + 1 < len(rec) and rec[li + 1][0] <= 32
        assert flags == (W <= 32) | (2 * (W <= 32 and narrow_next))
        assert first == n_entry
        n_entry += mc * W
        sums = {}
        for lam in range(W):
            r, sub = divmod(lam, spl)
            k = rows[rbase + r]
            s = y[k] if sub == 0 else 0.0
            for i in range(mc):
                slot = first + i * W + lam
                s -= lui[slot] * y[cols[slot]]
            sums.setdefault(r, []).append(s)
        for r, parts in sums.items():
            k = rows[rbase + r]
            v = sum(parts)
            y[k] = v * lui[dbase + r] if upper else v
    assert len(cols) >= n_entry
    return y, imap, slots


def _csr_solve(P, vals, b):
    rp, col, dg = P["lu_rowptr"], P["lu_col"], P["lu_diag"]
    y = b.copy()
    lp, lr = P["lev_ptr"], P["lev_rows"]
    for l in range(1, len(lp) - 1):
        for k in lr[lp[l]:lp[l + 1]]:
            y[k] -= sum(vals[s] * y[col[s]] for s in range(rp[k], dg[k]))
    up, ur = P["ulev_ptr"], P["ulev_rows"]
    for l in range(len(up) - 1):
        for k in ur[up[l]:up[l + 1]]:
            y[k] = (y[k] - sum(vals[s] * y[col[s]] for s in range(dg[k] + 1, rp[k + 1]))) * vals[dg[k]]
    return y


@pytest.mark.parametrize("which", ["rlc200", "rc300", "uneven6"])
def test_interleaved_solve_program_equals_row_solves(built_lib, which):
    """The interleaved ("ELL per level") solve program of the double-float engine (factors
    in global memory): every L entry of levels 1.. and every U entry appears exactly once,
    each U row's reciprocal diagonal once, pads are zero; emulated in FP64 it solves the
    same triangular systems as the row-descriptor program, for the three group-size layouts."""
    from krets_gb300.generators import rc_ladder_step, rlc_ladder, uneven_table
    if which == "rlc200":
        c = rlc_ladder(200)
        t, n = element_table(c), c.size
    elif which == "rc300":
        c = rc_ladder_step(300)
        t, n = element_table(c), c.size
    else:
        t, n = uneven_table(6)
    P = built_lib.symbolic_export(t, n, built_lib.MODE_TRAN, "tr", 1e-12)
    assert P["ipoff"][14] == 1
    rng = np.random.default_rng(3)
    nnz = len(P["lu_col"])
    vals = rng.uniform(-0.05, 0.05, nnz)
    vals[P["lu_diag"]] = rng.uniform(0.5, 1.5, n)
    b = rng.standard_normal(n)
    ref = _csr_solve(P, vals, b)
    rp, dg = P["lu_rowptr"], P["lu_diag"]
    level0 = set(P["lev_rows"][P["lev_ptr"][0]:P["lev_ptr"][1]].tolist())
    want = sorted([s for k in range(n) if k not in level0 for s in range(rp[k], dg[k])]
                  + [s for k in range(n) for s in range(dg[k] + 1, rp[k + 1])] + list(dg))
    for gi in (0, 1, 2):
        y, imap, slots = _il_solve(P, vals, b, gi)
        assert sorted(imap[imap >= 0].tolist()) == want
        np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("which", ["rlc200", "rc300", "uneven6", "rlc_sin"])
def test_direct_rhs_program_equals_gather(built_lib, which):
    """The direct right-hand side of the interleaved double-float step (every element
    writes the rows it feeds, unfed rows are zeroed) forms the same right-hand side as the
    gather pass over the step program's rhs operators, for any element values; a netlist
    with a row fed by two elements has no direct program."""
    from krets_gb300.generators import rc_ladder_step, rlc_ladder, uneven_table
    from krets_gb300.netlist import parse_circuit_description
    if which == "rlc200":
        c = rlc_ladder(200)
        t, n = element_table(c), c.size
    elif which == "rc300":
        c = rc_ladder_step(300)
        t, n = element_table(c), c.size
    elif which == "rlc_sin":
        # a floating capacitor (two rows, opposite signs) and a current source
        c = parse_circuit_description("V1 in 0 SIN(0 1 1e9 0 0 0)\nR1 in a 50\nL1 a b 1n\nC1 b 0 1p\n"
                                      "R2 b c 100\nC3 c d 1p\nR3 d 0 1k\nI1 e 0 1m\nR4 e 0 1k\n")
        t, n = element_table(c), c.size
    else:
        t, n = uneven_table(6)
    P = built_lib.symbolic_export(t, n, built_lib.MODE_TRAN, "tr", 1e-12)
    off, sp, spo = P["ipoff"], P["sprog"], P["spoff"]
    lean_off, n_zrow, n_ind, lean_ok = (int(v) for v in off[15:19])
    dyn = sp[spo[7]:spo[8]].reshape(-1, 4)
    nd = len(dyn)
    bd_ptr = sp[spo[8]:spo[8] + n + 1]
    bd_op = sp[spo[9]:spo[9] + int(bd_ptr[-1])]
    kinds = dyn[:, 0] >> 24
    fed_twice = np.any(np.diff(bd_ptr) > 1)
    if fed_twice:
        assert lean_ok == 0 and which == "uneven6"
        return
    assert lean_ok == 1
    ncap = int(np.sum(kinds == 2))   # KRETS_ELEM_C, then KRETS_ELEM_L
    assert np.all(kinds[:ncap] == 2) and np.all(kinds[ncap:ncap + n_ind] == 3) and n_ind == np.sum(kinds == 3)
    rng = np.random.default_rng(5)
    cb = rng.standard_normal(nd)
    ref = np.zeros(n)
    for k in range(n):
        for u in range(bd_ptr[k], bd_ptr[k + 1]):
            ref[k] += -cb[bd_op[u] >> 1] if bd_op[u] & 1 else cb[bd_op[u] >> 1]
    L = P["iprog"][lean_off:lean_off + 4 * nd].reshape(-1, 4)
    zrow = P["iprog"][lean_off + 4 * nd:lean_off + 4 * nd + n_zrow]
    b = np.full(n + 2, np.nan)
    for d in range(nd):
        if ncap <= d < ncap + n_ind:            # inductor: {p, m, branch, row << 1 | neg}
            p, m, w, rw = L[d]
            assert w == dyn[d][3] and {int(p), int(m)} <= set(range(n + 1))
            b[rw >> 1] = -cb[d] if rw & 1 else cb[d]
        else:                                   # {p, m | e|kind, 0, row +, row -}
            b[L[d][2]] = cb[d]
            b[L[d][3]] = -cb[d]
    b[zrow] = 0.0
    np.testing.assert_array_equal(b[:n], ref)


def test_orderings_of_a_path_joined_to_an_expander(built_lib):
    """A path whose first nested-dissection separator is one vertex, joined to a random
    expander whose own separators are large: every mode yields a full permutation (the
    dissection may stop early only at its first separator, and an ordering it left
    unfinished is never used)."""
    from krets_gb300.table import ELEM_DTYPE
    rng = np.random.default_rng(1)
    L, m, deg = 300, 400, 8
    edges = [(i, i + 1) for i in range(L)]
    E = set()
    while len(E) < m * deg // 2:
        a, b = rng.integers(0, m, 2)
        if a != b:
            E.add((L + min(a, b), L + max(a, b)))
    edges += sorted(E)
    nn = L + m
    t = np.zeros(1 + len(edges) + nn, dtype=ELEM_DTYPE)
    t["g"], t["b"] = -1, -1
    t[0]["kind"], t[0]["b"], t[0]["p"], t[0]["m"], t[0]["value"] = 4, 0, 1, -1, 1.0
    for r, (i, j) in enumerate(edges, start=1):
        t[r]["kind"], t[r]["p"], t[r]["m"], t[r]["value"] = 1, i + 1, j + 1, 1e3
    for k in range(nn):
        r = 1 + len(edges) + k
        t[r]["kind"], t[r]["p"], t[r]["m"], t[r]["value"] = 2, k + 1, -1, 1e-12
    for mode in (built_lib.MODE_DC, built_lib.MODE_TRAN):
        for ordering in (-1, 0x1ff):   # single-circuit and multi-circuit programs
            P = built_lib.symbolic_export(t, nn + 1, mode, "be", 1e-9, ordering=ordering)
            assert sorted(P["q"].tolist()) == list(range(nn + 1))
