"""CPU emulation (numpy) of the static program the host symbolic pass emits.

Test infrastructure: it executes the exported index arrays exactly the way the
device engine walks them (segmented stamp sums -> IKJ factor program -> level
ordered solves), so a mismatch against the oracle points at the symbolic pass
rather than at the CUDA code.  No solve path of the product calls this.
"""
import numpy as np

from krets_gb300 import _lib

PI = 3.14159265358979323846


def element_coefs(table, mode, method="be", h=1.0, freq=0.0, prev=None, t_src=0.0, icap=None):
    """Per-element (matrix coefficient, rhs coefficient), original unknown numbering."""
    ne = len(table)
    ca = np.zeros(ne, dtype=complex)
    cb = np.zeros(ne)
    tr = method == "tr"
    for e, el in enumerate(table):
        k, v = int(el["kind"]), float(el["value"])
        p, m, b = int(el["p"]), int(el["m"]), int(el["b"])
        if k == 1:
            ca[e] = v if el["flags"] & 1 else 1.0 / v
        elif k == 2:
            if mode == 1:
                ca[e] = 1j * (2.0 * PI * freq * v)
            elif mode == 2:
                vp = prev[p] if p >= 0 else 0.0
                vm = prev[m] if m >= 0 else 0.0
                if tr:
                    ca[e] = 2.0 * v / h
                    cb[e] = ca[e].real * (vp - vm) + icap[e]
                else:
                    ca[e] = v / h
                    cb[e] = -(-(v / h) * (vp - vm))
        elif k == 3:
            if mode == 1:
                ca[e] = 1j * (2.0 * PI * freq * v)
            elif mode == 2:
                ip = prev[b]
                if tr:
                    lh = 2.0 * v / h
                    vl = (prev[p] if p >= 0 else 0.0) - (prev[m] if m >= 0 else 0.0)
                    ca[e] = lh
                    cb[e] = -lh * ip - vl
                else:
                    ca[e] = v / h
                    cb[e] = -(v / h) * ip
        elif k == 4:
            if mode == 0:
                cb[e] = v
            elif mode == 1:
                cb[e] = float(el["ac"])
            else:
                from oracle import oracle as O
                w = el["wp"]
                cb[e] = O.pulse(w, t_src) if el["wave"] == 1 else (O.sin(w, t_src) if el["wave"] == 2 else v)
        elif k == 5:
            cb[e] = v
    return ca, cb


def emulate(prog, table, n, ca, cb, complex_=False):
    """Stamp, factor and solve with the program arrays; returns x in unknown order."""
    dt = complex if complex_ else float
    cav = ca if complex_ else ca.real
    nnz_lu = len(prog["lu_col"])
    lu = np.zeros(nnz_lu, dtype=dt)
    a_cptr, a_contrib = prog["a_cptr"], prog["a_contrib"]
    for t in range(len(prog["a_col"])):
        s = dt(0)
        for u in range(a_cptr[t], a_cptr[t + 1]):
            code = int(a_contrib[u])
            val = dt(1.0) if code & 2 else cav[code >> 2]
            s += -val if code & 1 else val
        lu[prog["a_slot"][t]] = s
    b = np.zeros(n, dtype=dt)
    for k in range(n):
        s = 0.0
        for u in range(prog["b_cptr"][k], prog["b_cptr"][k + 1]):
            code = int(prog["b_contrib"][u])
            s += -cb[code >> 1] if code & 1 else cb[code >> 1]
        b[k] = s
    piv = prog["piv"].reshape(-1, 4)
    upd = prog["upd"].reshape(-1, 2)
    diag = prog["lu_diag"]
    lev_ptr, lev_rows = prog["lev_ptr"], prog["lev_rows"]
    done = np.zeros(n, dtype=bool)
    for lv in range(len(lev_ptr) - 1):
        rows = lev_rows[lev_ptr[lv]:lev_ptr[lv + 1]]
        for k in rows:
            for pi in range(prog["piv_ptr"][k], prog["piv_ptr"][k + 1]):
                s, j, u0, u1 = piv[pi]
                assert done[j], "factor level order violated"
                l = lu[s] / lu[diag[j]]
                lu[s] = l
                for dst, src in upd[u0:u1]:
                    lu[dst] -= l * lu[src]
        for k in rows:
            done[k] = True
    rp, col = prog["lu_rowptr"], prog["lu_col"]
    y = b.copy()
    for lv in range(1, len(lev_ptr) - 1):
        for k in lev_rows[lev_ptr[lv]:lev_ptr[lv + 1]]:
            for u in range(rp[k], diag[k]):
                y[k] -= lu[u] * y[col[u]]
    ulp, ulr = prog["ulev_ptr"], prog["ulev_rows"]
    for lv in range(len(ulp) - 1):
        for k in ulr[ulp[lv]:ulp[lv + 1]]:
            s = y[k]
            for u in range(diag[k] + 1, rp[k + 1]):
                s -= lu[u] * y[col[u]]
            y[k] = s / lu[diag[k]]
    x = np.zeros(n, dtype=dt)
    x[prog["q"]] = y
    return x


def export(table, n, mode, method="be", h=1.0, freq=1e3, ordering=-1):
    return _lib.symbolic_export(table, n, mode, method, h, freq, ordering)


def factor_only(prog, n, ca, complex_=False):
    """Stamp and factor with the program (as emulate()); returns the LU value array."""
    dt = complex if complex_ else float
    cav = ca if complex_ else ca.real
    lu = np.zeros(len(prog["lu_col"]), dtype=dt)
    for t in range(len(prog["a_col"])):
        s = dt(0)
        for u in range(prog["a_cptr"][t], prog["a_cptr"][t + 1]):
            code = int(prog["a_contrib"][u])
            val = dt(1.0) if code & 2 else cav[code >> 2]
            s += -val if code & 1 else val
        lu[prog["a_slot"][t]] = s
    piv = prog["piv"].reshape(-1, 4)
    upd = prog["upd"].reshape(-1, 2)
    diag = prog["lu_diag"]
    lev_ptr, lev_rows = prog["lev_ptr"], prog["lev_rows"]
    for lv in range(len(lev_ptr) - 1):
        for k in lev_rows[lev_ptr[lv]:lev_ptr[lv + 1]]:
            for pi in range(prog["piv_ptr"][k], prog["piv_ptr"][k + 1]):
                s, j, u0, u1 = piv[pi]
                l = lu[s] / lu[diag[j]]
                lu[s] = l
                for dst, src in upd[u0:u1]:
                    lu[dst] -= l * lu[src]
    return lu


def transposed_solve(prog, n, lu, c):
    """Solve A^T y = c with the transposed program and the (unscaled-diagonal) LU values."""
    T = prog["tprog"]
    off = prog["tpoff"]
    ut_ptr = T[off[0]:off[0] + int(off[8]) + 1]
    ut_desc = T[off[1]:off[1] + 4 * n].reshape(n, 4)
    lt_ptr = T[off[2]:off[2] + int(off[9]) + 1]
    lt_desc = T[off[3]:off[3] + 4 * n].reshape(n, 4)
    ent = T[off[4]:off[5]].reshape(-1, 2)
    z = np.asarray(c, dtype=float)[prog["q"]].copy()      # c in position space (columns)
    for lv in range(len(ut_ptr) - 1):
        for t in range(ut_ptr[lv], ut_ptr[lv + 1]):
            r, first, dslot = ut_desc[t][0] & 0xffff, ut_desc[t][1], ut_desc[t][2]
            cnt = ut_desc[t][0] >> 16
            s = z[r]
            for e in range(first, first + cnt):
                s -= lu[ent[e][0]] * z[ent[e][1]]
            z[r] = s / lu[dslot]
    for lv in range(len(lt_ptr) - 1):
        for t in range(lt_ptr[lv], lt_ptr[lv + 1]):
            r, first, cnt = lt_desc[t][0] & 0xffff, lt_desc[t][1], lt_desc[t][0] >> 16
            s = z[r]
            for e in range(first, first + cnt):
                s -= lu[ent[e][0]] * z[ent[e][1]]
            z[r] = s
    y = np.zeros(n)
    y[prog["prow"]] = z                                      # position k <-> row prow[k]
    return y


def export_multi(table, n, mode, method="be", h=1e-9):
    """Program of the multi-circuit engine (dense trailing block, no update list)."""
    return _lib.symbolic_export(table, n, mode, method, h, 1e3, 0xff | 0x100)


def factor_multi(prog, n, ca):
    """Device factorisation of a multi-circuit program: rows merged in level order (rows of
    the dense trailing block only over their columns before it), then a dense LU of the
    block.  Returns the LU values (plain diagonal)."""
    lu = np.zeros(len(prog["lu_col"]))
    for t in range(len(prog["a_col"])):
        s = 0.0
        for u in range(prog["a_cptr"][t], prog["a_cptr"][t + 1]):
            code = int(prog["a_contrib"][u])
            val = 1.0 if code & 2 else ca[code >> 2].real
            s += -val if code & 1 else val
        lu[prog["a_slot"][t]] = s
    rp, col, dg = prog["lu_rowptr"], prog["lu_col"], prog["lu_diag"]
    t0, m = int(prog["meta"][7]), int(prog["meta"][8])
    lev_ptr, lev_rows = prog["lev_ptr"], prog["lev_rows"]
    nlev = len(lev_ptr) - 1
    done = np.zeros(n, dtype=bool)
    for lv in range(nlev):
        rows = lev_rows[lev_ptr[lv]:lev_ptr[lv + 1]]
        tail = m > 0 and lv == nlev - 1
        for k in rows:
            pos = {int(col[s]): s for s in range(rp[k], rp[k + 1])}
            lim = rp[k + 1] - m if tail else dg[k]
            for s in range(rp[k], lim):
                j = int(col[s])
                assert done[j], "factor level order violated"
                l = lu[s] / lu[dg[j]]
                lu[s] = l
                for u in range(dg[j] + 1, rp[j + 1]):
                    lu[pos[int(col[u])]] -= l * lu[u]
        for k in rows:
            done[k] = True
    if m:
        A = np.array([lu[rp[t0 + i + 1] - m:rp[t0 + i + 1]] for i in range(m)])
        for kk in range(m):
            A[kk + 1:, kk] /= A[kk, kk]
            A[kk + 1:, kk + 1:] -= np.outer(A[kk + 1:, kk], A[kk, kk + 1:])
        for i in range(m):
            lu[rp[t0 + i + 1] - m:rp[t0 + i + 1]] = A[i]
    return lu


def solve_multi(prog, n, lu, b):
    """Solve with the factors of factor_multi in the device's order: L levels (the last one
    = sparse parts of the dense block's rows), dense forward, dense backward, U levels.
    b in position-row order; returns x in unknown order."""
    rp, col, dg = prog["lu_rowptr"], prog["lu_col"], prog["lu_diag"]
    t0, m = int(prog["meta"][7]), int(prog["meta"][8])
    y = np.asarray(b, dtype=float).copy()
    lev_ptr, lev_rows = prog["lev_ptr"], prog["lev_rows"]
    nlev = len(lev_ptr) - 1
    for lv in range(1, nlev):
        tail = m > 0 and lv == nlev - 1
        new = {}
        for k in lev_rows[lev_ptr[lv]:lev_ptr[lv + 1]]:
            lim = rp[k + 1] - m if tail else dg[k]
            new[k] = y[k] - sum(lu[s] * y[col[s]] for s in range(rp[k], lim))
        for k, v in new.items():      # a level's rows are independent
            y[k] = v
    if m:
        D = np.array([lu[rp[t0 + i + 1] - m:rp[t0 + i + 1]] for i in range(m)])
        z = y[t0:].copy()
        for i in range(m):
            z[i] -= D[i, :i] @ z[:i]
        for i in range(m - 1, -1, -1):
            z[i] = (z[i] - D[i, i + 1:] @ z[i + 1:]) / D[i, i]
        y[t0:] = z
    ulp, ulr = prog["ulev_ptr"], prog["ulev_rows"]
    assert not m or not np.any(ulr >= t0)
    # border of the dense block (step program sections 14/15), then the U levels with the
    # entry counts of the step program's U descriptors
    sp, off = prog["sprog"], prog["spoff"]
    n_bchunk, n_brow = int(off[16]), int(off[17])
    chunks = sp[off[14]:off[14] + 2 * n_bchunk].reshape(-1, 2)
    brows = sp[off[15]:off[15] + 4 * n_brow].reshape(-1, 4)
    for row, first, nch, _ in brows:
        acc = 0.0
        for start, cnt in chunks[first:first + nch]:
            assert 0 < cnt <= 16 and np.all(col[start:start + cnt] >= t0)
            acc += sum(lu[q] * y[col[q]] for q in range(start, start + cnt))
        y[row] -= acc
    udesc = sp[off[3]:off[3] + 4 * len(ulr)].reshape(-1, 4)
    ucnt = {int(d[0]) & 0xffff: int(d[3]) + (int(d[0]) >> 16) for d in udesc}
    for lv in range(len(ulp) - 1):
        new = {}
        for k in ulr[ulp[lv]:ulp[lv + 1]]:
            e1 = dg[k] + 1 + ucnt[k]
            new[k] = (y[k] - sum(lu[s] * y[col[s]] for s in range(dg[k] + 1, e1))) / lu[dg[k]]
        for k, v in new.items():
            y[k] = v
    x = np.zeros(n)
    x[prog["q"]] = y
    return x
