"""Seeded synthetic workloads (netlists and Monte Carlo values) for the five
benchmark configurations and the tests.

All randomness comes from a counter-based splitmix64 stream (seed -> u64 ->
uniform in (0, 1]); normals use Box-Muller on consecutive uniform pairs.  The
generators are pure numpy and produce identical values on every machine.

Configurations (sizes as in the benchmark definitions):
  1  resistor ladder: V1 1 0 1; R_k k->k+1 (k < N), R_N N->0, all 1 kOhm, plus a
     1 kOhm shunt from every node to ground; N = 1000 gives 1001 unknowns
  2  RC low-pass ladder, 500 sections, R log-uniform 100 Ohm-10 kOhm, C
     log-uniform 1 pF-1 uF, AC 1 V source; 4096 log-spaced points 1 Hz-1 GHz
  3  RLC ladder Monte Carlo: 2048 instances x 200 sections (R 50 Ohm, L 10 nH,
     C 1 pF, each x (1 + 0.1 N(0,1))), 0-1 V pulse, 100 ps rise, 5 ns width
  4  uneven batch of random connected netlists (see random_netlist)
  5  RC ladder for adjoint sensitivities, 1000 sections
"""
from __future__ import annotations

import numpy as np

from .netlist import Circuit, parse_circuit_description
from .table import element_table

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """`count` consecutive splitmix64 outputs of the stream started at `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = (np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, count: int) -> np.ndarray:
    """Uniform doubles in (0, 1]: ((u >> 11) + 1) * 2^-53."""
    u = splitmix64(seed, count)
    return ((u >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)


def normal(seed: int, count: int) -> np.ndarray:
    """Standard normals by Box-Muller on consecutive uniform pairs."""
    m = (count + 1) // 2
    u = uniform(seed, 2 * m)
    u1, u2 = u[0::2], u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.empty(2 * m)
    z[0::2] = r * np.cos(2.0 * np.pi * u2)
    z[1::2] = r * np.sin(2.0 * np.pi * u2)
    return z[:count]


def log_uniform(seed: int, count: int, lo: float, hi: float) -> np.ndarray:
    return np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * uniform(seed, count))


# --------------------------------------------------------------------------- netlists
def resistor_ladder_netlist(n: int, shunts: bool = False) -> str:
    """The reference's resistor_ladder_<n>.cir element lines (plus optional shunts)."""
    lines = ["% N-sized resistor ladder", "V1 1 0 1"]
    for k in range(1, n):
        lines.append(f"R{k} {k} {k + 1} 1000")
    lines.append(f"R{n} {n} 0 1000")
    if shunts:
        for k in range(1, n + 1):
            lines.append(f"Rs{k} {k} 0 1000")
    return "\n".join(lines) + "\n"


def config1_circuit() -> Circuit:
    """Plain OP workload: 1000-section ladder with a shunt per node, 1001 unknowns."""
    return parse_circuit_description(resistor_ladder_netlist(1000, shunts=True))


def rc_ladder_ac(sections: int = 500, seed: int = 2) -> Circuit:
    """AC workload: V1 in 0 0 AC 1, R_k n_{k-1}->n_k, C_k n_k->0 (seeded values)."""
    r = log_uniform(seed, sections, 100.0, 1e4)
    c = log_uniform(seed + 1000003, sections, 1e-12, 1e-6)
    lines = ["* RC low-pass ladder", "V1 in 0 0 AC 1"]
    prev = "in"
    for k in range(1, sections + 1):
        lines.append(f"R{k} {prev} n{k} {float(r[k - 1])!r}")
        lines.append(f"C{k} n{k} 0 {float(c[k - 1])!r}")
        prev = f"n{k}"
    return parse_circuit_description("\n".join(lines) + "\n")


def rlc_ladder(sections: int = 200, rise: str = "100p", width: str = "5n") -> Circuit:
    """Nominal RLC ladder: R 50 Ohm n_{k-1}->m_k, L 10 nH m_k->n_k, C 1 pF n_k->0,
    driven by V1 in 0 dc 0 PULSE(0 1 0 <rise> <rise> <width> 1)."""
    lines = ["* RLC ladder", f"V1 in 0 dc 0 PULSE(0 1 0 {rise} {rise} {width} 1)"]
    prev = "in"
    for k in range(1, sections + 1):
        lines.append(f"R{k} {prev} m{k} 50")
        lines.append(f"L{k} m{k} n{k} 10n")
        lines.append(f"C{k} n{k} 0 1p")
        prev = f"n{k}"
    return parse_circuit_description("\n".join(lines) + "\n")


def monte_carlo_values(circuit: Circuit, n_inst: int, sigma: float = 0.1, seed: int = 3,
                       kinds=(1, 2, 3)) -> np.ndarray:
    """[n_inst][n_elem] element values: nominal x (1 + sigma N(0,1)) for R, C, L."""
    t = element_table(circuit)
    nominal = t["value"].copy()
    ne = len(t)
    z = normal(seed, n_inst * ne).reshape(n_inst, ne)
    mask = np.isin(t["kind"], kinds)
    vals = np.tile(nominal, (n_inst, 1))
    vals[:, mask] = nominal[mask] * (1.0 + sigma * z[:, mask])
    return vals


def rc_ladder_step(sections: int = 1000, seed: int = 5) -> Circuit:
    """Adjoint workload: R log-uniform 100 Ohm-10 kOhm, C log-uniform 1 pF-100 pF,
    1 V step input PULSE(0 1 0 1p 1p 1 2)."""
    r = log_uniform(seed, sections, 100.0, 1e4)
    c = log_uniform(seed + 1000003, sections, 1e-12, 1e-10)
    lines = ["* RC ladder, step input", "V1 in 0 dc 0 PULSE(0 1 0 1p 1p 1 2)"]
    prev = "in"
    for k in range(1, sections + 1):
        lines.append(f"R{k} {prev} n{k} {float(r[k - 1])!r}")
        lines.append(f"C{k} n{k} 0 {float(c[k - 1])!r}")
        prev = f"n{k}"
    return parse_circuit_description("\n".join(lines) + "\n")


def rc_ladder_step_values(circuit: Circuit, n_inst: int, seed: int = 5) -> np.ndarray:
    """[n_inst][n_elem] values of the adjoint workload's RC ladder, drawn per instance: R
    log-uniform 100 Ohm-10 kOhm, C log-uniform 1 pF-100 pF (instance i from seed
    seed + 7919 i, so instance 0 has the values of rc_ladder_step(seed=seed))."""
    t = element_table(circuit)
    r_pos = np.nonzero(t["kind"] == 1)[0]
    c_pos = np.nonzero(t["kind"] == 2)[0]
    vals = np.tile(t["value"].astype(np.float64), (n_inst, 1))
    for i in range(n_inst):
        s = seed + 7919 * i
        vals[i, r_pos] = log_uniform(s, len(r_pos), 100.0, 1e4)
        vals[i, c_pos] = log_uniform(s + 1000003, len(c_pos), 1e-12, 1e-10)
    return vals


# ---------------------------------------------------------------- uneven batch
UNEVEN_NODES = (10, 5000)


def _uneven_elements(index: int, seed: int = 4):
    """Element list [(letter, name, a, b, value, wave_params)] of uneven netlist `index`.

    Nodes N log-uniform in [10, 5000].  A random recursive spanning tree of resistors
    (node k attaches to a uniform earlier node, 0 = ground) plus N/2 extra random edges, so
    the mean degree is 3.  Tree edges are resistors; extra edges are R 10%, C 60%, L 30%, so
    that all edges together are 70% R, 20% C, 10% L.  Values: R log-U 1 Ohm-1 MOhm, C log-U
    1 fF-1 nF, L log-U 1 nH-1 uH.  1-4 voltage sources from distinct nodes to ground (DC in
    [-5, 5] V, or a pulse to that level, half of them), 1-4 current sources node to ground,
    DC in [-1, 1] mA.  An inductor or voltage source that would close a loop made only of
    inductors and voltage sources (a singular DC system) becomes a resistor.
    """
    base = seed * 1000003 + index * 7919
    u = uniform(base, 8)
    N = int(np.floor(np.exp(np.log(UNEVEN_NODES[0]) + u[0] * (np.log(UNEVEN_NODES[1] + 1) - np.log(UNEVEN_NODES[0])))))
    N = max(UNEVEN_NODES[0], min(UNEVEN_NODES[1], N))
    n_extra = N // 2
    n_v = 1 + int(u[1] * 4)
    n_i = 1 + int(u[2] * 4)
    r = uniform(base + 1, 4 * N + 8 * n_extra + 64)
    parent = np.floor(r[:N] * np.arange(1, N + 1)).astype(np.int64)   # in [0, k-1] for node k (1-based)
    ea = np.floor(r[N:N + n_extra] * (N + 1)).astype(np.int64)
    eb = np.floor(r[N + n_extra:N + 2 * n_extra] * (N + 1)).astype(np.int64)
    et = r[N + 2 * n_extra:N + 3 * n_extra]
    lv = r[N + 3 * n_extra:N + 4 * n_extra]
    tv = r[N + 4 * n_extra:2 * N + 4 * n_extra]
    src = r[2 * N + 4 * n_extra:]
    # union-find over the inductor / voltage-source graph (0 = ground)
    uf = list(range(N + 1))

    def find(a):
        while uf[a] != a:
            uf[a] = uf[uf[a]]
            a = uf[a]
        return a

    def nm(k):
        return "0" if k == 0 else f"n{k}"

    els = []
    vnodes = []
    for k in range(n_v):
        node = 1 + int(src[4 * k] * N)
        if node in vnodes or find(node) == find(0):
            continue
        vnodes.append(node)
        uf[find(node)] = find(0)
        level = float(-5.0 + 10.0 * src[4 * k + 1])
        if src[4 * k + 2] < 0.5:
            els.append(("V", str(k + 1), nm(node), "0", level, None))
        else:
            els.append(("V", str(k + 1), nm(node), "0", 0.0, [0.0, level, 1e-9 * (1 + int(src[4 * k + 3] * 100)),
                                                              1e-10, 1e-10, 5e-7, 1e-6]))
    for k in range(n_i):
        node = 1 + int(src[16 + 2 * k] * N)
        els.append(("I", str(k + 1), nm(node), "0", float(-1e-3 + 2e-3 * src[17 + 2 * k]), None))
    for k in range(1, N + 1):
        els.append(("R", f"t{k}", nm(k), nm(int(parent[k - 1])), float(np.exp(np.log(1.0) + tv[k - 1] * np.log(1e6))), None))
    for j in range(n_extra):
        a, b = int(ea[j]), int(eb[j])
        if a == b:
            b = (a + 1) % (N + 1)
        t = et[j]
        if t < 0.1:
            kind = "R"
        elif t < 0.7:
            kind = "C"
        else:
            kind = "L"
        if kind == "L":
            fa, fb = find(a), find(b)
            if fa == fb:
                kind = "R"
            else:
                uf[fa] = fb
        lo, hi = {"R": (1.0, 1e6), "C": (1e-15, 1e-9), "L": (1e-9, 1e-6)}[kind]
        val = float(np.exp(np.log(lo) + lv[j] * (np.log(hi) - np.log(lo))))
        els.append((kind, f"x{j}", nm(a), nm(b), val, None))
    return els, N


def uneven_netlist(index: int, seed: int = 4) -> str:
    """SPICE text of uneven netlist `index` (see _uneven_elements)."""
    els, _ = _uneven_elements(index, seed)
    lines = [f"* uneven netlist {index}"]
    for letter, name, a, b, v, w in els:
        if letter == "V":
            if w is None:
                lines.append(f"V{name} {a} {b} dc {v!r}")
            else:
                lines.append(f"V{name} {a} {b} dc 0 PULSE({' '.join(repr(float(x)) for x in w)})")
        else:
            lines.append(f"{letter}{name} {a} {b} {v!r}")
    return "\n".join(lines) + "\n"


def uneven_table(index: int, seed: int = 4):
    """(element table, n) of uneven netlist `index`, built without text parsing; the MNA
    numbering follows the parser's rule (branch unknowns of V/L/I in element order, each
    first-seen non-ground node after them)."""
    from .table import ELEM_DTYPE
    els, _ = _uneven_elements(index, seed)
    kinds = {"R": 1, "C": 2, "L": 3, "V": 4, "I": 5}
    t = np.zeros(len(els), dtype=ELEM_DTYPE)
    idx = {}
    counter = 0
    for k, (letter, name, a, b, v, w) in enumerate(els):
        rec = t[k]
        rec["kind"] = kinds[letter]
        rec["g"] = -1
        rec["b"] = -1
        if letter in "VLI":
            rec["b"] = counter
            counter += 1
        for nd in (a, b):
            if nd != "0" and nd not in idx:
                idx[nd] = counter
                counter += 1
        rec["p"] = idx.get(a, -1)
        rec["m"] = idx.get(b, -1)
        rec["value"] = v
        if w is not None:
            rec["wave"] = 1
            rec["wp"][:7] = w
    return t, counter


def dense_block_table(m: int, seed: int = 7):
    """(element table, n) of a netlist whose LU is dense: a 1 V source at node 1, a resistor
    between every pair of the m nodes (log-uniform 1 kOhm-100 kOhm) and a capacitor from
    every node to ground (1 pF); n = m + 1, and the LU ends in a dense block of m - 1 rows
    (the multi-circuit engine takes up to 65534 elements: m <= 361).  Used to time the
    dense-block set-up and solves of that engine as a function of m."""
    from .table import ELEM_DTYPE
    rng = np.random.default_rng(seed)
    pairs = [(i, j) for i in range(m) for j in range(i + 1, m)]
    t = np.zeros(1 + len(pairs) + m, dtype=ELEM_DTYPE)
    t["g"] = -1
    t["b"] = -1
    t[0]["kind"], t[0]["b"], t[0]["p"], t[0]["m"], t[0]["value"] = 4, 0, 1, -1, 1.0
    # node k (0-based) is unknown k + 1: node 1 first seen with the source, the others in
    # the order the pair list meets them, which is increasing
    for r, (i, j) in enumerate(pairs, start=1):
        t[r]["kind"], t[r]["p"], t[r]["m"] = 1, i + 1, j + 1
        t[r]["value"] = 10.0 ** rng.uniform(3, 5)
    for k in range(m):
        r = 1 + len(pairs) + k
        t[r]["kind"], t[r]["p"], t[r]["m"], t[r]["value"] = 2, k + 1, -1, 1e-12
    return t, m + 1
