"""Flattened element table: the record layout that crosses the C ABI
(`krets_element` in include/krets_gpu.h), built from a parsed Circuit.

Node and branch fields hold MNA unknown indices from the reference numbering
(crates/krets-parser/src/parser.rs:105-125); -1 marks ground or "not in the
index map", which is exactly the case where the reference's
`index_map.get(..)` returns None and the stamp entry is skipped.
"""
from __future__ import annotations

import numpy as np

from .netlist import (Circuit, KIND_C, KIND_D, KIND_I, KIND_L, KIND_M, KIND_Q, KIND_R, KIND_V)

ELEM_DTYPE = np.dtype([
    ("kind", "<i4"), ("p", "<i4"), ("m", "<i4"), ("b", "<i4"), ("g", "<i4"),
    ("flags", "<i4"), ("wave", "<i4"), ("pad", "<i4"),
    ("value", "<f8"), ("ac", "<f8"), ("wp", "<f8", (7,)),
])
assert ELEM_DTYPE.itemsize == 104

FLAG_G2 = 1
FLAG_NMOS_RESOLVED = 2


def element_table(circuit: Circuit, nmos_resolved: bool = False) -> np.ndarray:
    """Flatten the circuit into krets_element records.  nmos_resolved: NMOS devices stamp
    with their nodes resolved as V(<node>) (the reference looks bare names up and stamps
    nothing, stampable.rs:842-844)."""
    im = circuit.index_map
    t = np.zeros(len(circuit.elements), dtype=ELEM_DTYPE)
    for k, el in enumerate(circuit.elements):
        rec = t[k]
        rec["kind"] = el.kind
        rec["g"] = -1
        rec["b"] = im.get(f"I({el.identifier})", -1) if el.is_g2 else -1
        if el.kind == KIND_M:
            d, g, s = el.nodes
            rec["p"] = im.get(f"V({d})", -1)
            rec["g"] = im.get(f"V({g})", -1)
            rec["m"] = im.get(f"V({s})", -1)
            mdl = el.model
            rec["wp"][:5] = [mdl["vto"], mdl["kp"], mdl["lambda"], mdl["w"], mdl["l"]]
        elif el.kind == KIND_Q:
            rec["p"] = im.get(f"V({el.nodes[0]})", -1)
            rec["m"] = im.get(f"V({el.nodes[1]})", -1)
            rec["g"] = im.get(f"V({el.nodes[2]})", -1)
        else:
            rec["p"] = im.get(f"V({el.nodes[0]})", -1)
            rec["m"] = im.get(f"V({el.nodes[1]})", -1)
        rec["flags"] = FLAG_G2 if el.g2 else 0
        if el.kind == KIND_M and nmos_resolved:
            rec["flags"] |= FLAG_NMOS_RESOLVED
        rec["value"] = el.value
        if el.kind == KIND_V:
            rec["ac"] = el.ac
            rec["wave"] = el.wave
            if el.wave_params:
                rec["wp"][:len(el.wave_params)] = el.wave_params
        elif el.kind == KIND_D:
            rec["value"] = el.model["is"]
            rec["wp"][0] = el.model["n"]
    return t


def is_current_mask(circuit: Circuit) -> np.ndarray:
    """True for unknowns whose result key starts with 'I' (branch currents)."""
    mask = np.zeros(circuit.size, dtype=bool)
    for k, v in circuit.index_map.items():
        if k.startswith("I"):
            mask[v] = True
    return mask
