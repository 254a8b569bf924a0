"""Netlist front-end: the SPICE-subset grammar krets accepts, flattened to the
element table that crosses the C ABI.

This restates the reference front-end (crates/krets-parser) closely enough
that every fixture netlist parses to the same element list and, crucially,
the same MNA unknown numbering:

* line handling, `.control`/`.subckt`/`.model` blocks:   parser.rs:27-103
* unknown index assignment (Group-2 branch first, then
  first-seen non-ground nodes, element file order):     parser.rs:105-125
* element grammars: resistor.rs:35-51, capacitor.rs:166-183,
  inductor.rs:324-339, voltage_source.rs:106-235, current_source.rs:435-450,
  diode.rs:571-588, nmosfet.rs:382-434, bjt.rs (parse only),
  subcircuit.rs:33-157 (instance flattening, name/node prefixing)
* value suffixes: utils.rs:32-64;  `.model` cards: models.rs:39-94
* Group-2 membership: elements.rs:125-140; nonlinearity: elements.rs:143-148

Like the reference, an element line is parsed from its start and any trailing
text is ignored (the reference calls the nom parsers without
`all_consuming` from parser.rs:88).
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional

from .errors import ParseError

# Element kinds; the integer codes are the ones in include/krets_gpu.h.
KIND_R, KIND_C, KIND_L, KIND_V, KIND_I, KIND_D, KIND_M, KIND_Q = 1, 2, 3, 4, 5, 6, 7, 8
KIND_LETTER = {KIND_R: "R", KIND_C: "C", KIND_L: "L", KIND_V: "V", KIND_I: "I",
               KIND_D: "D", KIND_M: "M", KIND_Q: "Q"}

WAVE_NONE, WAVE_PULSE, WAVE_SIN = 0, 1, 2

# Boltzmann constant, elementary charge and temperature (constants.rs:1-4).
KB = 1.380649e-23
QE = 1.602176634e-19
TEMPERATURE = 300.0
THERMAL_VOLTAGE = KB * TEMPERATURE / QE


@dataclass
class Element:
    kind: int
    name: str                      # name without the kind letter ("1" for R1)
    nodes: List[str]               # plus, minus   (NMOS: drain, gate, source)
    value: float = 0.0             # R ohms, C farads, L henries, V dc, I amps
    g2: bool = False               # Group-2 flag (capacitor "G2" suffix)
    ac: float = 0.0                # V source AC amplitude
    wave: int = WAVE_NONE
    wave_params: List[float] = field(default_factory=list)
    model_name: str = ""
    bulk: str = ""
    # diode: saturation current, parasitic resistance, emission coefficient
    # nmos: w, l, vto, kp, lambda
    model: Dict[str, float] = field(default_factory=dict)

    @property
    def identifier(self) -> str:
        """`<letter><name>`, the key used for branch unknowns (I(V1))."""
        return KIND_LETTER[self.kind] + self.name

    @property
    def is_g2(self) -> bool:
        # elements.rs:125-140: V, L, I always; R and C when flagged.
        if self.kind in (KIND_V, KIND_L, KIND_I):
            return True
        if self.kind in (KIND_R, KIND_C):
            return self.g2
        return False

    @property
    def is_nonlinear(self) -> bool:
        return self.kind in (KIND_D, KIND_M, KIND_Q)


@dataclass
class Circuit:
    elements: List[Element]
    index_map: Dict[str, int]
    nodes: List[str]
    models: Dict[str, dict]

    @property
    def size(self) -> int:
        return len(self.index_map)

    def names_by_index(self) -> List[str]:
        names = [""] * len(self.index_map)
        for k, v in self.index_map.items():
            names[v] = k
        return names


# ----------------------------------------------------------------------------
# token helpers
_IDENT = re.compile(r"[A-Za-z0-9_]+")
_SPACE1 = re.compile(r"[ \t]+")
_VALUE_TOKEN = re.compile(r"[^ \t\r\n()]+")
# nom's `double`: optional sign, digits with optional fraction, optional exponent
_DOUBLE = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?")


def parse_value(s: str) -> float:
    """SPICE value with metric suffix (utils.rs:32-64)."""
    up = s.upper()
    mult = 1.0
    if up.endswith("MEG"):
        num, mult = up[:-3], 1e6
    elif up:
        suffix = {"F": 1e-15, "P": 1e-12, "N": 1e-9, "U": 1e-6, "M": 1e-3,
                  "K": 1e3, "G": 1e9, "T": 1e12}
        if up[-1] in suffix:
            num, mult = up[:-1], suffix[up[-1]]
        else:
            num = up
    else:
        num = up
    try:
        base = _rust_parse_f64(num)
    except ValueError:
        raise ParseError(f"Invalid numeric value '{s}'")
    return base * mult


def _rust_parse_f64(s: str) -> float:
    # Rust's f64::from_str: decimal / exponent forms, "inf", "nan", "infinity".
    if not re.fullmatch(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|[+-]?(?:inf|infinity|nan)", s,
                        flags=re.IGNORECASE):
        raise ValueError(s)
    return float(s)


class _Cursor:
    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def rest(self) -> str:
        return self.s[self.i:]

    def tag_ci(self, t: str) -> bool:
        if self.s[self.i:self.i + len(t)].lower() == t.lower():
            self.i += len(t)
            return True
        return False

    def tag(self, t: str) -> bool:
        if self.s.startswith(t, self.i):
            self.i += len(t)
            return True
        return False

    def ident(self) -> Optional[str]:
        m = _IDENT.match(self.s, self.i)
        if not m:
            return None
        self.i = m.end()
        return m.group(0)

    def space1(self) -> bool:
        m = _SPACE1.match(self.s, self.i)
        if not m:
            return False
        self.i = m.end()
        return True

    def space0(self) -> None:
        m = _SPACE1.match(self.s, self.i)
        if m:
            self.i = m.end()

    def sp_ident(self) -> Optional[str]:
        save = self.i
        if self.space1():
            v = self.ident()
            if v is not None:
                return v
        self.i = save
        return None

    def value(self) -> Optional[float]:
        m = _VALUE_TOKEN.match(self.s, self.i)
        if not m:
            return None
        try:
            v = parse_value(m.group(0))
        except ParseError:
            return None
        self.i = m.end()
        return v

    def sp_value(self) -> Optional[float]:
        save = self.i
        if self.space1():
            v = self.value()
            if v is not None:
                return v
        self.i = save
        return None

    def double(self) -> Optional[float]:
        m = _DOUBLE.match(self.s, self.i)
        if not m:
            return None
        self.i = m.end()
        return float(m.group(0))


def _two_nodes(c: _Cursor):
    plus = c.sp_ident()
    if plus is None:
        return None
    minus = c.sp_ident()
    if minus is None:
        return None
    return plus, minus


def _parse_rlci(c: _Cursor, letter: str, kind: int) -> Optional[Element]:
    if not c.tag_ci(letter):
        return None
    name = c.ident()
    if name is None:
        return None
    nodes = _two_nodes(c)
    if nodes is None:
        return None
    v = c.sp_value()
    if v is None:
        return None
    el = Element(kind, name, list(nodes), value=v)
    if kind == KIND_C:
        save = c.i
        if c.space1() and c.tag_ci("G2"):
            el.g2 = True
        else:
            c.i = save
    return el


def _parse_paren_values(c: _Cursor, count: int) -> Optional[List[float]]:
    c.space0()
    if not c.tag("("):
        return None
    vals = []
    for k in range(count):
        if k == 0:
            c.space0()
            v = c.value()
        else:
            v = c.sp_value()
        if v is None:
            return None
        vals.append(v)
    c.space0()
    if not c.tag(")"):
        return None
    return vals


def _parse_vsource(c: _Cursor) -> Optional[Element]:
    if not c.tag_ci("V"):
        return None
    name = c.ident()
    if name is None:
        return None
    nodes = _two_nodes(c)
    if nodes is None:
        return None
    el = Element(KIND_V, name, list(nodes))
    save = c.i
    implicit = None
    if c.space1():
        implicit = c.double()
    if implicit is None:
        c.i = save
    el.value = implicit if implicit is not None else 0.0
    while True:
        save = c.i
        if not c.space1():
            break
        if c.tag_ci("dc"):
            if c.space1():
                d = c.double()
                if d is not None:
                    el.value = d
                    continue
        c.i = save
        c.space1()
        if c.tag_ci("ac"):
            if c.space1():
                d = c.double()
                if d is not None:
                    el.ac = d
                    continue
        c.i = save
        c.space1()
        if c.tag_ci("pulse"):
            vals = _parse_paren_values(c, 7)
            if vals is not None:
                el.wave, el.wave_params = WAVE_PULSE, vals
                continue
        c.i = save
        c.space1()
        if c.tag_ci("sin"):
            vals = _parse_paren_values(c, 6)
            if vals is not None:
                el.wave, el.wave_params = WAVE_SIN, vals
                continue
        c.i = save
        break
    return el


def _parse_diode(c: _Cursor) -> Optional[Element]:
    if not c.tag_ci("D"):
        return None
    name = c.ident()
    if name is None:
        return None
    nodes = _two_nodes(c)
    if nodes is None:
        return None
    model = c.sp_ident()
    return Element(KIND_D, name, list(nodes), model_name=model or "default")


def _parse_bjt(c: _Cursor) -> Optional[Element]:
    if not c.tag_ci("Q"):
        return None
    if not (c.tag_ci("N") or c.tag_ci("P")):
        return None
    m = re.compile(r"[A-Za-z0-9]+").match(c.s, c.i)
    if not m:
        return None
    c.i = m.end()
    coll = c.sp_ident()
    base = c.sp_ident()
    emit = c.sp_ident()
    if None in (coll, base, emit):
        return None
    c.sp_value()
    return Element(KIND_Q, m.group(0), [coll, emit, base])


def _parse_nmos(c: _Cursor) -> Optional[Element]:
    if not c.tag_ci("MN"):
        return None
    name = c.ident()
    if name is None:
        return None
    ids = []
    for _ in range(5):
        v = c.sp_ident()
        if v is None:
            return None
        ids.append(v)
    drain, gate, source, bulk, model = ids
    el = Element(KIND_M, name, [drain, gate, source], bulk=bulk, model_name=model)
    return el


def _parse_xinst(c: _Cursor) -> Optional[Element]:
    if not c.tag_ci("x"):
        return None
    name = c.ident()
    if name is None:
        return None
    nodes = []
    while True:
        v = c.sp_ident()
        if v is None:
            break
        nodes.append(v)
    if not nodes:
        return None
    el = Element(0, name, nodes[:-1], model_name=nodes[-1])
    return el


def parse_element(line: str) -> Element:
    """First alternative that parses wins, in the order of elements.rs:44-65."""
    for fn in (lambda c: _parse_rlci(c, "R", KIND_R), lambda c: _parse_rlci(c, "C", KIND_C),
               lambda c: _parse_rlci(c, "L", KIND_L), _parse_vsource,
               lambda c: _parse_rlci(c, "I", KIND_I), _parse_diode, _parse_bjt, _parse_nmos,
               _parse_xinst):
        el = fn(_Cursor(line))
        if el is not None:
            return el
    raise ParseError(f"Failed to parse element from input '{line}'")


def parse_model(line: str) -> dict:
    """`.model NAME TYPE (k=v ...)` (models.rs:39-94). TYPE is case-sensitive."""
    text = line.split("%")[0].strip()
    c = _Cursor(text)
    if not c.tag_ci(".model") or not c.space1():
        raise ParseError(f"bad model card '{line}'")
    name = c.ident()
    if name is None or not c.space1():
        raise ParseError(f"bad model card '{line}'")
    for typ in ("NMOS", "PMOS", "D"):
        if c.tag(typ):
            break
    else:
        raise ParseError(f"unknown model type in '{line}'")
    c.space0()
    c.tag("(")
    params = {}
    while True:
        save = c.i
        c.space0()
        k = c.ident()
        if k is None:
            c.i = save
            break
        c.space0()
        if not c.tag("="):
            c.i = save
            break
        c.space0()
        v = c.value()
        if v is None:
            c.i = save
            break
        params[k] = v
    if typ == "D":
        m = {"type": "D", "name": name, "is": 1e-12, "rs": 0.0, "n": 1.0}
        for k, v in params.items():
            if k.lower() in ("is", "rs", "n"):
                m[k.lower()] = v
    else:
        m = {"type": typ, "name": name, "w": 1e-6, "l": 1e-6, "vto": 0.0,
             "kp": 2e-5 if typ == "NMOS" else 1e-5, "lambda": 0.02 if typ == "NMOS" else 0.01}
        for k, v in params.items():
            if k.lower() in ("w", "l", "vto", "kp", "lambda"):
                m[k.lower()] = v
    return m


def _parse_subcircuits(text: str) -> Dict[str, dict]:
    defs: Dict[str, dict] = {}
    inside, cur = False, ""
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("%") or line.startswith("*"):
            continue
        low = line.lower()
        if low.startswith(".subckt"):
            c = _Cursor(line)
            c.tag_ci(".subckt")
            name = c.sp_ident()
            if name is None:
                raise ParseError(f"Failed to parse subcircuit header: {line}")
            pins = []
            while True:
                p = c.sp_ident()
                if p is None:
                    break
                pins.append(p)
            defs[name] = {"pins": pins, "elements": []}
            cur, inside = name, True
            continue
        if low.startswith(".ends"):
            inside, cur = False, ""
            continue
        if inside:
            defs[cur]["elements"].append(parse_element(line))
    return defs


def _instantiate(inst: Element, defs: Dict[str, dict]) -> List[Element]:
    d = defs.get(inst.model_name)
    if d is None:
        raise ParseError(f"Undefined subcircuit definition: {inst.model_name}")
    if len(inst.nodes) != len(d["pins"]):
        raise ParseError(f"Node/port mismatch for instance {inst.name}")
    port = dict(zip(d["pins"], inst.nodes))
    out: List[Element] = []
    for sub in d["elements"]:
        e = Element(**{**sub.__dict__, "nodes": list(sub.nodes), "wave_params": list(sub.wave_params),
                       "model": dict(sub.model)})
        e.nodes = [port.get(n, f"{inst.name}_{n}") for n in e.nodes]
        e.name = f"{inst.name}_{e.name}"
        if e.kind == 0:
            out.extend(_instantiate(e, defs))
        else:
            out.append(e)
    return out


def parse_circuit_description(text: str) -> Circuit:
    """Parse a netlist and assign MNA unknown indices (parser.rs:27-154)."""
    defs = _parse_subcircuits(text)
    elements: List[Element] = []
    models: Dict[str, dict] = {}
    in_control = in_subckt = False
    for lineno, line in enumerate(text.splitlines(), 1):
        line = line.strip()
        if not line or line.startswith("%") or line.startswith("*"):
            continue
        low = line.lower()
        if low.startswith(".control"):
            in_control = True
            continue
        if low.startswith(".endc"):
            in_control = False
            continue
        if in_control:
            continue
        if low.startswith(".subckt"):
            in_subckt = True
            continue
        if low.startswith(".ends"):
            in_subckt = False
            continue
        if in_subckt:
            continue
        if low == ".end":
            continue
        try:
            if low.startswith(".model"):
                m = parse_model(line)
                models[m["name"]] = m
                continue
            el = parse_element(line)
        except ParseError as e:
            raise ParseError(f"Parse error on line {lineno}: {e}")
        if el.kind == 0:
            elements.extend(_instantiate(el, defs))
        else:
            elements.append(el)

    index_map: Dict[str, int] = {}
    seen = set()
    counter = 0
    for el in elements:
        if el.is_g2:
            index_map[f"I({el.identifier})"] = counter
            counter += 1
        for nd in el.nodes:
            if nd not in seen:
                seen.add(nd)
                if nd == "0":
                    continue
                index_map[f"V({nd})"] = counter
                counter += 1
    if not elements:
        raise ParseError("The netlist is empty")
    for el in elements:
        if el.kind == KIND_D:
            m = models.get(el.model_name)
            if m is None or m["type"] != "D":
                raise ParseError(f"Model '{el.model_name}' is not defined")
            el.model = {"is": m["is"], "rs": m["rs"], "n": m["n"]}
            el.value = m["is"]
        elif el.kind == KIND_M:
            m = models.get(el.model_name)
            if m is None or m["type"] != "NMOS":
                raise ParseError(f"Model '{el.model_name}' is not defined")
            el.model = {k: m[k] for k in ("w", "l", "vto", "kp", "lambda")}
    return Circuit(elements, index_map, sorted(seen), models)


def parse_circuit_description_file(path) -> Circuit:
    with open(path, "r") as f:
        return parse_circuit_description(f.read())


def diode_v_critical(is_: float, n: float) -> float:
    """Clamp voltage of diode.rs:65-70: n*VT*ln(f64::MAX * n*VT / Is)."""
    nvt = n * THERMAL_VOLTAGE
    return nvt * math.log(1.7976931348623157e308 * nvt / is_)
