"""Read, write and generate `sim.cfg` files (libconfig format).

The microswimmer driver is configured by a libconfig file whose schema is read
by src/libcilia/global.cpp:21-30 (root keys), src/simulation.cpp:614-673
(`md_objects`), src/sphere.h:14-17, src/cilia.h:11-24,
src/ConstantBeatCilia.h:14-21 and src/clami.cpp:32-118.  The reference writes
these files with pylibconfig2 (create.py:56-112, sr/sim_cfg.py:124-140); this
module reads and writes the same format without that dependency.

Groups map to dict, arrays and lists to list.  `Array` marks a libconfig array
(`[...]`) when writing; plain Python lists are written as lists (`(...)`)
unless all items are scalars.
"""
from __future__ import annotations

import math
import re

import numpy as np

__all__ = ["parse", "load", "dumps", "save", "fibonacci_clami", "plain_fluid", "baseline_config"]


class ParseError(ValueError):
    pass


_TOKEN = re.compile(
    r"""(?P<ws>\s+)|(?P<comment>\#[^\n]*|//[^\n]*|/\*.*?\*/)|
        (?P<str>"(?:[^"\\]|\\.)*")|
        (?P<float>[-+]?(?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|[-+]?\d+[eE][-+]?\d+)|
        (?P<hex>[-+]?0[xX][0-9a-fA-F]+L{0,2})|
        (?P<int>[-+]?\d+L{0,2})|
        (?P<bool>(?i:true|false)\b)|
        (?P<name>[A-Za-z*][-A-Za-z0-9_*]*)|
        (?P<punct>[=:;,{}\[\]()])""",
    re.VERBOSE | re.DOTALL,
)


def _tokens(text):
    pos = 0
    line = 1
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise ParseError(f"line {line}: syntax error near {text[pos:pos + 20]!r}")
        kind = m.lastgroup
        val = m.group(kind)
        if kind not in ("ws", "comment"):
            yield kind, val, line
        line += val.count("\n")
        pos = m.end()


def _unescape(s):
    out = []
    i = 0
    while i < len(s):
        c = s[i]
        if c == "\\" and i + 1 < len(s):
            e = s[i + 1]
            out.append({"n": "\n", "t": "\t", "r": "\r", "f": "\f", "\\": "\\", '"': '"'}.get(e, e))
            i += 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


class Array(list):
    """A libconfig array (homogeneous scalars, written with brackets)."""


class _Parser:
    def __init__(self, text):
        self.toks = list(_tokens(text))
        self.i = 0

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else (None, None, -1)

    def take(self, kind=None, val=None):
        t = self.peek()
        if t[0] is None or (kind and t[0] != kind) or (val and t[1] != val):
            raise ParseError(f"line {t[2]}: unexpected {t[1]!r}")
        self.i += 1
        return t

    def settings(self, close=None):
        out = {}
        while True:
            k, v, line = self.peek()
            if k is None:
                if close:
                    raise ParseError("unexpected end of file")
                return out
            if k == "punct" and v == close:
                return out
            name = self.take("name")[1]
            sep = self.take("punct")
            if sep[1] not in "=:":
                raise ParseError(f"line {sep[2]}: expected '=' or ':'")
            if name in out:
                raise ParseError(f"line {line}: duplicate setting {name}")
            out[name] = self.value()
            k, v, _ = self.peek()
            if k == "punct" and v in ";,":
                self.i += 1

    def value(self):
        k, v, line = self.peek()
        if k == "punct" and v == "{":
            self.i += 1
            g = self.settings("}")
            self.take("punct", "}")
            return g
        if k == "punct" and v in "[(":
            self.i += 1
            close = "]" if v == "[" else ")"
            items = Array() if v == "[" else []
            first = True
            while True:
                k2, v2, _ = self.peek()
                if k2 == "punct" and v2 == close:
                    self.i += 1
                    return items
                if not first:
                    self.take("punct", ",")
                first = False
                items.append(self.value())
        if k == "str":
            s = ""
            while self.peek()[0] == "str":
                s += _unescape(self.take("str")[1][1:-1])
            return s
        self.i += 1
        if k == "float":
            return float(v)
        if k == "int":
            return int(v.rstrip("L"))
        if k == "hex":
            return int(v.rstrip("L"), 16)
        if k == "bool":
            return v.lower() == "true"
        raise ParseError(f"line {line}: unexpected {v!r}")


def parse(text: str) -> dict:
    """Parse libconfig text into nested dict/list values."""
    return _Parser(text).settings()


def load(path) -> dict:
    with open(path) as f:
        return parse(f.read())


def _fmt_float(x: float) -> str:
    r = repr(float(x))
    if "inf" in r or "nan" in r:
        raise ValueError("libconfig cannot represent non-finite floats")
    return r if any(c in r for c in ".e") else r + ".0"


def _fmt(v, indent):
    pad = "  " * indent
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        return _fmt_float(v)
    if isinstance(v, str):
        return '"' + v.replace("\\", "\\\\").replace('"', '\\"').replace("\n", "\\n") + '"'
    if isinstance(v, dict):
        inner = "".join(f"{pad}  {k} = {_fmt(x, indent + 1)};\n" for k, x in v.items())
        return "{\n" + inner + pad + "}"
    if isinstance(v, (list, tuple, np.ndarray)):
        items = list(v)
        scalar = all(not isinstance(x, (dict, list, tuple, np.ndarray)) for x in items)
        if isinstance(v, Array) or (scalar and items and not isinstance(v, tuple)):
            return "[ " + ", ".join(_fmt(x, indent) for x in items) + " ]"
        if not items:
            return "( )"
        inner = (",\n").join(pad + "  " + _fmt(x, indent + 1) for x in items)
        return "(\n" + inner + "\n" + pad + ")"
    raise TypeError(f"cannot write {type(v)}")


def dumps(cfg: dict) -> str:
    return "".join(f"{k} = {_fmt(v, 0)};\n" for k, v in cfg.items())


def save(cfg: dict, path) -> None:
    with open(path, "w") as f:
        f.write(dumps(cfg))


# ---------------------------------------------------------------- generators --

def plain_fluid(L: int, *, tstep=0.1, desiredt=None, name="fluid") -> dict:
    """Periodic box of L^3 cells with no MD objects."""
    return {
        "name": name, "globalt": 0.0, "desiredt": float(desiredt if desiredt is not None else 1000 * tstep),
        "runtime": 86400.0, "tstep": float(tstep), "omega": 0.0,
        "sizex": int(L), "sizey": int(L), "sizez": int(L), "md_objects": (),
    }


def fibonacci_clami(n_cilia: int, *, radius: float, center, rodlength: int = 15,
                    springconstant: float = 5000.0, beatstrength: float = 0.17,
                    max_energy: float = 1.0, tau_power: float = 100.0 / 3.0,
                    tau_recovery: float = 200.0 / 3.0, m_speed: float = 5.3, seed: int = 0,
                    name: str = "volvox") -> dict:
    """A Clami with `n_cilia` cilia on a Fibonacci lattice over the sphere.

    The reference places cilia on rings (src/clami.cpp:81-101); a Fibonacci
    lattice is one ring per cilium.  Ring i has one cilium at latitude
    y_thetas[i] (degrees) and azimuth theta_offset[i], and the anchor is at
    r*(sin(thetaY), -cos(thetaY) sin(thetaX), cos(thetaX) cos(thetaY))
    (src/clami.cpp:126-129).  For the unit direction u of lattice point i this
    gives thetaY = asin(u_x) and thetaX = atan2(-u_y, u_z).  Phases are drawn
    uniformly in [0, 2 pi) and mapped to start delays as create.py:91-99 does
    (delay = phase / 2 pi * (tau_power + tau_recovery)).  The stall threshold
    `bending` is sqrt(2 E / k) (create.py:20).
    """
    rng = np.random.default_rng(seed)
    golden = math.pi * (3.0 - math.sqrt(5.0))
    y_thetas, offsets = [], []
    for i in range(n_cilia):
        z = 1.0 - 2.0 * (i + 0.5) / max(n_cilia, 1)
        r = math.sqrt(max(0.0, 1.0 - z * z))
        phi = golden * i
        u = (r * math.cos(phi), r * math.sin(phi), z)
        y_thetas.append(math.degrees(math.asin(max(-1.0, min(1.0, u[0])))))
        offsets.append(math.atan2(-u[1], u[2]))
    tau = tau_power + tau_recovery
    delays = [float(round(p / (2 * math.pi) * tau, 6)) for p in rng.uniform(0, 2 * math.pi, n_cilia)]
    cilia = {
        "type": "ConstantBeatCilia", "name": "cilia", "rodlength": int(rodlength),
        "beatstrength": float(beatstrength), "bending": float(math.sqrt(2 * max_energy / springconstant)),
        "min_bend": -0.7, "max_bend": 0.7, "m_speed": float(m_speed),
        "springconstant": float(springconstant), "position": Array([0.0, 0.0, 0.0]),
        "thetaX": 0.0, "thetaY": 0.0, "thetaZ": 0.0, "write_data": False,
        "power_stroke_duration": float(tau_power), "recovery_stroke_duration": float(tau_recovery),
        "start_delay": 0.0,
    }
    return {
        "type": "Clami", "name": name, "radius": float(radius), "springconstant": float(springconstant),
        "position": Array([float(c) for c in center]),
        "num_equators": Array([1] * n_cilia), "y_thetas": Array([float(x) for x in y_thetas]),
        "theta_offset": Array([float(x) for x in offsets]), "start_delays": Array(delays),
        "cilia": cilia,
    }


def swimmer_config(L: int, *, radius: float, n_cilia: int, rodlength: int = 15, seed: int = 0,
                   ststep: float = 0.002, name: str = "swimmer") -> dict:
    """A periodic L^3 box (10 particles per cell) with a Clami of `n_cilia`
    Fibonacci-lattice cilia at the centre (the ensemble and serving workloads)."""
    cfg = plain_fluid(int(L), name=name)
    cfg["ststep"] = float(ststep)
    cfg["md_objects"] = (fibonacci_clami(int(n_cilia), radius=float(radius), center=(L / 2, L / 2, L / 2),
                                         rodlength=int(rodlength), seed=seed),)
    return cfg


def ensemble_specs(n: int, seed: int = 0, edges=(16, 24, 32, 40, 48), max_cilia: int = 64,
                   rodlengths=(10, 15)) -> list:
    """Replica shapes of the batched ensemble: box edge uniform over `edges`,
    sphere radius edge/8, cilia count uniform in [0, max_cilia], rodlength
    uniform in [rodlengths[0], rodlengths[1]], independent seeds."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.choice(edges))
        out.append(dict(L=L, radius=L / 8.0, n_cilia=int(rng.integers(0, max_cilia + 1)),
                        rodlength=int(rng.integers(rodlengths[0], rodlengths[1] + 1)), seed=int(1000 * seed + i + 1)))
    return out


def baseline_config(which: str, **kw) -> dict:
    """Configurations of the benchmark workloads.

    plain32   : 32^3 periodic fluid, h = 0.1, no swimmer.
    swimmer64 : 64^3 fluid with a radius-8 Clami at the centre, 100 cilia of
                rodlength 15 on a Fibonacci lattice, spring constant 5000
                (stiffness 1e4 kT/a^2 for U = k (d - b)^2), beat period 1000
                MPC steps split 1:2, MD step 0.002 (50 substeps).
    swimmer128: 128^3 fluid, radius 16, 400 cilia of rodlength 20.
    """
    if which == "plain32":
        return plain_fluid(32, name="plain32")
    if which in ("swimmer64", "swimmer128"):
        L, R, nc, rl = (64, 8.0, 100, 15) if which == "swimmer64" else (128, 16.0, 400, 20)
        cfg = plain_fluid(L, name=which)
        cfg["ststep"] = 0.002
        cfg["md_objects"] = (fibonacci_clami(nc, radius=R, center=(L / 2, L / 2, L / 2), rodlength=rl,
                                             seed=kw.get("seed", 0)),)
        return cfg
    raise KeyError(which)
