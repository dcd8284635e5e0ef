"""NMODL front end for linear kinetic channels (the reference library's ``KINETIC`` files).

The reference parses NMODL with BlueBrain's ``nmodl`` library and hands a
``SOLVE ... METHOD sparse`` block to lti_sim (neuwon/rxd/nmodl/__init__.py:243-306,
313-325).  That parser is a third-party C++ package; this module reads the
subset of NMODL that the reference's ``nmodl_library/kinetic`` channels and
``artificial/passive.mod`` use, and turns a file into a ``Kinetic`` mechanism
whose scheme runs on the device:

* ``NEURON``: ``SUFFIX`` (the mechanism's name), ``USEION x ... WRITE ix`` (its
  conductance feeds species ``x``: conductances go to the species' accumulator,
  nmodl/__init__.py:168-208) or ``NONSPECIFIC_CURRENT i`` (a nonspecific
  conductance with the reversal potential parameter ``e``);
* ``PARAMETER``: values with units; the density ``gbar`` (or ``g``) is converted to
  S/cm2 from mho, S, mmho, mS, umho or uS per cm2;
* ``STATE``; ``INITIAL`` assignments other than states (``SOLVE ... STEADYSTATE``
  is the steady state the model computes);
* ``PROCEDURE`` and ``FUNCTION`` bodies of assignments, ``UNITSOFF``/``UNITSON``;
* ``KINETIC``: procedure calls, reactions ``~ A <-> B (kf, kb)``, ``CONSERVE``;
* ``BREAKPOINT``: the conductance ``g = gbar * (open states summed)``.

Expressions are NMODL arithmetic (``+ - * / ^``, parentheses, ``exp``, ``log``,
``fabs``, ``sqrt``, ``pow``, the file's functions) with unit annotations after
numbers removed; they are evaluated with numpy over arrays of voltages.
Anything else raises ``NotImplementedError`` naming the construct.
"""
import math
import os
import re

import numpy as np

# A numeric literal (not the tail of a name such as rates2) followed by a unit in parentheses.
_UNIT_AFTER_NUMBER = re.compile(r"(?<![\w.])((?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)\s*\(\s*[A-Za-z/][^()]*\)")
_NUMBER_UNITS = {"mho": 1.0, "s": 1.0, "siemens": 1.0, "mmho": 1e-3, "millimho": 1e-3, "ms": 1e-3,
                 "millisiemens": 1e-3, "umho": 1e-6, "micromho": 1e-6, "us": 1e-6, "microsiemens": 1e-6}
_MATH = {"exp": np.exp, "log": np.log, "log10": np.log10, "fabs": np.abs, "sqrt": np.sqrt, "pow": np.power,
         "sin": np.sin, "cos": np.cos, "tanh": np.tanh}


def _strip_comments(text):
    text = re.sub(r"\bCOMMENT\b.*?\bENDCOMMENT\b", "", text, flags=re.S)
    return re.sub(r":[^\n]*", "", text)


def _blocks(text):
    """Top-level blocks as (keyword, header, body) in file order."""
    out = []
    pos = 0
    head = re.compile(r"\b(NEURON|UNITS|PARAMETER|ASSIGNED|STATE|BREAKPOINT|INITIAL|DERIVATIVE|KINETIC|"
                      r"PROCEDURE|FUNCTION|NET_RECEIVE|CONSTANT|INDEPENDENT|TITLE)\b([^{\n]*)")
    while True:
        m = head.search(text, pos)
        if not m:
            break
        kw, header = m.group(1), m.group(2).strip()
        if kw == "TITLE":
            pos = m.end()
            continue
        brace = text.find("{", m.end() - len(m.group(2)))
        if brace < 0:
            raise NotImplementedError(f"NMODL: block {kw} without a body")
        depth, k = 0, brace
        while k < len(text):
            if text[k] == "{":
                depth += 1
            elif text[k] == "}":
                depth -= 1
                if depth == 0:
                    break
            k += 1
        out.append((kw, text[m.end(1):brace].strip(), text[brace + 1:k]))
        pos = k + 1
    return out


def _expr(src):
    """An NMODL expression as Python source."""
    src = _UNIT_AFTER_NUMBER.sub(r"\1", src)
    return src.replace("^", "**").strip()


def _split_top(src, sep=","):
    parts, depth, cur = [], 0, ""
    for ch in src:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def _statements(body):
    """Lines of a block body, without unit switches and empty lines."""
    out = []
    for line in body.split("\n"):
        line = line.strip()
        if not line or line in ("UNITSOFF", "UNITSON"):
            continue
        out.append(line)
    return out


def _assignment(line):
    m = re.match(r"^([A-Za-z_]\w*)\s*=\s*(.+)$", line)
    return (m.group(1), _expr(m.group(2))) if m else None


class KineticFile:
    """A parsed kinetic channel file; ``scheme()`` builds its KineticScheme."""

    def __init__(self, text, filename="<nmodl>"):
        self.filename = filename
        blocks = _blocks(_strip_comments(text))
        kinds = [b[0] for b in blocks]
        for bad in ("DERIVATIVE", "NET_RECEIVE"):
            if bad in kinds:
                raise NotImplementedError(f"{filename}: {bad} blocks have no device path")
        self.suffix, self.ion, self.nonspecific = None, None, False
        self.parameters, self.units, self.states = {}, {}, []
        self.initial, self.procedures, self.functions = [], {}, {}
        self.kinetic, self.breakpoint = None, []
        self.locals = []
        for kw, header, body in blocks:
            if kw == "NEURON":
                self._neuron(body)
            elif kw == "PARAMETER":
                # name = value (units) <range>, any number per line.
                for m in re.finditer(r"([A-Za-z_]\w*)\s*=\s*([-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)"
                                     r"\s*(?:\(([^)]*)\))?", body):
                    self.parameters[m.group(1)] = float(m.group(2))
                    self.units[m.group(1)] = (m.group(3) or "").strip()
            elif kw == "STATE":
                self.states = [s for s in re.findall(r"[A-Za-z_]\w*", re.sub(r"\([^)]*\)", "", body))]
            elif kw == "INITIAL":
                self.initial = _statements(body)
            elif kw == "PROCEDURE":
                name, args = self._signature(header)
                self.procedures[name] = (args, _statements(body))
            elif kw == "FUNCTION":
                name, args = self._signature(header)
                self.functions[name] = (args, _statements(body))
            elif kw == "KINETIC":
                self.kinetic = _statements(body)
            elif kw == "BREAKPOINT":
                self.breakpoint = _statements(body)
        text_nc = _strip_comments(text)
        for m in re.finditer(r"^\s*LOCAL\s+([^\n]+)", text_nc, flags=re.M):
            self.locals += [s.strip() for s in m.group(1).split(",")]
        if self.suffix is None:
            raise NotImplementedError(f"{filename}: no SUFFIX (point processes have no device path)")
        self._conductance()

    _NEURON_KEYWORDS = {"SUFFIX", "POINT_PROCESS", "ARTIFICIAL_CELL", "USEION", "NONSPECIFIC_CURRENT", "RANGE",
                        "GLOBAL", "POINTER", "BBCOREPOINTER", "EXTERNAL", "THREADSAFE", "ELECTRODE_CURRENT"}

    def _neuron(self, body):
        """NEURON statements, any number per line: each keyword's words up to the next keyword."""
        words = re.sub(r"\([^)]*\)", " ", body).replace(",", " ").split()
        stmts, cur = [], None
        for w in words:
            if w in self._NEURON_KEYWORDS:
                cur = [w]
                stmts.append(cur)
            elif cur is not None:
                cur.append(w)
        for st in stmts:
            if st[0] == "SUFFIX":
                self.suffix = st[1]
            elif st[0] in ("POINT_PROCESS", "ARTIFICIAL_CELL"):
                raise NotImplementedError(f"{self.filename}: {st[0]} has no device path")
            elif st[0] == "USEION":
                ion = st[1]
                write = []
                if "WRITE" in st:
                    write = st[st.index("WRITE") + 1:]
                    write = write[:write.index("VALENCE")] if "VALENCE" in write else write
                if f"e{ion}" in write:
                    raise NotImplementedError(f"{self.filename}: writes a reversal potential (hh-type mechanism)")
                if f"i{ion}" in write or f"g{ion}" in write:
                    if self.ion is not None:
                        raise NotImplementedError(f"{self.filename}: writes two ions")
                    self.ion = ion
            elif st[0] == "NONSPECIFIC_CURRENT":
                self.nonspecific = True
            elif st[0] == "POINTER":
                raise NotImplementedError(f"{self.filename}: POINTER variables have no device path")

    @staticmethod
    def _signature(header):
        m = re.match(r"^([A-Za-z_]\w*)\s*\((.*)\)\s*(?:\([^)]*\))?\s*$", header.strip())
        if not m:
            raise NotImplementedError(f"NMODL: cannot read the signature {header!r}")
        args = [re.sub(r"\(.*", "", a).strip() for a in _split_top(m.group(2))] if m.group(2).strip() else []
        return m.group(1), args

    def _conductance(self):
        """g = gbar * (sum of states) from BREAKPOINT; density in S/cm2."""
        self.open_states, self.gbar_name = None, None
        for line in self.breakpoint:
            a = _assignment(line)
            if not a or a[0] != "g":
                continue
            rhs = a[1].replace(" ", "")
            m = re.match(r"^([A-Za-z_]\w*)\*\(?([A-Za-z_]\w*(?:\+[A-Za-z_]\w*)*)\)?$", rhs)
            if not m or m.group(1) not in self.parameters:
                raise NotImplementedError(f"{self.filename}: conductance {a[1]!r} is not gbar * (open states)")
            self.gbar_name = m.group(1)
            self.open_states = m.group(2).split("+")
        if self.open_states is None:
            if self.states or not self.nonspecific:
                raise NotImplementedError(f"{self.filename}: no conductance 'g = gbar * ...' in BREAKPOINT")
            # A passive channel (passive.mod): i = g * (v - e) with g a density.
            self.gbar_name, self.open_states = "g", []
        if self.gbar_name not in self.parameters:
            raise NotImplementedError(f"{self.filename}: no density parameter {self.gbar_name!r}")
        unit = self.units.get(self.gbar_name, "").lower().replace(" ", "")
        scale = 1.0
        if unit:
            num = unit.split("/")[0]
            if num not in _NUMBER_UNITS or not unit.endswith("/cm2"):
                raise NotImplementedError(f"{self.filename}: density units {unit!r}")
            scale = _NUMBER_UNITS[num]
        self.gbar = self.parameters[self.gbar_name] * scale
        self.erev = self.parameters.get("e", 0.0) if self.nonspecific else 0.0

    # ------------------------------------------------------------ evaluation
    def _namespace(self, v, celsius):
        ns = dict(_MATH)
        ns.update(self.parameters)
        ns["v"], ns["celsius"] = v, float(celsius)
        for name, (args, body) in self.functions.items():
            ns[name] = self._function(name, args, body, ns)
        for line in self.initial:
            if line.startswith(("SOLVE", "STEADYSTATE")):
                continue
            a = _assignment(line)
            if a is None:
                raise NotImplementedError(f"{self.filename}: INITIAL statement {line!r}")
            if a[0] in self.states:
                continue
            ns[a[0]] = eval(a[1], {"__builtins__": {}}, ns)
        return ns

    def _function(self, name, args, body, ns):
        def fn(*vals):
            local = dict(ns)
            local.update(zip(args, vals))
            for line in body:
                a = _assignment(line)
                if a is None:
                    raise NotImplementedError(f"{self.filename}: FUNCTION {name} statement {line!r}")
                local[a[0]] = eval(a[1], {"__builtins__": {}}, local)
            return local[name]
        return fn

    def _call(self, line, ns):
        m = re.match(r"^([A-Za-z_]\w*)\s*\((.*)\)$", line)
        if not m or m.group(1) not in self.procedures:
            raise NotImplementedError(f"{self.filename}: statement {line!r}")
        args, body = self.procedures[m.group(1)]
        vals = [eval(_expr(x), {"__builtins__": {}}, ns) for x in _split_top(m.group(2))] if m.group(2) else []
        saved = {k: ns[k] for k in args if k in ns}
        ns.update(zip(args, vals))
        for stmt in body:
            a = _assignment(stmt)
            if a is None:
                self._call(stmt, ns)
            else:
                ns[a[0]] = eval(a[1], {"__builtins__": {}}, ns)
        ns.update(saved)

    def transitions(self, v, celsius):
        v = np.asarray(v, dtype=np.float64)
        ns = self._namespace(v, celsius)
        out, self.conserve_sum = [], None
        for line in self.kinetic or []:
            if line.startswith("~"):
                m = re.match(r"^~\s*([A-Za-z_]\w*)\s*<->\s*([A-Za-z_]\w*)\s*\((.*)\)\s*$", line)
                if not m:
                    raise NotImplementedError(f"{self.filename}: reaction {line!r}")
                kf, kb = _split_top(m.group(3))
                a, b = self.states.index(m.group(1)), self.states.index(m.group(2))
                ones = np.ones_like(v)
                out.append((a, b, ones * eval(_expr(kf), {"__builtins__": {}}, ns)))
                out.append((b, a, ones * eval(_expr(kb), {"__builtins__": {}}, ns)))
            elif line.startswith("CONSERVE"):
                continue
            else:
                self._call(line, ns)
        return out

    def conserve(self):
        for line in self.kinetic or []:
            if line.startswith("CONSERVE"):
                m = re.match(r"^CONSERVE\s+(.+?)\s*=\s*([-+]?[\d.]+(?:[eE][-+]?\d+)?)\s*$", line)
                names = set(s.strip() for s in m.group(1).split("+"))
                if names != set(self.states):
                    raise NotImplementedError(f"{self.filename}: CONSERVE must use all states")
                return float(m.group(2))
        return None

    def scheme(self):
        from .kinetic import KineticScheme
        if not self.states:
            return KineticScheme(self.suffix, ["O"], lambda v, celsius: [], open_states=["O"], conserve_sum=1.0)
        return KineticScheme(self.suffix, self.states, self.transitions, open_states=self.open_states,
                             conserve_sum=self.conserve())


def kinetic_mechanism(filename, text=None, **table):
    """The ``Kinetic`` mechanism class of an NMODL file (see the module docstring);
    table keywords (vmin, vmax, num_buckets, degree) override the voltage table,
    by default LinearInput -100..100 mV (nmodl/__init__.py:321-322) in 0.1 mV buckets."""
    from .kinetic import Kinetic
    if text is None:
        with open(filename, "rt") as f:
            text = f.read()
    kf = KineticFile(text, os.path.basename(str(filename)))
    params = dict(name=kf.suffix, scheme_factory=kf.scheme, gbar=kf.gbar, erev=kf.erev, ion=kf.ion,
                  vmin=-100.0, vmax=100.0, num_buckets=2000, degree=1)
    params.update(table)
    return Kinetic.configure(**params)
