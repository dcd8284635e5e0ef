"""Mechanism plugin API (neuwon/rxd/mechanisms.py:4-111) and the GPU mechanisms.

The reference compiles NMODL files into ``@Compute`` Python kernels.  Here a
mechanism is a host-side class that owns its instances' parameters; its
``advance`` runs inside the fused device step, so ``advance()`` on the class
is only a marker.  Mechanisms without a device kernel are rejected when the
model is created rather than silently run on the CPU.
"""
import math
import os
import re

import numpy as np


class Mechanism:
    """Abstract mechanism, same contract as neuwon/rxd/mechanisms.py:4-54."""
    omnipresent = False

    @classmethod
    def initialize(cls, model):
        """Set up this mechanism; may return a new Mechanism subclass."""
        return None

    @classmethod
    def get_name(cls):
        raise NotImplementedError(cls)

    @classmethod
    def other_mechanisms(cls):
        return []

    def __init__(self, segment, outside=None, magnitude=1.0, *other_mechanisms):
        raise NotImplementedError(type(self))

    @classmethod
    def advance(cls):
        """The device step advances every instance; nothing to do on the host."""
        return None


class HH(Mechanism):
    """Hodgkin-Huxley Na/K/leak channels, nmodl_library/artificial/hh.mod.

    Parameters follow the .mod file (S/cm2, mV); ``HH.configure(...)`` returns a
    subclass with other defaults (e.g. ena=50, ek=-77).  As compiled by the
    reference's NMODL front end (neuwon/rxd/nmodl/__init__.py:99-107, 168-208,
    492-500): each instance's conductance coefficient is gbar * 1e-8 * magnitude
    with magnitude = user magnitude * segment surface area (um2) at insertion
    time, and the three conductances are nonspecific (reversal potentials are
    class constants).  ``gnabar``/``gkbar``/``glbar`` may also be given per
    instance as keyword arguments (channel densities in S/cm2).
    """
    name = "hh"
    gnabar, gkbar, glbar = 0.12, 0.036, 0.0003
    ena, ek, el = 60.0, -88.0, -54.3
    _model = None

    @classmethod
    def configure(cls, **params):
        bad = set(params) - {"gnabar", "gkbar", "glbar", "ena", "ek", "el", "name"}
        if bad:
            raise ValueError(f"unknown HH parameters {sorted(bad)}")
        return type(cls.__name__, (cls,), dict(params))

    @classmethod
    def initialize(cls, model):
        bound = type(cls.__name__, (cls,), {"_model": model, "_instances": []})
        return bound

    @classmethod
    def get_name(cls):
        return cls.name

    def __init__(self, segment, outside=None, magnitude=1.0, *other_mechanisms,
                 gnabar=None, gkbar=None, glbar=None):
        model = type(self)._model
        if model is None:
            raise TypeError("mechanism class is not bound to a model; use model.mechanisms[name]")
        magnitude = float(magnitude)
        if not magnitude >= 0.0:
            raise ValueError("magnitude must be >= 0")
        self.segment = segment
        self.magnitude = magnitude
        self.index = model._add_mechanism_instance(
            type(self), segment, magnitude,
            dict(gnabar=gnabar, gkbar=gkbar, glbar=glbar))

    @classmethod
    def get_database_class(cls):
        return cls


def hh_steady_state(v, celsius=6.3):
    """Steady-state (m, h, n) of hh.mod at voltage v (INITIAL block, hh.mod:48-53)."""
    v = np.asarray(v, dtype=np.float64)

    def vtrap(x, y):
        with np.errstate(divide="ignore", invalid="ignore"):
            big = x / np.expm1(x / y)
        return np.where(np.abs(x / y) < 1e-6, y * (1 - x / y / 2), big)
    a = .1 * vtrap(-(v + 40), 10); b = 4 * np.exp(-(v + 65) / 18); m = a / (a + b)
    a = .07 * np.exp(-(v + 65) / 20); b = 1 / (np.exp(-(v + 35) / 10) + 1); h = a / (a + b)
    a = .01 * vtrap(-(v + 55), 10); b = .125 * np.exp(-(v + 65) / 80); n = a / (a + b)
    return m, h, n


def NMODL(filename, use_cache=True, **table):
    """NMODL front end: maps a .mod file onto a GPU mechanism.

    The reference parses NMODL with BlueBrain's nmodl library
    (neuwon/rxd/nmodl/parser.py).  Here ``SUFFIX hh`` becomes the HH mechanism
    with the file's PARAMETER defaults, and linear kinetic channels (KINETIC
    block, ``SOLVE ... METHOD sparse``) and passive channels become ``Kinetic``
    mechanisms through ``neuwon_gb300.nmodl`` (table keywords: vmin, vmax,
    num_buckets, degree); other files raise.
    """
    filename = os.path.abspath(str(filename))
    with open(filename, "rt") as f:
        text = f.read()
    text_nc = re.sub(r"COMMENT.*?ENDCOMMENT", "", text, flags=re.S)
    text_nc = re.sub(r":.*", "", text_nc)
    m = re.search(r"SUFFIX\s+(\w+)", text_nc)
    suffix = m.group(1) if m else None
    params = {}
    pm = re.search(r"PARAMETER\s*\{(.*?)\}", text_nc, flags=re.S)
    if pm:
        for name, value in re.findall(r"(\w+)\s*=\s*([-+]?[\d.]+(?:[eE][-+]?\d+)?)", pm.group(1)):
            params[name] = float(value)
    if suffix == "hh":
        keep = {k: v for k, v in params.items() if k in ("gnabar", "gkbar", "glbar", "ena", "ek", "el")}
        return HH.configure(**keep)
    from .nmodl import kinetic_mechanism
    return kinetic_mechanism(filename, text, **table)
