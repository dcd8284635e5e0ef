"""Drop-in backend for the reference's own ``RxD_Model.advance`` (neuwon/rxd/rxd_model.py:63-80).

A maintainer who keeps the reference's ``Database`` and its Python API installs

    model.advance = GB300Advance(model, hh={"hh": dict(gnabar=.12, gkbar=.036, glbar=.0003)})

after building the model.  Every call then runs one staggered step on the GPU
through the C ABI (include/neuwon_gb300.h) instead of the host path:

* the structure is read from the reference's ``Database`` after ``db.sort()``
  (``Database.sort``, database.py:189-222: segments neuron-contiguous, pointers
  valid until the next sort) -- parents, neuron of each segment, capacitance,
  axial resistance, voltage -- and re-read whenever the database was sorted
  again or grew;
* hh instances are read from their mechanism class (``segment``, ``magnitude``,
  gates ``m``/``h``/``n``; the reversal potentials from the class attributes of
  its nonspecific conductances, species.py:229-248); their densities, which the
  NMODL front end inlines into generated code, are given by the caller;
* electric species with constant reversal potentials (species.py:85-142) and
  kinetic mechanisms given as lti_sim tables feed the same accumulators as on
  the device;
* current clamps: ``Segment.inject_current`` plays a ``TimeSeries`` into
  ``Segment.sum_current`` on the input clock (electric.py:119-125,
  time.py:245-302); before each step the players registered on that clock are
  turned into device clamps for the step's two input ticks, then the clock is
  ticked, so the players advance as they would on the host;
* after each step the voltages and AP-detector flags are written back into the
  reference's arrays and the advance clock is ticked, so ``TimeSeries.record``,
  ``Segment.voltage`` and ``Neuron.AP_detected`` read as after the host step.

``extract`` returns the arrays read from the reference; ``GB300Advance.from_arrays``
installs such a set without a reference model (the test on the GPU replays
arrays recorded by running the reference).
"""
import ctypes

import numpy as np

from . import _lib
from .mechanisms import hh_steady_state
from .morphology import EPSILON

NULL = 0xFFFFFFFF          # neuwon/database/dtypes.py: NULL pointer (uint32)


def _db_array(db, name, dtype):
    a = db.get_data(name)
    return np.array(a, dtype=dtype, copy=True)


def extract(model, hh=None):
    """The arrays the C ABI needs, read from a reference ``RxD_Model`` after
    ``db.sort()``.  hh maps the names of hh-type mechanism classes to their
    densities (S/cm2: gnabar, gkbar, glbar)."""
    db = model.get_database()
    db.sort()
    parent = _db_array(db, "Segment.parent", np.int64)
    parent[parent == NULL] = -1
    neuron = _db_array(db, "Segment.neuron", np.int64)
    counts = np.bincount(neuron, minlength=int(neuron.max()) + 1 if len(neuron) else 0)
    out = {"parent": parent, "neuron_start": np.concatenate([[0], np.cumsum(counts)]).astype(np.int64),
           "capacitance": _db_array(db, "Segment.capacitance", np.float64),
           "axial_resistance": _db_array(db, "Segment.axial_resistance", np.float64),
           "voltage": _db_array(db, "Segment.voltage", np.float64),
           "time_step": float(model.get_time_step()), "celsius": float(model.get_temperature())}
    if np.any(np.diff(neuron) < 0):
        raise ValueError("Segment table is not sorted by neuron after db.sort()")
    for name, dens in (hh or {}).items():
        cls = db.get_class(name)
        seg = _db_array(db, f"{name}.segment", np.int64)
        mag = _db_array(db, f"{name}.magnitude", np.float64)
        rev = {ion: float(db.get_data(f"{name}.{ion}_reversal_potential")) for ion in ("na", "k", "l")}
        out["hh"] = {"segment": seg, "magnitude": mag,
                     "m": _db_array(db, f"{name}.m", np.float64), "h": _db_array(db, f"{name}.h", np.float64),
                     "n": _db_array(db, f"{name}.n", np.float64),
                     "gnabar": float(dens["gnabar"]), "gkbar": float(dens["gkbar"]), "glbar": float(dens["glbar"]),
                     "ena": rev["na"], "ek": rev["k"], "el": rev["l"], "name": cls.get_name()}
        break                               # the device holds one hh mechanism
    return out


def clamp_players(model, tick):
    """The current clamps playing into ``Segment.sum_current`` on the input clock,
    as device clamps (segment, amperes, first tick, ticks) for input ticks tick+1
    and tick+2: one clamp per player and tick, the value it will add then
    (TimeSeries._play_implementation, time.py:287-302, "+=" mode)."""
    out = []
    hook = model.input_hook._callbacks                  # Clock -> CallbackHook (time.py:13-41, 65)
    for cb in list(hook._callbacks):
        ts = getattr(cb, "__self__", None)
        if ts is None or getattr(ts, "play_data", None) is None:
            continue
        if getattr(ts, "component_name", None) != "sum_current" or ts.mode != "+=":
            raise NotImplementedError("only '+=' players of Segment.sum_current have a device path")
        seg = int(ts.db_object.get_unstable_index())
        idx, data = ts.play_index, ts.play_data
        for k in range(2):
            j = idx + k
            if j >= len(data):
                if not ts.play_loop:
                    break
                j %= len(data)
            out.append((seg, float(data[j]), tick + 1 + k, 1))
    return out


class GB300Advance:
    """``RxD_Model.advance`` on the GPU; see the module docstring."""

    def __init__(self, model=None, *, hh=None, precision="f64", device=0, propagator_tolerance=EPSILON,
                 arrays=None, write_back=True):
        self.model = model
        self.hh = hh
        self.precision = precision
        self.device = int(device)
        self.tolerance = float(propagator_tolerance)
        self.write_back = bool(write_back) and model is not None
        self.ctx = None
        self.ticks = 0
        self.arrays = arrays if arrays is not None else extract(model, hh)
        self._install()

    @classmethod
    def from_arrays(cls, arrays, **kw):
        """A backend for arrays ``extract`` produced (no reference model attached)."""
        return cls(None, arrays=arrays, **kw)

    def _install(self):
        a = self.arrays
        if self.ctx is not None:
            self.ctx.close()
        self.ctx = ctx = _lib.Context(self.device, self.precision)
        n = len(a["parent"])
        ns = len(a["neuron_start"]) - 1
        ctx.call("nw_model_init", n, ns, _lib.ptr(np.ascontiguousarray(a["neuron_start"])),
                 _lib.ptr(np.ascontiguousarray(a["parent"])), a["time_step"], a["celsius"])
        ctx.set_data("Segment.capacitance", a["capacitance"])
        ctx.set_data("Segment.axial_resistance", np.where(a["parent"] < 0, 1.0, a["axial_resistance"]))
        ctx.set_data("Segment.voltage", a["voltage"])
        nnz = ctypes.c_int64()
        ctx.call("nw_propagator_build", self.tolerance, ctypes.byref(nnz))   # electric.py:78-117
        ctx.set_option("propagator_format", 0)
        if "hh" in a:
            h = a["hh"]
            scale = 1e-8 * h["magnitude"]                                     # nmodl/__init__.py:103-107
            ctx.call("nw_hh_register", len(h["segment"]), _lib.ptr(np.ascontiguousarray(h["segment"])),
                     _lib.ptr(np.ascontiguousarray(h["gnabar"] * scale)),
                     _lib.ptr(np.ascontiguousarray(h["gkbar"] * scale)),
                     _lib.ptr(np.ascontiguousarray(h["glbar"] * scale)), h["ena"], h["ek"], h["el"],
                     float(a["voltage"][0]) if n else -70.0)
            for g in ("m", "h", "n"):
                ctx.set_data(f"hh.{g}", h[g])
        roots = np.asarray(a["neuron_start"][:-1], dtype=np.int64)
        ctx.call("nw_detectors_set", _lib.ptr(roots), _lib.ptr(np.full(ns, 20.0)))
        self.n = n
        self._clamps = None

    def _stale(self):
        """The reference re-sorted or grew its database since the arrays were read."""
        if self.model is None:
            return False
        db = self.model.get_database()
        return (not db.is_sorted()) or len(db.get_data("Segment.voltage")) != self.n

    def set_clamps(self, clamps):
        """Device clamps (segment, amperes, first tick, ticks) for the next step."""
        clamps = list(clamps)
        if clamps == self._clamps:
            return
        seg = np.array([c[0] for c in clamps], dtype=np.int64)
        amp = np.array([c[1] for c in clamps], dtype=np.float64)
        first = np.array([c[2] for c in clamps], dtype=np.int64)
        cnt = np.array([c[3] for c in clamps], dtype=np.int64)
        self.ctx.call("nw_clamps_set", len(clamps), _lib.ptr(seg), _lib.ptr(amp), _lib.ptr(first), _lib.ptr(cnt))
        self._clamps = clamps

    def step(self, clamps=()):
        """One step with the given device clamps (the path without a reference model)."""
        self.set_clamps(clamps)
        self.ctx.advance(1, _lib.PATH_BATCHED)
        self.ticks += 2

    def __call__(self):
        m = self.model
        if self._stale():
            self.arrays = extract(m, self.hh)
            self._install()
        self.set_clamps(clamp_players(m, self.ticks))
        self.ctx.advance(1, _lib.PATH_BATCHED)
        self.ticks += 2
        m.input_hook.tick()                   # the players move on by the step's two ticks
        m.input_hook.tick()
        if self.write_back:
            db = m.get_database()
            db.get_data("Segment.voltage")[:] = self.voltage()
            db.get_data("Neuron.AP_detected")[:] = self.ctx.get_data("Neuron.AP_detected",
                                                                     len(self.arrays["neuron_start"]) - 1, np.uint8)
        m.advance_hook.tick()                 # rxd_model.py:80: recorders read the written-back voltages

    def voltage(self):
        return self.ctx.get_data("Segment.voltage", self.n)

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None


def hh_initial_gates(v_init, celsius=6.3):
    """Steady-state gates of hh.mod's INITIAL block (for arrays built without a reference)."""
    return hh_steady_state(v_init, celsius)
