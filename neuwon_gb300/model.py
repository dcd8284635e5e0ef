"""Host-side mirror of the reference's model API around the GPU step.

``RxD_Model`` keeps the reference's public surface for the hot path
(neuwon/rxd/rxd_model.py:9-80): the constructor arguments, ``Neuron`` and
``Segment`` factories (neuwon/rxd/neuron/neuron.py:35-43,
segment.py:27-104), mechanism insertion (segment.py:124-160,
mechanisms.py:56-99), ``Segment.inject_current`` (electric.py:119-125),
AP detectors (neuron.py:65-75), the clocks (database/time.py:54-121) and
``TimeSeries.record`` of voltages (time.py:189-231).

The segment table is a structure of arrays in creation order.  Before the
first ``advance()`` (and again after any structural change) it is sorted by
neuron the way ``Database.sort()`` does (stable, database.py:589-646), its
geometry and passive properties are computed (morphology.geometry), and
everything is mirrored on the device; the propagator is then built on the
GPU.  After that ``advance()`` is a single C-ABI call.
"""
import math

import numpy as np

from . import _lib
from .morphology import EPSILON, Tree, device_order, geometry, passive_electric
from .kinetic import Kinetic
from .mechanisms import HH, Mechanism, hh_steady_state

MAX_KINETIC = 8     # kinetic mechanisms per model (the device's table of them)


class Clock:
    """Tick counter; neuwon/database/time.py:54-121."""

    def __init__(self, tick_period, units=""):
        self.dt = self.time_step = self.tick_period = float(tick_period)
        self.ticks = 0
        self.units = str(units)
        self._callbacks = []

    def get_time(self):
        return self.ticks * self.dt

    def __call__(self):
        return self.get_time()

    def get_ticks(self):
        return self.ticks

    def get_time_step(self):
        return self.dt

    def get_units(self):
        return self.units

    def is_now(self, time):
        return round(float(time) / self.dt) == self.ticks

    def register_callback(self, function):
        self._callbacks.append(function)

    def _tick(self, n=1):
        self.ticks += n
        if self._callbacks:
            self._callbacks = [f for f in self._callbacks if not f()]


class Segment:
    """Handle of one segment (a row of the segment table)."""
    __slots__ = ("_model", "_idx")

    def __init__(self, model, idx):
        idx = int(idx)
        if not 0 <= idx < model._n:
            raise IndexError(f"segment {idx} out of range (the model has {model._n} segments)")
        self._model = model
        self._idx = idx

    def __eq__(self, other):
        return isinstance(other, Segment) and other._model is self._model and other._idx == self._idx

    def __hash__(self):
        return hash((id(self._model), self._idx))

    def __repr__(self):
        return f"<Segment {self._idx}>"

    def get_unstable_index(self):
        return self._idx

    @property
    def parent(self):
        p = self._model._parent_of(self._idx)
        return None if p < 0 else Segment(self._model, p)

    @property
    def children(self):
        return [Segment(self._model, c) for c in self._model._children_of(self._idx)]

    @property
    def neuron(self):
        return self._model._neuron_handle(self._model._seg_neuron[self._idx])

    @property
    def coordinates(self):
        return self._model._coords[self._idx].copy()

    @property
    def diameter(self):
        return float(self._model._diam[self._idx])

    def is_root(self):
        return self._model._parent_of(self._idx) < 0

    is_sphere = is_root

    def is_cylinder(self):
        return not self.is_root()

    def _geom(self, name):
        return float(self._model._geometry()[name][self._idx])

    length = property(lambda self: self._geom("length"))
    surface_area = property(lambda self: self._geom("surface_area"))
    cross_sectional_area = property(lambda self: self._geom("cross_sectional_area"))
    volume = property(lambda self: self._geom("volume"))
    axial_resistance = property(lambda self: self._geom("axial_resistance"))
    capacitance = property(lambda self: self._geom("capacitance"))

    @property
    def voltage(self):
        return float(self._model._get_segment_values("Segment.voltage")[self._idx])

    @voltage.setter
    def voltage(self, value):
        self._model._set_segment_value("Segment.voltage", self._idx, float(value))

    def add_segment(self, coordinates, diameter, segment_type=None):
        return self._model.Segment(self, coordinates, diameter)

    def add_section(self, coordinates, diameter, maximum_segment_length=np.inf, segment_type=None):
        """segment.py:75-104: a straight section split into equal segments."""
        maximum_segment_length = float(maximum_segment_length)
        assert maximum_segment_length > 0
        coordinates = [float(x) for x in coordinates]
        diameter = float(diameter)
        displace = np.subtract(self.coordinates, coordinates)
        length = np.linalg.norm(displace)
        p_coords = np.array(self.coordinates)
        if self.is_sphere() or len(self.children) > 0:
            self_r = 0.5 * self.diameter
            if self_r < length - EPSILON:
                p_coords -= displace * (self_r / length)
                length -= self_r
        divisions = max(1, int(np.ceil(length / maximum_segment_length)))
        x = np.linspace(p_coords[0], coordinates[0], divisions + 1)
        y = np.linspace(p_coords[1], coordinates[1], divisions + 1)
        z = np.linspace(p_coords[2], coordinates[2], divisions + 1)
        d = np.linspace(self.diameter, diameter, divisions + 1)
        section, cur = [], self
        for (xx, yy, zz, dd) in list(zip(x, y, z, d))[1:]:
            cur = cur.add_segment((xx, yy, zz), dd)
            section.append(cur)
        return section

    def insert(self, mechanisms, outside=None):
        """segment.py:124-160."""
        if isinstance(mechanisms, dict):
            pass
        elif isinstance(mechanisms, str):
            mechanisms = {mechanisms: 1.0}
        else:
            mechanisms = {name: 1.0 for name in mechanisms}
        out = {}
        for name, magnitude in mechanisms.items():
            out[name] = self._model.mechanisms[name](self, outside, float(magnitude))
        return out

    def inject_current(self, current=1.0, duration=1.0):
        """electric.py:119-125: constant current (nA) for duration (ms), on the
        half-step input clock, starting with the next input tick."""
        current = float(current) * 1e-9
        duration = float(duration)
        assert duration >= 0
        count = math.ceil(duration / self._model.input_hook.dt)
        self._model._add_clamp(self._idx, current, self._model.input_hook.ticks + 1, count)

    def get_time_constant(self):
        raise NotImplementedError("sum_conductance is not kept on the device between steps")


class Neuron:
    """Handle of one neuron."""
    __slots__ = ("_model", "_nid")

    def __init__(self, model, nid):
        self._model = model
        self._nid = int(nid)

    def __eq__(self, other):
        return isinstance(other, Neuron) and other._model is self._model and other._nid == self._nid

    def __hash__(self):
        return hash((id(self._model), self._nid, "neuron"))

    @property
    def root(self):
        return Segment(self._model, self._model._neuron_root[self._nid])

    def set_AP_detector(self, segment=None, threshold=None):
        m = self._model
        if segment is not None:
            m._det_seg[self._nid] = segment._idx
        if threshold is not None:
            m._det_thr[self._nid] = float(threshold)
        m._dirty_detectors = True

    @property
    def AP_detected(self):
        return bool(self._model._get_neuron_values("Neuron.AP_detected")[self._nid])

    @property
    def spike_count(self):
        return int(self._model._get_neuron_values("Neuron.spike_count")[self._nid])


class TimeSeries:
    """Voltage recorder; the record half of neuwon/database/time.py:123-231."""

    def __init__(self):
        self._model = None
        self.data = []
        self.timestamps = []

    def record(self, segment, component="voltage", immediate=True):
        if component != "voltage":
            raise NotImplementedError("device probes record Segment.voltage only")
        self._model = segment._model
        self._model._add_probe(self, segment._idx, immediate)
        return self

    def stop(self):
        if self._model is not None:
            self._model._remove_probe(self)
        return self

    def get_data(self):
        if self._model is not None:
            self._model._flush_probes()
        return self.data

    def get_timestamps(self):
        if self._model is not None:
            self._model._flush_probes()
        return self.timestamps

    def __len__(self):
        return len(self.get_data())


class RxD_Model:
    """GPU-backed model with the reference's RxD_Model interface (rxd_model.py:9-80).

    Extra keyword arguments (not in the reference):
      precision             'f32' (default) or 'f64' state and step arithmetic
      device                CUDA device ordinal
      propagator_tolerance  prune |P_ij| below this (reference: machine epsilon)
      propagator_conserve   return the pruned mass of each row to its diagonal
                            (charge-conserving pruning; the reference does not)
      propagator_lump       move each pruned entry to the nearest kept entry on
                            the tree path to the row's segment (charge stays
                            near where it was: far smaller error than
                            propagator_conserve at the same tolerance)
      propagator_format     'rows' (every P_ij in its row, 16-bit column each),
                            'quads' (windows of 4 consecutive columns with one
                            16-bit base: ~16 % fewer bytes with the model's
                            depth-first numbering), 'windows' (windows of 8, 4,
                            2 or 1 consecutive columns, each the width of fewest
                            bytes per entry it covers) or 'pairs' (each coupling
                            stored once and applied to both segments through
                            detailed balance)
      path                  'batched' (fused persistent kernel, one CTA per neuron),
                            'wide' (whole-model launches per phase: neurons of any
                            size) or 'plain' (per-neuron launches)
      duplicates            'sum' (default: every instance of a mechanism on a
                            segment counts) or 'reference' (nonspecific
                            conductances count only the last instance of each
                            segment, as the reference's fancy-index "+=" does,
                            neuwon/rxd/species.py:256-260)

    ``species`` takes the reference's keyword dicts (``_SpeciesType``,
    species.py:90-142, see ``species.SpeciesType``) and ``Calcium`` objects; the
    electric ones are listed by name in ``model.species``.
    """

    def __init__(self, time_step=0.1, *, temperature=37, initial_voltage=-70,
                 cytoplasmic_resistance=100, membrane_capacitance=1,
                 extracellular_tortuosity=1.55, extracellular_max_distance=20e-6,
                 species=(), mechanisms=(), precision="f32", device=0,
                 propagator_tolerance=EPSILON, propagator_conserve=False, path="batched",
                 propagator_format="quads", propagator_lump=False, duplicates="sum"):
        from .species import Calcium, SpeciesType
        self._calcium = None
        self.species = {}
        for sp in species:
            if isinstance(sp, Calcium):
                ca = sp
            else:
                st = sp if isinstance(sp, SpeciesType) else SpeciesType(**dict(sp))
                if st.name in self.species:
                    raise ValueError(f"duplicate species {st.name}")
                self.species[st.name] = st
                ca = st.calcium
            if ca is not None:
                if self._calcium is not None:
                    raise NotImplementedError("one diffusing species (calcium) per model")
                self._calcium = ca
        if duplicates not in ("sum", "reference"):
            raise ValueError("duplicates must be 'sum' or 'reference'")
        self.duplicates = duplicates
        self.time_step = float(time_step)
        self.temperature = float(temperature)
        self.initial_voltage = float(initial_voltage)
        self.cytoplasmic_resistance = float(cytoplasmic_resistance)
        self.membrane_capacitance = float(membrane_capacitance)
        self.precision = precision
        self.device = int(device)
        self.propagator_tolerance = float(propagator_tolerance)
        self.propagator_conserve = bool(propagator_conserve)
        self.path = {"batched": _lib.PATH_BATCHED, "plain": _lib.PATH_PLAIN, "wide": _lib.PATH_WIDE}[path]
        self.propagator_format = {"rows": 0, "pairs": 1, "quads": 2, "windows": 3}[propagator_format]
        self.propagator_lump = bool(propagator_lump)
        self.input_hook = Clock(0.5 * self.time_step, units="ms")
        self.advance_hook = self.clock = Clock(self.time_step, units="ms")
        # Segment table (creation order).
        self._n = 0
        self._parent = np.empty(0, np.int64)
        self._coords = np.empty((0, 3))
        self._diam = np.empty(0)
        self._seg_neuron = np.empty(0, np.int64)
        self._neuron_root = []
        self._det_seg, self._det_thr = [], []
        # Mechanisms.
        self.mechanisms = {}
        self._mech_instances = {}
        for m in mechanisms:
            self._load_mechanism(m)
        self._clamps = []
        self._probes = []
        self._syn = None
        self._spike_partition = None
        self._dirty_synapses = False
        self._ctx = None
        self._order = None
        self._geom_cache = None
        self._dirty_structure = True
        self._dirty_clamps = True
        self._dirty_detectors = True
        self._dirty_probes = True
        self._pending = {}

    # ------------------------------------------------------ reference API
    def get_time_step(self):
        return self.time_step

    def get_temperature(self):
        return self.temperature

    def get_clock(self):
        return self.clock

    def get_mechanisms(self):
        return dict(self.mechanisms)

    def register_advance_callback(self, function):
        self.advance_hook.register_callback(function)

    def Neuron(self, coordinates, diameter, *, neuron_type=None, segment_type=None):
        nid = len(self._neuron_root)
        root = self._append(-1, coordinates, diameter, nid)
        self._neuron_root.append(root)
        self._det_seg.append(root)
        self._det_thr.append(20.0)
        return Neuron(self, nid)

    def Segment(self, parent, coordinates, diameter, *, segment_type=None):
        if parent is None:
            return self.Neuron(coordinates, diameter).root
        nid = int(self._seg_neuron[parent._idx])
        return Segment(self, self._append(parent._idx, coordinates, diameter, nid))

    def add_tree(self, tree):
        """Bulk-create one neuron from a ``morphology.Tree``; returns the Neuron."""
        nid = len(self._neuron_root)
        base = self._n
        par = np.where(tree.parent < 0, -1, tree.parent + base)
        self._grow(len(tree))
        sl = slice(base, base + len(tree))
        self._parent[sl] = par
        self._coords[sl] = tree.coordinates
        self._diam[sl] = tree.diameter
        self._seg_neuron[sl] = nid
        self._n += len(tree)
        self._neuron_root.append(base)
        self._det_seg.append(base)
        self._det_thr.append(20.0)
        self._dirty_structure = True
        return Neuron(self, nid)

    def insert_everywhere(self, name, magnitude=1.0, **per_instance):
        """Insert mechanism ``name`` on every segment (one vectorised call)."""
        cls = self.mechanisms[name]
        segs = np.arange(self._n, dtype=np.int64)
        if issubclass(cls, Kinetic):
            self._add_kinetic_instances(cls, segs, np.full(self._n, float(magnitude)), per_instance.get("gbar"))
        else:
            self._add_instances_bulk(cls, segs, np.full(self._n, float(magnitude)), per_instance)

    def advance(self, k_steps=1):
        """rxd_model.py:63-80, k_steps times, as one device launch."""
        self._sync()
        k = int(k_steps)
        if self._probes:
            self._ensure_probe_room(k)
        self._ctx.advance(k, self.path)
        self.input_hook.ticks += 2 * k
        self.advance_hook._tick(k)

    def _sync_calcium(self, g, order, par):
        ca = self._calcium
        nnz = _lib.ctypes.c_int64()
        A = np.ascontiguousarray(g["cross_sectional_area"][order], dtype=np.float64)
        L = np.ascontiguousarray(g["length"][order], dtype=np.float64)
        vol = np.ascontiguousarray(g["volume"][order], dtype=np.float64)
        self._ctx.call("nw_calcium_set", ca.diffusivity, _lib.ptr(A), _lib.ptr(L), _lib.ptr(vol), ca.initial,
                       self.propagator_tolerance, int(self.propagator_conserve or self.propagator_lump),
                       _lib.ctypes.byref(nnz))
        self.calcium_nnz = nnz.value
        geom_sorted = {k: np.asarray(v)[order] for k, v in g.items() if k in ("volume", "surface_area")}
        influx, efflux = (np.ascontiguousarray(x) for x in ca.coefficients(geom_sorted))
        if ca.pump:
            # Pump table generated on the GPU in FP64 (nw_lti_table_build).
            T = ca.degree + 1
            st0 = np.ascontiguousarray(ca.steady_state(ca.initial))
            self._ctx.call("nw_calcium_pump_set", _lib.ptr(influx), _lib.ptr(efflux),
                           _lib.ptr(np.zeros(ca.num_buckets * 9 * T)), ca.num_buckets, T, ca.log2_min(),
                           ca.bucket_frq(), ca.scale, _lib.ptr(st0))
            from .kinetic import gpu_table
            rates, fit = ca.table_inputs()
            gpu_table(self._ctx, rates, fit, ca.num_buckets, self.time_step, target=2)
        else:
            self._ctx.call("nw_calcium_pump_set", _lib.ptr(influx), _lib.ptr(efflux), None, 0, 0, 0.0, 0.0, 0.0,
                           None)

    def _calcium_values(self, name, count_per_segment=1):
        self._sync()
        n = self._n
        buf = np.empty(n * count_per_segment, dtype=np.float64)
        self._ctx.call("nw_calcium_data", name.encode(), _lib.ptr(buf), 1, len(buf), 0)
        if count_per_segment == 1:
            out = np.empty(n)
            out[self._order] = buf
            return out
        out = np.empty((n, count_per_segment))
        out[self._order] = buf.reshape(count_per_segment, n).T
        return out

    def set_spike_partition(self, total_neurons, neuron_offset, ring_steps=0):
        """This model holds neurons [neuron_offset, neuron_offset + its neurons) of a
        network of total_neurons split across ranks: presynaptic ids of
        add_synapses are global, and the spike ring covers every neuron (the
        ranks exchange it with replicas.SpikeExchange).  ring_steps forces a
        common ring length (a power of two above max + min delay of all ranks)."""
        self._spike_partition = (int(total_neurons), int(neuron_offset), int(ring_steps))
        self._dirty_synapses = self._syn is not None

    def add_synapses(self, pre_neurons, post_segments, w_ampa, w_nmda=None, delay=1.0, kinetics=None):
        """Synapses from neurons (handles or ids) onto segments (handles or creation
        indices) with AMPA / NMDA weights in nS and axonal delays in ms (rounded to
        whole steps, at least one).  Returns the new synapses' indices."""
        from .synapses import SynapseKinetics, delay_steps
        pre = np.array([getattr(p, "_nid", p) for p in np.atleast_1d(np.asarray(pre_neurons, dtype=object))],
                       dtype=np.int64)
        post = np.array([getattr(s, "_idx", s) for s in np.atleast_1d(np.asarray(post_segments, dtype=object))],
                        dtype=np.int64)
        m = len(pre)
        if len(post) != m:
            raise ValueError("pre_neurons and post_segments differ in length")
        n_pre = self._spike_partition[0] if self._spike_partition else len(self._neuron_root)
        if np.any(pre < 0) or np.any(pre >= n_pre):
            raise ValueError("presynaptic neuron out of range")
        if np.any(post < 0) or np.any(post >= self._n):
            raise ValueError("post segment out of range")
        wa = np.broadcast_to(np.asarray(w_ampa, dtype=np.float64), (m,))
        wn = wa if w_nmda is None else np.broadcast_to(np.asarray(w_nmda, dtype=np.float64), (m,))
        d = np.broadcast_to(delay_steps(delay, self.time_step), (m,))
        old = self._syn or {"pre": np.empty(0, np.int64), "post": np.empty(0, np.int64),
                            "wa": np.empty(0), "wn": np.empty(0), "delay": np.empty(0, np.int64),
                            "kinetics": SynapseKinetics()}
        if kinetics is not None:
            old["kinetics"] = kinetics
        first = len(old["pre"])
        self._syn = {"pre": np.concatenate([old["pre"], pre]), "post": np.concatenate([old["post"], post]),
                     "wa": np.concatenate([old["wa"], wa]), "wn": np.concatenate([old["wn"], wn]),
                     "delay": np.concatenate([old["delay"], d]), "kinetics": old["kinetics"]}
        self._dirty_synapses = True
        return np.arange(first, first + m)

    def _sync_synapses(self):
        sy = self._syn
        kin = sy["kinetics"]
        ao, af, no, nf = (np.ascontiguousarray(x, dtype=np.float64) for x in kin.matrices(self.time_step))
        post_dev = np.ascontiguousarray(self._inv[sy["post"]])
        if self._spike_partition is not None:
            total, offset, ring_steps = self._spike_partition
            self._ctx.set_option("spike_neurons", total)
            self._ctx.set_option("spike_neuron_offset", offset)
            self._ctx.set_option("spike_ring_steps", ring_steps)
        self._ctx.call("nw_synapses_set", len(sy["pre"]), _lib.ptr(np.ascontiguousarray(sy["pre"])),
                       _lib.ptr(post_dev), _lib.ptr(np.ascontiguousarray(sy["wa"] * 1e-9)),
                       _lib.ptr(np.ascontiguousarray(sy["wn"] * 1e-9)),
                       _lib.ptr(np.ascontiguousarray(sy["delay"], dtype=np.int32)),
                       _lib.ptr(ao), _lib.ptr(af), _lib.ptr(no), _lib.ptr(nf),
                       kin.pulse_steps(self.time_step), kin.e_syn, kin.mg)
        self._dirty_synapses = False

    def save_sqlite(self, filename):
        """Checkpoint the device state (neuwon/database/sql.py:78-101 layout)."""
        from .checkpoint import save_sqlite
        save_sqlite(self, filename)

    def load_sqlite(self, filename):
        """Restore a checkpoint written by ``save_sqlite`` (sql.py:103-129)."""
        from .checkpoint import load_sqlite
        load_sqlite(self, filename)

    def autotune(self, trial_steps=10):
        """Choose the batched path's lanes per row, threads per CTA and step-fusion
        depth by timing short runs of this model (state restored afterwards)."""
        self._sync()
        return self._ctx.autotune(trial_steps)

    # --------------------------------------------------- differentiation helpers
    def set_hh_densities(self, gnabar, gkbar, glbar):
        """Per-instance HH densities (S/cm2, registration order) without a rebuild."""
        self._sync()
        scale = 1e-8 * self._hh_magnitude                     # nmodl/__init__.py:103-107, 404-406
        for name, dens in (("hh.gna_coef", gnabar), ("hh.gk_coef", gkbar), ("hh.gl_coef", glbar)):
            d = np.broadcast_to(np.asarray(dens, dtype=np.float64), scale.shape)
            self._ctx.set_data(name, np.ascontiguousarray(d * scale))

    def hh_density_scale(self):
        """d coefficient (S) / d density (S/cm2) for every HH instance."""
        self._sync()
        return 1e-8 * self._hh_magnitude

    def set_cytoplasmic_resistance(self, ra):
        """Change Ra (ohm cm); the propagator is rebuilt before the next step."""
        ra = float(ra)
        if ra != self.cytoplasmic_resistance:
            self.cytoplasmic_resistance = ra
            self._geom_cache = None
            self._dirty_structure = True

    def reset_state(self):
        """Back to t = 0: initial voltage, steady-state gates, clock and detectors reset."""
        self._sync()
        n = self._n
        self._ctx.set_data("Segment.voltage", np.full(n, self.initial_voltage))
        for name, cls in self.mechanisms.items():
            if issubclass(cls, HH):
                m = self._instance_count(name)
                g = hh_steady_state(self.initial_voltage, self.temperature)
                for attr, val in zip(("hh.m", "hh.h", "hh.n"), g):
                    self._ctx.set_data(attr, np.full(m, float(val)))
            elif issubclass(cls, Kinetic):
                m = self._instance_count(name)
                init = cls.initial_state(self.initial_voltage, self.temperature)
                self._ctx.set_data(self.kinetic_state_name(name), np.tile(init, m))
        self._ctx.call("nw_set_option", b"reset_clock", 1)
        self.input_hook.ticks = 0
        self.advance_hook.ticks = 0
        self._flush_probes()

    def check(self):
        v = self.get_data("Segment.voltage")
        assert np.all(np.isfinite(v)), "non-finite voltage"

    def kinetic_state_name(self, mechanism):
        """The C-ABI attribute name of a kinetic mechanism's states ("kinetic.<q>.state")."""
        self._sync()
        return f"kinetic.{self._kin_index[mechanism]}.state"

    def get_data(self, name):
        """Whole-attribute read in creation order ('Segment.voltage', 'hh.m',
        'na11a.state', 'Segment.na_conductance', ...)."""
        if name.startswith("Segment.") and name.endswith("_conductance"):
            ion = name[len("Segment."):-len("_conductance")]
            if ion in self.species and self.species[ion].electric:
                # The species' conductance accumulator as the last mechanism phase
                # left it (species.py:129-133): device gather, creation order.
                self._sync()
                out = np.empty(self._n)
                self._ctx.call("nw_species_conductance", self._species_index[ion], _lib.ptr(out))
                return out[self._inv]
        if name.startswith("Segment."):
            return self._get_segment_values(name).copy()
        if name.startswith("Neuron."):
            return self._get_neuron_values(name).copy()
        if name in ("Species.ca", "Species.ca_derivative"):
            return self._calcium_values(name)
        if name == "CaPump.state":
            return self._calcium_values(name, 3)
        if name.startswith("Synapse."):
            self._sync()
            n = 0 if self._syn is None else len(self._syn["pre"])
            dt = np.int64 if name in ("Synapse.events", "Synapse.last_event", "Synapse.pulse_end") else np.float64
            return self._ctx.get_data(name, n, dt)
        mech, attr = name.split(".")
        self._sync()
        cls = self.mechanisms[mech]
        n = self._instance_count(cls.get_name())
        if issubclass(cls, Kinetic):
            if attr == "input":
                return self._ctx.get_data(self.kinetic_state_name(mech)[:-len("state")] + "input", n)
            S = len(cls.scheme_factory().states)
            return self._ctx.get_data(self.kinetic_state_name(mech), n * S).reshape(n, S)
        return self._ctx.get_data(f"hh.{attr}", n)

    def set_data(self, name, values):
        """Whole-attribute write in creation order: a kinetic mechanism's states
        ('<name>.state', instances x states) or the instance values of a two-input
        table ('<name>.input', e.g. NMDA_Mg.input: the glutamate concentration, mM)."""
        mech, attr = name.split(".")
        self._sync()
        cls = self.mechanisms.get(mech)
        if cls is None or not issubclass(cls, Kinetic) or attr not in ("state", "input"):
            raise KeyError(f"{name}: set_data takes '<kinetic mechanism>.state' or '.input'")
        n = self._instance_count(cls.get_name())
        values = np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64),
                                                      (n,) if attr == "input" else (n, len(cls.scheme_factory().states))))
        target = self.kinetic_state_name(mech)
        if attr == "input":
            target = target[:-len("state")] + "input"
        self._ctx.set_data(target, values.ravel())

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None

    # ------------------------------------------------------ internals
    def _load_mechanism(self, mechanism):
        if isinstance(mechanism, str):
            from .mechanisms import NMODL
            mechanism = NMODL(mechanism)
        if not (isinstance(mechanism, type) and issubclass(mechanism, Mechanism)):
            raise TypeError(f"not a Mechanism subclass: {mechanism!r}")
        bound = mechanism.initialize(self) or mechanism
        if not issubclass(bound, (HH, Kinetic)):
            raise NotImplementedError(f"mechanism {bound.get_name()} has no GPU kernel")
        name = bound.get_name()
        if name in self.mechanisms:
            raise ValueError(f"duplicate mechanism {name}")
        if issubclass(bound, HH) and any(issubclass(c, HH) for c in self.mechanisms.values()):
            raise NotImplementedError("one HH mechanism per model")
        if issubclass(bound, Kinetic):
            if sum(issubclass(c, Kinetic) for c in self.mechanisms.values()) >= MAX_KINETIC:
                raise NotImplementedError(f"at most {MAX_KINETIC} kinetic mechanisms per model")
            ion = bound.ion
            if ion is not None and not (ion in self.species and self.species[ion].electric):
                raise ValueError(f"mechanism {name} writes the conductance of ion {ion!r}, but the model declares no "
                                 f"electric species {ion!r} (species=[{{'name': {ion!r}, 'reversal_potential': ...}}])")
        self.mechanisms[name] = bound
        self._mech_instances[name] = {"seg": [], "mag": [], "n_at": [], "gnabar": [], "gkbar": [],
                                      "glbar": [], "gbar": []}

    def _grow(self, extra):
        need = self._n + extra
        cap = len(self._parent)
        if need <= cap:
            return
        cap = max(need, 2 * cap, 64)
        def grow(a, shape_tail=()):
            b = np.zeros((cap,) + shape_tail, dtype=a.dtype)
            b[:self._n] = a[:self._n]
            return b
        self._parent = grow(self._parent)
        self._coords = grow(self._coords, (3,))
        self._diam = grow(self._diam)
        self._seg_neuron = grow(self._seg_neuron)

    def _append(self, parent, coordinates, diameter, nid):
        self._grow(1)
        i = self._n
        self._parent[i] = parent
        self._coords[i] = np.asarray(coordinates, dtype=np.float64)
        self._diam[i] = float(diameter)
        self._seg_neuron[i] = nid
        self._n += 1
        self._dirty_structure = True
        self._geom_cache = None
        return i

    def _parent_of(self, i):
        return int(self._parent[i])

    def _children_of(self, i):
        return [int(c) for c in np.nonzero(self._parent[:self._n] == int(i))[0]]

    def _neuron_handle(self, nid):
        return Neuron(self, nid)

    def _geometry(self):
        if self._geom_cache is None or self._geom_cache["_n"] != self._n:
            tree = Tree(self._parent[:self._n], self._coords[:self._n], self._diam[:self._n])
            g = geometry(tree)
            R, C = passive_electric(g, self.cytoplasmic_resistance, self.membrane_capacitance)
            g["axial_resistance"] = R
            g["capacitance"] = C
            g["_n"] = self._n
            self._geom_cache = g
        return self._geom_cache

    def _area_at(self, n_at):
        """Surface areas of the first n_at segments with only their children then."""
        if n_at == self._n:
            return self._geometry()["surface_area"]
        t = Tree(self._parent[:n_at], self._coords[:n_at], self._diam[:n_at])
        return geometry(t)["surface_area"]

    def _add_mechanism_instance(self, cls, segment, magnitude, overrides):
        self._add_instances_bulk(cls, np.array([segment._idx]), np.array([magnitude]),
                                 {k: v for k, v in overrides.items() if v is not None})
        return self._instance_count(cls.get_name()) - 1

    def _instance_count(self, name):
        return sum(len(c) for c in self._mech_instances[name]["seg"])

    def _add_instances_bulk(self, cls, segs, mags, per_instance):
        """Append instances; per_instance maps gbar names to scalars or arrays."""
        rec = self._mech_instances[cls.get_name()]
        segs = np.asarray(segs, dtype=np.int64)
        m = len(segs)
        rec["seg"].append(segs)
        rec["mag"].append(np.broadcast_to(np.asarray(mags, dtype=np.float64), (m,)).copy())
        rec["n_at"].append(np.full(m, self._n, dtype=np.int64))
        for key in ("gnabar", "gkbar", "glbar"):
            v = per_instance.get(key)
            arr = np.full(m, np.nan) if v is None else np.broadcast_to(np.asarray(v, np.float64), (m,)).copy()
            rec[key].append(arr)
        self._dirty_structure = True

    def _add_kinetic_instances(self, cls, segs, mags, gbar):
        rec = self._mech_instances[cls.get_name()]
        segs = np.asarray(segs, dtype=np.int64)
        m = len(segs)
        rec["seg"].append(segs)
        rec["mag"].append(np.broadcast_to(np.asarray(mags, dtype=np.float64), (m,)).copy())
        rec["n_at"].append(np.full(m, self._n, dtype=np.int64))
        rec["gbar"].append(np.full(m, np.nan) if gbar is None
                           else np.broadcast_to(np.asarray(gbar, np.float64), (m,)).copy())
        self._dirty_structure = True
        return self._instance_count(cls.get_name()) - 1

    def _add_clamp(self, seg, amps, first_tick, count):
        self._clamps.append((int(seg), float(amps), int(first_tick), int(count)))
        self._dirty_clamps = True

    def _add_probe(self, ts, seg, immediate):
        rec = {"ts": ts, "seg": seg, "start_step": self.clock.ticks}
        self._flush_probes()
        self._probes.append(rec)
        if immediate:
            ts.data.append(self._get_segment_values("Segment.voltage")[seg])
            ts.timestamps.append(self.clock())
        self._dirty_probes = True

    def _remove_probe(self, ts):
        self._flush_probes()
        self._probes = [p for p in self._probes if p["ts"] is not ts]
        self._dirty_probes = True

    # --- device mirror ---------------------------------------------------
    def _sync(self):
        if self._ctx is None:
            self._ctx = _lib.Context(self.device, self.precision)
        if self._dirty_structure:
            self._sync_structure()
        if self._dirty_clamps:
            self._sync_clamps()
        if self._dirty_detectors:
            self._sync_detectors()
        if self._dirty_probes:
            self._sync_probes()
        if self._dirty_synapses:
            self._sync_synapses()

    def _sync_structure(self):
        ctx = self._ctx
        n = self._n
        if n == 0:
            raise RuntimeError("model has no segments")
        saved = None
        if self._order is not None:
            saved = self._save_state()
        # Database.sort() (stable by neuron), depth-first within each neuron.
        order = device_order(self._parent[:n], self._seg_neuron[:n], len(self._neuron_root))
        inv = np.empty(n, np.int64)
        inv[order] = np.arange(n)
        self._order, self._inv = order, inv
        nids = self._seg_neuron[:n][order]
        counts = np.bincount(nids, minlength=len(self._neuron_root))
        neuron_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        par = self._parent[:n][order]
        parent_dev = np.where(par < 0, -1, inv[np.maximum(par, 0)]).astype(np.int64)
        g = self._geometry()
        ctx.call("nw_model_init", n, len(self._neuron_root), _lib.ptr(neuron_start),
                 _lib.ptr(parent_dev), self.time_step, self.temperature)
        ctx.set_data("Segment.capacitance", g["capacitance"][order])
        ctx.set_data("Segment.axial_resistance", np.where(par < 0, 1.0, g["axial_resistance"][order]))
        ctx.set_data("Segment.voltage", np.full(n, self.initial_voltage))
        nnz = _lib.ctypes.c_int64()
        ctx.set_option("propagator_lump", int(self.propagator_lump))
        ctx.call("nw_propagator_build", self.propagator_tolerance, _lib.ctypes.byref(nnz))
        if self.propagator_conserve or self.propagator_lump:
            ctx.call("nw_propagator_conserve")
        ctx.set_option("propagator_format", self.propagator_format)
        self.propagator_nnz = nnz.value
        # Electric species, numbered in declaration order (species.py:90-142).
        electric = [s for s in self.species.values() if s.electric]
        self._species_index = {s.name: k for k, s in enumerate(electric)}
        erev = np.array([s.reversal_potential for s in electric], dtype=np.float64)
        ctx.call("nw_species_set", len(electric), _lib.ptr(erev) if len(erev) else None)
        ctx.set_option("duplicates", 1 if self.duplicates == "reference" else 0)
        ctx.call("nw_kinetic_clear")
        self._kin_index = {}
        for name, cls in self.mechanisms.items():
            if issubclass(cls, Kinetic):
                self._sync_kinetic(cls)
            else:
                self._sync_hh(cls)
        if self._calcium is not None:
            self._sync_calcium(g, order, par)
        self._dirty_structure = False
        self._dirty_clamps = self._dirty_detectors = self._dirty_probes = True
        self._dirty_synapses = self._syn is not None
        if saved is not None:
            self._restore_state(saved)
        for key, (name, values) in list(self._pending.items()):
            self._ctx.set_data(name, values[self._order])
        self._pending.clear()

    def _sync_hh(self, cls):
        rec = self._mech_instances[cls.get_name()]
        cat = lambda key, dt: (np.concatenate(rec[key]) if rec[key] else np.empty(0, dt))
        seg = cat("seg", np.int64)
        mag = cat("mag", np.float64)
        n_at = cat("n_at", np.int64)
        area = np.empty(len(seg))
        for k in np.unique(n_at):
            sel = n_at == k
            area[sel] = self._area_at(int(k))[seg[sel]]
        magnitude = mag * area                                 # nmodl/__init__.py:496-500

        def coef(key, default):
            v = cat(key, np.float64)
            v = np.where(np.isnan(v), default, v)
            return np.ascontiguousarray(v * 1e-8 * magnitude)  # nmodl/__init__.py:103-107, 404-406
        gna = coef("gnabar", cls.gnabar)
        gk = coef("gkbar", cls.gkbar)
        gl = coef("glbar", cls.glbar)
        self._hh_magnitude = magnitude.copy()
        seg_dev = np.ascontiguousarray(self._inv[seg]) if len(seg) else seg
        self._ctx.call("nw_hh_register", len(seg), _lib.ptr(seg_dev),
                       _lib.ptr(gna), _lib.ptr(gk), _lib.ptr(gl),
                       float(cls.ena), float(cls.ek), float(cls.el), self.initial_voltage)

    def _insertion_magnitude(self, rec):
        cat = lambda key, dt: (np.concatenate(rec[key]) if rec[key] else np.empty(0, dt))
        seg = cat("seg", np.int64)
        mag = cat("mag", np.float64)
        n_at = cat("n_at", np.int64)
        area = np.empty(len(seg))
        for k in np.unique(n_at):
            sel = n_at == k
            area[sel] = self._area_at(int(k))[seg[sel]]
        return seg, mag * area                                 # nmodl/__init__.py:496-500

    def _sync_kinetic(self, cls):
        rec = self._mech_instances[cls.get_name()]
        seg, magnitude = self._insertion_magnitude(rec)
        gbar = np.concatenate(rec["gbar"]) if rec["gbar"] else np.empty(0)
        gbar = np.where(np.isnan(gbar), cls.gbar, gbar)
        if cls.point_process:                  # S per instance times its magnitude (default 1)
            raw = np.concatenate(rec["mag"]) if rec["mag"] else np.empty(0)
            g = np.ascontiguousarray(gbar * raw)
        else:
            g = np.ascontiguousarray(gbar * 1e-8 * magnitude)
        # The table is generated on the GPU in FP64 (nw_lti_table_build) the first
        # time this mechanism, step and temperature are seen, then reused.
        sch = cls.scheme_factory()
        two = cls.inputs is not None
        if two:
            from .kinetic import canonical_terms
            terms = canonical_terms(cls.terms)
            nb, T = cls.inputs[0].num_buckets * cls.inputs[1].num_buckets, len(terms)
        else:
            nb, T = cls.num_buckets, cls.degree + 1
        key = (cls, self.time_step, self.temperature)
        cache = getattr(self, "_tables", {})
        self._tables = cache
        if cls.table is not None:
            cache[key] = np.asarray(cls.table, dtype=np.float64)
            if cache[key].shape != (nb, sch.num_states, sch.num_states, T):
                raise ValueError(f"{cls.get_name()}: table shape {cache[key].shape}, expected "
                                 f"{(nb, sch.num_states, sch.num_states, T)} [bucket][col][row][term]")
        layout = cache.get(key)
        placeholder = layout is None
        if placeholder:
            layout = np.zeros((nb, sch.num_states, sch.num_states, T))
        init = np.ascontiguousarray(cls.initial_state(self.initial_voltage, self.temperature))
        open_idx = np.asarray(sch.open_states, dtype=np.int32)
        seg_dev = np.ascontiguousarray(self._inv[seg]) if len(seg) else seg
        cs = float(sch.conserve_sum) if sch.conserve_sum is not None else 0.0
        frq = nb / (cls.vmax - cls.vmin)
        species = -1 if cls.ion is None else self._species_index[cls.ion]
        q = _lib.ctypes.c_int32()
        self._ctx.call("nw_kinetic_add", len(seg), _lib.ptr(seg_dev), _lib.ptr(g), sch.num_states,
                       len(open_idx), _lib.ptr(open_idx), float(cls.erev), species,
                       _lib.ptr(np.ascontiguousarray(layout.ravel())), nb, T, float(cls.vmin), frq, cs, _lib.ptr(init),
                       _lib.ctypes.byref(q))
        self._kin_index[cls.get_name()] = q.value
        if two:
            i1, i2 = cls.inputs
            inst = [inp for inp in cls.inputs if inp.kind != "voltage"]
            powers = np.ascontiguousarray(np.array(terms, dtype=np.int32).ravel())
            self._ctx.call("nw_kinetic_inputs", q.value, i1.code, i1.num_buckets, i1.minimum, i1.bucket_frq, i1.scale,
                           i2.code, i2.num_buckets, i2.minimum, i2.bucket_frq, i2.scale, T, _lib.ptr(powers),
                           float(inst[0].initial if inst else 0.0))
        if placeholder and len(seg):
            if two:
                from .kinetic import scheme_table_gpu2
                cache[key] = scheme_table_gpu2(self._ctx, sch, self.time_step, self.temperature, cls.inputs[0],
                                               cls.inputs[1], cls.terms, cls.samples_per_axis, target=16 + q.value)
            else:
                from .kinetic import scheme_table_gpu
                cache[key] = scheme_table_gpu(self._ctx, sch, self.time_step, self.temperature, cls.vmin, cls.vmax,
                                              nb, cls.degree, target=16 + q.value)

    def _sync_clamps(self):
        c = self._clamps
        seg = np.array([self._inv[x[0]] for x in c], dtype=np.int64)
        amp = np.array([x[1] for x in c], dtype=np.float64)
        first = np.array([x[2] for x in c], dtype=np.int64)
        cnt = np.array([x[3] for x in c], dtype=np.int64)
        self._ctx.call("nw_clamps_set", len(c), _lib.ptr(seg), _lib.ptr(amp), _lib.ptr(first), _lib.ptr(cnt))
        self._dirty_clamps = False

    def _sync_detectors(self):
        seg = self._inv[np.asarray(self._det_seg, dtype=np.int64)]
        thr = np.asarray(self._det_thr, dtype=np.float64)
        self._ctx.call("nw_detectors_set", _lib.ptr(np.ascontiguousarray(seg)), _lib.ptr(thr))
        self._dirty_detectors = False

    def _sync_probes(self, capacity=None):
        self._flush_probes()
        segs = np.array([self._inv[p["seg"]] for p in self._probes], dtype=np.int64)
        self._probe_cap = capacity or 4096
        self._ctx.call("nw_probes_set", len(segs), _lib.ptr(segs), self._probe_cap)
        self._probe_base_step = self.clock.ticks
        self._dirty_probes = False

    def _ensure_probe_room(self, k):
        steps = self._probe_steps()
        if steps + k > self._probe_cap:
            self._sync_probes(capacity=max(4096, k))

    def _probe_steps(self):
        if self._ctx is None or not self._probes or self._dirty_probes:
            return 0
        s = _lib.ctypes.c_int64()
        self._ctx.call("nw_probes_read", None, 2, 0, _lib.ctypes.byref(s))
        return s.value

    def _flush_probes(self):
        """Move device-recorded samples into the TimeSeries objects."""
        if self._ctx is None or not self._probes or self._dirty_probes:
            return
        steps = self._probe_steps()
        if steps == 0:
            return
        buf = np.empty((steps, len(self._probes)), dtype=np.float64)
        s = _lib.ctypes.c_int64()
        self._ctx.call("nw_probes_read", _lib.ptr(buf), 1, steps, _lib.ctypes.byref(s))
        for k, p in enumerate(self._probes):
            p["ts"].data.extend(buf[:, k].tolist())
            p["ts"].timestamps.extend(((self._probe_base_step + 1 + np.arange(steps)) * self.time_step).tolist())
        segs = np.array([self._inv[p["seg"]] for p in self._probes], dtype=np.int64)
        self._ctx.call("nw_probes_set", len(segs), _lib.ptr(segs), self._probe_cap)
        self._probe_base_step = self.clock.ticks

    def _save_state(self):
        st = {"V": self._ctx.get_data("Segment.voltage", len(self._order))[self._inv_prev()]}
        return st

    def _inv_prev(self):
        inv = np.empty(len(self._order), np.int64)
        inv[self._order] = np.arange(len(self._order))
        return inv

    def _restore_state(self, st):
        V = np.full(self._n, self.initial_voltage)
        V[:len(st["V"])] = st["V"]
        self._ctx.set_data("Segment.voltage", V[self._order])

    def _get_segment_values(self, name):
        if self._ctx is None or self._dirty_structure:
            if name == "Segment.voltage":
                v = np.full(self._n, self.initial_voltage)
                if "V" in self._pending:
                    v = self._pending["V"][1].copy()
                return v
            raise RuntimeError(f"{name} is available after the first advance()")
        dev = self._ctx.get_data(name, self._n)
        return dev[self._inv]

    def _set_segment_value(self, name, idx, value):
        vals = self._get_segment_values(name).copy()
        vals[idx] = value
        if self._ctx is None or self._dirty_structure:
            self._pending["V"] = (name, vals)
        else:
            self._ctx.set_data(name, vals[self._order])

    def _get_neuron_values(self, name):
        self._sync()
        return self._ctx.get_data(name, len(self._neuron_root))


Model = RxD_Model
