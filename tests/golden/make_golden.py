"""Generate golden fixtures by running the reference NEUWON itself.

Run from the repository root with the path of a checkout of the reference
as the first argument (or in the environment variable ``NEUWON_REFERENCE``):

    python tests/golden/make_golden.py <path of the reference checkout>

The reference imports four third-party packages that are absent here
(numba, graph_algorithms, matplotlib, BlueBrain nmodl).  They are replaced by
import-only stubs written to a temporary directory: numba's ``njit`` becomes
the identity and ``prange`` becomes ``range`` (so the reference's ``@Compute``
kernels run as plain Python; ``from_dtype`` gives the dtype's name, which is what the
host entry point needs to allocate local arrays), ``topological_sort`` is a ten-line
DFS, and the rest are empty modules.  None of them is on the computed path except the
identity JIT.

Because the NMODL parser is absent, the Hodgkin-Huxley channel is inserted
through the reference's Developers API (``neuwon/rxd/mechanisms.py:74-75``)
as a ``Mechanism`` subclass whose ``@Compute advance`` is what the NMODL
front end emits for ``nmodl_library/artificial/hh.mod`` (parameters scaled by
1e-8 * magnitude, exact exponential gate update, nonspecific conductances).

Outputs (numpy .npz, float64) go to ``tests/golden/``.
"""
import math
import os
import sys
import tempfile
import textwrap

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = None        # set by main() from argv[1] or NEUWON_REFERENCE

STUBS = {
    "numba/__init__.py": """
        def njit(*args, **kwargs):
            if args and callable(args[0]):
                return args[0]
            return lambda f: f
        jit = njit
        prange = range
        cuda = None
        def from_dtype(dtype):
            # The type's name: the host entry point allocates local arrays with
            # numpy.empty(size, dtype=numpy.<name>) (database/compute.py:317).
            import numpy
            return numpy.dtype(dtype).name
    """,
    "graph_algorithms/__init__.py": """
        def topological_sort(nodes, dependencies):
            order, seen = [], set()
            def visit(n):
                if id(n) in seen: return
                seen.add(id(n))
                for d in dependencies(n): visit(d)
                order.append(n)
            for n in nodes: visit(n)
            return order[::-1]
        def depth_first_traversal(*args, **kwargs):
            raise NotImplementedError
    """,
    "matplotlib/__init__.py": "",
    "matplotlib/pyplot.py": "",
    "nmodl/__init__.py": "",
    "nmodl/ast.py": """
        class _Any:
            def __getattr__(self, name): return name
        AstNodeType = _Any()
    """,
    "nmodl/dsl.py": """
        class _Any:
            def __getattr__(self, name): return _Any()
            def __call__(self, *a, **k): return _Any()
        visitor = _Any(); symtab = _Any(); to_nmodl = _Any(); NmodlDriver = _Any()
    """,
    "nmodl/symtab.py": "",
}


def reference_path(argv=None):
    """The reference checkout: first argument, else NEUWON_REFERENCE; no default."""
    argv = sys.argv[1:] if argv is None else argv
    path = argv[0] if argv else os.environ.get("NEUWON_REFERENCE")
    if not path or not os.path.isdir(os.path.join(path, "neuwon")):
        raise SystemExit("usage: make_golden.py <reference checkout> (or set NEUWON_REFERENCE)")
    return os.path.abspath(path)


def install_stubs():
    global REFERENCE
    if REFERENCE is None:
        REFERENCE = reference_path()
    root = tempfile.mkdtemp(prefix="neuwon_stubs_")
    for rel, src in STUBS.items():
        path = os.path.join(root, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(textwrap.dedent(src))
    sys.path.insert(0, REFERENCE)
    sys.path.insert(0, root)
    sys.path.insert(0, REPO)
    if not hasattr(np, "product"):
        np.product = np.prod            # removed in numpy 2; used by lti_sim/approx.py:78, 81


def make_hh(gnabar=.12, gkbar=.036, glbar=.0003, ena=60., ek=-88., el=-54.3):
    """Developers-API restatement of hh.mod, as the NMODL front end compiles it."""
    from neuwon.rxd.mechanisms import Mechanism
    from neuwon.database import Compute

    class hh(Mechanism):
        __slots__ = ()

        @classmethod
        def initialize(cls, model):
            db = model.get_database()
            celsius = model.get_temperature()
            dt = model.get_time_step()
            data = db.add_class(cls)
            data.add_attribute('segment', dtype='Segment')
            data.add_attribute('magnitude', units='um2')
            v0 = db.get('Segment.voltage').get_initial_value()
            q10 = 3.0 ** ((celsius - 6.3) / 10.0)

            def vtrap(x, y):
                if abs(x / y) < 1e-6:
                    return y * (1 - x / y / 2)
                return x / (math.exp(x / y) - 1)
            a = .1 * vtrap(-(v0 + 40), 10); b = 4 * math.exp(-(v0 + 65) / 18); m0 = a / (a + b)
            a = .07 * math.exp(-(v0 + 65) / 20); b = 1 / (math.exp(-(v0 + 35) / 10) + 1); h0 = a / (a + b)
            a = .01 * vtrap(-(v0 + 55), 10); b = .125 * math.exp(-(v0 + 65) / 80); n0 = a / (a + b)
            data.add_attribute('m', m0)
            data.add_attribute('h', h0)
            data.add_attribute('n', n0)
            cls_ = data.get_instance_type()
            model.register_nonspecific_conductance(cls_, 'na', ena)
            model.register_nonspecific_conductance(cls_, 'k', ek)
            model.register_nonspecific_conductance(cls_, 'l', el)
            G = dict(q10=q10, dt=dt, gna=gnabar * 1e-8, gk=gkbar * 1e-8, gl=glbar * 1e-8)

            @Compute
            def advance(self):
                v = self.segment.voltage
                x = -(v + 40)
                vt = 10 * (1 - x / 10 / 2) if abs(x / 10) < 1e-6 else x / (math.exp(x / 10) - 1)
                alpha = .1 * vt
                beta = 4 * math.exp(-(v + 65) / 18)
                mtau = 1 / (G['q10'] * (alpha + beta)); minf = alpha / (alpha + beta)
                alpha = .07 * math.exp(-(v + 65) / 20)
                beta = 1 / (math.exp(-(v + 35) / 10) + 1)
                htau = 1 / (G['q10'] * (alpha + beta)); hinf = alpha / (alpha + beta)
                x = -(v + 55)
                vt = 10 * (1 - x / 10 / 2) if abs(x / 10) < 1e-6 else x / (math.exp(x / 10) - 1)
                alpha = .01 * vt
                beta = .125 * math.exp(-(v + 65) / 80)
                ntau = 1 / (G['q10'] * (alpha + beta)); ninf = alpha / (alpha + beta)
                dt = G['dt']
                m = minf + (self.m - minf) * math.exp(-dt / mtau)
                h = hinf + (self.h - hinf) * math.exp(-dt / htau)
                n = ninf + (self.n - ninf) * math.exp(-dt / ntau)
                self.m = m
                self.h = h
                self.n = n
                mag = self.magnitude
                self.na_conductance += G['gna'] * mag * m * m * m * h
                self.k_conductance += G['gk'] * mag * n * n * n * n
                self.l_conductance += G['gl'] * mag
            cls_.advance = data.add_method(advance)
            return cls_

        @classmethod
        def get_name(cls):
            return 'hh'

        def __init__(self, segment, outside=None, magnitude=1.0):
            self.segment = segment
            self.magnitude = magnitude * segment.surface_area
    return hh


def make_kinetic(name, scheme, ion, gbar, num_buckets, v_init, record):
    """Developers-API kinetic channel whose step is the reference's own lti_sim
    output: LTI_Model + MatrixSamples + Approx1D build the table (seeded numpy RNG),
    Codegen._kernel emits the run-time kernel, and the advance method calls it and
    adds gbar * 1e-8 * magnitude * (open states) to the segment's {ion}_conductance
    accumulator, as the NMODL front end compiles a KINETIC mechanism
    (nmodl/__init__.py:298-306, 415-432).  The derivative is this package's
    restatement of the .mod file's KINETIC block (the NMODL parser is absent).
    record(key, value) receives the table, its sample inputs and the initial state."""
    from neuwon.rxd.mechanisms import Mechanism
    from neuwon.database import Compute
    from neuwon.rxd.lti_sim import LTI_Model, LinearInput
    from neuwon.rxd.lti_sim.approx import Approx1D, MatrixSamples
    from neuwon.rxd.lti_sim.codegen import Codegen
    from neuwon.rxd.nmodl.code_gen import exec_string

    class kinetic(Mechanism):
        __slots__ = ()

        @classmethod
        def initialize(cls, model):
            db = model.get_database()
            celsius = model.get_temperature()
            dt = model.get_time_step()

            def derivative(v, *state):
                return list(scheme.matrix([v], celsius)[0] @ np.array(state))
            inp = LinearInput('v', 'self.segment.voltage', -100, 100, initial=v_init)
            lti = LTI_Model(name, [inp], scheme.states, derivative, 1.0, dt)
            inp.set_num_buckets(num_buckets)
            samples = MatrixSamples(lti)
            approx = Approx1D(samples, 1)
            cg = Codegen.__new__(Codegen)              # Codegen.__init__ minus its timing run
            cg.model, cg.table, cg.polynomial, cg.target = lti, approx.table, approx.polynomial, 'host'
            cg.name, cg.inputs, cg.input_names = lti.name, lti.inputs, lti.input_names
            cg.state_names, cg.num_states, cg.conserve_sum = lti.state_names, lti.num_states, lti.conserve_sum
            cg.initial_state = lti.get_initial_state()
            table_data = cg._table_data()
            init = cg.initial_state
            record("table", np.asarray(table_data, dtype=np.float64).reshape(num_buckets, lti.num_states,
                                                                                lti.num_states, -1))
            record("samples", samples.inputs[0])
            record("init", np.array([init[s] for s in scheme.states]))
            data = db.add_class(cls)
            data.add_attribute('segment', dtype='Segment')
            data.add_attribute('magnitude', units='um2')
            for s in scheme.states:
                data.add_attribute(s, init[s])
            cls_ = data.get_instance_type()
            opened = " + ".join(f"self.{scheme.states[k]}" for k in scheme.open_states)
            # The NMODL front end emits one advance that calls the generated kernel
            # (nmodl/__init__.py:415-429); the reference's JIT does not pass that
            # kernel's local arrays (its Alloc annotations) through a nested call
            # (NameError at run time), so the kernel and the conductance write run
            # as two methods over all instances, in that order.
            src = (cg._kernel() + "\n"
                   "@Compute\n"
                   "def write_conductance(self):\n"
                   f"    self.segment.{ion}_conductance += {gbar * 1e-8!r} * self.magnitude * ({opened})\n")
            scope = {"Compute": Compute, "table": table_data, "numpy": np}
            exec_string(src, scope)
            lti_step = data.add_method(scope[f"{name}_advance"])
            write = data.add_method(scope["write_conductance"])

            def advance():
                lti_step()
                write()
            cls_.advance = staticmethod(advance)
            return cls_

        @classmethod
        def get_name(cls):
            return name

        def __init__(self, segment, outside=None, magnitude=1.0):
            self.segment = segment
            self.magnitude = magnitude * segment.surface_area
    kinetic.__name__ = kinetic.__qualname__ = name        # the database class is named after it
    return kinetic


def run_species(out):
    """Electric species (constant reversal potentials) fed by two kinetic channels of
    the reference library, Nav1.1 -> na and Kv1.1 -> k (tables and kernels from the
    reference's lti_sim), plus the restated hh with weaker sodium and potassium, on
    two neurons; a second Nav1.1 instance on two segments (a species accumulator
    counts both).  Records traces, spikes and each channel's table."""
    from neuwon.rxd.rxd_model import RxD_Model
    from neuwon_gb300.kinetic import kv11, nav11
    from neuwon_gb300.morphology import random_tree
    np.random.seed(4321)
    spec = dict(time_step=0.1, celsius=6.3, t_stop=25.0, v_init=-70.0,
                hh=dict(gnabar=0.12, gkbar=0.036, glbar=0.0003, ena=50.0, ek=-77.0, el=-54.3),
                nav=dict(gbar=0.03, buckets=2000), kv=dict(gbar=0.01, buckets=2000))
    rec = {}
    mechs = [make_hh(**spec["hh"]),
             make_kinetic("na11a", nav11(), "na", spec["nav"]["gbar"], spec["nav"]["buckets"], spec["v_init"],
                          lambda k, v: rec.__setitem__("nav_" + k, v)),
             make_kinetic("Kv11_6States_temperature2", kv11(), "k", spec["kv"]["gbar"], spec["kv"]["buckets"],
                          spec["v_init"], lambda k, v: rec.__setitem__("kv_" + k, v))]
    m = RxD_Model(time_step=spec["time_step"], temperature=spec["celsius"], initial_voltage=spec["v_init"],
                  species=[dict(name="na", charge=1, reversal_potential=50.0),
                           dict(name="k", charge=1, reversal_potential=-77.0)],
                  mechanisms=mechs)
    trees = [random_tree(80, seed=31), random_tree(50, seed=32)]
    all_segs = [build_reference_tree(m, t) for t in trees]
    flat = [s for segs in all_segs for s in segs]
    hh, nav, kv = (m.mechanisms[n] for n in ("hh", "na11a", "Kv11_6States_temperature2"))
    for s in flat:
        hh(s)
        nav(s)
    for k, s in enumerate(flat):
        if k % 7 != 3:                     # Kv1.1 on most segments only
            kv(s)
    dup = [5, 90]
    for k in dup:
        nav(flat[k])
    clamps = [(0, 0, 0.5, 2.0, 15.0), (1, 0, 0.4, 4.0, 12.0)]
    probes = [0, 10, 40, 79, 80, 100, 129]
    trace = [np.array([flat[p].voltage for p in probes])]
    ap = []
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    for k in range(steps):
        for (t, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                all_segs[t][s].inject_current(nA, dur)
        m.advance()
        trace.append(np.array([flat[p].voltage for p in probes]))
        ap.append(np.array(m.database.get_data("Neuron.AP_detected"), dtype=bool).copy())
        if k + 1 in (100, 250):
            out[f"species_snap{k + 1}"] = seg_array(m, "voltage")
            out[f"species_gna_snap{k + 1}"] = seg_array(m, "na_conductance")
            out[f"species_gk_snap{k + 1}"] = seg_array(m, "k_conductance")
    # Each channel's sample points and initial state in full; of its table every
    # 10th bucket (the full table is rebuilt from the sample points and checked
    # against these buckets).
    for key in ("nav", "kv"):
        out[f"species_{key}_samples"] = rec[f"{key}_samples"]
        out[f"species_{key}_init"] = rec[f"{key}_init"]
        out[f"species_{key}_table10"] = rec[f"{key}_table"][::10]
    out["species_trace"] = np.array(trace)
    out["species_probes"] = np.asarray(probes, dtype=np.int64)
    out["species_ap"] = np.array(ap)
    out["species_kv_skip"] = np.array([k for k in range(len(flat)) if k % 7 == 3], dtype=np.int64)
    out["species_dup"] = np.asarray(dup, dtype=np.int64)
    out["species_clamps"] = np.array(clamps, dtype=np.float64)
    out["species_meta"] = np.array([spec["time_step"], spec["celsius"], spec["t_stop"], spec["v_init"],
                                    spec["hh"]["gnabar"], spec["hh"]["gkbar"], spec["hh"]["glbar"],
                                    spec["hh"]["ena"], spec["hh"]["ek"], spec["hh"]["el"],
                                    spec["nav"]["gbar"], spec["kv"]["gbar"], 50.0, -77.0])


def run_dropin(out, prefix, tree, clamps, hh_kwargs, t_stop, insert_as_created):
    """The drop-in backend's view of a reference model: neuwon_gb300.dropin.extract
    (the arrays GB300Advance reads from the reference's Database after db.sort())
    at time 0, and before every step the device clamps clamp_players derives from
    the reference's own input-clock players, while the reference advances itself;
    plus the reference's voltages of every segment after every step."""
    from neuwon.rxd.rxd_model import RxD_Model
    from neuwon_gb300.dropin import clamp_players, extract
    m = RxD_Model(time_step=0.1, temperature=6.3, mechanisms=[make_hh(**hh_kwargs)])
    hh = m.mechanisms["hh"]
    segs = []
    for i in range(len(tree)):
        p = int(tree.parent[i])
        xyz = [float(x) for x in tree.coordinates[i]]
        d = float(tree.diameter[i])
        segs.append(m.Neuron(xyz, d).root if p < 0 else m.Segment(segs[p], xyz, d))
        if insert_as_created:
            hh(segs[-1])
    if not insert_as_created:
        for s in segs:
            hh(s)
    dens = {"hh": {k: hh_kwargs.get(k, d) for k, d in (("gnabar", .12), ("gkbar", .036), ("glbar", .0003))}}
    arrays = extract(m, dens)
    for key in ("parent", "neuron_start", "capacitance", "axial_resistance", "voltage"):
        out[f"{prefix}_{key}"] = arrays[key]
    for key in ("segment", "magnitude", "m", "h", "n"):
        out[f"{prefix}_hh_{key}"] = arrays["hh"][key]
    h = arrays["hh"]
    out[f"{prefix}_meta"] = np.array([arrays["time_step"], arrays["celsius"], h["gnabar"], h["gkbar"], h["glbar"],
                                      h["ena"], h["ek"], h["el"]])
    steps = int(round(t_stop / 0.1))
    played, volts = [], [seg_array(m, "voltage")]
    for k in range(steps):
        for (s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                segs[s].inject_current(nA, dur)
        for c in clamp_players(m, 2 * k):
            played.append((k,) + c)
        m.advance()
        volts.append(seg_array(m, "voltage"))
    out[f"{prefix}_clamps"] = np.array(played, dtype=np.float64).reshape(-1, 5)
    out[f"{prefix}_volts"] = np.array(volts)


def build_reference_tree(model, tree):
    """Create the tree's segments through the reference API, in order."""
    segs = []
    for i in range(len(tree)):
        p = int(tree.parent[i])
        xyz = [float(x) for x in tree.coordinates[i]]
        d = float(tree.diameter[i])
        if p < 0:
            segs.append(model.Neuron(xyz, d).root)
        else:
            segs.append(model.Segment(segs[p], xyz, d))
    return segs


def seg_array(model, name):
    return np.array(model.database.get_data(f"Segment.{name}"), dtype=np.float64).copy()


def run_geometry_and_propagator(out):
    from neuwon.rxd.rxd_model import RxD_Model
    from neuwon_gb300.morphology import random_tree
    tree = random_tree(120, seed=7)
    m = RxD_Model(time_step=0.1)
    build_reference_tree(m, tree)
    m.database.sort()
    seg_cls = m.Segment
    seg_cls._compute_propagator_matrix(0.05)
    P = m.database.get("Segment.electric_propagator_matrix").to_csr().get_data()
    # expm returns CSC, which the reference stores as is; normalise to CSR.
    import scipy.sparse
    P = scipy.sparse.csr_matrix(P)
    P.sort_indices()
    out["geom_parent"] = tree.parent
    out["geom_coordinates"] = tree.coordinates
    out["geom_diameter"] = tree.diameter
    for name in ("length", "surface_area", "cross_sectional_area", "volume",
                 "axial_resistance", "capacitance"):
        out["geom_" + name] = seg_array(m, name)
    out["geom_primary"] = np.array(m.database.get_data("Segment._primary"), dtype=bool)
    out["prop_indptr"] = np.asarray(P.indptr, dtype=np.int64)
    out["prop_indices"] = np.asarray(P.indices, dtype=np.int64)
    out["prop_data"] = np.asarray(P.data, dtype=np.float64)


def run_hh_tree(out, prefix, trees, *, time_step, celsius, t_stop, clamps, hh_kwargs,
                probes, snapshots, duplicate_segments=(), insert_as_created=False):
    """HH on every segment of every tree; clamps = [(tree, seg, nA, start, dur)].

    insert_as_created inserts each segment's hh instance right after creating the
    segment (as neuwon/rxd/tests/test_model.py:48-52 does), so its magnitude is the
    segment's area as a leaf; otherwise instances are inserted after the tree is grown."""
    from neuwon.rxd.rxd_model import RxD_Model
    m = RxD_Model(time_step=time_step, temperature=celsius, mechanisms=[make_hh(**hh_kwargs)])
    hh = m.mechanisms['hh']
    all_segs = []
    for tree in trees:
        if insert_as_created:
            segs = []
            for i in range(len(tree)):
                p = int(tree.parent[i])
                xyz = [float(x) for x in tree.coordinates[i]]
                d = float(tree.diameter[i])
                segs.append(m.Neuron(xyz, d).root if p < 0 else m.Segment(segs[p], xyz, d))
                hh(segs[-1])
        else:
            segs = build_reference_tree(m, tree)
        all_segs.append(segs)
    if not insert_as_created:
        for segs in all_segs:
            for s in segs:
                hh(s)
    for (t, s) in duplicate_segments:
        hh(all_segs[t][s])
    flat = [s for segs in all_segs for s in segs]
    trace = [np.array([flat[p].voltage for p in probes])]
    snaps = {}
    ap = []
    steps = int(round(t_stop / time_step))
    for k in range(steps):
        for (t, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                all_segs[t][s].inject_current(nA, dur)
        m.advance()
        trace.append(np.array([flat[p].voltage for p in probes]))
        ap.append(np.array(m.database.get_data("Neuron.AP_detected"), dtype=bool).copy())
        if (k + 1) in snapshots:
            snaps[k + 1] = seg_array(m, "voltage")
    out[prefix + "_trace"] = np.array(trace)
    out[prefix + "_probes"] = np.asarray(probes, dtype=np.int64)
    out[prefix + "_ap"] = np.array(ap)
    for k, v in snaps.items():
        out[f"{prefix}_snap{k}"] = v
    out[prefix + "_meta"] = np.array([time_step, celsius, t_stop])


def run_lti(out):
    """The reference's lti_sim table builder (approx.py) on the 8-state sodium scheme."""
    np.random.seed(1234)
    if not hasattr(np, "product"):
        np.product = np.prod            # removed in numpy 2; used by approx.py:81
    from neuwon.rxd.lti_sim import LTI_Model, LinearInput
    from neuwon.rxd.lti_sim.approx import Approx1D, MatrixSamples
    from neuwon_gb300.kinetic import na8
    sch = na8()

    def derivative(v, *state):
        return list(sch.matrix([v], 6.3)[0] @ np.array(state))
    inp = LinearInput('v', 'self.segment.voltage', -100, 60)
    model = LTI_Model('na8', [inp], sch.states, derivative, 1.0, 0.1)
    inp.set_num_buckets(1600)
    samples = MatrixSamples(model)
    approx = Approx1D(samples, 1)
    out["lti_table"] = approx.table
    out["lti_samples"] = samples.inputs[0]
    rng = np.random.default_rng(5)
    v = np.concatenate([rng.uniform(-110, 70, 300), [-100.0, -100.05, -100.2, 60.0, 75.0, -99.95]])
    st = rng.dirichlet(np.ones(8), len(v))
    new = []
    for vi, si in zip(v, st):
        x = approx.approximate_matrix(vi) @ si
        new.append(x * (1.0 / x.sum()))          # CONSERVE, codegen.py:95-102
    out["lti_v"], out["lti_state"], out["lti_new"] = v, st, np.array(new)


def run_lti2(out):
    """The reference's two-input table builder (Approx2D, approx.py:242-275) on the
    NMDA receptor scheme of nmodl_library/kinetic/NMDA.mod (restated as
    neuwon_gb300.kinetic.nmda, inputs sorted by name as lti_model.py:8 sorts them: C,
    then v), with quadratic terms on 4 x 8 buckets: its table, its random sample
    inputs, its approximate matrices at test points and its initial state."""
    np.random.seed(4321)
    if not hasattr(np, "product"):
        np.product = np.prod            # removed in numpy 2; used by approx.py:81
    from neuwon.rxd.lti_sim import LTI_Model, LinearInput, LogarithmicInput
    from neuwon.rxd.lti_sim.approx import Approx2D, MatrixSamples
    from neuwon_gb300.kinetic import nmda
    sch = nmda()

    def derivative(C, v, *state):
        return list(sch.matrix([C], [v], 6.3)[0] @ np.array(state))
    c_in = LogarithmicInput('C', 'self.C', 0, 1000)
    v_in = LinearInput('v', 'self.segment.voltage', -100, 100)
    model = LTI_Model('NMDA_Mg', [v_in, c_in], sch.states, derivative, 1.0, 0.1)
    c_in.set_num_buckets(4, scale=1e-2)
    v_in.set_num_buckets(8)
    terms = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2)]
    samples = MatrixSamples(model)
    approx = Approx2D(samples, terms)
    out["lti2_table"] = approx.table                               # [bC][bv][row][col][term]
    out["lti2_terms"] = np.array(approx.polynomial.terms)
    out["lti2_samples_C"], out["lti2_samples_v"] = samples.inputs[0], samples.inputs[1]
    rng = np.random.default_rng(9)
    C = np.concatenate([10.0 ** rng.uniform(-4, 3, 40), [0.0, 1000.0, 0.5]])
    v = np.concatenate([rng.uniform(-100, 100, 40), [-100.0, 100.0, 120.0]])
    out["lti2_C"], out["lti2_v"] = C, v
    out["lti2_approx"] = np.array([approx.approximate_matrix(c, x) for c, x in zip(C, v)])
    init = model.get_initial_state()
    out["lti2_init"] = np.array([init[x] for x in sch.states])     # at the inputs' minimum (C 0, v -100)


def scenarios():
    """Fixture groups by key prefix, each a function of the output dict."""
    from neuwon_gb300.morphology import random_tree, Tree

    def hh11(out):
        # The reference test's 11-segment HH scenario (test_model.py:35-66).
        coords = [[-1, 0, 7]] + [[x, 0, 7] for x in range(10)]
        t11 = Tree([-1] + list(range(10)), coords, [5.7] + [1.0] * 10)
        run_hh_tree(out, "hh11", [t11], time_step=0.1, celsius=6.3, t_stop=20.0,
                    clamps=[(0, 0, .1, 5.0, 1.0), (0, 0, .1, 15.0, 1.0)],
                    hh_kwargs={}, probes=list(range(11)), snapshots={100, 200}, insert_as_created=True)

    def hh200(out):
        # A 200-segment tree, workload parameters of the single-neuron config.
        run_hh_tree(out, "hh200", [random_tree(200, seed=11)], time_step=0.1, celsius=6.3, t_stop=30.0,
                    clamps=[(0, 0, 0.2, 5.0, 20.0)],
                    hh_kwargs=dict(ena=50.0, ek=-77.0, el=-54.3),
                    probes=[0, 1, 50, 100, 150, 199], snapshots={100, 300})

    def multi(out):
        # Three neurons (block-diagonal propagator), clamps on different segments,
        # plus a second hh instance on two segments (reference drops duplicates).
        ts = [random_tree(40, seed=21), random_tree(25, seed=22), random_tree(60, seed=23)]
        run_hh_tree(out, "multi", ts, time_step=0.1, celsius=6.3, t_stop=15.0,
                    clamps=[(0, 0, 0.3, 1.0, 6.0), (1, 5, 0.2, 2.0, 3.0), (2, 30, 0.25, 0.5, 8.0)],
                    hh_kwargs=dict(ena=50.0, ek=-77.0),
                    probes=[0, 10, 40, 45, 65, 95, 124], snapshots={150},
                    duplicate_segments=[(0, 3), (2, 30)])

    def c1(out):
        # The single-neuron configuration at full size: 2,000 segments (seed 0), HH
        # everywhere, 0.2 nA soma clamp 5-80 ms, dt 0.1 ms for 100 ms, the reference's
        # own epsilon-pruned propagator.  All segment voltages every 100 steps.
        run_hh_tree(out, "c1", [random_tree(2000, seed=0)], time_step=0.1, celsius=6.3, t_stop=100.0,
                    clamps=[(0, 0, 0.2, 5.0, 75.0)],
                    hh_kwargs=dict(ena=50.0, ek=-77.0, el=-54.3),
                    probes=[0, 1, 500, 1000, 1500, 1999],
                    snapshots={100 * i for i in range(1, 11)})

    def dropin(out):
        # The drop-in backend's arrays and clamps, read live from the reference:
        # the 11-segment cable (instances inserted as segments are created) and a
        # 200-segment tree.
        coords = [[-1, 0, 7]] + [[x, 0, 7] for x in range(10)]
        t11 = Tree([-1] + list(range(10)), coords, [5.7] + [1.0] * 10)
        run_dropin(out, "dropin_hh11", t11, [(0, .1, 5.0, 1.0), (0, .1, 15.0, 1.0)], {}, 20.0, True)
        run_dropin(out, "dropin_hh200", random_tree(200, seed=11), [(0, 0.2, 5.0, 20.0)],
                   dict(ena=50.0, ek=-77.0, el=-54.3), 30.0, False)

    return {"geom": run_geometry_and_propagator, "hh11": hh11, "hh200": hh200, "multi": multi, "c1": c1,
            "lti": run_lti, "lti2": run_lti2, "species": run_species, "dropin": dropin}


def main():
    """make_golden.py <reference checkout> [--only name,name]: with --only, the named
    groups are regenerated and merged into the existing fixture file."""
    args = sys.argv[1:]
    only = None
    if "--only" in args:
        k = args.index("--only")
        only = args[k + 1].split(",")
        del args[k:k + 2]
    global REFERENCE
    REFERENCE = reference_path(args)
    install_stubs()
    path = os.path.join(HERE, "reference_fixtures.npz")
    groups = scenarios()
    out = {}
    if only:
        prefixes = {"geom": ("geom_", "prop_")}
        with np.load(path) as old:
            for key in old.files:
                if not any(key.startswith(p) for g in only for p in prefixes.get(g, (g + "_",))):
                    out[key] = old[key]
    for name, fn in groups.items():
        if only is None or name in only:
            fn(out)
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
