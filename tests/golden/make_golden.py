"""Generate golden fixtures by running the reference NEUWON itself.

Run from the repository root with the path of a checkout of the reference
as the first argument (or in the environment variable ``NEUWON_REFERENCE``):

    python tests/golden/make_golden.py <path of the reference checkout>

The reference imports four third-party packages that are absent here
(numba, graph_algorithms, matplotlib, BlueBrain nmodl).  They are replaced by
import-only stubs written to a temporary directory: numba's ``njit`` becomes
the identity and ``prange`` becomes ``range`` (so the reference's ``@Compute``
kernels run as plain Python), ``topological_sort`` is a ten-line DFS, and the
rest are empty modules.  None of them is on the computed path except the
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


def main():
    install_stubs()
    from neuwon_gb300.morphology import random_tree, Tree
    out = {}
    run_geometry_and_propagator(out)

    # (1) The reference test's 11-segment HH scenario (test_model.py:35-66).
    coords = [[-1, 0, 7]] + [[x, 0, 7] for x in range(10)]
    t11 = Tree([-1] + list(range(10)), coords, [5.7] + [1.0] * 10)
    run_hh_tree(out, "hh11", [t11], time_step=0.1, celsius=6.3, t_stop=20.0,
                clamps=[(0, 0, .1, 5.0, 1.0), (0, 0, .1, 15.0, 1.0)],
                hh_kwargs={}, probes=list(range(11)), snapshots={100, 200}, insert_as_created=True)

    # (2) A 200-segment tree, workload parameters of the single-neuron config.
    t200 = random_tree(200, seed=11)
    run_hh_tree(out, "hh200", [t200], time_step=0.1, celsius=6.3, t_stop=30.0,
                clamps=[(0, 0, 0.2, 5.0, 20.0)],
                hh_kwargs=dict(ena=50.0, ek=-77.0, el=-54.3),
                probes=[0, 1, 50, 100, 150, 199], snapshots={100, 300})

    # (3) Three neurons (block-diagonal propagator), clamps on different segments,
    #     plus a second hh instance on two segments (reference drops duplicates).
    ts = [random_tree(40, seed=21), random_tree(25, seed=22), random_tree(60, seed=23)]
    run_hh_tree(out, "multi", ts, time_step=0.1, celsius=6.3, t_stop=15.0,
                clamps=[(0, 0, 0.3, 1.0, 6.0), (1, 5, 0.2, 2.0, 3.0), (2, 30, 0.25, 0.5, 8.0)],
                hh_kwargs=dict(ena=50.0, ek=-77.0),
                probes=[0, 10, 40, 45, 65, 95, 124], snapshots={150},
                duplicate_segments=[(0, 3), (2, 30)])

    # (4) The single-neuron configuration at full size: 2,000 segments (seed 0),
    #     HH everywhere, 0.2 nA soma clamp 5-80 ms, dt 0.1 ms for 100 ms, the
    #     reference's own epsilon-pruned propagator.  All segment voltages every
    #     100 steps.
    t2000 = random_tree(2000, seed=0)
    run_hh_tree(out, "c1", [t2000], time_step=0.1, celsius=6.3, t_stop=100.0,
                clamps=[(0, 0, 0.2, 5.0, 75.0)],
                hh_kwargs=dict(ena=50.0, ek=-77.0, el=-54.3),
                probes=[0, 1, 500, 1000, 1500, 1999],
                snapshots={100 * i for i in range(1, 11)})

    run_lti(out)

    path = os.path.join(HERE, "reference_fixtures.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
