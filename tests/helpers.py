"""Shared builders for oracle-vs-GPU parity cases."""
import numpy as np

from neuwon_gb300.morphology import Tree, geometry, passive_electric, random_tree
from oracle.reference_step import HHInstances, OracleModel, clamp_ticks

FIXTURES = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                      "reference_fixtures.npz")


def tree11():
    """The 11-segment cable of neuwon/rxd/tests/test_model.py:48-52."""
    coords = [[-1, 0, 7]] + [[x, 0, 7] for x in range(10)]
    return Tree([-1] + list(range(10)), coords, [5.7] + [1.0] * 10)


def concat(trees):
    parents, offs, off = [], [], 0
    for t in trees:
        parents.append(np.where(t.parent < 0, -1, t.parent + off))
        offs.append(off)
        off += len(t)
    geoms = [geometry(t) for t in trees]
    R = np.concatenate([passive_electric(g)[0] for g in geoms])
    C = np.concatenate([passive_electric(g)[1] for g in geoms])
    area = np.concatenate([g["surface_area"] for g in geoms])
    return np.concatenate(parents), R, C, area, offs


def kinetic_oracle(seg, area, time_step, celsius, gbar=0.012, erev=50.0, v_init=-70.0):
    """Na8 instances for the oracle, with the table and initial state the model uses."""
    from neuwon_gb300.kinetic import LTITable, na8
    from oracle.reference_step import KineticInstances
    sch = na8()
    tbl = LTITable(sch, time_step, celsius)
    init = sch.steady_state(v_init, celsius)
    return KineticInstances(seg, gbar * 1e-8 * area[seg], tbl.layout, tbl.vmin, tbl.bucket_frq,
                            sch.open_states, erev, sch.conserve_sum, init)


def oracle_case(trees, clamps, *, time_step=0.1, celsius=6.3, hh_kw=None, dups=(),
                duplicates="sum", prune=None, insert_as_created=False, kinetic=False):
    """clamps: [(tree, seg, nA, start_ms, dur_ms)]; dups: [(tree, seg)] extra hh instances.

    insert_as_created: instance magnitudes use each segment's area as a leaf
    (mechanism inserted right after the segment was created)."""
    parent, R, C, area, offs = concat(trees)
    if insert_as_created:
        area = np.concatenate([geometry(t)["creation_area"] for t in trees])
    n = len(parent)
    seg = np.array(list(range(n)) + [offs[a] + b for a, b in dups], dtype=np.int64)
    hh_kw = dict(hh_kw or {})
    hh = HHInstances(seg, area[seg], celsius=celsius, **hh_kw)
    cl = []
    for (ti, s, nA, start, dur) in clamps:
        f, c = clamp_ticks(start, dur, time_step)
        cl.append((offs[ti] + s, nA * 1e-9, f, c))
    det = [(o, 20.0) for o in offs]
    kw = {} if prune is None else {"prune": prune}
    if kinetic:
        kw["kinetic"] = kinetic_oracle(np.arange(n), area, time_step, celsius)
    om = OracleModel(parent, R, C, time_step=time_step, celsius=celsius, hh=hh, clamps=cl,
                     detectors=det, duplicates=duplicates, **kw)
    return om, dict(parent=parent, R=R, C=C, area=area, offs=offs, seg=seg, clamps=cl)


def gpu_model(trees, clamps, *, time_step=0.1, celsius=6.3, hh_kw=None, dups=(), precision="f32",
              path="batched", tolerance=None, probes=(), insert_as_created=False, kinetic=False,
              conserve=False):
    """The same case through the public RxD_Model API."""
    import neuwon_gb300 as nw
    hh_kw = dict(hh_kw or {})
    kw = {} if tolerance is None else {"propagator_tolerance": tolerance}
    if conserve:
        kw["propagator_conserve"] = True
    mechs = [nw.HH.configure(**hh_kw)] + ([nw.Kinetic] if kinetic else [])
    m = nw.RxD_Model(time_step=time_step, temperature=celsius, precision=precision, path=path,
                     mechanisms=mechs, **kw)
    hh = m.mechanisms["hh"]
    if insert_as_created:
        neurons = []
        for t in trees:
            segs = []
            for i in range(len(t)):
                p = int(t.parent[i])
                if p < 0:
                    neurons.append(m.Neuron(t.coordinates[i], t.diameter[i]))
                    segs.append(neurons[-1].root)
                else:
                    segs.append(m.Segment(segs[p], t.coordinates[i], t.diameter[i]))
                hh(segs[-1])
    else:
        neurons = [m.add_tree(t) for t in trees]
        m.insert_everywhere("hh")
        if kinetic:
            m.insert_everywhere("na8")
    offs = np.cumsum([0] + [len(t) for t in trees])[:-1]
    for (ti, s) in dups:
        hh(nw.Segment(m, offs[ti] + s))
    recs = [nw.TimeSeries().record(nw.Segment(m, p), "voltage") for p in probes]
    return m, neurons, offs, recs


def run_with_clamps(model, clamps, offs, steps):
    """Advance one step at a time, starting clamps like test_model.py:61-65."""
    import neuwon_gb300 as nw
    out = []
    for _ in range(steps):
        for (ti, s, nA, start, dur) in clamps:
            if model.clock.is_now(start):
                nw.Segment(model, offs[ti] + s).inject_current(nA, dur)
        model.advance()
    return out
