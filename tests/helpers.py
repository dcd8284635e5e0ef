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


def species_spec(fx):
    """The species scenario recorded from the reference (make_golden.run_species)."""
    meta = fx["species_meta"]
    return dict(time_step=float(meta[0]), celsius=float(meta[1]), t_stop=float(meta[2]), v_init=float(meta[3]),
                hh=dict(gnabar=meta[4], gkbar=meta[5], glbar=meta[6], ena=meta[7], ek=meta[8], el=meta[9]),
                nav_gbar=float(meta[10]), kv_gbar=float(meta[11]),
                species={"na": float(meta[12]), "k": float(meta[13])},
                trees=[random_tree(80, seed=31), random_tree(50, seed=32)],
                clamps=[(int(t), int(s), nA, start, dur) for t, s, nA, start, dur in fx["species_clamps"]],
                probes=fx["species_probes"], dup=fx["species_dup"], kv_skip=fx["species_kv_skip"])


def species_tables(fx):
    """The reference's Nav1.1 and Kv1.1 tables, rebuilt by this package's host table
    builder from the reference's own random sample points (equal to the reference's
    tables to 1e-12: tests/test_species.py), with the reference's initial states."""
    from neuwon_gb300.kinetic import LTITable, kv11, nav11
    meta = fx["species_meta"]
    out = {}
    for key, factory in (("nav", nav11), ("kv", kv11)):
        tbl = LTITable(factory(), float(meta[0]), float(meta[1]), -100.0, 100.0, 2000, 1,
                       sample_inputs=fx[f"species_{key}_samples"])
        out[key] = (tbl.layout, fx[f"species_{key}_init"])
    return out


def species_instances(spec):
    """Segments of the Nav1.1 instances (every segment, then the duplicates) and of the
    Kv1.1 instances (all but the skipped segments), in registration order."""
    n = sum(len(t) for t in spec["trees"])
    nav = np.concatenate([np.arange(n), spec["dup"]]).astype(np.int64)
    kv = np.setdiff1d(np.arange(n), spec["kv_skip"]).astype(np.int64)
    return nav, kv


def species_oracle(fx, tables=None):
    """Oracle of the species scenario: HH + Nav1.1 (-> na) + Kv1.1 (-> k) with the
    reference's tables and initial states (or ``tables`` = {"nav": (layout, init),
    "kv": (layout, init)})."""
    from oracle.reference_step import KineticInstances
    spec = species_spec(fx)
    parent, R, C, area, offs = concat(spec["trees"])
    n = len(parent)
    hh = HHInstances(np.arange(n), area, celsius=spec["celsius"], v_init=spec["v_init"],
                     **{k: float(v) for k, v in spec["hh"].items()})
    nav_seg, kv_seg = species_instances(spec)
    tables = tables or species_tables(fx)
    frq = 2000 / 200.0
    nav = KineticInstances(nav_seg, spec["nav_gbar"] * 1e-8 * area[nav_seg], tables["nav"][0], -100.0, frq, [2, 3],
                           0.0, 1.0, tables["nav"][1], species="na")
    kv = KineticInstances(kv_seg, spec["kv_gbar"] * 1e-8 * area[kv_seg], tables["kv"][0], -100.0, frq, [1],
                          0.0, 1.0, tables["kv"][1], species="k")
    cl = []
    for (ti, s, nA, start, dur) in spec["clamps"]:
        f, c = clamp_ticks(start, dur, spec["time_step"])
        cl.append((offs[ti] + s, nA * 1e-9, f, c))
    om = OracleModel(parent, R, C, time_step=spec["time_step"], celsius=spec["celsius"], v_init=spec["v_init"],
                     hh=hh, kinetic=[nav, kv], species=spec["species"], clamps=cl,
                     detectors=[(o, 20.0) for o in offs])
    return om, spec


def install_propagator(m, P, fmt=2):
    """Replace a synced model's propagator by P (scipy CSR over creation indices,
    e.g. the oracle's), permuted to the device's segment order."""
    import ctypes
    import scipy.sparse
    from neuwon_gb300 import _lib
    Pd = scipy.sparse.csr_matrix(P)[m._order][:, m._order].tocsr()
    Pd.sort_indices()
    rowptr = np.ascontiguousarray(Pd.indptr, dtype=np.int64)
    col = np.ascontiguousarray(Pd.indices, dtype=np.int64)
    val = np.ascontiguousarray(Pd.data, dtype=np.float64)
    m._ctx.call("nw_propagator_set_csr", m._n, _lib.ptr(rowptr), _lib.ptr(col), _lib.ptr(val), len(val))
    m._ctx.set_option("propagator_format", fmt)


def species_gpu(fx, precision="f64", path="batched", reference_tables=True, tolerance=None, propagator=None):
    """The species scenario through the public API: species declared with their
    reversal potentials, hh + Nav11 + Kv11 mechanisms.  propagator (scipy CSR over
    creation indices) replaces the one the model builds."""
    import neuwon_gb300 as nw
    spec = species_spec(fx)
    extra = {}
    if reference_tables:
        tables = species_tables(fx)
        nav_kw, kv_kw = dict(table=tables["nav"][0]), dict(table=tables["kv"][0])
    else:
        nav_kw, kv_kw = {}, {}
    if tolerance is not None:
        extra = dict(propagator_tolerance=tolerance, propagator_conserve=True)
    m = nw.RxD_Model(time_step=spec["time_step"], temperature=spec["celsius"], initial_voltage=spec["v_init"],
                     precision=precision, path=path,
                     species=[dict(name=k, charge=1, reversal_potential=v) for k, v in spec["species"].items()],
                     mechanisms=[nw.HH.configure(**{k: float(v) for k, v in spec["hh"].items()}),
                                 nw.Nav11.configure(gbar=spec["nav_gbar"], **nav_kw),
                                 nw.Kv11.configure(gbar=spec["kv_gbar"], **kv_kw)], **extra)
    offs = np.cumsum([0] + [len(t) for t in spec["trees"]])[:-1]
    for t in spec["trees"]:
        m.add_tree(t)
    m.insert_everywhere("hh")
    m.insert_everywhere("na11a")
    nav_seg, kv_seg = species_instances(spec)
    for s in nav_seg[len(nav_seg) - len(spec["dup"]):]:
        m.mechanisms["na11a"](nw.Segment(m, int(s)))
    for s in kv_seg:
        m.mechanisms["Kv11_6States_temperature2"](nw.Segment(m, int(s)))
    recs = [nw.TimeSeries().record(nw.Segment(m, int(p)), "voltage") for p in spec["probes"]]
    if propagator is not None:
        m._sync()
        install_propagator(m, propagator)
    return m, spec, offs, recs


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
              conserve=False, fmt="rows", duplicates="sum"):
    """The same case through the public RxD_Model API."""
    import neuwon_gb300 as nw
    hh_kw = dict(hh_kw or {})
    kw = {} if tolerance is None else {"propagator_tolerance": tolerance}
    kw["duplicates"] = duplicates
    if conserve == "lump":
        kw["propagator_lump"] = True
    elif conserve:
        kw["propagator_conserve"] = True
    kw["propagator_format"] = fmt
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


def network_case(sizes, num_synapses, *, seed=0, time_step=0.1, precision="f64", currents=None,
                 delay_lo=1.0, delay_hi=5.0, oracle=True, tolerance=None, path="batched", fmt="rows"):
    """Random trees wired by random_network; HH everywhere, a soma current per neuron.

    Returns (gpu model, oracle model or None, net dict, offsets)."""
    import neuwon_gb300 as nw
    from neuwon_gb300.synapses import SynapseKinetics, random_network
    from oracle.reference_step import SynapseInstances, synapse_matrices
    trees = [random_tree(int(n), seed=seed * 1000 + k) for k, n in enumerate(sizes)]
    net = random_network([len(t) for t in trees], num_synapses, seed, time_step=time_step,
                         delay_lo=delay_lo, delay_hi=delay_hi)
    rng = np.random.default_rng(seed + 7)
    amps = rng.uniform(0.05, 0.5, len(trees)) if currents is None else np.asarray(currents)
    clamps = [(k, 0, float(amps[k]), 0.0, 1e9) for k in range(len(trees))]
    hh_kw = dict(ena=50.0, ek=-77.0, el=-54.3)
    kw = {} if tolerance is None else {"propagator_tolerance": tolerance}
    m = nw.RxD_Model(time_step=time_step, temperature=6.3, precision=precision, path=path,
                     propagator_format=fmt, mechanisms=[nw.HH.configure(**hh_kw)], **kw)
    neurons = [m.add_tree(t) for t in trees]
    m.insert_everywhere("hh")
    offs = np.cumsum([0] + [len(t) for t in trees])[:-1]
    post = offs[net["post_neuron"]] + net["post_local"]
    kin = SynapseKinetics()
    m.add_synapses(net["pre"], post, net["weight_nS"], net["weight_nS"], net["delay_steps"] * time_step,
                   kinetics=kin)
    for (ti, s, nA, start, dur) in clamps:
        nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
    om = None
    if oracle:
        om, info = oracle_case(trees, clamps, time_step=time_step, hh_kw=hh_kw,
                               prune=tolerance if tolerance is not None else None)
        ao, af = synapse_matrices(time_step, kin.ampa_alpha, kin.ampa_beta, t_max=kin.t_max)
        no, nf = synapse_matrices(time_step, kin.nmda_alpha, kin.nmda_beta, kin.nmda_delta, kin.nmda_rho,
                                  t_max=kin.t_max)
        om.synapses = SynapseInstances(post, net["pre"], net["delay_steps"], net["weight_nS"] * 1e-9,
                                       net["weight_nS"] * 1e-9, ao, af, no, nf,
                                       kin.pulse_steps(time_step), kin.e_syn, kin.mg)
    return m, om, dict(net, post=post), offs


def calcium_case(trees, clamps, *, time_step=0.025, precision="f64", path="batched", tolerance=None,
                 conserve=False, oracle=True, calcium=None):
    """HH everywhere plus intracellular calcium (diffusion, pump, Na-fraction influx):
    the GPU model and the oracle with the same parameters."""
    import neuwon_gb300 as nw
    from oracle.reference_step import CalciumOracle
    ca = calcium or nw.Calcium()
    hh_kw = dict(ena=50.0, ek=-77.0, el=-54.3)
    kw = {} if tolerance is None else {"propagator_tolerance": tolerance}
    m = nw.RxD_Model(time_step=time_step, temperature=6.3, precision=precision, path=path, species=[ca],
                     propagator_conserve=conserve, mechanisms=[nw.HH.configure(**hh_kw)], **kw)
    neurons = [m.add_tree(t) for t in trees]
    m.insert_everywhere("hh")
    offs = np.cumsum([0] + [len(t) for t in trees])[:-1]
    for (ti, s, nA, start, dur) in clamps:
        nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
    om = None
    if oracle:
        om, info = oracle_case(trees, [(ti, s, nA, start, dur) for (ti, s, nA, start, dur) in clamps],
                               time_step=time_step, hh_kw=hh_kw, prune=tolerance)
        geoms = [geometry(t) for t in trees]
        cat = {k: np.concatenate([g[k] for g in geoms]) for k in ("cross_sectional_area", "length", "volume",
                                                                   "surface_area")}
        influx, efflux = ca.coefficients(cat)
        table = ca.table(time_step) if ca.pump else None
        om.calcium = CalciumOracle(info["parent"], cat["cross_sectional_area"], cat["length"], cat["volume"],
                                   ca.diffusivity, time_step, ca.initial, influx, efflux,
                                   table_step=(lambda c, st: ca.table_step(table, c, st)) if ca.pump else None,
                                   pump_state=ca.steady_state(ca.initial) if ca.pump else None,
                                   prune=tolerance if tolerance is not None else 2.220446049250313e-16)
    return m, om, offs
