"""GPU parity: the CUDA step through the C ABI against the FP64 oracle.

Tolerances:
  * FP64 contexts (batched and plain paths): 1e-7 mV max |dV| against the oracle.
  * FP32 batched path: 0.1 mV max |dV| (the metric's bound) on cases without
    spikes near the end of the window, equal spike counts always.
  * Propagator build (FP64, contour integral): 1e-13 absolute per entry.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse

import neuwon_gb300 as nw
from neuwon_gb300 import _lib
from neuwon_gb300.morphology import Tree, geometry, passive_electric, random_tree
from oracle.reference_step import EPSILON, propagator
from tests.helpers import FIXTURES, gpu_model, oracle_case, run_with_clamps, tree11

pytestmark = pytest.mark.gpu
F = np.load(FIXTURES)


def _ctx_with_tree(trees, precision="f64", dt=0.1):
    parent, R, C, area, offs = [], [], [], [], []
    from tests.helpers import concat
    parent, R, C, area, offs = concat(trees)
    n = len(parent)
    starts = np.array(list(offs) + [n], dtype=np.int64)
    ctx = _lib.Context(0, precision)
    ctx.call("nw_model_init", n, len(trees), _lib.ptr(starts), _lib.ptr(np.ascontiguousarray(parent)),
             dt, 6.3)
    ctx.set_data("Segment.capacitance", C)
    ctx.set_data("Segment.axial_resistance", np.where(parent < 0, 1.0, R))
    return ctx, parent, R, C


def _read_csr(ctx, n):
    nnz = ctypes.c_int64()
    ctx.call("nw_propagator_get_csr", None, None, None, ctypes.byref(nnz))
    rowptr = np.empty(n + 1, np.int64)
    col = np.empty(nnz.value, np.int64)
    val = np.empty(nnz.value, np.float64)
    ctx.call("nw_propagator_get_csr", _lib.ptr(rowptr), _lib.ptr(col), _lib.ptr(val), ctypes.byref(nnz))
    return scipy.sparse.csr_matrix((val, col, rowptr), shape=(n, n))


@pytest.mark.parametrize("tol", [EPSILON, 1e-9, 1e-6])
def test_propagator_build_matches_scipy_expm(tol):
    trees = [random_tree(300, seed=3), random_tree(1, seed=0), random_tree(120, seed=8)]
    ctx, parent, R, C = _ctx_with_tree(trees)
    nnz = ctypes.c_int64()
    ctx.call("nw_propagator_build", tol, ctypes.byref(nnz))
    P = _read_csr(ctx, len(parent))
    Pref = propagator(parent, R, C, 0.05, prune=0.0)
    diff = abs(P - Pref.multiply(abs(Pref) >= tol))
    # Entries within rounding of the threshold may land on either side.
    assert diff.max() < max(1e-13, 2 * tol)
    kept = abs(P).toarray() >= tol
    ref_kept = np.abs(Pref.toarray()) >= tol * (1 + 1e-6) + 1e-13
    assert np.all(kept[ref_kept])
    # Detailed balance c_i P_ij = c_j P_ji holds for the exact exponential.
    Pd = P.toarray()
    cp = C[:, None] * Pd
    both = (Pd != 0) & (Pd.T != 0)
    assert np.abs(cp - cp.T)[both].max() < 1e-13 * C.max()


@pytest.mark.parametrize("tol", [1e-8, 1e-6, 0.9])   # 0.9: every diagonal is below the tolerance
def test_lumped_propagator_matches_oracle(tol):
    """GPU lumping (pruned entries moved along the tree path to the nearest kept
    entry, then the unvisited remainder to the diagonal) equals the oracle's."""
    from oracle.reference_step import lump_and_conserve
    trees = [random_tree(300, seed=3), random_tree(1, seed=0), random_tree(120, seed=8)]
    ctx, parent, R, C = _ctx_with_tree(trees)
    ctx.set_option("propagator_lump", 1)
    nnz = ctypes.c_int64()
    ctx.call("nw_propagator_build", tol, ctypes.byref(nnz))
    ctx.call("nw_propagator_conserve")
    P = _read_csr(ctx, len(parent)).toarray()
    ref = lump_and_conserve(propagator(parent, R, C, 0.05, prune=0.0), parent, tol).toarray()
    assert np.abs(P - ref).max() < 1e-12
    assert np.abs(P.sum(axis=1) - 1.0).max() < 1e-12
    ctx.close()


@pytest.mark.parametrize("lump,tol", [(0, EPSILON), (0, 1e-8), (1, 1e-8), (1, 1e-6)])
def test_single_walk_build_equals_two_walks(lump, tol):
    """One walk per row into pool chunks gives the CSR of the counting and filling
    walks bit for bit; a pool too small for the rows falls back to two walks."""
    trees = [random_tree(300, seed=3), random_tree(1, seed=0), random_tree(120, seed=8), random_tree(700, seed=9)]
    out = []
    for once, chunks in ((0, 0), (1, 0), (1, 40)):
        ctx, parent, R, C = _ctx_with_tree(trees)
        ctx.set_option("propagator_lump", lump)
        ctx.set_option("propagator_single_walk", once)
        ctx.set_option("propagator_pool_chunks", chunks)
        nnz = ctypes.c_int64()
        ctx.call("nw_propagator_build", tol, ctypes.byref(nnz))
        walks = ctx.get_option("propagator_walks")
        P = _read_csr(ctx, len(parent))
        out.append((walks, P.indptr.copy(), P.indices.copy(), P.data.copy()))
        ctx.close()
    assert [o[0] for o in out] == [2, 1, 2]
    if tol <= 1e-8:
        assert np.diff(out[1][1]).max() > 2 * 64   # rows span several chunks
    for o in out[1:]:
        for x, y in zip(o[1:], out[0][1:]):
            assert np.array_equal(x, y)


def test_propagator_reference_fixture():
    t = Tree(F["geom_parent"], F["geom_coordinates"], F["geom_diameter"])
    ctx, parent, R, C = _ctx_with_tree([t])
    nnz = ctypes.c_int64()
    ctx.call("nw_propagator_build", EPSILON, ctypes.byref(nnz))
    P = _read_csr(ctx, len(t))
    Pr = scipy.sparse.csr_matrix((F["prop_data"], F["prop_indices"], F["prop_indptr"]), shape=P.shape)
    assert abs(P - Pr).max() < 1e-13


CASES = {
    "hh11": ([tree11()], [(0, 0, .1, 5., 1.), (0, 0, .1, 15., 1.)], {}, True),
    "hh200": ([random_tree(200, seed=11)], [(0, 0, 0.2, 5., 20.)], dict(ena=50., ek=-77., el=-54.3), False),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("path", ["batched", "plain", "wide"])
def test_f64_paths_match_reference_fixture(name, path):
    """The reference's own recorded voltages, reproduced by the FP64 GPU paths."""
    trees, clamps, hh_kw, as_created = CASES[name]
    ref = F[name + "_trace"]
    probes = F[name + "_probes"]
    m, neurons, offs, recs = gpu_model(trees, clamps, hh_kw=hh_kw, precision="f64", path=path,
                                       probes=list(probes), insert_as_created=as_created)
    run_with_clamps(m, clamps, offs, len(ref) - 1)
    got = np.array([r.get_data() for r in recs]).T
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() < 1e-7
    m.close()


def test_f64_multi_neuron_duplicates_sum():
    """Three neurons, two segments with two hh instances (summed, deterministic)."""
    trees = [random_tree(40, seed=21), random_tree(25, seed=22), random_tree(60, seed=23)]
    clamps = [(0, 0, 0.3, 1., 6.), (1, 5, 0.2, 2., 3.), (2, 30, 0.25, 0.5, 8.)]
    om, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3), (2, 30)])
    m, neurons, offs, _ = gpu_model(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3), (2, 30)],
                                    precision="f64")
    for k in range(150):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        om.advance()
    v = m.get_data("Segment.voltage")
    assert np.abs(v - om.voltage).max() < 1e-7
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    m.close()


def _c1_like(n=2000, t_ms=100.0, precision="f32", tol=EPSILON, seed=0):
    tree = random_tree(n, seed=seed)
    clamps = [(0, 0, 0.2, 5.0, 75.0)]
    hh_kw = dict(ena=50.0, ek=-77.0, el=-54.3)
    om, _ = oracle_case([tree], clamps, hh_kw=hh_kw, prune=tol)
    m, neurons, offs, _ = gpu_model([tree], clamps, hh_kw=hh_kw, precision=precision, tolerance=tol)
    steps = int(round(t_ms / 0.1))
    worst = 0.0
    for k in range(steps):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        om.advance()
        if k % 10 == 9:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
    spikes = (int(m.get_data("Neuron.spike_count")[0]), int(om.spike_count[0]))
    m.close()
    return worst, spikes


def test_f32_batched_single_neuron_config_short():
    """2,000-segment HH tree (the single-neuron config), 20 ms, FP32 vs FP64 oracle."""
    worst, (s_gpu, s_ref) = _c1_like(2000, 20.0)
    assert s_gpu == s_ref
    assert worst < 0.1, worst


@pytest.mark.parametrize("precision,tol,conserve,bound,path", [
    ("f32", 1e-6, "lump", 0.1, "batched"),
    ("f64", EPSILON, False, 1e-6, "batched"),
    ("f32", EPSILON, False, 0.1, "batched"),
    ("f32", 1e-8, True, 0.1, "batched"),
    ("f64", EPSILON, False, 1e-6, "wide"),
    ("f32", 1e-8, True, 0.1, "wide"),
])
def test_single_neuron_config_matches_reference(precision, tol, conserve, bound, path):
    """The single-neuron configuration at full size and length (2,000 segments, HH,
    0.2 nA soma clamp 5-80 ms, dt 0.1 ms for 100 ms): every segment's voltage every
    10 ms and the probed traces every step against the reference's own run; equal
    spike counts."""
    clamps = [(0, 0, 0.2, 5.0, 75.0)]
    probes = list(F["c1_probes"])
    m, neurons, offs, recs = gpu_model([random_tree(2000, seed=0)], clamps,
                                       hh_kw=dict(ena=50.0, ek=-77.0, el=-54.3), precision=precision,
                                       tolerance=tol, conserve=conserve, probes=probes, path=path)
    worst = 0.0
    for k in range(1000):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        if (k + 1) % 100 == 0:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - F[f"c1_snap{k + 1}"]).max())
    got = np.array([r.get_data() for r in recs]).T
    ref = F["c1_trace"]
    assert got.shape == ref.shape
    assert worst < bound, worst
    assert np.abs(got - ref).max() < bound
    assert int(m.get_data("Neuron.spike_count")[0]) == int(F["c1_ap"].sum())
    m.close()


@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_lanes_per_row_variants_agree(lanes):
    tree = random_tree(500, seed=2)
    clamps = [(0, 0, 0.3, 0.0, 10.0)]
    res = []
    for lpr in (lanes, 32):
        m, neurons, offs, _ = gpu_model([tree], clamps, precision="f64")
        m._sync()
        m._ctx.call("nw_set_tuning", lpr, 256, 0)
        run_with_clamps(m, clamps, offs, 60)
        res.append(m.get_data("Segment.voltage"))
        m.close()
    assert np.abs(res[0] - res[1]).max() < 1e-9


@pytest.mark.parametrize("bulk", [0, 1])
def test_batched_is_deterministic(bulk):
    trees = [random_tree(300, seed=s) for s in range(5)]
    clamps = [(k, 0, 0.3, 0.0, 20.0) for k in range(5)]
    outs = []
    for _ in range(2):
        m, neurons, offs, _ = gpu_model(trees, clamps, precision="f32")
        m._sync()
        m._ctx.call("nw_set_option", b"bulk_pipeline", bulk)
        run_with_clamps(m, clamps, offs, 100)
        outs.append(m.get_data("Segment.voltage"))
        m.close()
    assert np.array_equal(outs[0], outs[1])


def test_k_step_fusion_equals_single_steps():
    trees = [random_tree(250, seed=s) for s in range(3)]
    a, _, offs, _ = gpu_model(trees, [], precision="f64")
    b, _, _, _ = gpu_model(trees, [], precision="f64")
    for mm in (a, b):
        for k in range(3):
            nw.Segment(mm, offs[k]).inject_current(0.3, 8.0)
    a.advance(80)
    for _ in range(80):
        b.advance()
    assert np.abs(a.get_data("Segment.voltage") - b.get_data("Segment.voltage")).max() < 1e-12
    np.testing.assert_array_equal(a.get_data("Neuron.spike_count"), b.get_data("Neuron.spike_count"))


def test_passive_soma_only_and_no_mechanisms():
    """A lone sphere without mechanisms: injected charge ΔQ = I·t (test_electric.py:132-150)."""
    m = nw.RxD_Model(time_step=0.01, precision="f64")
    root = m.Neuron([0, 0, 0], 10).root
    m.advance(300)
    v0 = root.voltage
    init_Q = 1e-3 * v0 * root.capacitance
    root.inject_current(1, 2)
    m.advance(300)
    new_Q = 1e-3 * root.voltage * root.capacitance
    assert init_Q + 1e-9 * 2e-3 == pytest.approx(new_Q)
    m.close()


def test_nonfinite_voltage_is_reported():
    """A NaN injected from the host is flagged by the kernel, not silently propagated."""
    m, neurons, offs, _ = gpu_model([random_tree(50, seed=1)], [], precision="f32")
    m.advance()
    v = m.get_data("Segment.voltage")
    v[3] = np.nan
    m._ctx.set_data("Segment.voltage", v[m._order])
    with pytest.raises(_lib.NeuwonError, match="non-finite"):
        m.advance()
    m.close()


def test_bad_propagator_rejected():
    ctx, parent, R, C = _ctx_with_tree([random_tree(10, seed=1), random_tree(10, seed=2)])
    n = 20
    rowptr = np.arange(n + 1, dtype=np.int64)
    col = np.arange(n, dtype=np.int64)
    col[3] = 15          # couples neuron 0 to neuron 1
    val = np.ones(n)
    with pytest.raises(_lib.NeuwonError, match="couples two neurons"):
        ctx.call("nw_propagator_set_csr", n, _lib.ptr(rowptr), _lib.ptr(col), _lib.ptr(val), n)


@pytest.mark.parametrize("path", ["batched", "plain", "wide"])
def test_f64_hh_plus_na8_kinetic_matches_oracle(path):
    """HH + the 8-state Markov sodium scheme (voltage-table LTI step) vs the oracle."""
    trees = [random_tree(150, seed=31), random_tree(90, seed=32)]
    clamps = [(0, 0, 0.3, 1.0, 8.0), (1, 4, 0.2, 0.5, 5.0)]
    hh_kw = dict(ena=50., ek=-77.)
    om, _ = oracle_case(trees, clamps, hh_kw=hh_kw, kinetic=True)
    m, neurons, offs, _ = gpu_model(trees, clamps, hh_kw=hh_kw, precision="f64", path=path, kinetic=True)
    worst = 0.0
    for k in range(120):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        om.advance()
        if k % 20 == 19:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
    assert worst < 1e-7
    st = m.get_data("na8.state")
    assert np.abs(st - om.kinetic[0].state).max() < 1e-9
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    m.close()


def test_f32_hh_plus_na8_within_bound():
    trees = [random_tree(400, seed=41)]
    clamps = [(0, 0, 0.4, 0.0, 30.0)]
    om, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), kinetic=True)
    m, neurons, offs, _ = gpu_model(trees, clamps, hh_kw=dict(ena=50., ek=-77.), precision="f32", kinetic=True)
    worst = 0.0
    for k in range(300):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        om.advance()
        if k % 10 == 9:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
    assert worst < 0.1, worst
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    m.close()


def test_bulk_pipeline_matches_register_path():
    """The cp.async.bulk stream and the register stream compute the same step (FP32;
    only the assignment of entries to lanes, hence the rounding, differs)."""
    trees = [random_tree(1500, seed=51), random_tree(700, seed=52), random_tree(1, seed=0),
             random_tree(2600, seed=53)]
    clamps = [(0, 0, 0.4, 0.0, 20.0), (1, 0, 0.3, 1.0, 10.0), (3, 100, 0.5, 0.5, 15.0)]
    outs = []
    for bulk in (1, 0):
        m, neurons, offs, _ = gpu_model(trees, clamps, precision="f32", kinetic=True, tolerance=1e-9)
        m._sync()
        m._ctx.call("nw_set_option", b"bulk_pipeline", bulk)
        m._ctx.call("nw_set_tuning", 0 if bulk else 32, 1024, 0)
        active = ctypes.c_int64()
        m._ctx.call("nw_get_option", b"bulk_pipeline_active", ctypes.byref(active))
        assert active.value == bulk
        run_with_clamps(m, clamps, offs, 150)
        m.advance(50)
        outs.append((m.get_data("Segment.voltage"), m.get_data("na8.state"), m.get_data("Neuron.spike_count")))
        m.close()
    assert np.abs(outs[0][0] - outs[1][0]).max() < 1e-3
    assert np.abs(outs[0][1] - outs[1][1]).max() < 1e-5
    assert np.array_equal(outs[0][2], outs[1][2])
