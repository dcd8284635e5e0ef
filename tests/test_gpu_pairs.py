"""The pair format of the batched path: each coupling (i, j) stored once and
applied to both segments through detailed balance (c_i P_ij = c_j P_ji), with
fixed-point accumulation so the result does not depend on the order of the
atomic adds."""
import ctypes

import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300 import _lib
from neuwon_gb300.morphology import EPSILON, random_tree
from tests.helpers import FIXTURES, gpu_model, run_with_clamps, tree11

F = np.load(FIXTURES)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", ["pairs", "quads"])
@pytest.mark.parametrize("name", ["hh11", "hh200"])
def test_f64_pairs_match_reference_fixture(name, fmt):
    cases = {"hh11": ([tree11()], [(0, 0, .1, 5., 1.), (0, 0, .1, 15., 1.)], {}, True),
             "hh200": ([random_tree(200, seed=11)], [(0, 0, 0.2, 5., 20.)], dict(ena=50., ek=-77., el=-54.3), False)}
    trees, clamps, hh_kw, as_created = cases[name]
    ref = F[name + "_trace"]
    m, neurons, offs, recs = gpu_model(trees, clamps, hh_kw=hh_kw, precision="f64", probes=list(F[name + "_probes"]),
                                       insert_as_created=as_created, fmt=fmt)
    run_with_clamps(m, clamps, offs, len(ref) - 1)
    got = np.array([r.get_data() for r in recs]).T
    assert np.abs(got - ref).max() < 1e-7
    assert m._ctx.get_option("propagator_format") == {"pairs": 1, "quads": 2}[fmt]
    m.close()


@pytest.mark.parametrize("fmt", ["pairs", "quads"])
def test_f32_pairs_single_neuron_config_matches_reference(fmt):
    clamps = [(0, 0, 0.2, 5.0, 75.0)]
    m, _, offs, recs = gpu_model([random_tree(2000, seed=0)], clamps, hh_kw=dict(ena=50.0, ek=-77.0, el=-54.3),
                                 precision="f32", tolerance=1e-8, conserve=True, probes=list(F["c1_probes"]),
                                 fmt=fmt)
    worst = 0.0
    for k in range(1000):
        for (ti, s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance()
        if (k + 1) % 100 == 0:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - F[f"c1_snap{k + 1}"]).max())
    assert worst < 0.1, worst
    assert int(m.get_data("Neuron.spike_count")[0]) == int(F["c1_ap"].sum())
    m.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_pair_sums_in_global_memory_are_bit_identical(precision):
    """A 19,500-segment neuron keeps its sums in global memory (shared memory holds
    fewer), the small ones in shared memory; forcing every neuron to global memory
    gives the same bits (integer sums), and the pair format stays within pruning
    differences of the row format (pairs keep a coupling if either direction
    reaches the tolerance)."""
    trees = [random_tree(19500, seed=2), random_tree(3000, seed=3), random_tree(700, seed=4)]
    clamps = [(0, 0, 3.0, 0.0, 50.0), (1, 0, 0.5, 0.0, 50.0), (2, 0, 0.3, 0.0, 50.0)]
    out = []
    for fmt, limit in (("pairs", -1), ("pairs", 0), ("rows", -1)):
        m, _, offs, _ = gpu_model(trees, clamps, precision=precision, tolerance=1e-8, conserve=True, fmt=fmt,
                                  kinetic=True)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m._sync()
        m._ctx.set_option("pair_shared_limit", limit)
        m.advance(300)
        out.append((m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count")))
        m.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.abs(out[0][0] - out[2][0]).max() < 0.01
    assert np.array_equal(out[0][1], out[2][1])


@pytest.mark.parametrize("fmt", ["pairs", "quads"])
def test_pairs_are_deterministic(fmt):
    trees = [random_tree(800, seed=s) for s in range(6)]
    clamps = [(k, 0, 0.4, 0.0, 30.0) for k in range(6)]
    outs = []
    for _ in range(2):
        m, _, offs, _ = gpu_model(trees, clamps, precision="f32", tolerance=1e-8, conserve=True, fmt=fmt)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance(200)
        outs.append(m.get_data("Segment.voltage"))
        m.close()
    assert np.array_equal(outs[0], outs[1])


def test_pairs_need_a_built_propagator():
    m, _, _, _ = gpu_model([random_tree(50, seed=1)], [], precision="f64")
    m._sync()
    n = m._n
    rowptr = np.arange(n + 1, dtype=np.int64)
    col = np.arange(n, dtype=np.int64)
    val = np.ones(n)
    m._ctx.call("nw_propagator_set_csr", n, rowptr.ctypes.data_as(ctypes.c_void_p),
                col.ctypes.data_as(ctypes.c_void_p), val.ctypes.data_as(ctypes.c_void_p), n)
    rc = m._ctx.lib.nw_set_option(m._ctx.handle, b"propagator_format", 1)
    assert rc == -3                                                    # NW_ERR_STATE
    m.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_quads_equal_rows(precision):
    """The quad format holds exactly the row format's entries (zeros fill the
    windows), so results agree to rounding; with depth-first numbering a window
    holds about 3.5 of its 4 slots."""
    trees = [random_tree(n, seed=90 + n) for n in (2500, 600, 40, 4)]
    clamps = [(0, 0, 0.5, 0.0, 50.0), (1, 0, 0.3, 0.0, 50.0), (2, 0, 0.2, 0.0, 50.0)]
    out = []
    for fmt in ("rows", "quads"):
        m, _, offs, _ = gpu_model(trees, clamps, precision=precision, tolerance=1e-8, conserve=True, fmt=fmt,
                                  kinetic=True)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance(300)
        out.append((m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count")))
        if fmt == "quads":
            nq = m._ctx.get_option("quads")
            assert m.propagator_nnz - m._n <= 4 * nq < 1.25 * (m.propagator_nnz - m._n)
        m.close()
    tol = 1e-9 if precision == "f64" else 2e-3
    assert np.abs(out[0][0] - out[1][0]).max() < tol
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_windows_equal_rows(precision):
    """The windows format (windows of 8, 4, 2 or 1 consecutive columns, zeros where
    a column is not kept) holds exactly the row format's entries, so results agree
    to rounding; neurons of 1 to 7 segments put windows past their last segment,
    onto the zero padding of x."""
    trees = [random_tree(n, seed=90 + n) for n in (2500, 600, 40, 7, 4, 2, 1)]
    clamps = [(0, 0, 0.5, 0.0, 50.0), (1, 0, 0.3, 0.0, 50.0), (2, 0, 0.2, 0.0, 50.0), (3, 0, 0.05, 0.0, 50.0)]
    out = []
    for fmt in ("rows", "windows"):
        m, _, offs, _ = gpu_model(trees, clamps, precision=precision, tolerance=1e-8, conserve=True, fmt=fmt,
                                  kinetic=True)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance(300)
        out.append((m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count")))
        if fmt == "windows":
            assert m._ctx.get_option("propagator_format") == 3
            rows, nnz, stored, pbytes = (ctypes.c_int64() for _ in range(4))
            m._ctx.call("nw_propagator_stats", ctypes.byref(rows), ctypes.byref(nnz), ctypes.byref(stored),
                        ctypes.byref(pbytes))
            off_diag = m.propagator_nnz - m._n
            assert off_diag <= stored.value < 1.25 * off_diag
            nwin = m._ctx.get_option("windows")
            assert pbytes.value == stored.value * (8 if precision == "f64" else 4) + 2 * nwin + \
                m._n * (16 + (8 if precision == "f64" else 4))
        m.close()
    tol = 1e-9 if precision == "f64" else 2e-3
    assert np.abs(out[0][0] - out[1][0]).max() < tol
    assert np.array_equal(out[0][1], out[1][1])


def test_windows_fused_steps_and_graphs_bit_identical():
    """Fusion depth and graph replay change nothing in the windows format (FP32)."""
    trees = [random_tree(n, seed=300 + n) for n in (1800, 700, 9)]
    clamps = [(0, 0, 0.4, 0.0, 30.0), (1, 0, 0.3, 0.0, 30.0)]
    res = []
    for fusion, graph in ((1, 0), (7, 1), (0, 1)):
        m, _, offs, _ = gpu_model(trees, clamps, precision="f32", tolerance=3e-7, conserve="lump", fmt="windows",
                                  kinetic=True)
        m._sync()
        m._ctx.set_option("fusion_depth", fusion)
        m._ctx.set_option("cuda_graph", graph)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance(60)
        res.append(m.get_data("Segment.voltage"))
        m.close()
    assert np.array_equal(res[0], res[1]) and np.array_equal(res[0], res[2])


def test_windows_need_sorted_rows():
    """A propagator whose rows are not sorted by column is refused by the windows
    format (the quad and row formats take it)."""
    m, _, _, _ = gpu_model([random_tree(30, seed=5)], [], precision="f64", fmt="windows")
    m._sync()
    n = m._n
    cols, vals, ptr = [], [], [0]
    for i in range(n):                       # row 0 lists column 1 before its diagonal
        if i == 0:
            cols += [1, 0]
            vals += [1e-3, 1 - 1e-3]
        elif i == 1:
            cols += [0, 1]
            vals += [1e-3, 1 - 1e-3]
        else:
            cols += [i]
            vals += [1.0]
        ptr.append(len(cols))
    rowptr = np.array(ptr, dtype=np.int64)
    col = np.array(cols, dtype=np.int64)
    val = np.array(vals)
    m._ctx.call("nw_propagator_set_csr", n, _lib.ptr(rowptr), _lib.ptr(col), _lib.ptr(val), len(val))
    m._ctx.set_option("propagator_format", 3)
    rc = m._ctx.lib.nw_advance(m._ctx.handle, 1, _lib.PATH_BATCHED)
    assert rc == -3                                                    # NW_ERR_STATE
    m._ctx.set_option("propagator_format", 2)
    m._ctx.advance(1)
    m.close()


def test_quads_lanes_split_by_row_length():
    """Neurons of short rows (mean quads per row below "lanes_split") take half the
    lanes per row: the same windows summed in another order, so FP32 results agree
    to rounding with equal spikes, and fusion depth and graph replay still change
    no bit."""
    trees = [random_tree(n, seed=400 + n) for n in (3000, 900, 120, 30)]
    clamps = [(0, 0, 0.5, 0.0, 40.0), (1, 0, 0.3, 0.0, 40.0), (2, 0, 0.2, 0.0, 40.0)]
    out = {}
    for split, fusion, graph in ((0, 7, 1), (65535, 1, 0), (65535, 7, 1)):
        m, _, offs, _ = gpu_model(trees, clamps, precision="f32", tolerance=3e-7, conserve="lump", fmt="quads",
                                  kinetic=True)
        m._sync()
        m._ctx.call("nw_set_tuning", 16, 1024, 0)
        m._ctx.set_option("lanes_split", split)
        m._ctx.set_option("fusion_depth", fusion)
        m._ctx.set_option("cuda_graph", graph)
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m.advance(150)
        assert m._ctx.get_option("narrow_neurons") == (4 if split else 0)
        out[(split, fusion)] = (m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count"))
        m.close()
    assert np.array_equal(out[(65535, 1)][0], out[(65535, 7)][0])
    assert np.abs(out[(0, 7)][0] - out[(65535, 7)][0]).max() < 2e-3
    assert np.array_equal(out[(0, 7)][1], out[(65535, 7)][1])


def test_autotune_reports_lanes_split():
    trees = [random_tree(n, seed=500 + n) for n in (2500, 1500, 300, 60)]
    m, _, _, _ = gpu_model(trees, [], precision="f32", tolerance=3e-7, conserve="lump", fmt="quads", kinetic=True)
    m._sync()
    v0 = m.get_data("Segment.voltage")
    tuned = m.autotune(3)
    assert set(tuned) >= {"lanes_per_row", "threads", "fusion_depth", "ms_per_step", "lanes_split", "narrow_neurons"}
    assert m._ctx.get_option("lanes_split") == tuned["lanes_split"]
    assert np.array_equal(m.get_data("Segment.voltage"), v0)       # state restored
    m.close()
