"""The wide path: neurons beyond the batched path's limits (more than 65,535
segments, or more than shared memory holds), whole-model launches per phase."""
import ctypes

import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300 import _lib
from neuwon_gb300.morphology import random_tree
from tests.helpers import gpu_model, run_with_clamps

pytestmark = pytest.mark.gpu


def test_wide_equals_batched_in_f64():
    trees = [random_tree(n, seed=40 + n) for n in (300, 1200, 50)]
    clamps = [(0, 0, 0.3, 1.0, 30.0), (1, 0, 0.4, 0.0, 50.0), (2, 3, 0.1, 2.0, 5.0)]
    out = []
    for path in ("batched", "wide"):
        m, neurons, offs, recs = gpu_model(trees, clamps, precision="f64", path=path, kinetic=True, probes=[0, 400])
        run_with_clamps(m, clamps, offs, 300)
        out.append((m.get_data("Segment.voltage"), m.get_data("na8.state"), m.get_data("Neuron.spike_count"),
                    np.array([r.get_data() for r in recs])))
        m.close()
    for a, b in zip(*out):
        assert np.abs(np.asarray(a, float) - np.asarray(b, float)).max() < 1e-9


def test_wide_runs_a_neuron_beyond_the_batched_limit():
    """A 70,000-segment tree: the batched path refuses it (16-bit columns), the
    wide path runs it; FP32 stays within 0.1 mV of FP64 and spikes agree."""
    tree = random_tree(70000, seed=9)
    res = {}
    for precision in ("f64", "f32"):
        m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision=precision, path="wide",
                         propagator_tolerance=1e-8, propagator_conserve=True,
                         mechanisms=[nw.HH.configure(ena=50.0, ek=-77.0, el=-54.3)])
        nr = m.add_tree(tree)
        m.insert_everywhere("hh")
        nr.root.inject_current(5.0, 1e6)
        m._sync()
        if precision == "f32":
            rc = m._ctx.lib.nw_advance(m._ctx.handle, 1, _lib.PATH_BATCHED)
            assert rc == -6                                   # NW_ERR_LIMIT
        m.advance(400)
        res[precision] = (m.get_data("Segment.voltage"), int(m.get_data("Neuron.spike_count")[0]))
        m.close()
    assert res["f64"][1] == res["f32"][1] and res["f64"][1] > 0
    assert np.abs(res["f64"][0] - res["f32"][0]).max() < 0.1


def test_wide_graph_chunks_are_bit_identical_to_direct_launches():
    trees = [random_tree(700, seed=s) for s in (1, 2)]
    clamps = [(0, 0, 0.3, 0.0, 100.0), (1, 0, 0.35, 0.0, 100.0)]
    out = []
    for graph in (0, 1):
        m, _, offs, _ = gpu_model(trees, clamps, precision="f32", path="wide")
        for (ti, s, nA, start, dur) in clamps:
            nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
        m._sync()
        m._ctx.set_option("cuda_graph", graph)
        m.advance(70)          # two 32-step graphs and a 6-step one
        m.advance(70)          # replays
        out.append(m.get_data("Segment.voltage"))
        if graph:
            assert m._ctx.get_option("graph_captures") == 2
        m.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_wide_quads_equal_wide_rows(precision):
    """The wide path's quad format (global 32-bit window bases) holds the row
    format's entries; a 2-segment neuron's windows reach into its neighbour."""
    trees = [random_tree(n, seed=30 + n) for n in (1500, 2, 400)]
    out = []
    for fmt in ("rows", "quads"):
        m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision=precision, path="wide", propagator_tolerance=1e-8,
                         propagator_conserve=True, propagator_format=fmt,
                         mechanisms=[nw.HH.configure(ena=50.0, ek=-77.0, el=-54.3)])
        for t in trees:
            nr = m.add_tree(t)
            nr.root.inject_current(0.4, 1e6)
        m.insert_everywhere("hh")
        m.advance(200)
        out.append((m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count")))
        m.close()
    tol = 1e-9 if precision == "f64" else 2e-3
    assert np.abs(out[0][0] - out[1][0]).max() < tol
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_wide_fused_half_steps_equal_phase_launches(precision):
    """One launch per half step (propagator rows, then each segment's mechanisms
    and next x in the same launch) against one launch per phase: HH + na8 and HH +
    calcium models agree to rounding (the calcium rows are summed in another
    order), spikes and probes included."""
    from tests.helpers import calcium_case
    trees = [random_tree(n, seed=60 + n) for n in (900, 2500, 40)]
    clamps = [(0, 0, 0.4, 0.0, 1e6), (1, 0, 0.6, 1.0, 40.0), (2, 3, 0.1, 2.0, 5.0)]
    tol = 1e-9 if precision == "f64" else 2e-3
    for case in ("kinetic", "calcium"):
        out = []
        for fusion in (0, 1):
            if case == "kinetic":
                m, _, offs, recs = gpu_model(trees, clamps, precision=precision, path="wide", kinetic=True,
                                             probes=[0, 950])
            else:
                m, _, offs = calcium_case(trees, clamps, precision=precision, path="wide", oracle=False)
                recs = []
            m._sync()
            m._ctx.set_option("wide_fusion", fusion)
            if case == "kinetic":
                run_with_clamps(m, clamps, offs, 250)
            else:
                m.advance(250)
            res = [m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count")]
            res.append(m.get_data("na8.state") if case == "kinetic" else m.get_data("Species.ca"))
            res += [np.asarray(r.get_data()) for r in recs]
            out.append(res)
            m.close()
        assert np.array_equal(out[0][1], out[1][1]) and out[0][1].sum() > 0
        assert np.abs(out[0][0] - out[1][0]).max() < tol                       # voltages (mV)
        a, b = np.asarray(out[0][2], float), np.asarray(out[1][2], float)
        scale = np.abs(a).max() if case == "calcium" else 1.0                  # calcium: relative
        assert np.abs(a - b).max() < tol * scale, (case, np.abs(a - b).max())
        for a, b in zip(out[0][3:], out[1][3:]):                               # probe traces
            assert np.abs(np.asarray(a, float) - np.asarray(b, float)).max() < tol
