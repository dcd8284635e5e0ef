"""Launch machinery of the batched path: CUDA-graph replay, step-fusion depth and
the autotuner.  None of them may change a result: graph replay and fusion depth
are bit-identical to direct single launches; the autotuner restores the state it
stepped through and only picks among launch shapes whose results agree."""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.morphology import random_tree
from tests.helpers import gpu_model, run_with_clamps

pytestmark = pytest.mark.gpu


def _case(precision="f32", probes=(0, 5, 400)):
    trees = [random_tree(n, seed=s) for s, n in ((3, 400), (4, 150), (5, 900))]
    clamps = [(0, 0, 0.3, 0.0, 30.0), (1, 0, 0.25, 2.0, 10.0), (2, 0, 0.4, 1.0, 40.0)]
    m, neurons, offs, recs = gpu_model(trees, clamps, precision=precision, probes=list(probes), kinetic=True)
    for (ti, s, nA, start, dur) in clamps:
        nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
    m._sync()
    return m, recs


def _state(m):
    return (m.get_data("Segment.voltage"), m.get_data("hh.m"), m.get_data("na8.state"),
            m.get_data("Neuron.spike_count"))


@pytest.mark.parametrize("fusion", [1, 7, 25, 0])
def test_graph_replay_and_fusion_are_bit_identical(fusion):
    ref, ref_recs = _case()
    ref._ctx.set_option("cuda_graph", 0)
    ref._ctx.set_option("fusion_depth", 1)
    for _ in range(3):
        ref.advance(40)
    m, recs = _case()
    m._ctx.set_option("cuda_graph", 1)
    m._ctx.set_option("fusion_depth", fusion)
    for _ in range(3):
        m.advance(40)
    assert m._ctx.get_option("graph_captures") == 1
    assert m._ctx.get_option("graph_replays") == 3
    for a, b in zip(_state(ref), _state(m)):
        assert np.array_equal(a, b)
    for ra, rb in zip(ref_recs, recs):
        assert np.array_equal(np.asarray(ra.get_data()), np.asarray(rb.get_data()))
    assert m._ctx.clock() == ref._ctx.clock()
    ref.close(); m.close()


def _quad_case(precision):
    trees = [random_tree(n, seed=s) for s, n in ((3, 400), (4, 150), (5, 900))]
    clamps = [(0, 0, 0.3, 0.0, 30.0), (1, 0, 0.25, 2.0, 10.0), (2, 0, 0.4, 1.0, 40.0)]
    m, neurons, offs, recs = gpu_model(trees, clamps, precision=precision, kinetic=True, fmt="quads")
    for (ti, s, nA, start, dur) in clamps:
        nw.Segment(m, offs[ti] + s).inject_current(nA, dur)
    m._sync()
    m._ctx.set_option("fusion_depth", 1)
    return m


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_conductance_cache_carries_over_calls_until_the_model_changes(precision):
    """One-step calls start from the conductances the previous call's fused pass
    cached; any change made between calls (gates, densities, kinetic states,
    another path's steps) makes the next launch gather them again.  Bit-identical
    to a model whose cache is dropped after every call."""
    from neuwon_gb300 import _lib
    runs = []
    for drop in (False, True):
        m = _quad_case(precision)
        used = []

        def steps(k):
            for _ in range(k):
                m.advance(1)
                used.append(m._ctx.get_option("conductance_cache_valid"))
                if drop:
                    m._ctx.set_option("cuda_graph", 1)      # every option call drops the cache
        steps(6)
        gm = m._ctx.get_data("hh.m", m._instance_count("hh"))
        gm[::3] *= 0.7
        m._ctx.set_data("hh.m", gm)
        steps(4)
        k = m._instance_count("hh")
        m.set_hh_densities(np.full(k, 0.15), 0.036, np.full(k, 0.0004))
        steps(4)
        st = m.get_data("na8.state")
        m.set_data("na8.state", np.roll(st, 1, axis=0))
        steps(4)
        m._ctx.advance(2, _lib.PATH_PLAIN)
        m.input_hook.ticks += 4
        m.advance_hook._tick(2)
        steps(4)
        if not drop:
            assert all(u == 1 for u in used)             # the cache was in use after every call
        runs.append(_state(m))
        m.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_claimed_rows_give_the_static_schedule_bits(precision):
    """Quad rows taken by the warps from a shared counter: every row is summed by the
    same lanes in the same order as under the static schedule."""
    runs = []
    for claimed in (0, 1):
        m = _quad_case(precision)
        m._ctx.set_option("fusion_depth", 7)
        m._ctx.set_option("rows_claimed", claimed)
        m._ctx.call("nw_set_tuning", 8, 256, 0)     # many rows per warp
        m.advance(30)
        m._ctx.call("nw_set_tuning", 16, 1024, 0)
        m.advance(20)
        assert m._ctx.get_option("rows_claimed") == claimed
        runs.append(_state(m))
        m.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_graph_cache_follows_launch_shape():
    m, _ = _case(probes=())
    m._ctx.set_option("fusion_depth", 10)
    m.advance(20)
    m.advance(20)
    assert m._ctx.get_option("graph_captures") == 1
    m._ctx.call("nw_set_tuning", 8, 512, 0)        # a new launch shape: a new graph
    m.advance(20)
    assert m._ctx.get_option("graph_captures") == 2
    m.advance(5)                                     # a new step count: a new graph
    assert m._ctx.get_option("graph_captures") == 3
    m._ctx.call("nw_set_tuning", 0, 1024, 0)
    m._ctx.set_option("fusion_depth", 10)
    m.advance(20)                                    # the first shape again: replayed
    assert m._ctx.get_option("graph_captures") == 3
    assert m._ctx.get_option("graphs_cached") == 3
    m._ctx.set_option("clear_graphs", 1)
    assert m._ctx.get_option("graphs_cached") == 0
    m.close()


def test_graph_sees_host_side_changes_between_replays():
    """Clamp amplitudes and the clock live in device memory: a replayed graph uses
    the current ones."""
    a, _ = _case("f64")
    b, _ = _case("f64")
    b._ctx.set_option("cuda_graph", 0)
    for mm in (a, b):
        mm.advance(30)
        nw.Segment(mm, 0).inject_current(0.6, 5.0)       # new clamp list between replays
        mm.advance(30)
        mm.advance(30)
    for x, y in zip(_state(a), _state(b)):
        assert np.array_equal(x, y)
    a.close(); b.close()


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_autotune_restores_state_and_keeps_results(precision):
    m, recs = _case(precision)
    m.advance(20)
    before = _state(m)
    clock = m._ctx.clock()
    best = m.autotune(trial_steps=4)
    assert best["lanes_per_row"] in (0, 4, 8, 16, 32)
    assert best["threads"] in (512, 768, 1024)
    assert best["fusion_depth"] in (1, 2, 5, 10, 20, 25, 50, 100, 200, 500)
    assert best["ms_per_step"] > 0
    for x, y in zip(before, _state(m)):
        assert np.array_equal(x, y)
    assert m._ctx.clock() == clock
    assert len(recs[0].get_data()) == 21
    # The chosen shape gives the same trajectory as the default one.
    ref, _ = _case(precision)
    ref.advance(20)
    m.advance(60)
    ref.advance(60)
    tol = 1e-9 if precision == "f64" else 2e-3
    assert np.abs(m.get_data("Segment.voltage") - ref.get_data("Segment.voltage")).max() < tol
    assert np.array_equal(m.get_data("Neuron.spike_count"), ref.get_data("Neuron.spike_count"))
    m.close(); ref.close()
