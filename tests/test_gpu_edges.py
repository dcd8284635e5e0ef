"""Edge cases of the step: zero-step calls, one-segment neurons, mechanisms on a
subset of segments (non-identity instance layouts, several instances per
segment), many clamps on one neuron, limits that must be refused."""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.morphology import Tree, geometry, random_tree
from oracle.reference_step import HHInstances, OracleModel, clamp_ticks
from tests.helpers import concat, kinetic_oracle

pytestmark = pytest.mark.gpu

HH_KW = dict(ena=50.0, ek=-77.0, el=-54.3)


def _subset_case(path, precision="f64"):
    trees = [random_tree(120, seed=71), Tree([-1], [[0, 0, 0]], [15.0]), random_tree(60, seed=72)]
    parent, R, C, area, offs = concat(trees)
    n = len(parent)
    rng = np.random.default_rng(3)
    hh_seg = np.sort(np.concatenate([rng.choice(n, n // 2, replace=False), [offs[1]], rng.choice(n, 10)]))
    kin_seg = np.sort(rng.choice(n, n // 3, replace=False))
    clamps = [(offs[0] + 5, 0.3, 0.0, 8.0), (offs[0] + 5, 0.2, 2.0, 3.0), (offs[1], 0.05, 0.0, 20.0),
              (offs[2] + 40, 0.4, 1.0, 6.0)] + [(offs[0] + k, 0.01, 0.5 * k, 1.0) for k in range(10)]
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision=precision, path=path,
                     mechanisms=[nw.HH.configure(**HH_KW), nw.Kinetic])
    for t in trees:
        m.add_tree(t)
    for s in hh_seg:
        nw.Segment(m, s).insert("hh")
    for s in kin_seg:
        nw.Segment(m, s).insert("na8")
    cl = []
    for (s, nA, start, dur) in clamps:
        f, c = clamp_ticks(start, dur, 0.1)
        cl.append((s, nA * 1e-9, f, c))
    hh = HHInstances(hh_seg, area[hh_seg], celsius=6.3, **HH_KW)
    om = OracleModel(parent, R, C, time_step=0.1, celsius=6.3, hh=hh, clamps=cl,
                     detectors=[(o, 20.0) for o in offs], kinetic=kinetic_oracle(kin_seg, area, 0.1, 6.3))
    return m, om, clamps


@pytest.mark.parametrize("path", ["batched", "wide", "plain"])
def test_subsets_duplicates_one_segment_neuron_and_many_clamps(path):
    m, om, clamps = _subset_case(path)
    worst = 0.0
    for k in range(150):
        for (s, nA, start, dur) in clamps:
            if m.clock.is_now(start):
                nw.Segment(m, s).inject_current(nA, dur)
        m.advance()
        om.advance()
        if k % 10 == 9:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
    assert worst < 1e-7, worst
    assert np.abs(m.get_data("na8.state") - om.kinetic[0].state).max() < 1e-9
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    m.close()


def test_zero_steps_is_a_no_op():
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision="f64", mechanisms=[nw.HH])
    nr = m.add_tree(random_tree(50, seed=1))
    m.insert_everywhere("hh")
    nr.root.inject_current(0.3, 10.0)
    m.advance(3)
    v = m.get_data("Segment.voltage")
    clock = m._ctx.clock()
    m.advance(0)
    assert m._ctx.clock() == clock
    assert np.array_equal(v, m.get_data("Segment.voltage"))
    m.close()


def test_limits_are_refused():
    from neuwon_gb300 import _lib
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision="f32", mechanisms=[nw.HH])
    m.add_tree(random_tree(40, seed=2))
    m.insert_everywhere("hh")
    for k in range(17):                                  # 17 clamps on one neuron
        nw.Segment(m, k).inject_current(0.01, 1.0)
    with pytest.raises(_lib.NeuwonError):
        m.advance(1)
    m.close()
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision="f32", mechanisms=[nw.HH])
    m.add_tree(random_tree(40, seed=2))
    m._sync()
    rc = m._ctx.lib.nw_advance(m._ctx.handle, -1, _lib.PATH_BATCHED)
    assert rc == -1                                      # NW_ERR_ARG
    rc = m._ctx.lib.nw_advance(m._ctx.handle, 1, 7)
    assert rc == -1
    m.close()


def test_largest_batched_neuron_equals_wide():
    """56,000 segments: near the largest FP32 neuron whose x fits in one CTA's shared
    memory (227 KB); the batched path matches the wide path to rounding."""
    tree = random_tree(56000, seed=5)
    out = []
    for path in ("batched", "wide"):
        m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision="f32", path=path, propagator_tolerance=1e-6,
                         propagator_conserve=True, mechanisms=[nw.HH.configure(**HH_KW)])
        nr = m.add_tree(tree)
        m.insert_everywhere("hh")
        nr.root.inject_current(5.0, 1e6)
        m.advance(100)
        out.append(m.get_data("Segment.voltage"))
        m.close()
    assert np.abs(out[0] - out[1]).max() < 2e-3
