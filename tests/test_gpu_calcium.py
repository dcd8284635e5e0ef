"""Intracellular calcium on the GPU (diffusion, pump, sodium-fraction influx)
against the oracle, and the FP32 precision study of the 1 M-segment
configuration at reduced size (FP32 + compensated sums vs FP64, both on the
GPU, tolerances 1e-6 and 1e-9)."""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.morphology import random_tree
from tests.helpers import calcium_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", ["batched", "wide"])
def test_f64_calcium_matches_oracle(path):
    trees = [random_tree(300, seed=12), random_tree(120, seed=13)]
    clamps = [(0, 0, 0.5, 0.0, 1e6), (1, 0, 0.3, 0.0, 1e6)]
    m, om, offs = calcium_case(trees, clamps, path=path)
    worst_v = worst_c = 0.0
    for k in range(600):
        m.advance(1)
        om.advance()
        if k % 50 == 49:
            worst_v = max(worst_v, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
            c = m.get_data("Species.ca")
            worst_c = max(worst_c, (np.abs(c - om.calcium.c) / om.calcium.c).max())
    assert worst_v < 1e-7, worst_v
    assert worst_c < 1e-9, worst_c
    assert np.abs(m.get_data("CaPump.state") - om.calcium.state).max() < 1e-9
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert om.spike_count.sum() > 0 and om.calcium.c.max() > 10 * 5e-5    # spikes raised calcium
    m.close()


@pytest.mark.parametrize("tol", [1e-6, 1e-9])
def test_f32_precision_study_reduced(tol):
    """20,000-segment tree, HH + calcium, dt 0.025 ms for 50 ms on the wide path:
    FP32 vs FP64 max |dV| <= 0.1 mV and max relative d[Ca] <= 1e-3."""
    tree = random_tree(20000, seed=100)
    clamps = [(0, 0, 1.0, 0.0, 1e6)]
    res = {}
    for precision in ("f64", "f32"):
        m, _, _ = calcium_case([tree], clamps, precision=precision, path="wide", tolerance=tol, conserve=True,
                               oracle=False)
        m.advance(2000)
        res[precision] = (m.get_data("Segment.voltage"), m.get_data("Species.ca"),
                          int(m.get_data("Neuron.spike_count")[0]))
        m.close()
    dv = np.abs(res["f64"][0] - res["f32"][0]).max()
    dca = (np.abs(res["f64"][1] - res["f32"][1]) / res["f64"][1]).max()
    print(f"tolerance {tol}: max |dV| {dv:.3g} mV, max rel d[Ca] {dca:.3g}, spikes {res['f64'][2]}")
    assert res["f64"][2] == res["f32"][2] and res["f64"][2] > 0
    assert dv < 0.1, dv
    assert dca < 1e-3, dca
