"""Two-input kinetic tables on the GPU (lti_sim's Approx2D): the reference
library's NMDA receptor (nmodl_library/kinetic/NMDA.mod, restated as
neuwon_gb300.kinetic.nmda) as point processes whose table runs over the glutamate
concentration (an instance value) and the voltage, against the FP64 oracle."""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.kinetic import NMDA, LTITable2, canonical_terms, nmda
from neuwon_gb300.morphology import random_tree

pytestmark = pytest.mark.gpu

HH_KW = dict(ena=50.0, ek=-77.0, el=-54.3)
SYN_SEGS = [0, 5, 40, 120, 40]          # segment 40 carries two receptors


def _model(tree, precision, path):
    m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision=precision, path=path,
                     mechanisms=[nw.HH.configure(**HH_KW), NMDA])
    nr = m.add_tree(tree)
    m.insert_everywhere("hh")
    for s in SYN_SEGS:
        m.mechanisms["NMDA_Mg"](nw.Segment(m, s))
    nr.root.inject_current(0.05, 1e6)
    return m


def _oracle(tree, glu):
    from oracle.reference_step import HHInstances, KineticInstances, OracleModel, clamp_ticks
    from tests.helpers import concat
    parent, R, C, area, offs = concat([tree])
    n = len(tree)
    i1, i2 = NMDA.inputs
    tbl = LTITable2(nmda(), 0.1, 6.3, i1, i2, NMDA.terms, NMDA.samples_per_axis)
    ki = KineticInstances(np.array(SYN_SEGS), NMDA.gbar, tbl.layout, 0.0, 1.0, nmda().open_states, NMDA.erev, 1.0,
                          NMDA.initial_state(-70.0, 6.3),
                          inputs=[(i.kind, i.num_buckets, i.minimum, i.bucket_frq, i.scale) for i in (i1, i2)],
                          powers=canonical_terms(NMDA.terms), input_values=glu)
    f, c = clamp_ticks(0.0, 1e6, 0.1)
    return OracleModel(parent, R, C, time_step=0.1, celsius=6.3, hh=HHInstances(np.arange(n), area, celsius=6.3, **HH_KW),
                       kinetic=[ki], clamps=[(0, 0.05e-9, f, c)], detectors=[(0, 20.0)])


@pytest.mark.parametrize("path", ["batched", "wide", "plain"])
def test_nmda_point_processes_match_oracle(path):
    """FP64: glutamate 1 mM at the synapses for 20 ms, then washed out; voltages
    within 1e-7 mV of the oracle, receptor states within 1e-9, spikes equal."""
    tree = random_tree(200, seed=8)
    m = _model(tree, "f64", path)
    glu = np.array([1.0, 0.5, 2.0, 1.0, 0.3])
    m.set_data("NMDA_Mg.input", glu)
    assert np.array_equal(m.get_data("NMDA_Mg.input"), glu)
    om = _oracle(tree, glu)
    worst_v = worst_s = 0.0
    for k in range(400):
        if k == 200:
            m.set_data("NMDA_Mg.input", np.zeros(len(SYN_SEGS)))
            om.kinetic[0].input_values = np.zeros(len(SYN_SEGS))
        m.advance(1)
        om.advance()
        if k % 20 == 19:
            worst_v = max(worst_v, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
            worst_s = max(worst_s, np.abs(m.get_data("NMDA_Mg.state") - om.kinetic[0].state).max())
    assert worst_v < 1e-7, worst_v
    assert worst_s < 1e-9, worst_s
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert om.spike_count[0] >= 1
    m.close()


def test_nmda_f32_within_tolerance_of_f64():
    tree = random_tree(300, seed=9)
    out = {}
    for precision in ("f64", "f32"):
        m = _model(tree, precision, "batched")
        m.set_data("NMDA_Mg.input", np.full(len(SYN_SEGS), 1.0))
        m.advance(300)
        out[precision] = (m.get_data("Segment.voltage"), m.get_data("Neuron.spike_count"))
        m.close()
    assert np.abs(out["f64"][0] - out["f32"][0]).max() < 0.1
    assert np.array_equal(out["f64"][1], out["f32"][1]) and out["f64"][1].sum() > 0


def test_two_input_gpu_table_equals_host_table():
    """nw_lti_table_build over the flat bucket pairs (FP64 expm and fit on the GPU)
    equals the host FP64 build on the same grid."""
    from neuwon_gb300.kinetic import scheme_table_gpu2
    m = _model(random_tree(200, seed=1), "f64", "batched")
    m._sync()
    i1, i2 = NMDA.inputs
    gpu = scheme_table_gpu2(m._ctx, nmda(), 0.1, 6.3, i1, i2, NMDA.terms, NMDA.samples_per_axis)
    host = LTITable2(nmda(), 0.1, 6.3, i1, i2, NMDA.terms, NMDA.samples_per_axis)
    assert np.abs(gpu - host.layout).max() < 1e-11
    m.close()
