"""Spike-event routing and synapse kinetics on the host (oracle side).

The reference has no event delivery; the oracle's priority queue is the
definition the GPU's spike-ring routing must reproduce exactly."""
import numpy as np
import pytest

from neuwon_gb300.synapses import SynapseKinetics, delay_steps, random_network
from oracle.reference_step import EventQueue, synapse_matrices


def _brute_force(pre, delay, spikes):
    out = set()
    for (j, t) in spikes:
        for k in np.flatnonzero(pre == j):
            out.add((t + int(delay[k]), int(k)))
    return out


def test_event_queue_matches_enumeration():
    rng = np.random.default_rng(0)
    N, M = 50, 3000
    pre = rng.integers(0, N, M)
    delay = rng.integers(1, 40, M)
    q = EventQueue(pre, delay)
    spikes = sorted({(int(rng.integers(0, N)), int(t)) for t in rng.integers(0, 300, 400)}, key=lambda x: x[1])
    got = set()
    by_step = {}
    for (j, t) in spikes:
        by_step.setdefault(t, []).append(j)
    for step in range(400):
        for k in q.pop(step):
            got.add((step, k))
        q.push(step, by_step.get(step, []))
    assert got == _brute_force(pre, delay, spikes)


def test_kinetics_matrices_agree_with_oracle_and_conserve():
    kin = SynapseKinetics()
    for dt in (0.025, 0.1):
        ao, af, no, nf = kin.matrices(dt)
        ro = synapse_matrices(dt, kin.ampa_alpha, kin.ampa_beta, t_max=kin.t_max)
        rn = synapse_matrices(dt, kin.nmda_alpha, kin.nmda_beta, kin.nmda_delta, kin.nmda_rho, t_max=kin.t_max)
        for a, b in zip((ao, af, no, nf), ro + rn):
            assert np.abs(a - b).max() < 1e-15
        for M in (ao, af, no, nf):
            assert np.abs(M.sum(axis=0) - 1).max() < 1e-14       # probability conserved
            assert M.min() >= 0
    # Transmitter absent: the AMPA open state decays with rate beta.
    ao, af, _, _ = kin.matrices(0.1)
    assert af[1, 1] == pytest.approx(np.exp(-kin.ampa_beta * 0.1), rel=1e-14)


def test_delays_and_network_are_seeded():
    assert list(delay_steps([0.01, 0.1, 0.149, 0.151, 20.0], 0.1)) == [1, 1, 1, 2, 200]
    a = random_network([200, 300, 500], 1000, 3)
    b = random_network([200, 300, 500], 1000, 3)
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert np.all(a["pre"] != a["post_neuron"])
    sizes = np.array([200, 300, 500])
    assert np.all(a["post_local"] < sizes[a["post_neuron"]])
    assert np.all((a["delay_steps"] >= 10) & (a["delay_steps"] <= 200))


def test_oracle_network_delivers_at_delay():
    """A spike of the presynaptic neuron opens its synapses exactly delay steps later."""
    from tests.helpers import network_case
    m, om, net, offs = network_case([120, 80], 40, seed=1, currents=[0.6, 0.0], delay_lo=1.0, delay_hi=2.0)
    spikes = []
    for step in range(250):
        om.advance()
        spikes += [(int(j), step) for j in np.flatnonzero(om.AP_detected)]
    assert any(j == 0 for j, _ in spikes)
    expect = _brute_force(net["pre"], net["delay_steps"], [s for s in spikes if s[1] + 1 < 250])
    got = {(t, k) for (t, k) in om.synapses.delivered}
    assert got == {(t, k) for (t, k) in expect if t < 250}
    k = om.synapses.delivered[0][1]
    assert om.synapses.events[k] >= 1
