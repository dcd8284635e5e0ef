"""Spike events and synapses on the GPU against the oracle's priority queue.

Routing is integer work and must be bit-exact: given the spike list the GPU
produced, the oracle queue delivers the same events to the same synapses at
the same steps (per-synapse event counts and last delivery step).  Dynamics
(HH + AMPA/NMDA) in FP64 match the oracle's voltages."""
import numpy as np
import pytest

from oracle.reference_step import EventQueue
from tests.helpers import network_case

pytestmark = pytest.mark.gpu


def _replay_queue(net, spikes, steps):
    """Per-synapse (events, last_event) from the oracle queue fed with a spike list."""
    q = EventQueue(net["pre"], net["delay_steps"])
    by_step = {}
    for j, t in spikes:
        by_step.setdefault(t, []).append(j)
    M = len(net["pre"])
    events = np.zeros(M, np.int64)
    last = np.full(M, -1, np.int64)
    for step in range(steps):
        for k in q.pop(step):
            events[k] += 1
            last[k] = step
        q.push(step, by_step.get(step, []))
    return events, last


def _run_recording(m, steps):
    spikes = []
    for step in range(steps):
        m.advance(1)
        ap = m.get_data("Neuron.AP_detected")
        spikes += [(int(j), step) for j in np.flatnonzero(ap)]
    return spikes


@pytest.mark.parametrize("path,fmt", [("batched", "rows"), ("batched", "quads"), ("wide", "rows")])
def test_f64_network_matches_oracle(path, fmt):
    m, om, net, offs = network_case([150, 90, 200, 60], 300, seed=2, delay_lo=1.0, delay_hi=4.0, path=path,
                                    fmt=fmt)
    steps = 400
    spikes = []
    worst = 0.0
    for step in range(steps):
        m.advance(1)
        om.advance()
        spikes += [(int(j), step) for j in np.flatnonzero(m.get_data("Neuron.AP_detected"))]
        if step % 20 == 19:
            worst = max(worst, np.abs(m.get_data("Segment.voltage") - om.voltage).max())
    assert worst < 1e-6, worst
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert len(spikes) > 4
    ev, last = _replay_queue(net, spikes, steps)
    np.testing.assert_array_equal(m.get_data("Synapse.events"), om.synapses.events)
    np.testing.assert_array_equal(m.get_data("Synapse.events"), ev)
    np.testing.assert_array_equal(m.get_data("Synapse.last_event"), last)
    assert ev.sum() > 0
    for name, ref in (("Synapse.ampa_open", om.synapses.ampa[:, 1]), ("Synapse.nmda_open", om.synapses.nmda[:, 1]),
                      ("Synapse.nmda_desensitized", om.synapses.nmda[:, 2])):
        assert np.abs(m.get_data(name) - ref).max() < 1e-9
    m.close()


def test_fusion_is_capped_by_the_shortest_delay():
    """Fusing more steps than the shortest delay would read spikes not yet written;
    the library caps it, so any requested depth gives the single-step result."""
    res = []
    for fusion in (1, 50):
        m, _, net, _ = network_case([300, 200, 250, 100, 400], 2000, seed=3, precision="f32", oracle=False,
                                    delay_lo=1.0, delay_hi=3.0)
        m._sync()
        m._ctx.set_option("fusion_depth", fusion)
        m.advance(300)
        res.append((m.get_data("Segment.voltage"), m.get_data("Synapse.events"), m.get_data("Neuron.spike_count")))
        m.close()
    for a, b in zip(*res):
        assert np.array_equal(a, b)
    assert res[0][1].sum() > 0


def test_f32_routing_is_bit_exact_given_the_spike_list():
    """A larger FP32 network (64 neurons, 20,000 synapses, delays 1-20 ms, 300 ms):
    every synapse's delivery count and last delivery step equal the oracle queue's
    for the spikes the GPU produced."""
    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(200), np.log(1500), 64)).astype(int)
    m, _, net, _ = network_case(sizes, 20000, seed=4, precision="f32", oracle=False, delay_lo=1.0, delay_hi=20.0,
                                tolerance=1e-8)
    steps = 3000
    spikes = _run_recording(m, steps)
    ev, last = _replay_queue(net, spikes, steps)
    assert len(spikes) > 50 and ev.sum() > 1000
    np.testing.assert_array_equal(m.get_data("Synapse.events"), ev)
    np.testing.assert_array_equal(m.get_data("Synapse.last_event"), last)
    m.close()


def test_autotune_restores_synapse_state():
    m, _, net, _ = network_case([300, 200, 250], 800, seed=5, precision="f32", oracle=False, delay_lo=1.0,
                                delay_hi=3.0)
    m.advance(200)
    names = ("Synapse.events", "Synapse.last_event", "Synapse.pulse_end", "Synapse.ampa_open", "Synapse.nmda_open")
    before = [m.get_data(n) for n in names]
    ref, _, _, _ = network_case([300, 200, 250], 800, seed=5, precision="f32", oracle=False, delay_lo=1.0,
                                delay_hi=3.0)
    ref.advance(200)
    m.autotune(trial_steps=4)
    for n, b in zip(names, before):
        assert np.array_equal(m.get_data(n), b)
    m.advance(200)
    ref.advance(200)
    np.testing.assert_array_equal(m.get_data("Synapse.events"), ref.get_data("Synapse.events"))
    m.close(); ref.close()


def test_partitioned_network_equals_one_model():
    """A network split into two models (emulated ranks on one GPU, each advancing an
    epoch of the shortest delay, then summing spike rings on the host) gives the
    single model's voltages, spikes and deliveries bit for bit."""
    import neuwon_gb300 as nw
    from neuwon_gb300.morphology import random_tree
    from neuwon_gb300.replicas import SpikeExchange
    from neuwon_gb300.synapses import random_network
    sizes = [300, 250, 400, 150, 350, 200]
    trees = [random_tree(n, seed=60 + k) for k, n in enumerate(sizes)]
    amps = [0.5, 0.4, 0.6, 0.3, 0.45, 0.55]
    net = random_network(sizes, 1200, 9, delay_lo=1.0, delay_hi=4.0)
    E = int(net["delay_steps"].min())

    def build(neuron_ids, syn_ids, partition=None):
        m = nw.RxD_Model(time_step=0.1, temperature=6.3, precision="f64", mechanisms=[nw.HH.configure(ena=50.0, ek=-77.0)])
        offs, o = {}, 0
        for j in neuron_ids:
            nr = m.add_tree(trees[j])
            offs[j] = o
            o += sizes[j]
            nr.root.inject_current(amps[j], 1e9)
        m.insert_everywhere("hh")
        if partition is not None:
            m.set_spike_partition(*partition)
        post = np.array([offs[net["post_neuron"][k]] + net["post_local"][k] for k in syn_ids])
        m.add_synapses(net["pre"][syn_ids], post, net["weight_nS"][syn_ids], net["weight_nS"][syn_ids],
                       net["delay_steps"][syn_ids] * 0.1)
        m._sync()
        return m

    all_syn = np.arange(1200)
    full = build(range(6), all_syn)
    R = 32 * full._ctx.get_option("synapse_ring_words")
    a_syn = all_syn[net["post_neuron"] < 3]
    b_syn = all_syn[net["post_neuron"] >= 3]
    A = build(range(3), a_syn, (6, 0, R))
    B = build(range(3, 6), b_syn, (6, 3, R))
    ranks = [SpikeExchange(A), SpikeExchange(B)]
    total = lambda _: sum(r.own() for r in ranks)
    for r in ranks:
        r.reduce = total
    for epoch in range(40):
        A.advance(E)
        B.advance(E)
        summed = total(None)
        for r in ranks:
            r.install(summed)
        full.advance(E)
    v_full = full.get_data("Segment.voltage")
    v_parts = np.concatenate([A.get_data("Segment.voltage"), B.get_data("Segment.voltage")])
    assert np.array_equal(v_full, v_parts)
    ev = full.get_data("Synapse.events")
    assert np.array_equal(ev[a_syn], A.get_data("Synapse.events"))
    assert np.array_equal(ev[b_syn], B.get_data("Synapse.events"))
    assert ev.sum() > 0 and (ev[a_syn] > 0).any() and (ev[b_syn] > 0).any()
    np.testing.assert_array_equal(full.get_data("Neuron.spike_count"),
                                  np.concatenate([A.get_data("Neuron.spike_count"), B.get_data("Neuron.spike_count")]))
    for m in (full, A, B):
        m.close()
