"""Synapses driven by spike events.

The reference grows synapse geometry (neuwon/rxd/synapses.py) but has no
synaptic kinetics and no event delivery: no mechanism in it has a NET_RECEIVE
block.  This module defines them for the GPU path.  A spike is the AP
detector's output (neuwon/rxd/neuron/neuron.py:72-75); it reaches each
outgoing synapse after that synapse's axonal delay, rounded to whole steps.
An arrival keeps transmitter present for ``pulse`` ms (Destexhe, Mainen &
Sejnowski 1994).  Each synapse has a 2-state AMPA scheme C <-> O and a
3-state NMDA scheme C -> O -> D -> C with the magnesium block of Jahr &
Stevens (1990).  Both schemes are linear with piecewise-constant rates, so
they advance exactly by one precomputed transition matrix per step
(transmitter present or absent), built here in FP64.
"""
import numpy as np
import scipy.linalg


class SynapseKinetics:
    """Rates in 1/ms (alpha in 1/(mM ms)), transmitter t_max (mM) for ``pulse`` ms.

    Defaults: AMPA and NMDA binding/unbinding from Destexhe, Mainen & Sejnowski
    (1998, "Kinetic models of synaptic transmission", table 1); the NMDA
    desensitisation (delta) and recovery (rho) rates are this project's choice."""

    def __init__(self, ampa_alpha=1.1, ampa_beta=0.19, nmda_alpha=0.072, nmda_beta=0.0066,
                 nmda_delta=0.0084, nmda_rho=0.0068, t_max=1.0, pulse=1.0, e_syn=0.0, mg=1.0):
        self.ampa_alpha, self.ampa_beta = float(ampa_alpha), float(ampa_beta)
        self.nmda_alpha, self.nmda_beta = float(nmda_alpha), float(nmda_beta)
        self.nmda_delta, self.nmda_rho = float(nmda_delta), float(nmda_rho)
        self.t_max, self.pulse = float(t_max), float(pulse)
        self.e_syn, self.mg = float(e_syn), float(mg)

    def generators(self, transmitter):
        """Rate matrices Q (d state / dt = Q state) of the AMPA and NMDA schemes."""
        T = float(transmitter)
        a, b = self.ampa_alpha, self.ampa_beta
        qa = np.array([[-a * T, b], [a * T, -b]])
        a, b, d, r = self.nmda_alpha, self.nmda_beta, self.nmda_delta, self.nmda_rho
        qn = np.array([[-a * T, b, r], [a * T, -b - d, 0.0], [0.0, d, -r]])
        return qa, qn

    def matrices(self, time_step):
        """(ampa_on, ampa_off, nmda_on, nmda_off): expm(Q * dt), FP64, row-major."""
        on = [scipy.linalg.expm(q * time_step) for q in self.generators(self.t_max)]
        off = [scipy.linalg.expm(q * time_step) for q in self.generators(0.0)]
        return on[0], off[0], on[1], off[1]

    def pulse_steps(self, time_step):
        return max(1, int(round(self.pulse / time_step)))


def delay_steps(delay_ms, time_step):
    """Axonal delays in whole steps (at least one)."""
    d = np.rint(np.asarray(delay_ms, dtype=np.float64) / time_step).astype(np.int64)
    return np.maximum(d, 1)


def random_network(neuron_sizes, num_synapses, seed, *, time_step=0.1, w_mu=-1.0, w_sigma=0.5,
                   delay_lo=1.0, delay_hi=20.0):
    """Seeded random connectivity: pre neuron uniform, post neuron uniform among
    the others, post segment uniform in the post neuron (neuron-relative index),
    weights lognormal (mu, sigma of the log, in nS), delays uniform (ms)."""
    rng = np.random.default_rng(seed)
    sizes = np.asarray(neuron_sizes, dtype=np.int64)
    N = len(sizes)
    pre = rng.integers(0, N, num_synapses)
    post = rng.integers(0, N - 1, num_synapses)
    post = post + (post >= pre)
    local = (rng.random(num_synapses) * sizes[post]).astype(np.int64)
    w = np.exp(rng.normal(w_mu, w_sigma, num_synapses))
    delay = rng.uniform(delay_lo, delay_hi, num_synapses)
    return dict(pre=pre, post_neuron=post, post_local=local, weight_nS=w,
                delay_steps=delay_steps(delay, time_step))
