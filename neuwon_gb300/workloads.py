"""Seeded synthetic workloads with the shapes of the benchmark configurations.

single_neuron: one 2,000-segment random binary tree (seed 0), HH everywhere,
    0.2 nA soma clamp from 5 to 80 ms, dt 0.1 ms, 100 ms.
batched: 1,024 trees (seeds 1..1024) with log-uniform sizes in [500, 20000]
    (sizes drawn with seed 0), HH and the 8-state Markov sodium scheme (na8,
    gbar 0.012 S/cm2, ENa 50 mV, voltage table on a 0.1 mV grid over
    -100..60 mV) everywhere, a soma current per neuron drawn uniformly in
    [0.05, 0.5] nA (seed 0), dt 0.1 ms.

HH parameters for both: gNa 0.12, gK 0.036, gL 0.0003 S/cm2, ENa 50, EK -77,
EL -54.3 mV, 6.3 degC; Ra 100 ohm-cm, Cm 1 uF/cm2.
"""
import multiprocessing

import numpy as np

from .kinetic import Kinetic
from .mechanisms import HH
from .morphology import neuron_sizes, random_tree

HH_PARAMS = dict(gnabar=0.12, gkbar=0.036, glbar=0.0003, ena=50.0, ek=-77.0, el=-54.3)
CELSIUS = 6.3
TIME_STEP = 0.1


def _tree(args):
    n, seed = args
    return random_tree(int(n), seed=int(seed))


def batched_trees(num_neurons=1024, seed=0, first=0, count=None, processes=None, lo=500, hi=20000):
    """Trees [first, first+count) of the batched workload (built in parallel).

    Neuron k has sizes[k] segments (sizes drawn with ``seed``) and tree seed
    k + 1 + seed * num_neurons, so every rank of a weak-scaling run gets its
    own neurons."""
    sizes = neuron_sizes(num_neurons, seed=seed, lo=lo, hi=hi)
    last = num_neurons if count is None else min(num_neurons, first + count)
    jobs = [(sizes[k], k + 1 + seed * num_neurons) for k in range(first, last)]
    if processes == 1 or len(jobs) < 8:
        return [_tree(j) for j in jobs]
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(processes) as pool:
        return pool.map(_tree, jobs, chunksize=4)


def batched_currents(num_neurons=1024, seed=0):
    """Soma current per neuron, nA."""
    return np.random.default_rng(seed).uniform(0.05, 0.5, num_neurons)


def build_model(trees, currents_nA, *, precision="f32", tolerance=1e-7, conserve=True,
                duration_ms=1e9, path="batched", device=0, kinetic=True, fmt="rows", lump=False):
    """RxD_Model with HH (and na8) on every segment and a constant soma clamp per neuron."""
    from .model import RxD_Model
    mechs = [HH.configure(**HH_PARAMS)] + ([Kinetic] if kinetic else [])
    m = RxD_Model(time_step=TIME_STEP, temperature=CELSIUS, precision=precision, device=device,
                  propagator_tolerance=tolerance, propagator_conserve=conserve, path=path,
                  propagator_format=fmt, propagator_lump=lump, mechanisms=mechs)
    neurons = [m.add_tree(t) for t in trees]
    m.insert_everywhere("hh")
    if kinetic:
        m.insert_everywhere("na8")
    for nrn, amp in zip(neurons, currents_nA):
        nrn.root.inject_current(float(amp), duration_ms)
    return m, neurons
