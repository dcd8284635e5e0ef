"""FP64 numpy restatement of the reference's staggered time step (test oracle).

Each function names the reference lines it follows (paths relative to the
reference project).  Units follow the reference: voltages mV, currents A,
conductances S, capacitances F, time ms.
"""
import math
import numpy as np
import scipy.linalg
import scipy.sparse
import scipy.sparse.linalg

EPSILON = float(np.finfo(np.float64).eps)   # neuwon/database/dtypes.py:4


def coefficient_coo(parent, R, C, time_step_ms):
    """COO of dV/dt coefficients; neuwon/rxd/neuron/electric.py:85-109.

    Four entries per (child, parent) edge, in the reference's append order.
    Returns (dst, src, coef) so that ``matrix[dst, src] = coef`` (duplicates sum).
    """
    dt = time_step_ms * 1e-3
    src, dst, coef = [], [], []
    for child, p in enumerate(parent):
        if p < 0:
            continue
        r = R[child]; c_parent = C[p]; c_child = C[child]
        src.append(child); dst.append(p);     coef.append(+dt / (r * c_parent))
        src.append(child); dst.append(child); coef.append(-dt / (r * c_child))
        src.append(p);     dst.append(child); coef.append(+dt / (r * c_child))
        src.append(p);     dst.append(p);     coef.append(-dt / (r * c_parent))
    return (np.asarray(dst, dtype=np.int64), np.asarray(src, dtype=np.int64),
            np.asarray(coef, dtype=np.float64))


def propagator(parent, R, C, time_step_ms, prune=EPSILON, dense_above=400):
    """expm of the coefficient matrix, pruned below ``prune``; electric.py:78-117.

    The reference calls ``scipy.sparse.linalg.expm`` on a CSC matrix; above
    ``dense_above`` segments the same exponential is taken with the dense
    ``scipy.linalg.expm`` (same mathematics, far faster).  Independent trees
    (separate neurons) are exponentiated block by block, which is exact for a
    block-diagonal matrix.  Returns a scipy CSR matrix.
    """
    parent = np.asarray(parent, dtype=np.int64)
    n = len(parent)
    dst, src, coef = coefficient_coo(parent, R, C, time_step_ms)
    # Block boundaries: trees are contiguous ranges starting at each root.
    roots = np.nonzero(parent < 0)[0]
    bounds = list(roots) + [n]
    blocks = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        sel = (dst >= a) & (dst < b)
        m = b - a
        if m <= dense_above:
            A = scipy.sparse.csc_matrix((coef[sel], (dst[sel] - a, src[sel] - a)),
                                        shape=(m, m), dtype=np.float64)
            P = scipy.sparse.linalg.expm(A)
            P = scipy.sparse.csr_matrix(P) if scipy.sparse.issparse(P) else scipy.sparse.csr_matrix(np.atleast_2d(P))
            P = P.toarray()
        else:
            A = np.zeros((m, m))
            np.add.at(A, (dst[sel] - a, src[sel] - a), coef[sel])
            P = scipy.linalg.expm(A)
        P[np.abs(P) < prune] = 0.0
        blocks.append(scipy.sparse.csr_matrix(P))
    P = scipy.sparse.block_diag(blocks, format="csr") if len(blocks) > 1 else blocks[0]
    P.eliminate_zeros()
    P.sort_indices()
    return P


def lump_and_conserve(P, parent, tol, explore_factor=1e-2):
    """Pruning that keeps charge where it belongs (this project's option; the
    reference drops |P_ij| < epsilon, electric.py:114-115): walking the tree
    outward from each row's segment i, expanding nodes whose |P_ij| reaches
    tol * explore_factor, a visited entry below tol is added to the nearest kept
    entry on the path back to i; what the walk never reaches is returned to the
    diagonal.  Rows keep their sums.  Dense input, CSR output."""
    A = np.asarray(P.toarray() if scipy.sparse.issparse(P) else P, dtype=np.float64)
    parent = np.asarray(parent, dtype=np.int64)
    n = len(A)
    children = [[] for _ in range(n)]
    for c, p in enumerate(parent):
        if p >= 0:
            children[p].append(c)
    explore = tol * explore_factor
    out = np.zeros_like(A)
    for i in range(n):
        total = A[i].sum()
        stack = [(i, -1, i)]                      # (node, came from, nearest kept toward i)
        while stack:
            u, w, t = stack.pop()
            v = A[i, u]
            if abs(v) >= tol or u == i:
                out[i, u] += v
                t = u
            else:
                out[i, t] += v
            if abs(v) < explore and u != i:
                continue
            nbrs = children[u] + ([parent[u]] if parent[u] >= 0 else [])
            for x in nbrs:
                if x != w:
                    stack.append((x, u, t))
        out[i, i] += total - out[i].sum()
    return scipy.sparse.csr_matrix(out)


# ---------------------------------------------------------------- HH (hh.mod)

def _vtrap(x, y):
    """nmodl_library/artificial/hh.mod:88-94."""
    x = np.asarray(x, dtype=np.float64)
    small = np.abs(x / y) < 1e-6
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        big = x / (np.exp(x / y) - 1.0)
    return np.where(small, y * (1.0 - x / y / 2.0), big)


def hh_rates(v, celsius):
    """PROCEDURE rates(v); nmodl_library/artificial/hh.mod:62-86.

    Returns (minf, mtau, hinf, htau, ninf, ntau)."""
    q10 = 3.0 ** ((celsius - 6.3) / 10.0)
    alpha = 0.1 * _vtrap(-(v + 40.0), 10.0)
    beta = 4.0 * np.exp(-(v + 65.0) / 18.0)
    s = alpha + beta
    mtau = 1.0 / (q10 * s); minf = alpha / s
    alpha = 0.07 * np.exp(-(v + 65.0) / 20.0)
    beta = 1.0 / (np.exp(-(v + 35.0) / 10.0) + 1.0)
    s = alpha + beta
    htau = 1.0 / (q10 * s); hinf = alpha / s
    alpha = 0.01 * _vtrap(-(v + 55.0), 10.0)
    beta = 0.125 * np.exp(-(v + 65.0) / 80.0)
    s = alpha + beta
    ntau = 1.0 / (q10 * s); ninf = alpha / s
    return minf, mtau, hinf, htau, ninf, ntau


class HHInstances:
    """``hh`` mechanism instances as the NMODL front end would lay them out.

    * gbar parameters in S/cm2 are converted to S/um2 (x1e-8) and multiplied
      by the instance magnitude (um2); neuwon/rxd/nmodl/__init__.py:99-107, 404-406;
    * ``USEION na WRITE gna, ena`` writes the equilibrium, so each conductance
      is a *nonspecific* conductance stored on the instance and scattered to
      its segment; nmodl/__init__.py:179-208, species.py:229-263;
    * ``SOLVE states`` without METHOD uses the exact solution of the linear
      gate ODEs, x <- xinf + (x - xinf)*exp(-dt/xtau); nmodl/solver.py:48-55,105-106.
    """

    def __init__(self, segment, magnitude, *, gnabar=0.12, gkbar=0.036, glbar=0.0003,
                 ena=60.0, ek=-88.0, el=-54.3, v_init=-70.0, celsius=6.3):
        self.segment = np.asarray(segment, dtype=np.int64)
        m = len(self.segment)
        mag = np.broadcast_to(np.asarray(magnitude, dtype=np.float64), (m,)).copy()
        self.gna_coef = np.broadcast_to(np.asarray(gnabar, np.float64) * 1e-8, (m,)) * mag
        self.gk_coef = np.broadcast_to(np.asarray(gkbar, np.float64) * 1e-8, (m,)) * mag
        self.gl_coef = np.broadcast_to(np.asarray(glbar, np.float64) * 1e-8, (m,)) * mag
        self.E = {"na": float(ena), "k": float(ek), "l": float(el)}
        minf, _, hinf, _, ninf, _ = hh_rates(np.full(m, float(v_init)), celsius)
        self.m, self.h, self.n = minf.copy(), hinf.copy(), ninf.copy()
        self.g = {"na": np.zeros(m), "k": np.zeros(m), "l": np.zeros(m)}

    def zero_accumulators(self):
        """species.py:252-254 (nonspecific conductances reset before mechanisms run)."""
        for g in self.g.values():
            g.fill(0.0)

    def advance(self, voltage, dt, celsius):
        """BREAKPOINT block of hh.mod:41-46 after NMODL's solve and IO fixups."""
        v = voltage[self.segment]
        minf, mtau, hinf, htau, ninf, ntau = hh_rates(v, celsius)
        m = minf + (self.m - minf) * np.exp(-dt / mtau)
        h = hinf + (self.h - hinf) * np.exp(-dt / htau)
        n = ninf + (self.n - ninf) * np.exp(-dt / ntau)
        self.m, self.h, self.n = m, h, n
        self.g["na"] += self.gna_coef * m * m * m * h
        self.g["k"] += self.gk_coef * n * n * n * n
        self.g["l"] += self.gl_coef


class KineticInstances:
    """Instances of one lti_sim kinetic mechanism, stepped as the kernel that
    neuwon/rxd/lti_sim/codegen.py:39-106 generates, with its conductance
    gbar*magnitude*(open states) written by the BREAKPOINT block after the
    LTI call (nmodl/__init__.py:415-429): into the accumulator of its ion's
    species (``species`` = the species name, USEION, nmodl/__init__.py:168-208;
    ``erev`` unused) or, with ``species`` None, as a nonspecific conductance with
    reversal potential ``erev``.

    ``layout`` is the flattened table [bucket][col][row][term] (codegen.py:29-37)."""

    def __init__(self, segment, g_coef, layout, vmin, bucket_frq, open_states, erev,
                 conserve_sum, init_state, species=None, inputs=None, powers=None, input_values=None):
        """Two-input tables (lti_sim Approx2D, approx.py:242-337): ``inputs`` is a pair
        of (kind, num_buckets, minimum, bucket_frq, scale) with kind "voltage",
        "log" (LogarithmicInput) or "linear", ``powers`` the terms' (p1, p2), and
        ``input_values`` the instances' value of the non-voltage input; the layout
        is [b1 * nb2 + b2][col][row][term]."""
        self.species = species
        self.inputs = inputs
        self.powers = None if powers is None else [tuple(p) for p in powers]
        self.input_values = None if input_values is None else np.asarray(input_values, dtype=np.float64)
        self.segment = np.asarray(segment, dtype=np.int64)
        m = len(self.segment)
        self.g_coef = np.broadcast_to(np.asarray(g_coef, np.float64), (m,)).copy()
        self.layout = np.asarray(layout, dtype=np.float64)
        self.nb, S, S2, self.T = self.layout.shape
        assert S == S2
        self.S = S
        self.vmin, self.frq = float(vmin), float(bucket_frq)
        self.open_states = list(open_states)
        self.erev = float(erev)
        self.conserve_sum = conserve_sum
        self.state = np.tile(np.asarray(init_state, dtype=np.float64), (m, 1))   # [inst][state]
        self.g = np.zeros(m)

    def zero_accumulators(self):
        self.g.fill(0.0)

    def _locate2(self, voltage):
        """Flat bucket and the basis of every instance for a two-input table
        (codegen.py:43-70: inputs located one by one, flat index b1 * nb2 + b2)."""
        v = voltage[self.segment]
        locs, buckets = [], []
        for kind, nb, minimum, frq, scale in self.inputs:
            x = v if kind == "voltage" else self.input_values
            if kind == "log":
                pos = (np.log2(x + scale) - np.log2(minimum + scale)) * frq          # codegen.py:47-48
            else:
                pos = (x - minimum) * frq                                          # codegen.py:45
            b = np.trunc(pos).astype(np.int64)
            hi = b > nb - 1
            lo = (~hi) & (b < 0)
            locs.append(np.where(hi, 1.0, np.where(lo, 0.0, pos - b)))
            buckets.append(np.where(hi, nb - 1, np.where(lo, 0, b)))
        flat = buckets[0] * self.inputs[1][1] + buckets[1]
        basis = []
        for a, b in self.powers:                                   # factors in order, codegen.py:64-69
            x = np.ones(len(v))
            for k in range(a):
                x = locs[0] if k == 0 else x * locs[0]
            for k in range(b):
                x = locs[1] if (k == 0 and a == 0) else x * locs[1]
            basis.append(x)
        return flat, basis

    def advance(self, voltage):
        if self.inputs is not None:
            flat, basis = self._locate2(voltage)
            tbl = self.layout[flat]
            scratch = np.zeros((len(flat), self.S))
            for col in range(self.S):
                s = self.state[:, col]
                for row in range(self.S):
                    poly = np.zeros(len(flat))
                    for t, (a, b) in enumerate(self.powers):
                        poly = poly + (tbl[:, col, row, t] if a == 0 and b == 0 else basis[t] * tbl[:, col, row, t])
                    scratch[:, row] += poly * s
            if self.conserve_sum is not None:
                total = scratch[:, 0].copy()
                for x in range(1, self.S):
                    total += scratch[:, x]
                scratch *= (self.conserve_sum / total)[:, None]
            self.state = scratch
            self.g += self.g_coef * self.state[:, self.open_states].sum(axis=1)
            return
        v = voltage[self.segment]
        inp = (v - self.vmin) * self.frq                         # codegen.py:45
        bucket = np.trunc(inp).astype(np.int64)                  # int(input0)
        hi = bucket > self.nb - 1
        lo = (~hi) & (bucket < 0)
        loc = np.where(hi, 1.0, np.where(lo, 0.0, inp - bucket))
        bucket = np.where(hi, self.nb - 1, np.where(lo, 0, bucket))
        tbl = self.layout[bucket]                                # [inst][col][row][term]
        terms = [None] + [loc ** p for p in range(1, self.T)]
        scratch = np.zeros((len(v), self.S))
        for col in range(self.S):
            s = self.state[:, col]
            for row in range(self.S):
                poly = 0.0 + tbl[:, col, row, 0]
                for t in range(1, self.T):
                    poly = poly + terms[t] * tbl[:, col, row, t]
                scratch[:, row] += poly * s
        if self.conserve_sum is not None:
            total = scratch[:, 0].copy()
            for x in range(1, self.S):
                total += scratch[:, x]
            scratch *= (self.conserve_sum / total)[:, None]
        self.state = scratch
        self.g += self.g_coef * self.state[:, self.open_states].sum(axis=1)


# --------------------------------------------------------------------- synapses
# The reference has no synaptic kinetics and no event delivery (its
# neuwon/rxd/synapses.py only grows synapse geometry; there is no NET_RECEIVE).
# What follows is this project's definition, restated here as the oracle for the
# GPU kernels: spikes are the AP detector's output (neuron.py:72-75), routed
# through a priority queue to synapses after an axonal delay of whole steps.

def synapse_matrices(time_step, alpha, beta, delta=None, rho=None, t_max=1.0):
    """Exact per-step transition matrices (row-major, new state from old) of the
    2-state AMPA scheme C <-> O or the 3-state NMDA scheme C -> O -> D -> C
    (C -> O at alpha*T, O -> C at beta, O -> D at delta, D -> C at rho), with the
    transmitter present (T = t_max) and absent (T = 0)."""
    import scipy.linalg
    out = []
    for T in (t_max, 0.0):
        if delta is None:
            Q = np.array([[-alpha * T, beta], [alpha * T, -beta]])
        else:
            Q = np.array([[-alpha * T, beta, rho],
                          [alpha * T, -beta - delta, 0.0],
                          [0.0, delta, -rho]])
        out.append(scipy.linalg.expm(Q * time_step))
    return out


class EventQueue:
    """Spike (neuron, step) -> deliveries (step + delay, synapse), kept in a heap."""

    def __init__(self, pre, delay):
        import heapq
        self._heapq = heapq
        self.pre = np.asarray(pre, dtype=np.int64)
        self.delay = np.asarray(delay, dtype=np.int64)
        order = np.argsort(self.pre, kind="stable")
        self._out = {}
        for k in order:
            self._out.setdefault(int(self.pre[k]), []).append(int(k))
        self._heap = []

    def push(self, step, neurons):
        for j in neurons:
            for k in self._out.get(int(j), ()):
                self._heapq.heappush(self._heap, (step + int(self.delay[k]), k))

    def pop(self, step):
        got = []
        while self._heap and self._heap[0][0] <= step:
            when, k = self._heapq.heappop(self._heap)
            assert when == step, "event in the past"
            got.append(k)
        return sorted(got)


class SynapseInstances:
    """AMPA (C, O) + NMDA (C, O, D) per synapse, on post segments.

    g = w_ampa * O_ampa + w_nmda * O_nmda * B(V),  B(V) = 1 / (1 + exp(-0.062 V) mg / 3.57)
    (Jahr & Stevens 1990), reversal e_syn.  A delivery at step s keeps transmitter
    present for the mechanism updates of steps s .. s + pulse_steps - 1."""

    def __init__(self, segment, pre, delay_steps, w_ampa, w_nmda, ampa_on, ampa_off, nmda_on, nmda_off,
                 pulse_steps, e_syn=0.0, mg=1.0):
        self.segment = np.asarray(segment, dtype=np.int64)
        self.pre = np.asarray(pre, dtype=np.int64)
        self.delay = np.asarray(delay_steps, dtype=np.int64)
        self.w_ampa = np.asarray(w_ampa, dtype=np.float64)
        self.w_nmda = np.asarray(w_nmda, dtype=np.float64)
        self.Ma = (np.asarray(ampa_on), np.asarray(ampa_off))
        self.Mn = (np.asarray(nmda_on), np.asarray(nmda_off))
        self.pulse_steps = int(pulse_steps)
        self.e_syn = float(e_syn)
        self.mg = float(mg)
        m = len(self.segment)
        self.ampa = np.zeros((m, 2)); self.ampa[:, 0] = 1.0
        self.nmda = np.zeros((m, 3)); self.nmda[:, 0] = 1.0
        self.pulse_end = np.zeros(m, dtype=np.int64)
        self.events = np.zeros(m, dtype=np.int64)
        self.last_event = np.full(m, -1, dtype=np.int64)
        self.queue = EventQueue(self.pre, self.delay)
        self.delivered = []                      # (step, synapse) log

    def conductance(self, voltage):
        v = voltage[self.segment]
        block = 1.0 / (1.0 + np.exp(-0.062 * v) * (self.mg / 3.57))
        return self.w_ampa * self.ampa[:, 1] + self.w_nmda * self.nmda[:, 1] * block

    def advance(self, step):
        for k in self.queue.pop(step):
            self.pulse_end[k] = step + self.pulse_steps
            self.events[k] += 1
            self.last_event[k] = step
            self.delivered.append((step, k))
        on = step < self.pulse_end
        for Mx, st in ((self.Ma, self.ampa), (self.Mn, self.nmda)):
            new_on = st @ Mx[0].T
            new_off = st @ Mx[1].T
            st[:] = np.where(on[:, None], new_on, new_off)


# --------------------------------------------------------------------- calcium
class CalciumOracle:
    """Intracellular calcium for the oracle: species.py:56-70's update after every
    electric half step (c <- max(0, c + dcdt h), then c <- M c) with M = expm of the
    diffusion operator built like electric.py:85-109 (resistance 1e-3 L / (D A),
    capacity = volume), and the pump / sodium-fraction influx writing dc/dt in the
    mechanism phase (the pump steps through the same tabled propagator as the
    device, given as ``table_step(c, states)``)."""

    def __init__(self, parent, cross_area, length, volume, diffusivity, time_step, initial, influx, efflux,
                 table_step=None, pump_state=None, prune=EPSILON):
        parent = np.asarray(parent, dtype=np.int64)
        n = len(parent)
        res = np.where(parent < 0, 1.0, 1e-3 * np.asarray(length) / (diffusivity * np.asarray(cross_area)))
        self.M = propagator(parent, res, np.asarray(volume, dtype=np.float64), 0.5 * time_step, prune)
        self.volume = np.asarray(volume, dtype=np.float64)
        self.c = np.full(n, float(initial))
        self.dcdt = np.zeros(n)
        self.influx = np.asarray(influx, dtype=np.float64)
        self.efflux = np.asarray(efflux, dtype=np.float64)
        self.table_step = table_step
        self.state = None if pump_state is None else np.tile(np.asarray(pump_state, dtype=np.float64), (n, 1))
        self.half_step = 0.5 * time_step

    def advance_half(self):
        self.c = self.M.dot(np.maximum(0.0, self.c + self.dcdt * self.half_step))

    def mechanisms(self, voltage, hh):
        ina = np.zeros(len(self.c))
        if hh is not None:
            np.add.at(ina, hh.segment, hh.g["na"] * (voltage[hh.segment] - hh.E["na"]))
        d = -self.influx * ina
        if self.table_step is not None:
            self.state = self.table_step(self.c, self.state)
            d = d - self.efflux * self.state[:, 1]
        self.dcdt = d


class OracleModel:
    """FP64 restatement of ``RxD_Model.advance()`` (neuwon/rxd/rxd_model.py:63-80).

    Inputs are plain arrays for the segments (creation order, neurons
    contiguous as after ``Database.sort()``).  ``clamps`` is a list of
    (segment, amperes, first_tick, num_ticks) in input-hook ticks (half steps);
    ``detectors`` is a list of (segment, threshold_mV) per neuron.

    ``duplicates='sum'`` adds every mechanism instance's conductance into its
    segment.  ``duplicates='numpy'`` reproduces the reference's fancy-index
    ``a[idx] += b`` (species.py:256-260), under which only one of several
    instances on the same segment is counted (nonspecific conductances; species
    accumulators are written per instance and count every one).

    ``species`` maps electric species names to constant reversal potentials (mV),
    in declaration order (the ``_SpeciesType`` accumulators, species.py:85-160);
    ``kinetic`` is one ``KineticInstances`` or a list of them.
    """

    def __init__(self, parent, R, C, *, time_step=0.1, celsius=6.3, v_init=-70.0,
                 prune=EPSILON, propagator_matrix=None, hh=None, clamps=(),
                 detectors=(), duplicates="sum", kinetic=None, synapses=None, calcium=None, species=None):
        self.parent = np.asarray(parent, dtype=np.int64)
        self.n = len(self.parent)
        self.R = np.asarray(R, dtype=np.float64)
        self.C = np.asarray(C, dtype=np.float64)
        self.time_step = float(time_step)
        self.half_step = 0.5 * self.time_step     # rxd_model.py:21, species.py:273
        self.celsius = float(celsius)
        self.voltage = np.full(self.n, float(v_init))
        self.integral_voltage = np.zeros(self.n)
        self.nonspecific_current = np.zeros(self.n)
        self.sum_current = np.zeros(self.n)
        self.sum_conductance = np.zeros(self.n)
        self.driving_voltage = np.zeros(self.n)
        self.P = propagator_matrix if propagator_matrix is not None else \
            propagator(self.parent, self.R, self.C, self.half_step, prune)
        self.hh = hh
        self.kinetic = [] if kinetic is None else (list(kinetic) if isinstance(kinetic, (list, tuple)) else [kinetic])
        self.species = dict(species or {})
        # {name}_current / {name}_conductance segment accumulators (species.py:125-133).
        self.species_current = {s: np.zeros(self.n) for s in self.species}
        self.species_conductance = {s: np.zeros(self.n) for s in self.species}
        for k in self.kinetic:
            assert k.species is None or k.species in self.species, f"undeclared species {k.species}"
        self.synapses = synapses
        self.calcium = calcium
        self.clamps = [(int(s), float(a), int(f), int(k)) for (s, a, f, k) in clamps]
        self.detectors = [(int(s), float(t)) for (s, t) in detectors]
        self.AP_detected = np.zeros(len(self.detectors), dtype=bool)
        self._AP_true_state = np.zeros(len(self.detectors), dtype=bool)
        self.spike_count = np.zeros(len(self.detectors), dtype=np.int64)
        self.input_ticks = 0
        self.steps = 0
        self.duplicates = duplicates

    # rxd_model.py:91-113
    def _advance_species(self):
        self.sum_current[:] = self.nonspecific_current
        self.sum_conductance.fill(0.0)
        self.driving_voltage.fill(0.0)
        # _SpeciesType._apply_accumulators (species.py:155-160), declared species
        # first, then the nonspecific conductances the mechanisms registered.
        for name, erev in self.species.items():
            g = self.species_conductance[name]
            self.sum_current += self.species_current[name]
            self.sum_conductance += g
            self.driving_voltage += g * erev
        if self.hh is not None:
            seg = self.hh.segment
            for ion in ("na", "k", "l"):
                g = self.hh.g[ion]
                if self.duplicates == "numpy":
                    self.sum_conductance[seg] += g
                    self.driving_voltage[seg] += g * self.hh.E[ion]
                else:
                    np.add.at(self.sum_conductance, seg, g)
                    np.add.at(self.driving_voltage, seg, g * self.hh.E[ion])
        for k in self.kinetic:
            if k.species is not None:
                continue
            if self.duplicates == "numpy":
                self.sum_conductance[k.segment] += k.g
                self.driving_voltage[k.segment] += k.g * k.erev
            else:
                np.add.at(self.sum_conductance, k.segment, k.g)
                np.add.at(self.driving_voltage, k.segment, k.g * k.erev)
        if self.synapses is not None:
            sy = self.synapses
            g = sy.conductance(self.voltage)
            np.add.at(self.sum_conductance, sy.segment, g)
            np.add.at(self.driving_voltage, sy.segment, g * sy.e_syn)
        # input_hook.tick(): Clock.tick then TimeSeries._play_implementation
        # (database/time.py:114-117, 287-302), current clamps in "+=" mode.
        self.input_ticks += 1
        t = self.input_ticks
        for seg, amps, first, count in self.clamps:
            if first <= t < first + count:
                self.sum_current[seg] += amps
        with np.errstate(divide="ignore", invalid="ignore"):
            self.driving_voltage /= self.sum_conductance
        self.driving_voltage[:] = np.nan_to_num(self.driving_voltage)
        self._advance_electric(self.half_step)
        if self.calcium is not None:
            self.calcium.advance_half()

    # neuwon/rxd/neuron/electric.py:56-76
    def _advance_electric(self, time_step):
        dt = time_step * 1e-3
        dv_currents = time_step * self.sum_current / self.C
        exponent = -dt * self.sum_conductance / self.C
        alpha = np.exp(exponent)
        diff_v = self.driving_voltage - self.voltage
        self.voltage[:] = self.P.dot(self.driving_voltage - diff_v * alpha + dv_currents)
        self.integral_voltage[:] = (dt * self.driving_voltage - exponent * diff_v * alpha
                                    + (.5 * dt * dv_currents))

    # rxd_model.py:115-123
    def _advance_mechanisms(self):
        self.nonspecific_current.fill(0.0)
        if self.hh is not None:
            self.hh.zero_accumulators()
            self.hh.advance(self.voltage, self.time_step, self.celsius)
        for acc in list(self.species_current.values()) + list(self.species_conductance.values()):
            acc.fill(0.0)                                   # species.py:147-153
        for k in self.kinetic:
            k.zero_accumulators()
            k.advance(self.voltage)
            if k.species is not None:
                # self.segment.{ion}_conductance += g, one instance at a time.
                np.add.at(self.species_conductance[k.species], k.segment, k.g)
        if self.synapses is not None:
            self.synapses.advance(self.steps)
        if self.calcium is not None:
            self.calcium.mechanisms(self.voltage, self.hh)

    # neuwon/rxd/neuron/neuron.py:72-75
    def _advance_AP_detector(self):
        for k, (seg, thr) in enumerate(self.detectors):
            over = self.voltage[seg] >= thr
            self.AP_detected[k] = over and not self._AP_true_state[k]
            self._AP_true_state[k] = over
            self.spike_count[k] += int(self.AP_detected[k])
        if self.synapses is not None:
            self.synapses.queue.push(self.steps, np.flatnonzero(self.AP_detected))

    def advance(self):
        """rxd_model.py:63-80: species(dt/2) -> mechanisms(dt) -> species(dt/2) -> AP."""
        self._advance_species()
        self._advance_mechanisms()
        self._advance_species()
        self._advance_AP_detector()
        self.steps += 1


def clamp_ticks(start_ms, duration_ms, time_step):
    """Ticks on which ``Segment.inject_current`` adds its current.

    ``inject_current`` (electric.py:119-125) plays a two-point constant wave on
    the half-step input clock with ``immediate=False`` (time.py:245-285): it
    fires on the ``ceil(duration/half_step)`` ticks after the call.  A call made
    when the model clock reads ``start_ms`` (i.e. before the advance that starts
    at ``start_ms``) therefore covers ticks [2k+1, 2k+1+count) with
    k = round(start_ms / time_step).
    """
    half = 0.5 * time_step
    count = math.ceil(float(duration_ms) / half)
    k = round(float(start_ms) / time_step)
    return 2 * k + 1, count
