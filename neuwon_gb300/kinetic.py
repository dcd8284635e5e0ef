"""Linear kinetic schemes solved by exact integration with voltage tables.

Restates the reference's lti_sim pipeline (neuwon/rxd/lti_sim/):

* the propagator of one step is expm(A(v) dt) with every column renormalised
  to sum to 1 (lti_model.py:51-65);
* the input range is cut into equal buckets (inputs.py:26-48, 72-83) and, in every
  bucket, each matrix entry is fitted by least squares with a polynomial in
  the location within the bucket (approx.py:159-174, polynomial.py:3-20);
* at run time an instance locates its voltage, evaluates the polynomials and
  multiplies its state vector, then rescales the states to the CONSERVE sum
  (codegen.py:39-106).  The table is stored as [bucket][col][row][term]
  (codegen.py:29-37).

The exact matrices are sampled at deterministic points (the midpoints of
``samples_per_bucket`` equal sub-buckets) instead of the reference's one
random point per sub-bucket; ``build_table(sample_inputs=...)`` accepts the
reference's own sample points to reproduce its table.

The 8-state sodium scheme ``na8`` is the Markov form of the Hodgkin-Huxley
sodium channel: states (k, h) with k = 0..3 open m-gates and h = 1 (available)
or 0 (inactivated); k -> k+1 at (3-k) alpha_m, k+1 -> k at (k+1) beta_m,
available -> inactivated at beta_h, back at alpha_h, rates of
nmodl_library/artificial/hh.mod scaled by q10.  Started from the binomial
distribution of (m, h), its open state (3, 1) equals m^3 h exactly.
"""
import math

import numpy as np
import scipy.linalg

from .mechanisms import Mechanism


class KineticScheme:
    """A linear kinetic scheme dS/dt = A(v) S."""

    def __init__(self, name, states, transitions, open_states, conserve_sum=1.0):
        """transitions(v, celsius) -> list of (src, dst, rate) with numpy rates."""
        self.name = str(name)
        self.states = list(states)
        self.num_states = len(self.states)
        self.transitions = transitions
        self.open_states = [self.states.index(s) for s in open_states]
        self.conserve_sum = conserve_sum

    def matrix(self, v, celsius):
        """A(v) for an array of voltages: shape (len(v), S, S)."""
        v = np.atleast_1d(np.asarray(v, dtype=np.float64))
        S = self.num_states
        A = np.zeros((len(v), S, S))
        for src, dst, rate in self.transitions(v, celsius):
            A[:, dst, src] += rate
            A[:, src, src] -= rate
        return A

    def exact_propagator(self, v, dt, celsius):
        """expm(A(v) dt) with columns renormalised to sum 1 (lti_model.py:51-65)."""
        M = scipy.linalg.expm(self.matrix(v, celsius) * dt)
        M /= M.sum(axis=1, keepdims=True)
        return M

    def steady_state(self, v, celsius):
        """State after an hour at voltage v from equal occupancies summing to the
        conserve sum, through the column-renormalised propagator
        (LTI_Model.get_initial_state, neuwon/rxd/lti_sim/lti_model.py:67-78)."""
        M = scipy.linalg.expm(self.matrix([v], celsius)[0] * 3600e3)
        M = M / M.sum(axis=0, keepdims=True)
        s = M @ np.full(self.num_states, (self.conserve_sum or 1.0) / self.num_states)
        return s


def _vtrap(x, y):
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        big = x / (np.exp(x / y) - 1.0)
    return np.where(np.abs(x / y) < 1e-6, y * (1.0 - x / y / 2.0), big)


def hh_sodium_rates(v, celsius):
    """alpha/beta of the m and h gates (hh.mod:62-86), times q10."""
    q10 = 3.0 ** ((celsius - 6.3) / 10.0)
    am = 0.1 * _vtrap(-(v + 40.0), 10.0)
    bm = 4.0 * np.exp(-(v + 65.0) / 18.0)
    ah = 0.07 * np.exp(-(v + 65.0) / 20.0)
    bh = 1.0 / (np.exp(-(v + 35.0) / 10.0) + 1.0)
    return q10 * am, q10 * bm, q10 * ah, q10 * bh


def na8():
    states = ["C3", "C2", "C1", "O", "I3", "I2", "I1", "I"]   # (k, h): k = index % 4, h = index < 4

    def transitions(v, celsius):
        am, bm, ah, bh = hh_sodium_rates(v, celsius)
        out = []
        for row in (0, 4):
            for k in range(3):
                out.append((row + k, row + k + 1, (3 - k) * am))
                out.append((row + k + 1, row + k, (k + 1) * bm))
        for k in range(4):
            out.append((k, 4 + k, bh))
            out.append((4 + k, k, ah))
        return out
    return KineticScheme("na8", states, transitions, open_states=["O"], conserve_sum=1.0)


def _boltzmann(v, b, vv, k):
    """FUNCTION rates2 of nmodl_library/kinetic/Nav11.mod:144-146: b / (1 + exp((v - vv) / k))."""
    with np.errstate(over="ignore"):
        return b / (1.0 + np.exp((v - vv) / k))


def nav11():
    """Six-state Nav1.1 channel of nmodl_library/kinetic/Nav11.mod (SUFFIX na11a,
    USEION na): states C1 C2 O1 O2 I1 I2, open = O1 + O2, CONSERVE sum 1; rate
    constants of its PARAMETER block (Nav11.mod:21-87), q10 = 3^((celsius - 20)/10)
    (INITIAL, :120) and PROCEDURE rates (:148-163), reactions of KINETIC kin (:131-142)."""
    states = ["C1", "C2", "O1", "O2", "I1", "I2"]
    C1, C2, O1, O2, I1, I2 = range(6)

    def transitions(v, celsius):
        q = 3.0 ** ((celsius - 20.0) / 10.0)
        r = lambda *terms: q * sum(_boltzmann(v, *t) for t in terms)
        c1c2 = r((18.0, -7.0, -10.0))
        c2c1 = r((3.0, -37.0, 10.0), (18.0, -7.0, -10.0))
        c2o1 = r((18.0, -7.0, -10.0))
        o1c2 = r((3.0, -37.0, 10.0), (18.0, -7.0, -10.0))
        c2o2 = r((0.08, -10.0, -15.0))
        o2c2 = r((2.0, -50.0, 7.0), (0.2, -20.0, -10.0))
        o1i1 = r((8.0, -37.0, 13.0), (17.0, -7.0, -15.0))
        i1o1 = r((0.00001, -37.0, 10.0))
        i1c1 = r((0.21, -61.0, 7.0))
        c1i1 = r((0.3, -61.0, -5.5))
        i1i2 = r((0.0015, -90.0, -5.0))
        i2i1 = r((0.0075, -90.0, 15.0))
        return [(C1, C2, c1c2), (C2, C1, c2c1), (C2, O1, c2o1), (O1, C2, o1c2), (C2, O2, c2o2), (O2, C2, o2c2),
                (O1, I1, o1i1), (I1, O1, i1o1), (I1, C1, i1c1), (C1, I1, c1i1), (I1, I2, i1i2), (I2, I1, i2i1)]
    return KineticScheme("na11a", states, transitions, open_states=["O1", "O2"], conserve_sum=1.0)


# PARAMETER block of nmodl_library/kinetic/Kv11.mod:10-34 (temperature factors per degC).
_KV11 = dict(Hkc=0.12166, Hki=0.44916, Hkn=-0.85022, Hri=0.0026028, Hric_n=-0.066541, Hrn=-0.048079,
             Hvc=0.91934, Hvic_c=-0.71121, Hvic_n=-0.29515, Hvn_ic=0.94495, Ri=0.78718, Rn=1.6611,
             Vc=-17.6122, Zc=1.6756, kc=0.030179, ki=0.00025091, kn=0.010089, ric_c=0.01189, ric_n=5.55,
             vc_ic=1.6111, vic_c=999.9351, vic_n=0.66208, vn_ic=0.10006)


def kv11():
    """Six-state Kv1.1 channel of nmodl_library/kinetic/Kv11.mod (SUFFIX
    Kv11_6States_temperature2, USEION k): states CS OS IC1 CIC1 IN INC1, open = OS,
    CONSERVE sum 1; INITIAL constants F = 96.485, A = 8.134 (celsius + 273.15),
    rc_ic = ric_c, rn_ic = ric_n, Hrn_ic = Hric_n (:55-62), PROCEDURE rates (:76-79),
    reactions of KINETIC kin (:64-74)."""
    states = ["CS", "OS", "IC1", "CIC1", "IN", "INC1"]
    CS, OS, IC1, CIC1, IN, INC1 = range(6)
    p = _KV11

    def transitions(v, celsius):
        t = celsius - 25.0
        FA = 96.485 / (8.134 * (celsius + 273.15))
        e = lambda x: math.exp(x * t)
        shift = v - p["Vc"] - p["Hvc"] * t
        kco = p["kc"] * np.exp(p["Zc"] * FA * shift) * e(p["Hkc"])
        koc = p["kc"] * np.exp(-p["Zc"] * FA * shift) * e(p["Hkc"])
        rc_ic, rn_ic, Hrn_ic = p["ric_c"], p["ric_n"], p["Hric_n"]
        ki_t, kn_t = p["ki"] * e(p["Hki"]), p["kn"] * e(p["Hkn"])
        one = np.ones_like(kco)
        return [
            (CS, OS, kco), (OS, CS, koc),
            (CIC1, IC1, p["vc_ic"] * kco), (IC1, CIC1, rc_ic * p["vc_ic"] * koc),
            (CS, CIC1, one * p["ric_c"] * p["vic_c"] * ki_t * e(p["Hvic_c"])),
            (CIC1, CS, one * p["vic_c"] * ki_t * p["Ri"] * e(p["Hri"]) * e(p["Hvic_c"])),
            (OS, IC1, one * ki_t), (IC1, OS, one * ki_t * p["Ri"] * e(p["Hri"])),
            (OS, IN, one * kn_t), (IN, OS, one * kn_t * p["Rn"] * e(p["Hrn"])),
            (IC1, INC1, one * p["vn_ic"] * rn_ic * kn_t * e(Hrn_ic) * e(p["Hvn_ic"])),
            (INC1, IC1, one * p["vn_ic"] * kn_t * p["Rn"] * e(p["Hrn"]) * e(p["Hvn_ic"])),
            (IN, INC1, one * p["ric_n"] * p["vic_n"] * ki_t * e(p["Hric_n"]) * e(p["Hvic_n"])),
            (INC1, IN, one * p["vic_n"] * ki_t * p["Ri"] * e(p["Hri"]) * e(p["Hvic_n"])),
        ]
    return KineticScheme("Kv11_6States_temperature2", states, transitions, open_states=["OS"], conserve_sum=1.0)


class TableInput:
    """One input of a kinetic table, located as lti_sim's inputs locate theirs
    (neuwon/rxd/lti_sim/inputs.py): the segment voltage ("voltage", LinearInput),
    an instance value on a log2 scale ("log", LogarithmicInput: minimum 0, bucket
    value (log2(x + scale) - log2(minimum + scale)) * frq) or on a linear one
    ("linear")."""

    KINDS = {"voltage": 0, "log": 1, "linear": 2}

    def __init__(self, name, kind, minimum, maximum, num_buckets, scale=1.0, initial=None):
        if kind not in self.KINDS:
            raise ValueError(f"input kind {kind!r}: one of {sorted(self.KINDS)}")
        self.name, self.kind = str(name), kind
        self.code = self.KINDS[kind]
        self.minimum, self.maximum = float(minimum), float(maximum)
        self.num_buckets = int(num_buckets)
        self.scale = float(scale)
        self.initial = self.minimum if initial is None else float(initial)
        if kind == "log":
            self.offset = math.log2(self.minimum + self.scale)                        # inputs.py:90-96
            span = math.log2(self.maximum + self.scale) - self.offset
        else:
            self.offset = self.minimum                                                # inputs.py:74-77
            span = self.maximum - self.minimum
        self.bucket_frq = self.num_buckets / span
        self.bucket_width = span / self.num_buckets

    def position(self, x):
        x = np.asarray(x, dtype=np.float64)
        if self.kind == "log":
            return (np.log2(x + self.scale) - self.offset) * self.bucket_frq
        return (x - self.offset) * self.bucket_frq

    def value(self, pos):
        y = self.offset + np.asarray(pos, dtype=np.float64) * self.bucket_width
        return 2.0 ** y - self.scale if self.kind == "log" else y

    def locate(self, x):
        """(bucket, location) clamped to the table (codegen.py:43-59)."""
        pos = self.position(x)
        b = np.trunc(pos).astype(np.int64)
        hi, lo = b > self.num_buckets - 1, b < 0
        loc = np.where(hi, 1.0, np.where(lo, 0.0, pos - b))
        return np.where(hi, self.num_buckets - 1, np.where(lo, 0, b)), loc


def canonical_terms(terms):
    """Polynomial terms in lti_sim's canonical order (polynomial.py:19-20): by total
    degree, then by the reversed powers."""
    return sorted({tuple(int(p) for p in t) for t in terms}, key=lambda t: (sum(t), tuple(reversed(t))))


class KineticScheme2(KineticScheme):
    """A linear kinetic scheme dS/dt = A(x1, x2) S over two table inputs, in table
    order (lti_sim sorts a model's inputs by name, lti_model.py:8)."""

    def __init__(self, name, states, transitions, open_states, input_names, conserve_sum=1.0):
        """transitions(x1, x2, celsius) -> list of (src, dst, rate) with numpy rates."""
        super().__init__(name, states, transitions, open_states, conserve_sum)
        self.input_names = tuple(input_names)

    def matrix(self, x1, x2, celsius):
        x1 = np.atleast_1d(np.asarray(x1, dtype=np.float64))
        x2 = np.broadcast_to(np.asarray(x2, dtype=np.float64), x1.shape)
        S = self.num_states
        A = np.zeros((len(x1), S, S))
        for src, dst, rate in self.transitions(x1, x2, celsius):
            A[:, dst, src] += rate
            A[:, src, src] -= rate
        return A

    def exact_propagator(self, x1, x2, dt, celsius):
        M = scipy.linalg.expm(self.matrix(x1, x2, celsius) * dt)
        M /= M.sum(axis=1, keepdims=True)
        return M

    def steady_state(self, x1, x2, celsius):
        M = scipy.linalg.expm(self.matrix([x1], [x2], celsius)[0] * 3600e3)
        M = M / M.sum(axis=0, keepdims=True)
        return M @ np.full(self.num_states, (self.conserve_sum or 1.0) / self.num_states)


def nmda():
    """Ten-state NMDA receptor with magnesium block of nmodl_library/kinetic/NMDA.mod
    (Kampa et al. 2004; POINT_PROCESS NMDA_Mg): rate constants of its PARAMETER block
    (mg = 1 mM, valence -2, memb_fraction 0.8), the voltage- and glutamate-dependent
    rates and the thirteen reactions of KINETIC kstates, CONSERVE sum 1, open state O.
    Inputs in lti_sim's order (sorted by name): C (glutamate, mM) then v (mV)."""
    states = ["U", "Cl", "D1", "D2", "O", "UMg", "ClMg", "D1Mg", "D2Mg", "OMg"]
    U, Cl, D1, D2, O, UMg, ClMg, D1Mg, D2Mg, OMg = range(10)
    P = dict(Rb=10e-3, Ru=5.6e-3, Ro=10e-3, Rc=273e-3, Rd1=2.2e-3, Rr1=1.6e-3, Rd2=0.43e-3, Rr2=0.5e-3,
             Rmb=0.05e-3, Rmu=12800e-3, Rmc1b=0.00005e-3, Rmc1u=2.438312e-3, Rmc2b=0.00005e-3,
             Rmc2u=5.041915e-3, Rmd1b=0.00005e-3, Rmd1u=2.98874e-3, Rmd2b=0.00005e-3, Rmd2u=2.953408e-3,
             RbMg=10e-3, RuMg=17.1e-3, RoMg=10e-3, RcMg=548e-3, Rd1Mg=2.1e-3, Rr1Mg=0.87e-3, Rd2Mg=0.26e-3,
             Rr2Mg=0.42e-3, mg=1.0, valence=-2.0, memb_fraction=0.8)

    def transitions(C, v, celsius):
        p = P
        block = np.exp((v - 40.0) * p["valence"] * p["memb_fraction"] / 25.0)
        unblock = np.exp(-1.0 * (v - 40.0) * p["valence"] * (1.0 - p["memb_fraction"]) / 25.0)
        rb = p["Rb"] * 1e3 * C
        rbMg = p["RbMg"] * 1e3 * C
        rmb, rmu = p["Rmb"] * p["mg"] * 1e3 * block, p["Rmu"] * unblock
        rmc1b, rmc1u = p["Rmc1b"] * p["mg"] * 1e3 * block, p["Rmc1u"] * unblock
        rmc2b, rmc2u = p["Rmc2b"] * p["mg"] * 1e3 * block, p["Rmc2u"] * unblock
        rmd1b, rmd1u = p["Rmd1b"] * p["mg"] * 1e3 * block, p["Rmd1u"] * unblock
        rmd2b, rmd2u = p["Rmd2b"] * p["mg"] * 1e3 * block, p["Rmd2u"] * unblock
        one = np.ones_like(v)
        pairs = [(U, Cl, rb, p["Ru"] * one), (Cl, O, p["Ro"] * one, p["Rc"] * one),
                 (Cl, D1, p["Rd1"] * one, p["Rr1"] * one), (D1, D2, p["Rd2"] * one, p["Rr2"] * one),
                 (O, OMg, rmb, rmu), (UMg, ClMg, rbMg, p["RuMg"] * one), (ClMg, OMg, p["RoMg"] * one, p["RcMg"] * one),
                 (ClMg, D1Mg, p["Rd1Mg"] * one, p["Rr1Mg"] * one), (D1Mg, D2Mg, p["Rd2Mg"] * one, p["Rr2Mg"] * one),
                 (U, UMg, rmc1b, rmc1u), (Cl, ClMg, rmc2b, rmc2u), (D1, D1Mg, rmd1b, rmd1u), (D2, D2Mg, rmd2b, rmd2u)]
        out = []
        for a, b, kf, kb in pairs:
            out.append((a, b, kf))
            out.append((b, a, kb))
        return out
    return KineticScheme2("NMDA_Mg", states, transitions, open_states=["O"], input_names=("C", "v"), conserve_sum=1.0)


class LTITable2:
    """Two-input polynomial approximation of the per-step propagator (lti_sim's
    Approx2D, approx.py:242-275): per bucket pair (b1, b2), every matrix entry is
    fitted by least squares over samples in the bucket with the terms
    loc1^p1 * loc2^p2.  Samples sit on a grid of ``samples_per_axis`` sub-bucket
    midpoints per input, or are given (``sample_inputs`` = (x1, x2), e.g. the
    reference's own random samples).  ``layout`` is [b1 * nb2 + b2][col][row][term]."""

    def __init__(self, scheme, dt, celsius, input1, input2, terms, samples_per_axis=4, sample_inputs=None):
        self.scheme, self.dt, self.celsius = scheme, float(dt), float(celsius)
        self.inputs = (input1, input2)
        self.terms = canonical_terms(terms)
        self.powers = np.array(self.terms, dtype=np.int32)
        S, T = scheme.num_states, len(self.terms)
        nb1, nb2 = input1.num_buckets, input2.num_buckets
        if sample_inputs is None:
            sub = (np.arange(samples_per_axis) + 0.5) / samples_per_axis
            g1, g2 = np.meshgrid(sub, sub, indexing="ij")
            p1 = (np.arange(nb1)[:, None, None] + np.zeros(nb2)[None, :, None] + g1.ravel()[None, None, :]).ravel()
            p2 = (np.zeros(nb1)[:, None, None] + np.arange(nb2)[None, :, None] + g2.ravel()[None, None, :]).ravel()
            x1, x2 = input1.value(p1), input2.value(p2)
        else:
            x1, x2 = (np.asarray(x, dtype=np.float64) for x in sample_inputs)
        exact = scheme.exact_propagator(x1, x2, self.dt, self.celsius)
        pos1, pos2 = input1.position(x1), input2.position(x2)
        b1, b2 = pos1.astype(np.int64), pos2.astype(np.int64)                  # approx.py:16-18
        flat = b1 * nb2 + b2
        order = np.argsort(flat, kind="stable")
        flat, pos1, pos2, b1, b2, exact = flat[order], pos1[order], pos2[order], b1[order], b2[order], exact[order]
        bounds = np.searchsorted(flat, np.arange(nb1 * nb2 + 1))
        table = np.empty((nb1 * nb2, S, S, T))
        for f in range(nb1 * nb2):
            lo, hi = bounds[f], bounds[f + 1]
            l1, l2 = pos1[lo:hi] - b1[lo:hi], pos2[lo:hi] - b2[lo:hi]
            A = np.stack([l1 ** a * l2 ** b for a, b in self.terms], axis=1)
            coef = np.linalg.lstsq(A, exact[lo:hi].reshape(-1, S * S), rcond=None)[0]
            table[f] = coef.reshape(T, S, S).transpose(1, 2, 0)
        self.table = table                                                     # [b][row][col][term]
        self.layout = np.ascontiguousarray(table.transpose(0, 2, 1, 3))        # [b][col][row][term]

    def basis(self, loc1, loc2):
        out = []
        for a, b in self.terms:
            x = np.ones_like(loc1)
            for k in range(a):
                x = loc1 if k == 0 else x * loc1
            for k in range(b):
                x = loc2 if (k == 0 and a == 0) else x * loc2
            out.append(x)
        return np.stack(out, axis=-1)

    def approximate(self, x1, x2):
        """The table's matrices at inputs (x1, x2): shape (n, row, col)."""
        (b1, l1), (b2, l2) = self.inputs[0].locate(x1), self.inputs[1].locate(x2)
        f = b1 * self.inputs[1].num_buckets + b2
        return np.einsum("ncrt,nt->nrc", self.layout[f], self.basis(l1, l2))

    def max_error(self, samples_per_axis=5):
        """Max |table - exact| over a grid of points in every bucket pair."""
        i1, i2 = self.inputs
        sub = (np.arange(samples_per_axis) + 0.37) / samples_per_axis
        p1 = (np.arange(i1.num_buckets)[:, None] + sub[None, :]).ravel()
        p2 = (np.arange(i2.num_buckets)[:, None] + sub[None, :]).ravel()
        P1, P2 = np.meshgrid(p1, p2, indexing="ij")
        x1, x2 = i1.value(P1.ravel()), i2.value(P2.ravel())
        err = 0.0
        for k in range(0, len(x1), 20000):
            exact = self.scheme.exact_propagator(x1[k:k + 20000], x2[k:k + 20000], self.dt, self.celsius)
            err = max(err, float(np.abs(self.approximate(x1[k:k + 20000], x2[k:k + 20000]) - exact).max()))
        return err


def table_inputs2(scheme, celsius, input1, input2, terms, samples_per_axis=4):
    """Rate matrices at the grid samples of every bucket pair (bucket-major, flat bucket
    b1 * nb2 + b2) and the pseudo-inverse of the two-input fit (the same for every
    bucket pair): the inputs of nw_lti_table_build for a two-input table."""
    terms = canonical_terms(terms)
    k = int(samples_per_axis)
    sub = (np.arange(k) + 0.5) / k
    g1, g2 = np.meshgrid(sub, sub, indexing="ij")
    g1, g2 = g1.ravel(), g2.ravel()
    nb1, nb2 = input1.num_buckets, input2.num_buckets
    p1 = (np.arange(nb1)[:, None, None] + np.zeros(nb2)[None, :, None] + g1[None, None, :]).ravel()
    p2 = (np.zeros(nb1)[:, None, None] + np.arange(nb2)[None, :, None] + g2[None, None, :]).ravel()
    rates = np.ascontiguousarray(scheme.matrix(input1.value(p1), input2.value(p2), celsius), dtype=np.float64)
    A = np.stack([g1 ** a * g2 ** b for a, b in terms], axis=1)
    fit = np.ascontiguousarray(np.linalg.pinv(A))
    return rates, fit, terms


def scheme_table_gpu2(ctx, scheme, dt, celsius, input1, input2, terms, samples_per_axis=4, target=0):
    """A two-input table built on the GPU in FP64 (nw_lti_table_build over the flat
    bucket pairs)."""
    rates, fit, terms = table_inputs2(scheme, celsius, input1, input2, terms, samples_per_axis)
    return gpu_table(ctx, rates, fit, input1.num_buckets * input2.num_buckets, dt, target)


def binomial_state(m, h):
    """Na8 occupancy equivalent to HH gates (m, h)."""
    s = np.zeros(8)
    for k in range(4):
        p = math.comb(3, k) * m ** k * (1 - m) ** (3 - k)
        s[k] = p * h
        s[4 + k] = p * (1 - h)
    return s


class LTITable:
    """Voltage-bucketed polynomial approximation of the per-step propagator."""

    def __init__(self, scheme, dt, celsius, vmin=-100.0, vmax=60.0, num_buckets=1600, degree=1,
                 samples_per_bucket=20, sample_inputs=None):
        self.scheme = scheme
        self.dt, self.celsius = float(dt), float(celsius)
        self.vmin, self.vmax = float(vmin), float(vmax)
        self.num_buckets = int(num_buckets)
        self.num_terms = int(degree) + 1
        self.bucket_frq = self.num_buckets / (self.vmax - self.vmin)       # inputs.py:74-77
        self.bucket_width = (self.vmax - self.vmin) / self.num_buckets
        S, T, nb = scheme.num_states, self.num_terms, self.num_buckets
        if sample_inputs is None:
            sub = (np.arange(samples_per_bucket) + 0.5) / samples_per_bucket
            loc = (np.arange(nb)[:, None] + sub[None, :]).ravel()
            sample_inputs = self.vmin + loc * self.bucket_width
        v = np.asarray(sample_inputs, dtype=np.float64)
        exact = scheme.exact_propagator(v, self.dt, self.celsius)             # (n, S, S)
        pos = (v - self.vmin) * self.bucket_frq
        bucket = pos.astype(np.int32)                                         # approx.py:16-18
        order = np.argsort(bucket, kind="stable")
        bucket, pos, exact = bucket[order], pos[order], exact[order]
        table = np.empty((nb, S, S, T))
        bounds = np.searchsorted(bucket, np.arange(nb + 1))
        for b in range(nb):
            lo, hi = bounds[b], bounds[b + 1]
            loc = pos[lo:hi] - b
            A = loc[:, None] ** np.arange(T)[None, :]
            B = exact[lo:hi].reshape(-1, S * S)
            coef = np.linalg.lstsq(A, B, rcond=None)[0]
            table[b] = coef.reshape(T, S, S).transpose(1, 2, 0)
        self.table = table                                   # [bucket][row][col][term]
        self.layout = np.ascontiguousarray(table.transpose(0, 2, 1, 3))   # [bucket][col][row][term]

    def locate(self, v):
        """Bucket index and location, as the generated kernel computes them (codegen.py:43-59)."""
        x = (np.asarray(v, dtype=np.float64) - self.vmin) * self.bucket_frq
        b = np.trunc(x).astype(np.int64)
        loc = x - b
        hi = b > self.num_buckets - 1
        lo = b < 0
        b = np.where(hi, self.num_buckets - 1, np.where(lo, 0, b))
        loc = np.where(hi, 1.0, np.where(lo, 0.0, loc))
        return b, loc

    def advance(self, v, states):
        """One step for arrays of instances: states (n, S) -> new states (codegen.py:74-106)."""
        b, loc = self.locate(v)
        basis = loc[:, None] ** np.arange(self.num_terms)[None, :]           # (n, T)
        M = np.einsum("ncrt,nt->nrc", self.layout[b], basis)                  # (n, row, col)
        new = np.einsum("nrc,nc->nr", M, states)
        cs = self.scheme.conserve_sum
        if cs is not None:
            new *= (cs / new.sum(axis=1))[:, None]
        return new

    def max_error(self, samples=64):
        """Max |table - exact| over points spread through every bucket."""
        sub = (np.arange(samples) + 0.37) / samples
        v = (self.vmin + (np.arange(self.num_buckets)[:, None] + sub[None, :]) * self.bucket_width).ravel()
        exact = self.scheme.exact_propagator(v, self.dt, self.celsius)
        b, loc = self.locate(v)
        basis = loc[:, None] ** np.arange(self.num_terms)[None, :]
        approx = np.einsum("nrct,nt->nrc", self.table[b], basis)
        return float(np.abs(approx - exact).max())


def table_inputs(rate_fn, to_input, num_buckets, degree, samples_per_bucket):
    """Sample rate matrices and the per-bucket least-squares fit weights of a table:
    sample k of bucket b sits at location (k + 1/2) / samples_per_bucket in the
    bucket (input value to_input(b + location)); the fit of approx.py:159-174 is
    then the same pseudo-inverse for every bucket.  Returns (rates, fit)."""
    nb, spb, T = int(num_buckets), int(samples_per_bucket), int(degree) + 1
    sub = (np.arange(spb) + 0.5) / spb
    pos = (np.arange(nb)[:, None] + sub[None, :]).ravel()
    rates = np.ascontiguousarray(rate_fn(to_input(pos)), dtype=np.float64)
    fit = np.ascontiguousarray(np.linalg.pinv(sub[:, None] ** np.arange(T)[None, :]))
    return rates, fit


def gpu_table(ctx, rates, fit, num_buckets, dt, target=0):
    """lti_sim table generated on the GPU in FP64 (nw_lti_table_build); layout
    [bucket][col][row][term]."""
    from . import _lib
    S = rates.shape[-1]
    T, spb = fit.shape
    table = np.empty((num_buckets, S, S, T))
    ctx.call("nw_lti_table_build", S, int(num_buckets), int(spb), int(T), _lib.ptr(rates), _lib.ptr(fit),
             float(dt), int(target), _lib.ptr(table))
    return table


def scheme_table_gpu(ctx, scheme, dt, celsius, vmin, vmax, num_buckets, degree, samples_per_bucket=20, target=0):
    """The voltage table of a kinetic scheme (LinearInput over [vmin, vmax]) built on the GPU."""
    width = (vmax - vmin) / num_buckets
    rates, fit = table_inputs(lambda v: scheme.matrix(v, celsius), lambda pos: vmin + pos * width,
                              num_buckets, degree, samples_per_bucket)
    return gpu_table(ctx, rates, fit, num_buckets, dt, target)


def optimize_table(ctx, scheme, dt, celsius, accuracy, vmin=-100.0, vmax=60.0, degrees=(1, 2, 3),
                   start_buckets=10, samples_per_bucket=20, test_points=16, max_table_bytes=8 << 20):
    """Smallest table meeting ``accuracy`` (max |table - exact| entry error), as
    lti_sim's optimizer searches it (optimizer.py:184-213): per polynomial degree
    grow the bucket count by max(1.5, 1.7^orders of magnitude of the excess) until
    the error is met, then shrink by 0.9 while it still is.  Tables and the exact
    reference propagators come from the GPU (FP64).  Among the degrees, the one
    with fewest terms per entry whose FP32 table fits ``max_table_bytes`` wins
    (fewer bytes on ties).  Returns dict(num_buckets, degree, max_error, table)."""
    from . import _lib
    S = scheme.num_states

    def error_of(nb, degree):
        table = scheme_table_gpu(ctx, scheme, dt, celsius, vmin, vmax, nb, degree, samples_per_bucket)
        width = (vmax - vmin) / nb
        sub = (np.arange(test_points) + 0.37) / test_points
        pos = (np.arange(nb)[:, None] + sub[None, :]).ravel()
        Q = np.ascontiguousarray(scheme.matrix(vmin + pos * width, celsius))
        exact = np.empty_like(Q)
        ctx.call("nw_lti_expm", S, len(Q), _lib.ptr(Q), float(dt), _lib.ptr(exact))
        exact /= exact.sum(axis=1, keepdims=True)
        b = pos.astype(np.int64)
        loc = pos - b
        basis = loc[:, None] ** np.arange(degree + 1)[None, :]
        approx = np.einsum("ncrt,nt->nrc", table[b], basis)
        return float(np.abs(approx - exact).max()), table

    best = None
    for degree in degrees:
        nb = float(start_buckets)
        err, table = error_of(int(round(nb)), degree)
        lo = 1
        while err > accuracy:
            lo = int(round(nb))
            nb *= max(1.5, 1.7 ** np.log10(err / accuracy))
            if nb > 1e6:
                break
            new_err, new_table = error_of(int(round(nb)), degree)
            if not new_err < err:
                break
            err, table = new_err, new_table
        if err > accuracy:
            continue
        cur = (int(round(nb)), err, table)
        while True:
            nb *= 0.9
            if int(round(nb)) <= lo or int(round(nb)) == cur[0]:
                break
            e2, t2 = error_of(int(round(nb)), degree)
            if e2 > accuracy:
                break
            cur = (int(round(nb)), e2, t2)
        nbytes = cur[0] * S * S * (degree + 1) * 4
        cand = {"num_buckets": cur[0], "degree": degree, "max_error": cur[1], "table": cur[2], "bytes": nbytes}
        key = (nbytes > max_table_bytes, degree + 1, nbytes)
        if best is None or key < best[0]:
            best = (key, cand)
    if best is None:
        raise RuntimeError("no table meets the accuracy")
    return best[1]


class Kinetic(Mechanism):
    """A kinetic-scheme channel with one conductance.

    conductance = gbar[S/cm2] * 1e-8 * magnitude[um2] * sum(open states).  With
    ``ion`` None it is a nonspecific conductance with reversal potential ``erev``;
    with ``ion`` the name of an electric species of the model (``USEION``,
    neuwon/rxd/nmodl/__init__.py:168-208) it is written into that species'
    conductance accumulator and takes the species' reversal potential
    (species.py:155-160).  The step uses a voltage table (LinearInput over
    [vmin, vmax]) built on the GPU for the model's dt and temperature when the
    model is first advanced, or ``table``: a table made elsewhere for that dt and
    temperature, in lti_sim's layout [bucket][col][row][term] (e.g. the
    ``table_data`` lti_sim's code generator emits, reshaped; codegen.py:29-37).
    """
    name = "na8"
    scheme_factory = staticmethod(na8)
    gbar = 0.012
    erev = 50.0
    ion = None
    table = None
    vmin, vmax, num_buckets, degree = -100.0, 60.0, 1600, 1
    # Two-input schemes (KineticScheme2): the table inputs (TableInput, in the
    # scheme's input order), the polynomial terms (powers per input) and the grid
    # samples per input and bucket; the instance value input starts at its
    # TableInput's initial value and reads / writes as "<name>.input".
    inputs, terms, samples_per_axis = None, None, 4
    # A point process (POINT_PROCESS): gbar in S per instance, times the instance's
    # magnitude, instead of a density in S/cm2 times its area.
    point_process = False
    _model = None

    @classmethod
    def configure(cls, **params):
        ok = {"name", "scheme_factory", "gbar", "erev", "ion", "table", "vmin", "vmax", "num_buckets", "degree",
              "inputs", "terms", "samples_per_axis", "point_process"}
        bad = set(params) - ok
        if bad:
            raise ValueError(f"unknown kinetic parameters {sorted(bad)}")
        if "scheme_factory" in params:
            params["scheme_factory"] = staticmethod(params["scheme_factory"])
        return type(cls.__name__, (cls,), dict(params))

    @classmethod
    def initialize(cls, model):
        return type(cls.__name__, (cls,), {"_model": model})

    @classmethod
    def get_name(cls):
        return cls.name

    def __init__(self, segment, outside=None, magnitude=1.0, *other_mechanisms, gbar=None):
        model = type(self)._model
        if model is None:
            raise TypeError("mechanism class is not bound to a model; use model.mechanisms[name]")
        self.segment = segment
        self.magnitude = float(magnitude)
        self.index = model._add_kinetic_instances(type(self), np.array([segment._idx]),
                                                  np.array([self.magnitude]), gbar)

    @classmethod
    def get_database_class(cls):
        return cls

    @classmethod
    def build_table(cls, dt, celsius):
        if cls.inputs is not None:
            return LTITable2(cls.scheme_factory(), dt, celsius, cls.inputs[0], cls.inputs[1], cls.terms,
                             cls.samples_per_axis)
        return LTITable(cls.scheme_factory(), dt, celsius, cls.vmin, cls.vmax, cls.num_buckets, cls.degree)

    @classmethod
    def initial_state(cls, voltage, celsius):
        """The steady state at the initial inputs (voltage; instance values at their
        TableInput's initial value)."""
        sch = cls.scheme_factory()
        if cls.inputs is None:
            return sch.steady_state(voltage, celsius)
        x = [voltage if inp.kind == "voltage" else inp.initial for inp in cls.inputs]
        return sch.steady_state(x[0], x[1], celsius)


# The reference library's kinetic channels restated above, as mechanisms: the
# conductance feeds the channel's ion species (USEION na / USEION k), gbar is the
# PARAMETER default in S/cm2 (Nav11.mod: 0.1 mho/cm2; Kv11.mod: 36 mmho/cm2), and
# the voltage table spans the range the reference's NMODL front end gives a
# voltage input (LinearInput -100..100 mV, neuwon/rxd/nmodl/__init__.py:321-322),
# in 0.1 mV buckets with linear polynomials.
Nav11 = Kinetic.configure(name="na11a", scheme_factory=nav11, gbar=0.1, ion="na", vmin=-100.0, vmax=100.0,
                          num_buckets=2000, degree=1)
Kv11 = Kinetic.configure(name="Kv11_6States_temperature2", scheme_factory=kv11, gbar=0.036, ion="k",
                         vmin=-100.0, vmax=100.0, num_buckets=2000, degree=1)

# The reference library's NMDA receptor (nmodl_library/kinetic/NMDA.mod, POINT_PROCESS
# NMDA_Mg): gmax 500 pS per synapse, Erev 5 mV, NONSPECIFIC_CURRENT; a two-input table
# over the glutamate concentration C (LogarithmicInput 0..1000 mM, the range the
# reference's NMODL front end gives a POINTER, nmodl/__init__.py:323-324; log scale
# 0.01 mM, 30 buckets) and the voltage (LinearInput -100..100 mV, 100 buckets), with
# quadratic polynomials: max entry error 7e-5 at dt 0.1 ms, below the 1e-4 the
# reference's front end asks of lti_sim (nmodl/__init__.py:305).
NMDA = Kinetic.configure(name="NMDA_Mg", scheme_factory=nmda, gbar=500e-12, erev=5.0, point_process=True,
                         inputs=(TableInput("C", "log", 0.0, 1000.0, 30, scale=1e-2),
                                 TableInput("v", "voltage", -100.0, 100.0, 100)),
                         terms=[(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2)])
