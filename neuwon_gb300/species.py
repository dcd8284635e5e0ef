"""Intracellular calcium: a diffusing species with a pump and a sodium-coupled influx.

The reference declares species with ``RxD_Model(species=[...])`` keyword sets of
``_SpeciesType`` (neuwon/rxd/species.py:90-142) and advances each non-constant
intracellular one after every electric half step (species.py:56-70):
``c <- max(0, c + dc/dt * dt/2)`` then ``c <- M c``.  Its builder of the
diffusion propagator M (species.py:74-83) is unfinished; here M is built on
the GPU by the electric propagator's builder (FP64, pruned) from
``d c_i/dt = D A_i / (L_i vol_i) (c_parent - c_i)``.

The mechanisms writing ``dc/dt`` are new (the reference library has a Ca pump
only as NMODL source): a 3-state pump E1 <-> E1Ca -> E2 -> E1 on every segment,
advanced exactly per step by a table over a logarithmic concentration input
(lti_sim's LogarithmicInput, neuwon/rxd/lti_sim/inputs.py:85-109), and an
influx equal to a fraction of the segment's HH sodium current.
"""
import numpy as np
import scipy.linalg

FARADAY = 96485.3321233100184      # C/mol (species.py:8)


class SpeciesType:
    """One entry of ``RxD_Model(species=[...])``: the keywords of the reference's
    ``_SpeciesType`` (neuwon/rxd/species.py:90-142).

    A species with a ``reversal_potential`` is electric: mechanisms that name it as
    their ion write its per-segment conductance accumulator, which enters every
    segment's total conductance and conductance-weighted driving voltage with the
    species' constant reversal potential (``_apply_accumulators``,
    species.py:155-160).  The device computes exactly that sum per segment (no
    mechanism here writes a current into a species: conductances go in,
    nmodl/__init__.py:185).  Keywords without a device path raise instead of
    being ignored:

    * ``reversal_potential="nerst"`` / ``"ghk"``: the reference computes neither
      (``_compute_reversal_potential`` is ``1/0`` past the constant case,
      species.py:165);
    * ``outside_global_constant=False``: extracellular concentrations are not
      stepped on the device;
    * ``inside_global_constant=False`` for a species other than calcium, and a
      finite ``decay_period``: intracellular calcium (``Calcium``) is the one
      diffusing species with a device path.
    """

    def __init__(self, name, *, charge=0, reversal_potential=None, diffusivity=0.0, decay_period=np.inf,
                 inside_initial_concentration=0.0, inside_global_constant=True,
                 outside_initial_concentration=0.0, outside_global_constant=True):
        self.name = str(name)
        self.charge = int(charge)
        self.electric = reversal_potential is not None
        self.reversal_potential = None
        if self.electric:
            try:
                self.reversal_potential = float(reversal_potential)
            except (TypeError, ValueError):
                raise NotImplementedError(
                    f"species {self.name}: reversal potential {reversal_potential!r} has no device path (the "
                    "reference's own Nernst/GHK computation is unfinished); give a constant in mV") from None
            if not np.isfinite(self.reversal_potential):
                raise ValueError(f"species {self.name}: reversal potential must be finite")
        self.diffusivity = float(diffusivity)
        self.decay_period = float(decay_period)
        self.inside_initial_concentration = float(inside_initial_concentration)
        self.inside_global_constant = bool(inside_global_constant)
        self.outside_initial_concentration = float(outside_initial_concentration)
        self.outside_global_constant = bool(outside_global_constant)
        assert self.decay_period > 0.0 and self.diffusivity >= 0.0      # species.py:20-21
        if not self.outside_global_constant:
            raise NotImplementedError(f"species {self.name}: extracellular concentrations have no device path")
        self.calcium = None
        if not self.inside_global_constant:
            if self.name.lower() != "ca":
                raise NotImplementedError(f"species {self.name}: only intracellular calcium is stepped on the device")
            if self.decay_period < np.inf:
                raise NotImplementedError("species ca: a decay period has no device path (diffusion does)")
            self.calcium = Calcium(diffusivity=self.diffusivity, initial=self.inside_initial_concentration,
                                   na_fraction=0.0, pump=False)

    def __repr__(self):
        return f"<Species: {self.name}>"


class Calcium:
    """Parameters of the calcium system (units: um2/ms, mM, 1/ms, mol/um2).

    Rates: E1 -> E1Ca at k1 * c, E1Ca -> E1 at km1, E1Ca -> E2 at k2 (one ion
    out), E2 -> E1 at k3.  ``na_fraction`` of the sodium current enters as Ca2+.
    ``pump_density`` is pump sites per membrane area."""
    name = "ca"

    def __init__(self, diffusivity=0.6, initial=5e-5, na_fraction=0.005, pump=True, pump_density=4e-23,
                 k1=200.0, km1=0.5, k2=1.0, k3=2.0, c_max=1.0, scale=1e-6, num_buckets=400, degree=2,
                 samples_per_bucket=16):
        self.diffusivity = float(diffusivity)
        self.initial = float(initial)
        self.na_fraction = float(na_fraction)
        self.pump = bool(pump)
        self.pump_density = float(pump_density)
        self.k1, self.km1, self.k2, self.k3 = float(k1), float(km1), float(k2), float(k3)
        self.c_max, self.scale = float(c_max), float(scale)
        self.num_buckets, self.degree = int(num_buckets), int(degree)
        self.samples_per_bucket = int(samples_per_bucket)

    # -------------------------------------------------------------- pump
    def generator(self, c):
        """Rate matrices Q(c) (d state/dt = Q state), shape (len(c), 3, 3)."""
        c = np.atleast_1d(np.asarray(c, dtype=np.float64))
        Q = np.zeros((len(c), 3, 3))
        Q[:, 0, 0] = -self.k1 * c
        Q[:, 1, 0] = self.k1 * c
        Q[:, 0, 1] = self.km1
        Q[:, 1, 1] = -(self.km1 + self.k2)
        Q[:, 2, 1] = self.k2
        Q[:, 2, 2] = -self.k3
        Q[:, 0, 2] = self.k3
        return Q

    def exact_propagator(self, c, dt):
        return np.array([scipy.linalg.expm(q * dt) for q in self.generator(c)])

    def steady_state(self, c):
        Q = self.generator([c])[0]
        A = np.vstack([Q, np.ones(3)])
        b = np.array([0.0, 0.0, 0.0, 1.0])
        return np.linalg.lstsq(A, b, rcond=None)[0]

    def log2_min(self):
        return float(np.log2(0.0 + self.scale))

    def bucket_frq(self):
        return self.num_buckets / (np.log2(self.c_max + self.scale) - self.log2_min())

    def locate(self, c):
        """Bucket and in-bucket location as the device computes them."""
        x = (np.log2(np.asarray(c, dtype=np.float64) + self.scale) - self.log2_min()) * self.bucket_frq()
        b = np.trunc(x).astype(np.int64)
        loc = x - b
        hi = b > self.num_buckets - 1
        lo = b < 0
        return np.where(hi, self.num_buckets - 1, np.where(lo, 0, b)), np.where(hi, 1.0, np.where(lo, 0.0, loc))

    def table(self, dt):
        """Least-squares polynomial per bucket of the exact step, layout
        [bucket][col][row][term] (lti_sim/approx.py:159-174, codegen.py:35-37)."""
        nb, T, spb = self.num_buckets, self.degree + 1, self.samples_per_bucket
        sub = (np.arange(spb) + 0.5) / spb
        pos = (np.arange(nb)[:, None] + sub[None, :]).ravel()
        c = 2.0 ** (self.log2_min() + pos / self.bucket_frq()) - self.scale
        exact = self.exact_propagator(c, dt)                      # (n, row, col)
        table = np.empty((nb, 3, 3, T))
        for b in range(nb):
            sel = slice(b * spb, (b + 1) * spb)
            loc = pos[sel] - b
            A = loc[:, None] ** np.arange(T)[None, :]
            coef = np.linalg.lstsq(A, exact[sel].reshape(spb, 9), rcond=None)[0]
            table[b] = coef.reshape(T, 3, 3).transpose(1, 2, 0)   # [row][col][term]
        return np.ascontiguousarray(table.transpose(0, 2, 1, 3))  # [bucket][col][row][term]

    def table_inputs(self):
        """Sample rate matrices and fit weights for the GPU table builder (same
        sample points and fit as ``table``)."""
        from .kinetic import table_inputs
        frq, lo = self.bucket_frq(), self.log2_min()
        return table_inputs(self.generator, lambda pos: 2.0 ** (lo + pos / frq) - self.scale,
                            self.num_buckets, self.degree, self.samples_per_bucket)

    def table_step(self, table, c, states):
        """One step of the tabled pump for arrays of instances (the device's arithmetic)."""
        b, loc = self.locate(c)
        basis = loc[:, None] ** np.arange(table.shape[-1])[None, :]
        M = np.einsum("ncrt,nt->nrc", table[b], basis)
        new = np.einsum("nrc,nc->nr", M, states)
        return new / new.sum(axis=1, keepdims=True)

    # -------------------------------------------------------- coefficients
    def coefficients(self, geom):
        """Per-segment influx (mM/ms per A of Na current) and efflux (mM/ms per bound
        pump fraction) coefficients from the segment geometry (um, um2, um3)."""
        vol_L = np.asarray(geom["volume"], dtype=np.float64) * 1e-15
        influx = self.na_fraction / (2.0 * FARADAY) / vol_L
        sites = self.pump_density * np.asarray(geom["surface_area"], dtype=np.float64)
        efflux = sites * self.k2 * 1e3 / vol_L if self.pump else np.zeros_like(vol_L)
        return influx, efflux
