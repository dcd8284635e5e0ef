"""Electric species and several kinetic mechanisms, pinned against the reference (CPU).

The fixture group ``species_*`` (tests/golden/make_golden.py: run_species) was
recorded by running the reference itself: species ``na`` and ``k`` declared
with constant reversal potentials (neuwon/rxd/species.py:85-160), the restated
hh (nonspecific conductances), and the reference library's Nav1.1 and Kv1.1
channels whose tables and run-time kernels come from the reference's own lti_sim
(LTI_Model, MatrixSamples, Approx1D, Codegen), writing the ``na`` / ``k``
conductance accumulators; two neurons, a duplicated Nav1.1 instance.
"""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.kinetic import LTITable, kv11, nav11
from tests.helpers import FIXTURES, species_oracle

F = np.load(FIXTURES)


def test_oracle_species_matches_reference():
    """1e-8 mV, the bound of the other oracle-vs-reference traces: the reference
    exponentiates both neurons as one matrix, the oracle block by block, and the
    rounding difference grows through the action potentials' upstrokes."""
    om, spec = species_oracle(F)
    probes = spec["probes"]
    trace = F["species_trace"]
    assert np.abs(om.voltage[probes] - trace[0]).max() == 0.0
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    ap = []
    for k in range(steps):
        om.advance()
        assert np.abs(om.voltage[probes] - trace[k + 1]).max() < 1e-8, k
        ap.append(om.AP_detected.copy())
        if k + 1 in (100, 250):
            assert np.abs(om.voltage - F[f"species_snap{k + 1}"]).max() < 1e-8
            for sp, key in (("na", "gna"), ("k", "gk")):
                want = F[f"species_{key}_snap{k + 1}"]
                assert np.abs(om.species_conductance[sp] - want).max() <= 1e-9 * np.abs(want).max()
    assert np.array_equal(np.array(ap), F["species_ap"])
    assert np.array_equal(F["species_ap"].sum(axis=0), [1, 1])     # both neurons fire


@pytest.mark.parametrize("factory, key", [(nav11, "nav"), (kv11, "kv")])
def test_library_channel_tables_match_reference_lti_sim(factory, key):
    """This package's table builder, given the reference's sample points, equals the
    reference's Approx1D table (approx.py:159-174); the initial state equals
    LTI_Model.get_initial_state (lti_model.py:67-78)."""
    spec_meta = F["species_meta"]
    dt, celsius, v_init = spec_meta[0], spec_meta[1], spec_meta[3]
    sch = factory()
    tbl = LTITable(sch, dt, celsius, -100.0, 100.0, 2000, 1, sample_inputs=F[f"species_{key}_samples"])
    ref = F[f"species_{key}_table10"]                     # every 10th bucket of the reference's table
    assert tbl.layout.shape == (2000, 6, 6, 2) and ref.shape == (200, 6, 6, 2)
    assert np.abs(tbl.layout[::10] - ref).max() < 1e-12
    assert np.abs(sch.steady_state(v_init, celsius) - F[f"species_{key}_init"]).max() < 1e-12


def test_library_channel_tables_meet_reference_accuracy():
    """lti_sim's target is 1e-4 max entry error (nmodl/__init__.py:305); the 0.1 mV
    linear tables of the restated channels meet it."""
    for factory in (nav11, kv11):
        tbl = LTITable(factory(), 0.1, 20.0, -100.0, 100.0, 2000, 1)
        assert tbl.max_error(samples=4) < 1e-4


def test_species_keywords_on_the_model():
    m = nw.RxD_Model(species=[dict(name="na", charge=1, reversal_potential=50),
                              dict(name="k", charge=1, reversal_potential=-77), dict(name="cl", charge=-1)],
                     mechanisms=[nw.Nav11, nw.Kv11])
    assert list(m.species) == ["na", "k", "cl"]
    assert m.species["na"].reversal_potential == 50.0 and not m.species["cl"].electric
    assert set(m.mechanisms) == {"na11a", "Kv11_6States_temperature2"}
    with pytest.raises(ValueError, match="electric species 'na'"):
        nw.RxD_Model(mechanisms=[nw.Nav11])
    with pytest.raises(ValueError, match="electric species 'k'"):
        nw.RxD_Model(species=[dict(name="k", charge=1)], mechanisms=[nw.Kv11])
    with pytest.raises(NotImplementedError):
        nw.RxD_Model(species=[dict(name="na", reversal_potential="ghk")])
    with pytest.raises(ValueError):
        nw.RxD_Model(duplicates="drop")


def test_many_kinetic_mechanisms_allowed_up_to_the_device_limit():
    mechs = [nw.Kinetic.configure(name=f"k{i}") for i in range(8)]
    nw.RxD_Model(mechanisms=mechs)
    with pytest.raises(NotImplementedError):
        nw.RxD_Model(mechanisms=mechs + [nw.Kinetic.configure(name="k8")])
    with pytest.raises(NotImplementedError):
        nw.RxD_Model(mechanisms=[nw.HH, nw.HH.configure(name="hh2")])


def test_oracle_duplicates_count_in_species_but_not_nonspecific():
    """A species accumulator is written instance by instance (every duplicate counts);
    a nonspecific conductance is scattered with a fancy-index "+=", which keeps one
    (species.py:256-260)."""
    from oracle.reference_step import KineticInstances, OracleModel
    from neuwon_gb300.morphology import geometry, passive_electric, random_tree
    t = random_tree(12, seed=3)
    R, C = passive_electric(geometry(t))
    layout = np.zeros((4, 1, 1, 1)); layout[...] = 1.0           # one always-open state
    seg = np.array([0, 1, 2, 2])
    for species, dup, want in ((None, "numpy", 1.0), (None, "sum", 2.0), ("x", "numpy", 2.0)):
        k = KineticInstances(seg, np.full(4, 1e-9), layout, -100.0, 0.02, [0], 10.0, 1.0, [1.0], species=species)
        om = OracleModel(t.parent, R, C, kinetic=[k], duplicates=dup, species={"x": 10.0})
        om._advance_mechanisms()
        om.sum_conductance.fill(0.0)
        om._advance_species()
        # The pre-division sum on segment 2: sum_conductance keeps it after the step.
        assert om.sum_conductance[2] == pytest.approx(want * 1e-9)
