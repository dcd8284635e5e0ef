"""Electric species and several kinetic mechanisms on the GPU, through the C ABI.

The scenario (species ``na`` and ``k`` with constant reversal potentials; the
restated hh plus the reference library's Nav1.1 -> na and Kv1.1 -> k channels;
two neurons; a duplicated Nav1.1 instance) was recorded by running the
reference itself (tests/golden/make_golden.py: run_species).

Tolerances (the tables are the reference's lti_sim tables, rebuilt from its
sample points and installed as given):
  * FP64 paths against the FP64 oracle, with the oracle's propagator installed on
    the device: 1e-7 mV, species conductance accumulators 1e-9 relative;
  * FP64 paths with the propagator the GPU builds, against the voltages the
    reference recorded: 5e-7 mV.  The build equals scipy's expm to about 1e-13 per
    entry (tests/test_gpu_parity.py); the upstrokes of the scenario's two action
    potentials amplify that difference to 1.2e-7 mV at most;
  * FP32 against the FP64 oracle: 0.1 mV with equal spike counts.
"""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.kinetic import LTITable, kv11, nav11
from tests.helpers import FIXTURES, gpu_model, oracle_case, run_with_clamps, species_gpu, species_oracle

pytestmark = pytest.mark.gpu
F = np.load(FIXTURES)


def _run(m, spec, offs, recs):
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    snaps = {}
    for k in range(steps):
        run_with_clamps(m, spec["clamps"], offs, 1)
        if k + 1 in (100, 250):
            snaps[k + 1] = (m.get_data("Segment.voltage"), m.get_data("Segment.na_conductance"),
                            m.get_data("Segment.k_conductance"))
    return np.array([r.get_data() for r in recs]).T, snaps


@pytest.mark.parametrize("path", ["batched", "wide", "plain"])
def test_species_f64_matches_oracle(path):
    om, spec = species_oracle(F)
    m, spec, offs, recs = species_gpu(F, precision="f64", path=path, propagator=om.P)
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    for k in range(steps):
        run_with_clamps(m, spec["clamps"], offs, 1)
        om.advance()
        if k % 25 == 24:
            assert np.abs(m.get_data("Segment.voltage") - om.voltage).max() < 1e-7, k
            for sp in ("na", "k"):
                want = om.species_conductance[sp]
                got = m.get_data(f"Segment.{sp}_conductance")
                assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert np.array_equal(om.spike_count, [1, 1])
    m.close()


@pytest.mark.parametrize("path", ["batched", "wide", "plain"])
def test_species_f64_matches_reference(path):
    m, spec, offs, recs = species_gpu(F, precision="f64", path=path)
    got, snaps = _run(m, spec, offs, recs)
    ref = F["species_trace"]
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() < 5e-7
    for k, (v, gna, gk) in snaps.items():
        assert np.abs(v - F[f"species_snap{k}"]).max() < 5e-7
        for g, key in ((gna, "gna"), (gk, "gk")):
            want = F[f"species_{key}_snap{k}"]
            assert np.abs(g - want).max() <= 1e-6 * np.abs(want).max()
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), F["species_ap"].sum(axis=0))
    m.close()


@pytest.mark.parametrize("path", ["batched", "wide"])
def test_species_f32_matches_oracle(path):
    om, spec = species_oracle(F)
    m, spec, offs, _ = species_gpu(F, precision="f32", path=path)
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    worst = 0.0
    for k in range(steps):
        run_with_clamps(m, spec["clamps"], offs, 1)
        om.advance()
        if k % 10 == 9:
            worst = max(worst, float(np.abs(m.get_data("Segment.voltage") - om.voltage).max()))
    assert worst < 0.1, worst
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert om.spike_count.sum() >= 2
    m.close()


def test_species_with_gpu_built_tables_matches_oracle():
    """Without given tables the model builds the Nav1.1 / Kv1.1 tables on the GPU (FP64);
    against the oracle holding the host FP64 build of the same tables: 1e-7 mV."""
    spec_meta = F["species_meta"]
    dt, celsius, v_init = float(spec_meta[0]), float(spec_meta[1]), float(spec_meta[3])
    tables = {}
    for key, factory in (("nav", nav11), ("kv", kv11)):
        sch = factory()
        tables[key] = (LTITable(sch, dt, celsius, -100.0, 100.0, 2000, 1).layout, sch.steady_state(v_init, celsius))
    om, spec = species_oracle(F, tables=tables)
    m, spec, offs, _ = species_gpu(F, precision="f64", reference_tables=False)
    steps = int(round(spec["t_stop"] / spec["time_step"]))
    for k in range(steps):
        run_with_clamps(m, spec["clamps"], offs, 1)
        om.advance()
    assert np.abs(m.get_data("Segment.voltage") - om.voltage).max() < 1e-7
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    states = m.get_data("na11a.state")
    assert states.shape == (len(om.kinetic[0].segment), 6)
    assert np.abs(states - om.kinetic[0].state).max() < 1e-9
    m.close()


def test_species_checkpoint_roundtrip(tmp_path):
    """Save mid-run, continue, restore, continue again: bit-identical, for two kinetic mechanisms."""
    m, spec, offs, _ = species_gpu(F, precision="f32")
    run_with_clamps(m, spec["clamps"], offs, 60)
    path = str(tmp_path / "species.sqlite")
    m.save_sqlite(path)
    run_with_clamps(m, spec["clamps"], offs, 40)
    v1 = m.get_data("Segment.voltage")
    kv1 = m.get_data("Kv11_6States_temperature2.state")
    m.load_sqlite(path)
    run_with_clamps(m, spec["clamps"], offs, 40)
    assert np.array_equal(m.get_data("Segment.voltage"), v1)
    assert np.array_equal(m.get_data("Kv11_6States_temperature2.state"), kv1)
    m.close()


@pytest.mark.parametrize("path", ["batched", "plain", "wide"])
def test_duplicates_reference_mode_matches_reference_fixture(path):
    """duplicates='reference': of several hh instances on one segment only the last
    counts, as the reference's fancy-index "+=" (species.py:256-260) gives; the
    reference's own recorded traces of the three-neuron case with two duplicated
    instances are reproduced to 1e-7 mV."""
    trees = [nw.random_tree(40, seed=21), nw.random_tree(25, seed=22), nw.random_tree(60, seed=23)]
    clamps = [(0, 0, 0.3, 1., 6.), (1, 5, 0.2, 2., 3.), (2, 30, 0.25, 0.5, 8.)]
    ref = F["multi_trace"]
    m, neurons, offs, recs = gpu_model(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3), (2, 30)],
                                       precision="f64", path=path, probes=list(F["multi_probes"]),
                                       duplicates="reference")
    run_with_clamps(m, clamps, offs, len(ref) - 1)
    got = np.array([r.get_data() for r in recs]).T
    assert np.abs(got - ref).max() < 1e-7
    assert np.abs(m.get_data("Segment.voltage") - F["multi_snap150"]).max() < 1e-7
    om, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3), (2, 30)], duplicates="sum")
    for _ in range(len(ref) - 1):
        om.advance()
    assert np.abs(m.get_data("Segment.voltage") - om.voltage).max() > 1e-3    # the modes differ on this case
    m.close()


def test_nmodl_channels_on_device_match_oracle(tmp_path):
    """Channel files read by the NMODL front end (a three-state K channel feeding
    species k, a passive leak) run on the device next to HH: FP64 against the
    oracle holding the host build of the same tables, 1e-7 mV."""
    from neuwon_gb300.kinetic import LTITable
    from oracle.reference_step import HHInstances, KineticInstances, OracleModel, clamp_ticks
    from tests.helpers import concat
    from tests.test_nmodl import KTEST, PASSIVE
    (tmp_path / "ktest.mod").write_text(KTEST)
    (tmp_path / "leak.mod").write_text(PASSIVE)
    tree = nw.random_tree(150, seed=3)
    celsius, dt, steps = 6.3, 0.1, 300
    hh_kw = dict(ena=50.0, ek=-77.0, el=-54.3)
    m = nw.RxD_Model(time_step=dt, temperature=celsius, precision="f64",
                     species=[dict(name="k", charge=1, reversal_potential=-80.0)],
                     mechanisms=[nw.HH.configure(**hh_kw), str(tmp_path / "ktest.mod"), str(tmp_path / "leak.mod")])
    nr = m.add_tree(tree)
    for name in ("hh", "ktest", "leak"):
        m.insert_everywhere(name)
    nr.root.inject_current(1.0, 20.0)
    parent, R, C, area, offs = concat([tree])
    n = len(tree)
    seg = np.arange(n)
    kins = []
    for name, species, erev in (("ktest", "k", 0.0), ("leak", None, m.mechanisms["leak"].erev)):
        cls = m.mechanisms[name]
        sch = cls.scheme_factory()
        tbl = LTITable(sch, dt, celsius, -100.0, 100.0, 2000, 1)
        kins.append(KineticInstances(seg, cls.gbar * 1e-8 * area, tbl.layout, -100.0, tbl.bucket_frq,
                                     sch.open_states, erev, sch.conserve_sum, sch.steady_state(-70.0, celsius),
                                     species=species))
    f, c = clamp_ticks(0.0, 20.0, dt)
    om = OracleModel(parent, R, C, time_step=dt, celsius=celsius, hh=HHInstances(seg, area, celsius=celsius, **hh_kw),
                     kinetic=kins, species={"k": -80.0}, clamps=[(0, 1.0e-9, f, c)], detectors=[(0, 20.0)])
    m.advance(steps)
    for _ in range(steps):
        om.advance()
    assert np.abs(m.get_data("Segment.voltage") - om.voltage).max() < 1e-7
    assert np.abs(m.get_data("ktest.state") - om.kinetic[0].state).max() < 1e-9
    np.testing.assert_array_equal(m.get_data("Neuron.spike_count"), om.spike_count)
    assert om.spike_count[0] >= 1
    m.close()
