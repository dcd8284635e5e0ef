"""Kinetic schemes (lti_sim): the table builder and run-time step against the
reference's own lti_sim output, and the 8-state sodium scheme against HH."""
import numpy as np
import pytest
import scipy.linalg

from neuwon_gb300.kinetic import LTITable, binomial_state, hh_sodium_rates, na8
from oracle.reference_step import KineticInstances, hh_rates
from tests.helpers import FIXTURES

F = np.load(FIXTURES)


def test_table_matches_reference_lti_sim():
    """Same sample points as the reference's MatrixSamples -> same least-squares table."""
    t = LTITable(na8(), 0.1, 6.3, sample_inputs=F["lti_samples"])
    assert np.abs(t.table - F["lti_table"]).max() < 1e-13


def test_runtime_step_matches_reference_approximation():
    t = LTITable(na8(), 0.1, 6.3, sample_inputs=F["lti_samples"])
    new = t.advance(F["lti_v"], F["lti_state"])
    assert np.abs(new - F["lti_new"]).max() < 1e-14


def test_oracle_kinetic_step_matches_reference():
    """The oracle's codegen restatement on the reference's own table."""
    sch = na8()
    layout = F["lti_table"].transpose(0, 2, 1, 3)
    v = F["lti_v"]
    ki = KineticInstances(np.arange(len(v)), 1.0, layout, -100.0, 1600 / 160.0, sch.open_states, 50.0,
                          1.0, np.zeros(8))
    ki.state = F["lti_state"].copy()
    ki.advance(v)
    assert np.abs(ki.state - F["lti_new"]).max() < 1e-14


def test_deterministic_table_error_within_reference_target():
    """The reference optimises tables to 1e-4 max error (nmodl/__init__.py:305)."""
    t = LTITable(na8(), 0.1, 6.3)
    assert t.max_error(16) < 1e-5


def test_na8_is_the_markov_form_of_hh_sodium():
    """With exact propagators, the open state of Na8 equals m^3 h along any voltage path."""
    sch = na8()
    rng = np.random.default_rng(0)
    v_path = np.concatenate([np.full(20, -65.0), rng.uniform(-90, 40, 200)])
    m0, _, h0, _, _, _ = hh_rates(np.array([-65.0]), 6.3)
    m, h = m0[0], h0[0]
    s = binomial_state(m, h)
    dt = 0.1
    for v in v_path:
        P = scipy.linalg.expm(sch.matrix([v], 6.3)[0] * dt)
        s = P @ s
        am, bm, ah, bh = hh_sodium_rates(np.array([v]), 6.3)
        minf, mt = am[0] / (am[0] + bm[0]), 1 / (am[0] + bm[0])
        hinf, ht = ah[0] / (ah[0] + bh[0]), 1 / (ah[0] + bh[0])
        m = minf + (m - minf) * np.exp(-dt / mt)
        h = hinf + (h - hinf) * np.exp(-dt / ht)
        assert abs(s[3] - m ** 3 * h) < 1e-12
    assert abs(s.sum() - 1.0) < 1e-12


def test_locate_matches_generated_kernel_rules():
    """Truncation toward zero and clamping (codegen.py:43-59)."""
    t = LTITable(na8(), 0.1, 6.3)
    b, loc = t.locate(np.array([-100.0, -100.05, -100.2, 59.99, 60.0, 70.0, -50.0]))
    assert list(b[:3]) == [0, 0, 0]
    assert loc[0] == 0.0 and loc[1] == pytest.approx(-0.5) and loc[2] == 0.0
    assert b[3] == 1599 and b[4] == 1599 and loc[4] == 1.0 and loc[5] == 1.0
    assert b[6] == 500 and loc[6] == pytest.approx(0.0, abs=1e-9)


def test_table_inputs_fit_equals_host_least_squares():
    """The GPU builder's inputs (sample rate matrices, one pseudo-inverse for every
    bucket) reproduce the host table when the exponentials are taken on the host."""
    import scipy.linalg
    from neuwon_gb300.kinetic import LTITable, na8, table_inputs
    sch = na8()
    nb, deg, spb = 200, 1, 20
    rates, fit = table_inputs(lambda v: sch.matrix(v, 6.3), lambda pos: -100.0 + pos * 160.0 / nb, nb, deg, spb)
    P = np.array([scipy.linalg.expm(q * 0.1) for q in rates])
    P /= P.sum(axis=1, keepdims=True)
    table = np.einsum("ts,bsrc->bcrt", fit, P.reshape(nb, spb, 8, 8))
    host = LTITable(sch, 0.1, 6.3, num_buckets=nb, degree=deg, samples_per_bucket=spb)
    assert np.abs(table - host.layout).max() < 1e-12


def _nmda_inputs(nb_c=4, nb_v=8):
    from neuwon_gb300.kinetic import TableInput
    return (TableInput("C", "log", 0.0, 1000.0, nb_c, scale=1e-2), TableInput("v", "voltage", -100.0, 100.0, nb_v))


def test_two_input_table_matches_reference_approx2d():
    """NMDA.mod's scheme on the reference's own random samples: the least-squares
    table, the approximate matrices at test points (clamped outside the table) and
    the canonical term order equal the reference's Approx2D."""
    from neuwon_gb300.kinetic import LTITable2, canonical_terms, nmda
    terms = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2)]
    assert [tuple(t) for t in F["lti2_terms"]] == canonical_terms(terms)
    i1, i2 = _nmda_inputs()
    t = LTITable2(nmda(), 0.1, 6.3, i1, i2, terms, sample_inputs=(F["lti2_samples_C"], F["lti2_samples_v"]))
    ref = F["lti2_table"].reshape(t.table.shape)
    assert np.abs(t.table - ref).max() < 1e-10 * max(1.0, np.abs(ref).max())
    assert np.abs(t.approximate(F["lti2_C"], F["lti2_v"]) - F["lti2_approx"]).max() < 1e-9


def test_two_input_initial_state_matches_reference():
    from neuwon_gb300.kinetic import nmda
    assert np.abs(nmda().steady_state(0.0, -100.0, 6.3) - F["lti2_init"]).max() < 1e-10


def test_oracle_two_input_step_matches_reference_approximation():
    """The oracle's restatement of the generated two-input kernel, on the reference's
    table: state' = M(C, v) state, then CONSERVE."""
    from neuwon_gb300.kinetic import nmda
    sch = nmda()
    i1, i2 = _nmda_inputs()
    layout = F["lti2_table"].reshape(32, 10, 10, 6).transpose(0, 2, 1, 3)
    C, v = F["lti2_C"], F["lti2_v"]
    ki = KineticInstances(np.arange(len(v)), 1.0, layout, 0.0, 1.0, sch.open_states, 5.0, 1.0, np.zeros(10),
                          inputs=[("log", 4, 0.0, i1.bucket_frq, 1e-2), ("voltage", 8, -100.0, i2.bucket_frq, 1.0)],
                          powers=F["lti2_terms"], input_values=C)
    rng = np.random.default_rng(3)
    st = rng.dirichlet(np.ones(10), len(v))
    ki.state = st.copy()
    ki.advance(v)
    want = np.einsum("nrc,nc->nr", F["lti2_approx"], st)
    want /= want.sum(axis=1, keepdims=True)
    assert np.abs(ki.state - want).max() < 1e-12


def test_nmda_table_within_reference_target():
    """The default NMDA table (30 log buckets of C, 100 of v, quadratic) meets the
    1e-4 max entry error the reference's front end asks of lti_sim."""
    from neuwon_gb300.kinetic import NMDA
    t = NMDA.build_table(0.1, 6.3)
    assert t.max_error(2) < 1e-4
