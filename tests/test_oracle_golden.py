"""The oracle pinned against the reference (CPU only).

Fixtures in tests/golden/reference_fixtures.npz were produced by running the
reference NEUWON itself (tests/golden/make_golden.py).  The reference test
suite's own golden HH trace (neuwon/rxd/tests/test_model.py:77-113) is
restated below as data with its tolerance.
"""
import math

import numpy as np
import pytest
import scipy.sparse

from neuwon_gb300.morphology import Tree, geometry, passive_electric, random_tree
from oracle.reference_step import OracleModel, clamp_ticks, propagator
from tests.helpers import FIXTURES, concat, oracle_case, tree11

F = np.load(FIXTURES)

# neuwon/rxd/tests/test_model.py:77-97: tip voltage every 0.1 ms for 20 ms,
# rounded to 0.01 mV by the reference's author; the test allows 30 mV.
GOLDEN_TIP = [
    -70.0, -69.75, -69.5, -69.26, -69.02, -68.8, -68.58, -68.37, -68.16, -67.97, -67.78,
    -67.59, -67.42, -67.25, -67.08, -66.92, -66.77, -66.63, -66.48, -66.35, -66.22,
    -66.09, -65.98, -65.86, -65.75, -65.65, -65.55, -65.46, -65.37, -65.29, -65.21,
    -65.14, -65.07, -65.01, -64.96, -64.9, -64.86, -64.82, -64.79, -64.76, -64.73, -64.72,
    -64.7, -64.7, -64.7, -64.7, -64.71, -64.73, -64.75, -64.77, -64.8, -57.95, -51.25,
    -44.26, -35.5, -20.62, 10.85, 48.59, 55.34, 53.32, 50.03, 44.2, 39.32, 33.97,
    28.32, 22.52, 16.68, 10.88,
    5.19, -0.39, -5.83, -11.15, -16.38, -21.56, -26.77, -32.15, -37.95, -44.6, -52.76,
    -63.07, -74.33, -82.23, -85.48, -86.52, -86.82, -86.89, -86.88, -86.83, -86.77,
    -86.7, -86.63, -86.55, -86.47, -86.38, -86.3, -86.2, -86.1, -86.0, -85.9, -85.78,
    -85.67, -85.55, -85.43, -85.3, -85.16, -85.03, -84.88, -84.74, -84.58, -84.43, -84.27,
    -84.1, -83.93, -83.76, -83.58, -83.4, -83.21, -83.02, -82.82, -82.62, -82.42, -82.21,
    -82.0, -81.79, -81.57, -81.36, -81.13, -80.91, -80.68, -80.45, -80.22, -79.99, -79.76,
    -79.52, -79.28, -79.05, -78.81, -78.57, -78.33, -78.09, -77.85, -77.61, -77.37,
    -77.13, -76.89, -76.66, -76.42, -76.19, -75.95, -75.72, -75.49, -68.42, -61.74,
    -55.41, -49.28, -42.78, -34.19, -18.72, 14.02, 49.11, 54.24, 50.38, 46.96,
    42.66, 37.71, 32.32, 26.67, 20.9, 15.11, 9.39,
    3.76, -1.74, -7.12, -12.39, -17.58, -22.74, -27.97, -33.41, -39.35, -46.28, -54.92,
    -65.71, -76.65, -83.36, -85.87, -86.65, -86.87, -86.9, -86.88, -86.83, -86.77, -86.7,
    -86.62, -86.54, -86.46, -86.38, -86.29, -86.19, -86.09, -85.99, -85.88]


def test_geometry_matches_reference():
    t = Tree(F["geom_parent"], F["geom_coordinates"], F["geom_diameter"])
    g = geometry(t)
    R, C = passive_electric(g)
    for k in ("length", "surface_area", "cross_sectional_area", "volume"):
        np.testing.assert_allclose(g[k], F["geom_" + k], rtol=1e-13)
    np.testing.assert_allclose(R, F["geom_axial_resistance"], rtol=1e-13)
    np.testing.assert_allclose(C, F["geom_capacitance"], rtol=1e-13)
    assert np.array_equal(g["primary"], F["geom_primary"])


def test_propagator_matches_reference():
    t = Tree(F["geom_parent"], F["geom_coordinates"], F["geom_diameter"])
    R, C = passive_electric(geometry(t))
    P = propagator(t.parent, R, C, 0.05)
    Pr = scipy.sparse.csr_matrix((F["prop_data"], F["prop_indices"], F["prop_indptr"]))
    assert abs(P - Pr).max() < 1e-14
    # Charge conservation check of neuwon/rxd/tests/test_electric.py:84-85.
    assert np.sum(P.data) / P.shape[0] == pytest.approx(1.0)


CASES = [
    ("hh11", [tree11()], [(0, 0, .1, 5., 1.), (0, 0, .1, 15., 1.)], {}, (), True),
    ("hh200", [random_tree(200, seed=11)], [(0, 0, 0.2, 5., 20.)],
     dict(ena=50., ek=-77., el=-54.3), (), False),
    ("multi", [random_tree(40, seed=21), random_tree(25, seed=22), random_tree(60, seed=23)],
     [(0, 0, 0.3, 1., 6.), (1, 5, 0.2, 2., 3.), (2, 30, 0.25, 0.5, 8.)],
     dict(ena=50., ek=-77.), [(0, 3), (2, 30)], False),
]


@pytest.mark.parametrize("prefix,trees,clamps,hh_kw,dups,as_created", CASES)
def test_oracle_traces_match_reference(prefix, trees, clamps, hh_kw, dups, as_created):
    om, _ = oracle_case(trees, clamps, hh_kw=hh_kw, dups=dups, duplicates="numpy",
                        insert_as_created=as_created)
    ref = F[prefix + "_trace"]
    probes = F[prefix + "_probes"]
    mine = [om.voltage[probes].copy()]
    for _ in range(len(ref) - 1):
        om.advance()
        mine.append(om.voltage[probes].copy())
    assert np.abs(np.array(mine) - ref).max() < 1e-8
    np.testing.assert_array_equal(om.AP_detected, F[prefix + "_ap"][-1])


def test_oracle_single_neuron_config_matches_reference():
    """The single-neuron configuration at full size: 2,000 segments, HH, 0.2 nA soma
    clamp 5-80 ms, dt 0.1 ms for 100 ms; every segment's voltage every 10 ms against
    the reference's own run (epsilon-pruned propagator on both sides)."""
    clamps = [(0, 0, 0.2, 5.0, 75.0)]
    om, _ = oracle_case([random_tree(2000, seed=0)], clamps, hh_kw=dict(ena=50., ek=-77., el=-54.3),
                        duplicates="numpy")
    probes = F["c1_probes"]
    trace = [om.voltage[probes].copy()]
    worst = 0.0
    for k in range(1000):
        om.advance()
        trace.append(om.voltage[probes].copy())
        if (k + 1) % 100 == 0:
            worst = max(worst, np.abs(om.voltage - F[f"c1_snap{k + 1}"]).max())
    assert worst < 1e-8, worst
    assert np.abs(np.array(trace) - F["c1_trace"]).max() < 1e-8
    assert int(om.spike_count[0]) == int(F["c1_ap"].sum())


def test_duplicate_instances_reference_drops_one():
    """species.py:256-260 drops duplicate segment indices; the sum differs."""
    trees = [random_tree(40, seed=21), random_tree(25, seed=22), random_tree(60, seed=23)]
    clamps = [(0, 0, 0.3, 1., 6.), (1, 5, 0.2, 2., 3.), (2, 30, 0.25, 0.5, 8.)]
    a, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3)], duplicates="numpy")
    b, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), dups=[(0, 3)], duplicates="sum")
    for _ in range(50):
        a.advance(); b.advance()
    assert np.abs(a.voltage - b.voltage).max() > 1e-3


def test_oracle_against_reference_test_golden_trace():
    """neuwon/rxd/tests/test_model.py:35-128 with its 30 mV tolerance."""
    om, _ = oracle_case([tree11()], [(0, 0, .1, 5., 1.), (0, 0, .1, 15., 1.)], insert_as_created=True)
    trace = [om.voltage[10]]
    for _ in range(200):
        om.advance()
        trace.append(om.voltage[10])
    diff = np.abs(np.array(trace) - np.array(GOLDEN_TIP))
    assert diff.max() < 30
    assert diff.max() < 3.0    # observed 2.98 mV (the reference changed after the golden was taken)
    assert om.spike_count[0] == 2


def _sphere(diameter=20.0):
    return Tree([-1], [[0, 0, 0]], [diameter])


def test_time_constant():
    """neuwon/rxd/tests/test_electric.py:28-46."""
    t = _sphere(20.0)
    R, C = passive_electric(geometry(t))
    G = 1e-10
    tau = C[0] / G
    nstep = 1000
    dt = tau / nstep * 1e3
    om = OracleModel(t.parent, R, C, time_step=2 * dt, celsius=6.3, v_init=0.0)
    # _advance_electric(dt) directly with driving voltage 1 and conductance G.
    for _ in range(nstep):
        om.sum_current[:] = 0.0
        om.sum_conductance[:] = G
        om.driving_voltage[:] = 1.0
        om._advance_electric(dt)
    assert om.voltage[0] == pytest.approx(1 - 1 / np.e)


def test_inject_current_charge():
    """neuwon/rxd/tests/test_electric.py:132-150: delta Q = I t on a passive sphere."""
    t = _sphere(10.0)
    R, C = passive_electric(geometry(t))
    f, c = clamp_ticks(3.0, 2.0, 0.01)
    om = OracleModel(t.parent, R, C, time_step=0.01, celsius=37, clamps=[(0, 1e-9, f, c)])
    for _ in range(300):
        om.advance()
    init_Q = 1e-3 * om.voltage[0] * C[0]
    for _ in range(300):
        om.advance()
    new_Q = 1e-3 * om.voltage[0] * C[0]
    assert init_Q + 1e-9 * 2e-3 == pytest.approx(new_Q)


@pytest.mark.parametrize("diam,rm,max_len,dt,ptol", [(1, 4e11, 2, .01, .05), (.9, 2e11, 10, .025, .15)])
def test_length_constant(diam, rm, max_len, dt, ptol):
    """neuwon/rxd/tests/test_electric.py:48-130 on a 3 mm cable."""
    from neuwon_gb300 import RxD_Model
    m = RxD_Model()
    root = m.Neuron([0, 0, 0], diam).root
    section = [root] + root.add_section([3000, 0, 0], diam, max_len)
    idx = np.array([s.get_unstable_index() for s in section])
    g = m._geometry()
    parent = m._parent[:m._n]
    R, C = g["axial_resistance"], g["capacitance"]
    om = OracleModel(parent, R, C, time_step=2 * dt, celsius=37, v_init=0.0)
    G = g["surface_area"] / rm
    probe = len(section) // 2
    rm_len = 1.0 / (G[probe] / g["length"][probe])
    ri = R[probe] / g["length"][probe]
    lam = (rm_len / ri) ** 0.5
    for _ in range(round(10 / dt)):
        om.voltage[probe] = 1.0
        om.sum_current[:] = 0.0
        om.sum_conductance[:] = G
        om.driving_voltage[:] = 0.0
        om._advance_electric(dt)
    xs = m._coords[idx, 0]
    import bisect
    test = bisect.bisect_left(list(xs), xs[probe] + lam)
    ratio = om.voltage[test] / om.voltage[probe]
    assert ratio == pytest.approx(1 / np.e, ptol)
    assert np.sum(om.P.data) / om.P.shape[0] == pytest.approx(1)


def test_c_oracle_matches_numpy_oracle():
    from oracle.cpu_oracle import CpuOracle
    om, d = oracle_case([random_tree(150, seed=5), random_tree(90, seed=6)],
                        [(0, 0, 0.3, 1., 10.), (1, 10, 0.25, 2., 5.)], hh_kw=dict(ena=50., ek=-77.))
    P = om.P
    co = CpuOracle(P.indptr, P.indices, P.data, d["C"], time_step=0.1, celsius=6.3,
                   hh=dict(segment=d["seg"], gna=om.hh.gna_coef, gk=om.hh.gk_coef, gl=om.hh.gl_coef,
                           ena=50., ek=-77., el=-54.3),
                   clamps=d["clamps"], detectors=[(o, 20.0) for o in d["offs"]])
    for _ in range(200):
        om.advance()
        co.advance()
    assert np.abs(om.voltage - co.V).max() < 1e-9
    np.testing.assert_array_equal(om.spike_count, co.spike_count)


def test_c_oracle_with_kinetic_matches_numpy_oracle():
    """The C oracle's kinetic step (table lookup, CONSERVE) equals the numpy oracle's."""
    from oracle.cpu_oracle import CpuOracle
    om, d = oracle_case([random_tree(150, seed=5), random_tree(90, seed=6)],
                        [(0, 0, 0.3, 1., 10.), (1, 10, 0.25, 2., 5.)], hh_kw=dict(ena=50., ek=-77.),
                        kinetic=True)
    P = om.P
    k = om.kinetic[0]
    co = CpuOracle(P.indptr, P.indices, P.data, d["C"], time_step=0.1, celsius=6.3,
                   hh=dict(segment=d["seg"], gna=om.hh.gna_coef, gk=om.hh.gk_coef, gl=om.hh.gl_coef,
                           ena=50., ek=-77., el=-54.3),
                   clamps=d["clamps"], detectors=[(o, 20.0) for o in d["offs"]],
                   kinetic=dict(segment=k.segment, gcoef=k.g_coef, table=k.layout, vmin=k.vmin,
                                bucket_frq=k.frq, open=k.open_states, erev=k.erev, conserve=k.conserve_sum,
                                init=k.state[0].copy()))
    for _ in range(200):
        om.advance()
        co.advance()
    assert np.abs(om.voltage - co.V).max() < 1e-9
    assert np.abs(om.kinetic[0].state - co.kstate.T).max() < 1e-12
    np.testing.assert_array_equal(om.spike_count, co.spike_count)


def test_clamp_ticks_match_reference_timeseries():
    """time.py:276-279: ceil(duration / half_step) plays, first on the next tick."""
    assert clamp_ticks(5.0, 1.0, 0.1) == (101, 20)
    assert clamp_ticks(5.0, 75.0, 0.1) == (101, math.ceil(75.0 / 0.05))
    assert clamp_ticks(0.0, 0.3, 0.1) == (1, 6)


def test_lumped_pruning_keeps_rows_and_beats_dropping():
    """Moving each pruned entry to the nearest kept entry on the tree path keeps
    every row sum and is far closer to the unpruned step than returning the
    pruned mass to the diagonal."""
    from oracle.reference_step import lump_and_conserve
    trees = [random_tree(200, seed=41), random_tree(120, seed=42)]
    clamps = [(0, 0, 0.4, 0.0, 30.0), (1, 0, 0.5, 0.0, 30.0)]
    parent, R, C, area, offs = concat(trees)
    full = propagator(parent, R, C, 0.05, prune=0.0)
    tol = 1e-6
    L = lump_and_conserve(full, parent, tol)
    assert np.abs(np.asarray(L.sum(axis=1)).ravel() - np.asarray(full.sum(axis=1)).ravel()).max() < 1e-13
    D = full.toarray().copy()
    drop = np.abs(D) < tol
    np.fill_diagonal(drop, False)
    D[np.arange(len(D)), np.arange(len(D))] += np.where(drop, D, 0).sum(axis=1)
    D[drop] = 0.0
    assert (L.toarray() != 0).sum() <= (D != 0).sum()
    errs = []
    for P in (L, scipy.sparse.csr_matrix(D)):
        ref, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.), prune=0.0)
        om, _ = oracle_case(trees, clamps, hh_kw=dict(ena=50., ek=-77.))
        om.P = P
        worst = 0.0
        for _ in range(300):
            ref.advance(); om.advance()
            worst = max(worst, np.abs(ref.voltage - om.voltage).max())
        errs.append(worst)
    assert errs[0] < errs[1] / 5, errs


def test_lumping_keeps_the_row_entry_at_any_tolerance():
    """Every diagonal below the tolerance: lumping still keeps each row's own entry
    (the target of everything dropped near it), so the result is the identity."""
    from oracle.reference_step import lump_and_conserve
    t = random_tree(120, seed=8)
    parent, R, C, area, offs = concat([t])
    full = propagator(parent, R, C, 0.05, prune=0.0)
    assert full.diagonal().max() < 0.9
    L = lump_and_conserve(full, parent, 0.9).toarray()
    assert np.abs(L - np.eye(len(L))).max() < 1e-13


@pytest.mark.parametrize("tol", [1e-8, 3e-7, 1e-5])
def test_c_lumping_matches_numpy_lumping(tol):
    """The C walk the CPU baseline prunes with equals the oracle's lump_and_conserve."""
    from oracle.cpu_oracle import lump
    from oracle.reference_step import lump_and_conserve
    t = random_tree(250, seed=5)
    parent, R, C, area, offs = concat([t])
    full = propagator(parent, R, C, 0.05, prune=0.0).toarray()
    a = lump_and_conserve(full, parent, tol).toarray()
    b = lump(full, parent, tol)
    assert np.array_equal(a != 0, b != 0)
    assert np.abs(a - b).max() < 1e-13
