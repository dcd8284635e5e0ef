"""Calcium system on the host: pump table, logarithmic input, diffusion oracle."""
import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.morphology import geometry, random_tree
from oracle.reference_step import CalciumOracle


def test_log_input_matches_lti_sim_definition():
    """Bucket value = (log2(c + scale) - log2(min + scale)) * num_buckets / log2 range,
    min = 0 (neuwon/rxd/lti_sim/inputs.py:91-105)."""
    ca = nw.Calcium(num_buckets=300, c_max=2.0, scale=1e-5)
    c = np.array([0.0, 1e-6, 3e-4, 0.1, 1.99, 2.0, 5.0])
    lo, hi = np.log2(0 + 1e-5), np.log2(2.0 + 1e-5)
    x = (np.log2(c + 1e-5) - lo) * 300 / (hi - lo)
    b, loc = ca.locate(c)
    expect_b = np.minimum(np.trunc(x).astype(int), 299)
    assert np.array_equal(b, expect_b)
    assert np.allclose(np.where(x >= 300, 1.0, x - np.trunc(x)), loc)


def test_pump_table_and_steady_state():
    ca = nw.Calcium()
    dt = 0.025
    table = ca.table(dt)
    rng = np.random.default_rng(0)
    c = np.concatenate([10 ** rng.uniform(-7, 0, 400), [0.0, 1.0]])
    st = rng.dirichlet(np.ones(3), len(c))
    exact = np.einsum("nrc,nc->nr", ca.exact_propagator(c, dt), st)
    got = ca.table_step(table, c, st)
    assert np.abs(got - exact).max() < 1e-6
    s0 = ca.steady_state(5e-5)
    assert np.abs(ca.exact_propagator([5e-5], dt)[0] @ s0 - s0).max() < 1e-14
    assert abs(s0.sum() - 1) < 1e-14


def test_diffusion_conserves_calcium():
    tree = random_tree(250, seed=4)
    g = geometry(tree)
    ca = CalciumOracle(tree.parent, g["cross_sectional_area"], g["length"], g["volume"], 0.6, 0.025, 5e-5,
                       np.zeros(250), np.zeros(250))
    ca.c[17] = 0.01                                   # a local load spreads and keeps its total
    total = (ca.c * ca.volume).sum()
    for _ in range(400):
        ca.advance_half()
    assert abs((ca.c * ca.volume).sum() - total) < 1e-12 * total
    assert ca.c[17] < 0.01 and ca.c.min() >= 0


def test_reference_species_keywords():
    """The _SpeciesType keywords (species.py:90-142): every one is kept or refused, none dropped."""
    from neuwon_gb300.species import SpeciesType
    sp = SpeciesType(name="ca", charge=2, reversal_potential=120.0, diffusivity=0.6,
                     inside_initial_concentration=1e-4, inside_global_constant=False)
    assert sp.charge == 2 and sp.electric and sp.reversal_potential == 120.0
    ca = sp.calcium
    assert ca.diffusivity == 0.6 and ca.initial == 1e-4 and not ca.pump
    na = SpeciesType(name="na", charge=1, reversal_potential=50)
    assert na.electric and na.reversal_potential == 50.0 and na.calcium is None
    assert not SpeciesType(name="cl", charge=-1).electric
    with pytest.raises(NotImplementedError):
        SpeciesType(name="na", inside_global_constant=False)
    with pytest.raises(NotImplementedError):
        SpeciesType(name="k", reversal_potential="nerst")
    with pytest.raises(NotImplementedError):
        SpeciesType(name="k", outside_global_constant=False)
    with pytest.raises(NotImplementedError):
        SpeciesType(name="ca", inside_global_constant=False, decay_period=10.0)
    with pytest.raises(TypeError):
        SpeciesType(name="k", bogus=1)
