"""The drop-in backend for the reference's own RxD_Model (neuwon_gb300.dropin), on the CPU.

The fixture groups ``dropin_hh11`` / ``dropin_hh200`` hold what the backend's
``extract`` read from the reference's Database and the device clamps
``clamp_players`` derived from the reference's input-clock players, recorded by
running the reference (tests/golden/make_golden.py: run_dropin).  With a
checkout of the reference named by NEUWON_REFERENCE the live test rebuilds the
model through the reference and compares; without it that test is skipped (the
GPU test replays the recorded arrays either way).
"""
import os

import numpy as np
import pytest

from neuwon_gb300.dropin import NULL, clamp_players, extract
from tests.helpers import FIXTURES

F = np.load(FIXTURES)


def test_fixture_arrays_are_consistent():
    for p, n in (("dropin_hh11", 11), ("dropin_hh200", 200)):
        parent = F[f"{p}_parent"]
        assert len(parent) == n and parent[0] == -1 and np.all(parent[1:] < np.arange(1, n))
        assert list(F[f"{p}_neuron_start"]) == [0, n]
        assert np.all(F[f"{p}_capacitance"] > 0) and np.all(F[f"{p}_hh_magnitude"] > 0)
        assert np.array_equal(F[f"{p}_hh_segment"], np.arange(n))
        cl = F[f"{p}_clamps"]
        assert np.all(cl[:, 4] == 1) and np.all(cl[:, 3] == 2 * cl[:, 0] + 1 + (np.arange(len(cl)) % 2))
    assert NULL == 0xFFFFFFFF


@pytest.mark.skipif(not os.environ.get("NEUWON_REFERENCE"), reason="needs a reference checkout (NEUWON_REFERENCE)")
def test_live_extraction_matches_fixture():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    make_golden.REFERENCE = make_golden.reference_path([os.environ["NEUWON_REFERENCE"]])
    make_golden.install_stubs()
    from neuwon_gb300.morphology import random_tree
    out = {}
    make_golden.run_dropin(out, "dropin_hh200", random_tree(200, seed=11), [(0, 0.2, 5.0, 20.0)],
                           dict(ena=50.0, ek=-77.0, el=-54.3), 30.0, False)
    for key, val in out.items():
        assert np.array_equal(val, F[key]), key
