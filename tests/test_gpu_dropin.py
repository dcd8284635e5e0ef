"""The drop-in backend for the reference's own RxD_Model, on the GPU.

The arrays ``neuwon_gb300.dropin.extract`` read from the reference's Database
after db.sort() and the device clamps ``clamp_players`` derived from the
reference's own input-clock players were recorded by running the reference
(tests/golden/make_golden.py: run_dropin), together with the voltage of every
segment after every step of the reference's own ``advance()``.  Replayed through
``GB300Advance`` (the C ABI, FP64, batched path) they must give the reference's
voltages to 1e-7 mV.
"""
import numpy as np
import pytest

from neuwon_gb300.dropin import GB300Advance
from tests.helpers import FIXTURES

pytestmark = pytest.mark.gpu
F = np.load(FIXTURES)


def _arrays(p):
    meta = F[f"{p}_meta"]
    a = {k: F[f"{p}_{k}"] for k in ("parent", "neuron_start", "capacitance", "axial_resistance", "voltage")}
    a.update(time_step=float(meta[0]), celsius=float(meta[1]))
    a["hh"] = {k: F[f"{p}_hh_{k}"] for k in ("segment", "magnitude", "m", "h", "n")}
    a["hh"].update(gnabar=meta[2], gkbar=meta[3], glbar=meta[4], ena=meta[5], ek=meta[6], el=meta[7])
    return a


@pytest.mark.parametrize("prefix", ["dropin_hh11", "dropin_hh200"])
def test_dropin_backend_reproduces_reference_advance(prefix):
    backend = GB300Advance.from_arrays(_arrays(prefix), precision="f64")
    volts = F[f"{prefix}_volts"]
    clamps = F[f"{prefix}_clamps"]
    assert np.abs(backend.voltage() - volts[0]).max() == 0.0
    worst = 0.0
    for k in range(len(volts) - 1):
        step = [(int(s), float(a), int(f), int(c)) for (kk, s, a, f, c) in clamps if int(kk) == k]
        backend.step(step)
        worst = max(worst, float(np.abs(backend.voltage() - volts[k + 1]).max()))
    assert worst < 1e-7, worst
    assert volts.max() > 0.0                   # the clamp fired the neuron
    backend.close()
