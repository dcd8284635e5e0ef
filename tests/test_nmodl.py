"""The NMODL front end for kinetic channels (neuwon_gb300.nmodl), on the CPU.

A channel file written here (not from the reference) exercises every construct
the front end reads; with NEUWON_REFERENCE naming a checkout of the reference,
every kinetic channel of its nmodl_library is parsed too, and Nav1.1 / Kv1.1
are compared with the restated schemes the device tests use.
"""
import glob
import math
import os

import numpy as np
import pytest

import neuwon_gb300 as nw
from neuwon_gb300.nmodl import KineticFile, kinetic_mechanism

# A three-state potassium channel, C <-> O <-> I, in the library's style.
KTEST = """
TITLE test channel
COMMENT
three states, rates from a FUNCTION and a PROCEDURE
ENDCOMMENT
NEURON {
    SUFFIX ktest
    USEION k READ ek WRITE ik
    RANGE gbar, g
}
UNITS { (mV) = (millivolt) }
PARAMETER {
    v (mV)
    celsius (degC)
    gbar = 20 (mS/cm2)   : 0.02 S/cm2
    a0 = 0.5 (/ms)
    vh = -30 (mV)
    s = 9 (mV)
    kin = 0.02 (/ms)
}
ASSIGNED { ik (mA/cm2) g (mS/cm2) kco (/ms) koc (/ms) }
STATE { C O I }
LOCAL q
INITIAL {
    q = 2^((celsius - 22(degC))/10 (degC))
    SOLVE kin STEADYSTATE sparse
}
BREAKPOINT {
    SOLVE kin METHOD sparse
    g = gbar*O
    ik = g*(v - ek)*(1e-3)
}
KINETIC kin {
    rates(v)
    ~ C <-> O (kco, koc)
    ~ O <-> I (q*kin, q*kin*0.1)
    CONSERVE C + O + I = 1
}
FUNCTION boltz(x, h, w) {
    boltz = 1/(1 + exp(-(x - h)/w))
}
PROCEDURE rates(v(mV)) {
UNITSOFF
    kco = q*a0*boltz(v, vh, s)
    koc = q*a0*(1 - boltz(v, vh, s))
UNITSON
}
"""

PASSIVE = """
NEURON { SUFFIX leak  NONSPECIFIC_CURRENT i  RANGE g, e }
PARAMETER { g = .0005 (S/cm2) <0,1e9>  e = -65 (mV) }
ASSIGNED { v (mV) i (mA/cm2) }
BREAKPOINT { i = g*(v - e) }
"""


def _ktest_matrix(v, celsius):
    q = 2.0 ** ((celsius - 22.0) / 10.0)
    b = 1 / (1 + np.exp(-(v + 30.0) / 9.0))
    kco, koc = q * 0.5 * b, q * 0.5 * (1 - b)
    A = np.zeros((len(v), 3, 3))
    for src, dst, r in ((0, 1, kco), (1, 0, koc), (1, 2, q * 0.02 + 0 * v), (2, 1, q * 0.02 * 0.1 + 0 * v)):
        A[:, dst, src] += r
        A[:, src, src] -= r
    return A


def test_parses_a_kinetic_channel():
    kf = KineticFile(KTEST, "ktest.mod")
    assert kf.suffix == "ktest" and kf.ion == "k" and not kf.nonspecific
    assert kf.gbar == pytest.approx(0.02) and kf.states == ["C", "O", "I"]
    sch = kf.scheme()
    assert sch.open_states == [1] and sch.conserve_sum == 1.0
    v = np.linspace(-100, 100, 21)
    for celsius in (6.3, 22.0, 35.0):
        assert np.abs(sch.matrix(v, celsius) - _ktest_matrix(v, celsius)).max() < 1e-14


def test_parses_a_passive_channel():
    kf = KineticFile(PASSIVE, "leak.mod")
    assert kf.nonspecific and kf.ion is None
    assert kf.gbar == pytest.approx(5e-4) and kf.erev == -65.0
    sch = kf.scheme()
    assert sch.num_states == 1 and sch.open_states == [0]
    assert np.all(sch.matrix([-70.0, 0.0], 6.3) == 0.0)


def test_nmodl_loads_channels_into_a_model(tmp_path):
    path = tmp_path / "ktest.mod"
    path.write_text(KTEST)
    leak = tmp_path / "leak.mod"
    leak.write_text(PASSIVE)
    m = nw.RxD_Model(species=[dict(name="k", charge=1, reversal_potential=-80.0)],
                     mechanisms=[str(path), str(leak)])
    assert set(m.mechanisms) == {"ktest", "leak"}
    cls = m.mechanisms["ktest"]
    assert cls.ion == "k" and cls.gbar == pytest.approx(0.02) and (cls.vmin, cls.vmax) == (-100.0, 100.0)
    with pytest.raises(ValueError, match="electric species 'k'"):
        nw.RxD_Model(mechanisms=[str(path)])


@pytest.mark.parametrize("text, what", [
    (KTEST.replace("SUFFIX ktest", "POINT_PROCESS ktest"), "POINT_PROCESS"),
    (KTEST.replace("g = gbar*O", "g = gbar*O*O"), "conductance"),
    (KTEST.replace("(mS/cm2)   :", "(mA/cm2)   :"), "density units"),
    (KTEST.replace("~ O <-> I", "~ O + C <-> I"), "reaction"),
])
def test_rejects_what_it_cannot_run(text, what):
    with pytest.raises(NotImplementedError, match=what):
        KineticFile(text, "x.mod").scheme().matrix([0.0], 6.3)


REF = os.environ.get("NEUWON_REFERENCE")


@pytest.mark.skipif(not REF, reason="needs a reference checkout (NEUWON_REFERENCE)")
def test_reference_library_channels():
    """Every kinetic channel of the reference's nmodl_library parses into a
    conserving generator; Nav1.1 and Kv1.1 equal the restated schemes."""
    files = sorted(glob.glob(os.path.join(REF, "nmodl_library", "kinetic", "*.mod")))
    parsed = 0
    for f in files:
        text = open(f).read()
        if "POINT_PROCESS" in text:
            continue                                 # AMPA / NMDA synapses: point processes
        sch = KineticFile(text, os.path.basename(f)).scheme()
        A = sch.matrix(np.linspace(-100, 100, 21), 20.0)
        assert np.abs(A.sum(axis=1)).max() <= 1e-12 * np.abs(A).max()
        parsed += 1
    assert parsed >= 30
    v = np.linspace(-100, 100, 81)
    for name, restated in (("Nav11.mod", nw.nav11()), ("Kv11.mod", nw.kv11())):
        mech = kinetic_mechanism(os.path.join(REF, "nmodl_library", "kinetic", name))
        sch = mech.scheme_factory()
        for celsius in (6.3, 20.0, 37.0):
            a, b = sch.matrix(v, celsius), restated.matrix(v, celsius)
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    assert kinetic_mechanism(os.path.join(REF, "nmodl_library", "kinetic", "Kv11.mod")).gbar == pytest.approx(0.036)
