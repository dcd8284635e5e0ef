"""ctypes driver of the C oracle (oracle/cpu_step.c) -- test infrastructure / CPU baseline."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle_step.so")


def build():
    src = os.path.join(HERE, "cpu_step.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


class _Model(ctypes.Structure):
    _fields_ = [(n, t) for n, t in [
        ("n_seg", ctypes.c_int64),
        ("rowptr", ctypes.c_void_p), ("col", ctypes.c_void_p), ("val", ctypes.c_void_p),
        ("V", ctypes.c_void_p), ("Vint", ctypes.c_void_p), ("C", ctypes.c_void_p), ("Inonspec", ctypes.c_void_p),
        ("time_step", ctypes.c_double),
        ("m", ctypes.c_int64), ("hh_seg_ptr", ctypes.c_void_p), ("hh_seg", ctypes.c_void_p),
        ("gm", ctypes.c_void_p), ("gh", ctypes.c_void_p), ("gn", ctypes.c_void_p),
        ("cna", ctypes.c_void_p), ("ck", ctypes.c_void_p), ("cl", ctypes.c_void_p),
        ("ena", ctypes.c_double), ("ek", ctypes.c_double), ("el", ctypes.c_double), ("celsius", ctypes.c_double),
        ("clamp_ptr", ctypes.c_void_p), ("clamp_amp", ctypes.c_void_p), ("clamp_first", ctypes.c_void_p),
        ("clamp_count", ctypes.c_void_p),
        ("n_neuron", ctypes.c_int64), ("det_seg", ctypes.c_void_p), ("det_thr", ctypes.c_void_p),
        ("ap_state", ctypes.c_void_p), ("ap_detected", ctypes.c_void_p), ("spike_count", ctypes.c_void_p),
        ("x", ctypes.c_void_p), ("input_ticks", ctypes.c_int64), ("g_valid", ctypes.c_int),
        ("km", ctypes.c_int64), ("kin_seg_ptr", ctypes.c_void_p), ("kin_seg", ctypes.c_void_p),
        ("kstate", ctypes.c_void_p), ("kgcoef", ctypes.c_void_p), ("ktable", ctypes.c_void_p),
        ("kS", ctypes.c_int64), ("kT", ctypes.c_int64), ("knb", ctypes.c_int64), ("knopen", ctypes.c_int64),
        ("kopen", ctypes.c_void_p),
        ("kvmin", ctypes.c_double), ("kfrq", ctypes.c_double), ("kcs", ctypes.c_double), ("kerev", ctypes.c_double),
    ]]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class CpuOracle:
    """FP64 OpenMP step over a CSR propagator (with diagonal) and HH instances.

    hh: dict(segment, gna, gk, gl (S), ena, ek, el); clamps: list of
    (segment, amps, first_tick, num_ticks); detectors: list of (segment, thr);
    kinetic: dict(segment, gcoef (S), table [bucket][col][row][term], vmin,
    bucket_frq, open (state indices), erev, conserve (0: none), init (S,)).
    """

    def __init__(self, csr_indptr, csr_indices, csr_data, C, *, time_step, celsius, v_init=-70.0,
                 hh=None, clamps=(), detectors=(), m0=None, kinetic=None):
        self.lib = ctypes.CDLL(build())
        self.lib.oracle_advance.argtypes = [ctypes.POINTER(_Model), ctypes.c_int]
        self.lib.oracle_threads.restype = ctypes.c_int
        n = len(C)
        self.n = n
        self.rowptr = np.ascontiguousarray(csr_indptr, dtype=np.int64)
        self.col = np.ascontiguousarray(csr_indices, dtype=np.int32)
        self.val = np.ascontiguousarray(csr_data, dtype=np.float64)
        self.C = np.ascontiguousarray(C, dtype=np.float64)
        self.V = np.full(n, float(v_init))
        self.Vint = np.zeros(n)
        self.x = np.zeros(n)
        M = _Model()
        M.n_seg = n
        M.rowptr, M.col, M.val = _p(self.rowptr), _p(self.col), _p(self.val)
        M.V, M.Vint, M.C, M.Inonspec = _p(self.V), _p(self.Vint), _p(self.C), None
        M.time_step = float(time_step)
        M.celsius = float(celsius)
        if hh is not None:
            seg = np.asarray(hh["segment"], dtype=np.int64)
            order = np.argsort(seg, kind="stable")
            self.hh_seg = np.ascontiguousarray(seg[order])
            self.hh_seg_ptr = np.zeros(n + 1, np.int64)
            np.add.at(self.hh_seg_ptr, self.hh_seg + 1, 1)
            self.hh_seg_ptr = np.cumsum(self.hh_seg_ptr)
            m = len(seg)
            from .reference_step import hh_rates
            minf, _, hinf, _, ninf, _ = hh_rates(np.full(m, float(v_init)), celsius)
            self.gm, self.gh, self.gn = minf.copy(), hinf.copy(), ninf.copy()
            self.cna = np.ascontiguousarray(np.asarray(hh["gna"], np.float64)[order])
            self.ck = np.ascontiguousarray(np.asarray(hh["gk"], np.float64)[order])
            self.cl = np.ascontiguousarray(np.asarray(hh["gl"], np.float64)[order])
            M.m = m
            M.hh_seg_ptr, M.hh_seg = _p(self.hh_seg_ptr), _p(self.hh_seg)
            M.gm, M.gh, M.gn = _p(self.gm), _p(self.gh), _p(self.gn)
            M.cna, M.ck, M.cl = _p(self.cna), _p(self.ck), _p(self.cl)
            M.ena, M.ek, M.el = float(hh["ena"]), float(hh["ek"]), float(hh["el"])
        else:
            self.hh_seg_ptr = np.zeros(n + 1, np.int64)
            M.m = 0
            M.hh_seg_ptr = _p(self.hh_seg_ptr)
        if clamps:
            cs = sorted(range(len(clamps)), key=lambda k: clamps[k][0])
            self.clamp_ptr = np.zeros(n + 1, np.int64)
            for k in cs:
                self.clamp_ptr[clamps[k][0] + 1] += 1
            self.clamp_ptr = np.cumsum(self.clamp_ptr)
            self.clamp_amp = np.array([clamps[k][1] for k in cs], np.float64)
            self.clamp_first = np.array([clamps[k][2] for k in cs], np.int64)
            self.clamp_count = np.array([clamps[k][3] for k in cs], np.int64)
            M.clamp_ptr, M.clamp_amp = _p(self.clamp_ptr), _p(self.clamp_amp)
            M.clamp_first, M.clamp_count = _p(self.clamp_first), _p(self.clamp_count)
        self.det_seg = np.array([d[0] for d in detectors], np.int64)
        self.det_thr = np.array([d[1] for d in detectors], np.float64)
        self.ap_state = np.zeros(len(detectors), np.uint8)
        self.ap_detected = np.zeros(len(detectors), np.uint8)
        self.spike_count = np.zeros(len(detectors), np.int64)
        M.n_neuron = len(detectors)
        M.det_seg, M.det_thr = _p(self.det_seg), _p(self.det_thr)
        M.ap_state, M.ap_detected, M.spike_count = _p(self.ap_state), _p(self.ap_detected), _p(self.spike_count)
        M.x = _p(self.x)
        if kinetic is not None:
            seg = np.asarray(kinetic["segment"], dtype=np.int64)
            order = np.argsort(seg, kind="stable")
            self.kin_seg = np.ascontiguousarray(seg[order])
            self.kin_seg_ptr = np.zeros(n + 1, np.int64)
            np.add.at(self.kin_seg_ptr, self.kin_seg + 1, 1)
            self.kin_seg_ptr = np.cumsum(self.kin_seg_ptr)
            table = np.ascontiguousarray(kinetic["table"], dtype=np.float64)
            nb, S, _, T = table.shape
            km = len(seg)
            self.kstate = np.ascontiguousarray(np.repeat(np.asarray(kinetic["init"], np.float64)[:, None], km, 1))
            self.kgcoef = np.ascontiguousarray(np.asarray(kinetic["gcoef"], np.float64)[order])
            self.ktable = table
            self.kopen = np.ascontiguousarray(kinetic["open"], dtype=np.int64)
            M.km = km
            M.kin_seg_ptr, M.kin_seg = _p(self.kin_seg_ptr), _p(self.kin_seg)
            M.kstate, M.kgcoef, M.ktable = _p(self.kstate), _p(self.kgcoef), _p(self.ktable)
            M.kS, M.kT, M.knb, M.knopen = S, T, nb, len(self.kopen)
            M.kopen = _p(self.kopen)
            M.kvmin, M.kfrq = float(kinetic["vmin"]), float(kinetic["bucket_frq"])
            M.kcs, M.kerev = float(kinetic.get("conserve") or 0.0), float(kinetic["erev"])
        self.M = M

    def advance(self, k=1):
        self.lib.oracle_advance(ctypes.byref(self.M), int(k))

    def threads(self):
        return int(self.lib.oracle_threads())


def lump(P, parent, tol, explore_factor=1e-2):
    """Lumped pruning of one neuron's dense propagator in C (oracle_lump in
    oracle/cpu_step.c; the same walk as reference_step.lump_and_conserve).
    Returns a dense array."""
    lib = ctypes.CDLL(build())
    lib.oracle_lump.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                                ctypes.c_double, ctypes.c_void_p]
    lib.oracle_lump.restype = ctypes.c_int
    P = np.ascontiguousarray(P, dtype=np.float64)
    parent = np.ascontiguousarray(parent, dtype=np.int64)
    out = np.empty_like(P)
    rc = lib.oracle_lump(_p(P), _p(parent), len(parent), float(tol), float(explore_factor), _p(out))
    if rc != 0:
        raise MemoryError("oracle_lump: scratch allocation failed")
    return out
