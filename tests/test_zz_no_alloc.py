"""The allocation-free half step, called through the C ABI on caller-owned arrays.

Callers whose device memory all comes from their own pool allocator, or whose
time loop must not allocate, cannot let a library call cudaMalloc;
nw_electric_half_step_noalloc runs the membrane update and propagator
multiply of one half step on arrays they provide, with its scratch vector in
a static device array.  Here pairs of calls in a row (full steps of a model
with a leak conductance on every segment and a current clamp) must reproduce
what the existing entry point nw_advance (plain FP64 path) computes, within the
FP64 parity tolerance of the other GPU tests (1e-7 mV): voltages and integral
voltages, over three pairs, so the shared scratch array is reused, and the
exponential branch exp(-dt G / C) is exercised with nonzero G and E.  Free
device memory must not change across the calls.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MV = 1e-7


def _propagator(model):
    from neuwon_gb300 import _lib
    ctx = model._ctx
    n = model._n
    nnz = ctypes.c_int64()
    ctx.call("nw_propagator_get_csr", None, None, None, ctypes.byref(nnz))
    rowptr = np.empty(n + 1, np.int64)
    col = np.empty(nnz.value, np.int64)
    val = np.empty(nnz.value, np.float64)
    ctx.call("nw_propagator_get_csr", _lib.ptr(rowptr), _lib.ptr(col), _lib.ptr(val), ctypes.byref(nnz))
    return rowptr, col.astype(np.int32), val


def test_noalloc_half_step_matches_advance_on_two_calls():
    import torch
    import neuwon_gb300 as nw
    from neuwon_gb300 import _lib
    from neuwon_gb300.morphology import random_tree

    tree = random_tree(400, seed=77)
    el = -54.3
    # HH with only its leak: a constant conductance gl on every segment with reversal el.
    m = nw.RxD_Model(time_step=0.1, precision="f64", path="plain",
                     mechanisms=[nw.HH.configure(gnabar=0.0, gkbar=0.0, glbar=0.002, el=el)])
    m.add_tree(tree)
    m.insert_everywhere("hh")
    nw.Segment(m, 0).inject_current(0.3, 10.0)            # active on ticks 1..200
    m._sync()
    rowptr, col, val = _propagator(m)
    n = m._n
    C = m._geometry()["capacitance"][m._order]            # device order (depth-first within the neuron)
    gl = np.empty(n)
    gl[m._inv] = m.get_data("hh.gl_coef")                  # instance k sits on creation segment k
    assert gl.min() > 0
    lib = _lib.load()

    dev = torch.device("cuda", 0)
    to_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = {k: to_dev(v) for k, v in dict(rowptr=rowptr, col=col, val=val, C=C, V=np.full(n, -70.0),
                                       Vint=np.zeros(n), G0=np.zeros(n), E0=np.zeros(n),
                                       G=gl, E=np.full(n, el)).items()}
    I = np.zeros(n)
    I[m._inv[0]] = 0.3e-9
    d["I"] = to_dev(I)
    p = lambda t: ctypes.c_void_p(t.data_ptr())

    def half_step(G, E):
        rc = lib.nw_electric_half_step_noalloc(
            n, p(d["rowptr"]), p(d["col"]), p(d["val"]), p(d["V"]), p(d["C"]), p(G), p(E), p(d["I"]),
            p(d["Vint"]), 0.05, None)
        assert rc == 0

    for k in range(3):
        # The first half step of the first step sees no mechanism conductance yet
        # (rxd_model.py:63-80: the accumulators are filled by the mechanism phase).
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        half_step(d["G0"] if k == 0 else d["G"], d["E0"] if k == 0 else d["E"])
        half_step(d["G"], d["E"])
        torch.cuda.synchronize()
        used = free0 - torch.cuda.mem_get_info(0)[0]
        if k == 0:
            # With lazy module loading the first call loads the library's device code
            # on this GPU, which creates the 8 MiB static scratch array (and no more).
            assert 0 <= used <= (8 << 20) + (2 << 20)
        else:
            assert used == 0                              # nothing allocated by the two calls
        m.advance(1)
        want = m.get_data("Segment.voltage")              # creation order
        got = d["V"].cpu().numpy()[m._inv]
        assert np.abs(got - want).max() < TOL_MV
        assert np.abs(got + 70.0).max() > 1e-3            # the clamp and the leak moved the voltage
        want_int = m.get_data("Segment.integral_voltage")
        got_int = d["Vint"].cpu().numpy()[m._inv]
        assert np.abs(got_int - want_int).max() < TOL_MV * 1e-3
        assert np.abs(got_int).max() > 0
    m.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from neuwon_gb300 import _lib
    lib = _lib.load()
    dummy = ctypes.c_void_p(1)
    rc = lib.nw_electric_half_step_noalloc((1 << 20) + 1, dummy, dummy, dummy, dummy, dummy, dummy,
                                           dummy, dummy, None, 0.05, None)
    assert rc == -6   # NW_ERR_LIMIT, checked before anything is launched
