"""The allocation-free half step, called through the C ABI on caller-owned arrays.

Callers whose device memory all comes from their own allocator cannot let a
library call cudaMalloc; nw_electric_half_step_noalloc runs the membrane
update and propagator multiply of one half step on arrays they provide, with
its scratch in a static device array.  Here two calls in a row (one full step
of a passive model with a current clamp) must reproduce what the existing
entry point nw_advance (plain FP64 path) computes, within the FP64 parity
tolerance of the other GPU tests (1e-7 mV); and again for a second pair of
calls, so the shared scratch array is reused.
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
    amps = 0.3e-9
    m = nw.RxD_Model(time_step=0.1, precision="f64", path="plain")
    m.add_tree(tree)
    nw.Segment(m, 0).inject_current(0.3, 10.0)            # active on ticks 1..200
    m._sync()
    rowptr, col, val = _propagator(m)
    C = m._geometry()["capacitance"][m._order]            # device order (depth-first within the neuron)
    n = m._n
    lib = _lib.load()

    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in dict(
        rowptr=rowptr, col=col, val=val, C=C, G=np.zeros(n), E=np.zeros(n),
        V=np.full(n, -70.0)).items()}
    I = np.zeros(n)
    I[0] = amps
    d["I"] = torch.from_numpy(I).to(dev)

    def half_step():
        torch.cuda.synchronize()
        rc = lib.nw_electric_half_step_noalloc(
            n, ctypes.c_void_p(d["rowptr"].data_ptr()), ctypes.c_void_p(d["col"].data_ptr()),
            ctypes.c_void_p(d["val"].data_ptr()), ctypes.c_void_p(d["V"].data_ptr()),
            ctypes.c_void_p(d["C"].data_ptr()), ctypes.c_void_p(d["G"].data_ptr()),
            ctypes.c_void_p(d["E"].data_ptr()), ctypes.c_void_p(d["I"].data_ptr()), 0.05, None)
        torch.cuda.synchronize()
        assert rc == 0

    for _ in range(2):
        half_step()
        half_step()
        m.advance(1)
        want = m.get_data("Segment.voltage")              # creation order
        got = d["V"].cpu().numpy()[m._inv]
        assert np.abs(got - want).max() < TOL_MV
        assert np.abs(got + 70.0).max() > 1e-6        # the clamp moved the voltage
    m.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from neuwon_gb300 import _lib
    lib = _lib.load()
    dummy = ctypes.c_void_p(1)
    rc = lib.nw_electric_half_step_noalloc((1 << 20) + 1, dummy, dummy, dummy, dummy, dummy, dummy,
                                           dummy, dummy, 0.05, None)
    assert rc == -6   # NW_ERR_LIMIT, checked before anything is launched
