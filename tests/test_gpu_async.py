"""nw_advance_host_async: the end-to-end step with host buffers whose voltage copies
run on a second stream while the next step computes.  Every step's voltages must
equal those of the synchronous nw_advance_host bit for bit (same kernels, same
inputs), with pinned output buffers, one per step, read after nw_synchronize."""
import numpy as np
import pytest

from neuwon_gb300 import _lib
from neuwon_gb300.morphology import random_tree
from tests.helpers import gpu_model

pytestmark = pytest.mark.gpu


def _model():
    trees = [random_tree(n, seed=900 + n) for n in (1500, 400, 30)]
    m, neurons, _, _ = gpu_model(trees, [], precision="f32", tolerance=3e-7, conserve="lump", fmt="quads",
                                 kinetic=True)
    for nr in neurons:
        nr.root.inject_current(0.3, 1e9)
    m._sync()
    return m


def test_async_host_steps_equal_sync_steps():
    import torch
    steps = 20
    stim = np.array([0.4e-9, 0.2e-9, 0.01e-9])           # one amplitude per clamp (A)
    m1 = _model()
    ref = []
    for _ in range(steps):
        v = np.empty(m1._n, dtype=np.float32)
        m1._ctx.call("nw_advance_host", 1, _lib.ptr(stim), _lib.ptr(v), 2)
        ref.append(v)
    m1.close()
    m2 = _model()
    stim_p = torch.from_numpy(stim).pin_memory()
    outs = [torch.empty(m2._n, dtype=torch.float32).pin_memory() for _ in range(steps)]
    for k in range(steps):
        m2._ctx.call("nw_advance_host_async", 1, stim_p.data_ptr(), outs[k].data_ptr(), 2)
    m2._ctx.call("nw_synchronize")
    for k in range(steps):
        assert np.array_equal(outs[k].numpy(), ref[k]), k
    assert not np.array_equal(ref[0], ref[-1])             # the voltages do move
    rc = m2._ctx.lib.nw_advance_host_async(m2._ctx.handle, 1, None, outs[0].data_ptr(), 1)
    assert rc == -1                                         # FP64 output of an FP32 context: refused
    m2.close()
