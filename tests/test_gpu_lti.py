"""Kinetic tables generated on the GPU in FP64 against the host FP64 build
(itself pinned to the reference's lti_sim Approx1D) and scipy's expm."""
import numpy as np
import pytest
import scipy.linalg

import neuwon_gb300 as nw
from neuwon_gb300 import _lib
from neuwon_gb300.kinetic import LTITable, na8, optimize_table, scheme_table_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = _lib.Context(0, "f64")
    yield c
    c.close()


def test_expm_matches_scipy(ctx):
    rng = np.random.default_rng(0)
    for S in (2, 3, 8, 13, 16):
        Q = rng.uniform(0, 5, (50, S, S))
        for q in Q:
            np.fill_diagonal(q, 0.0)
            q[np.diag_indices(S)] = -q.sum(axis=0)
        Q *= np.logspace(-3, 2, 50)[:, None, None]           # norms from tiny to large (squaring)
        Q = np.ascontiguousarray(Q)
        out = np.empty_like(Q)
        ctx.call("nw_lti_expm", S, len(Q), _lib.ptr(Q), 0.1, _lib.ptr(out))
        ref = np.array([scipy.linalg.expm(q * 0.1) for q in Q])
        assert np.abs(out - ref).max() < 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("dt,celsius", [(0.1, 6.3), (0.025, 6.3), (0.1, 37.0)])
def test_na8_table_matches_host_build(ctx, dt, celsius):
    sch = na8()
    host = LTITable(sch, dt, celsius)
    gpu = scheme_table_gpu(ctx, sch, dt, celsius, -100.0, 60.0, 1600, 1)
    assert np.abs(gpu - host.layout).max() < 1e-12


def test_calcium_pump_table_matches_host_build(ctx):
    ca = nw.Calcium()
    from neuwon_gb300.kinetic import gpu_table
    rates, fit = ca.table_inputs()
    gpu = gpu_table(ctx, rates, fit, ca.num_buckets, 0.025)
    assert np.abs(gpu - ca.table(0.025)).max() < 1e-12


def test_optimizer_meets_accuracy(ctx):
    sch = na8()
    res = optimize_table(ctx, sch, 0.1, 6.3, accuracy=1e-4)
    assert res["max_error"] <= 1e-4
    host = LTITable(sch, 0.1, 6.3, num_buckets=res["num_buckets"], degree=res["degree"])
    assert host.max_error(16) <= 1e-4 * 1.05
    # A bucket count 20 % smaller misses the accuracy (the search stops near the edge).
    smaller = LTITable(sch, 0.1, 6.3, num_buckets=int(res["num_buckets"] * 0.8), degree=res["degree"])
    assert smaller.max_error(16) > 0.5e-4
