"""Adjoint kernels: gradients of the soma-trace loss with respect to per-segment
gNa/gK/gL densities and Ra, checked against plain FP64 PyTorch autograd through
the same step and against FP64 central differences (relative tolerance 1e-4,
the target for the adjoint)."""
import numpy as np
import pytest
import torch

import neuwon_gb300 as nw
from neuwon_gb300._lib import NeuwonError
from neuwon_gb300.adjoint import loss_and_gradients, trace_loss
from neuwon_gb300.morphology import random_tree
from tests import torch_reference

pytestmark = pytest.mark.gpu

DT, CELSIUS = 0.025, 6.3
HH_KW = dict(ena=50.0, ek=-77.0, el=-54.3)


def _model(trees, precision="f64", amps=(0.4,), tol=nw.EPSILON):
    m = nw.RxD_Model(time_step=DT, temperature=CELSIUS, precision=precision, propagator_tolerance=tol,
                     mechanisms=[nw.HH.configure(**HH_KW)])
    neurons = [m.add_tree(t) for t in trees]
    m.insert_everywhere("hh")
    for nr, a in zip(neurons, amps):
        nr.root.inject_current(a, 1e6)
    m._sync()
    return m, neurons


def _target(m, steps, rng, spread=0.3):
    """Soma traces of the same model with densities drawn +-spread around the defaults."""
    k = m._instance_count("hh")
    dens = [rng.uniform(1 - spread, 1 + spread, k) * d for d in (0.12, 0.036, 0.0003)]
    m.set_hh_densities(*dens)
    m.reset_state()
    tr = []
    for _ in range(steps):
        m.advance()
        v = m.get_data("Segment.voltage")
        tr.append([v[r] for r in m._neuron_root])
    m.set_hh_densities(0.12, 0.036, 0.0003)
    return np.array(tr)


def test_adjoint_matches_fp64_torch_autograd():
    tree = random_tree(120, seed=61)
    steps = 240
    m, neurons = _model([tree])
    target = _target(m, steps, np.random.default_rng(0))
    loss, gna, gk, gl, gra = loss_and_gradients(m, steps, target, checkpoint_every=50)
    g = m._geometry()
    k = m._instance_count("hh")
    dens = [torch.full((k,), d, dtype=torch.float64, requires_grad=True) for d in (0.12, 0.036, 0.0003)]
    ra = torch.tensor(100.0, dtype=torch.float64, requires_grad=True)
    clamps = [(c[0], c[1], c[2], c[3]) for c in m._clamps]
    L = torch_reference.trace_loss(m._parent[:m._n], g["axial_resistance"], g["capacitance"], g["surface_area"],
                                   100.0, dens[0], dens[1], dens[2], ra, dt=DT, celsius=CELSIUS, steps=steps,
                                   clamps=clamps, det=m._neuron_root, target=target, **HH_KW)
    L.backward()
    assert loss == pytest.approx(L.item(), rel=1e-10)
    for mine, ref in ((gna, dens[0].grad), (gk, dens[1].grad), (gl, dens[2].grad)):
        ref = ref.numpy()
        assert np.abs(mine - ref).max() <= 1e-6 * np.abs(ref).max()
    assert gra == pytest.approx(ra.grad.item(), rel=1e-6)
    m.close()


def test_adjoint_matches_central_differences():
    trees = [random_tree(150, seed=71), random_tree(90, seed=72)]
    steps = 200
    m, neurons = _model(trees, amps=(0.4, 0.3))
    target = _target(m, steps, np.random.default_rng(1))
    loss, gna, gk, gl, gra = loss_and_gradients(m, steps, target, checkpoint_every=64)
    rng = np.random.default_rng(2)
    k = m._instance_count("hh")
    base = {"gna": np.full(k, 0.12), "gk": np.full(k, 0.036), "gl": np.full(k, 0.0003)}
    grads = {"gna": gna, "gk": gk, "gl": gl}

    def loss_at(d):
        m.set_hh_densities(d["gna"], d["gk"], d["gl"])
        val = loss_and_gradients(m, steps, target, checkpoint_every=64)[0]
        return val

    for name in ("gna", "gk", "gl"):
        idx = rng.choice(k, 4, replace=False)
        idx[0] = 0                                   # always include a soma
        for i in idx:
            h = 1e-4 * base[name][i]
            d = {kk: v.copy() for kk, v in base.items()}
            d[name][i] += h
            lp = loss_at(d)
            d[name][i] -= 2 * h
            lm = loss_at(d)
            fd = (lp - lm) / (2 * h)
            assert grads[name][i] == pytest.approx(fd, rel=1e-4, abs=1e-9 * abs(loss) / base[name][i])
    m.set_hh_densities(base["gna"], base["gk"], base["gl"])
    h = 1e-4 * 100.0
    m.set_cytoplasmic_resistance(100.0 + h)
    lp = loss_and_gradients(m, steps, target, checkpoint_every=64)[0]
    m.set_cytoplasmic_resistance(100.0 - h)
    lm = loss_and_gradients(m, steps, target, checkpoint_every=64)[0]
    assert gra == pytest.approx((lp - lm) / (2 * h), rel=1e-4)
    m.close()


def test_checkpoint_interval_does_not_change_gradients():
    tree = random_tree(200, seed=81)
    m, _ = _model([tree])
    target = np.full((150, 1), -60.0)
    a = loss_and_gradients(m, 150, target, checkpoint_every=150)
    b = loss_and_gradients(m, 150, target, checkpoint_every=37)
    assert a[0] == pytest.approx(b[0], rel=1e-13)
    for x, y in zip(a[1:4], b[1:4]):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(x).max()
    assert a[4] == pytest.approx(b[4], rel=1e-12)
    m.close()


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_overlapped_recompute_gives_the_serial_gradients(precision):
    """The recompute of checkpoint segment k-1 on a second stream beside the reverse
    sweep of segment k (two tapes) changes no operation: bit-identical to one stream."""
    trees = [random_tree(120 + 37 * i, seed=300 + i) for i in range(12)]
    steps, K = 230, 40
    m, _ = _model(trees, precision=precision, amps=tuple(0.2 + 0.03 * i for i in range(12)))
    target = np.random.default_rng(4).uniform(-70.0, -55.0, (steps, len(trees)))
    runs = []
    for overlap in (0, 1, 1):
        m._ctx.set_option("adjoint_overlap", overlap)
        m.reset_state()
        runs.append(loss_and_gradients(m, steps, target, checkpoint_every=K))
        runs[-1] = runs[-1] + (m.get_data("Segment.voltage").copy(),)
    assert m._ctx.get_option("adjoint_overlap") == 1
    for r in runs[1:]:
        assert r[0] == runs[0][0] and r[4] == runs[0][4]
        for x, y in zip(r[1:4], runs[0][1:4]):
            assert np.array_equal(x, y)
        assert np.array_equal(r[5], runs[0][5])
    m.close()


def test_fp32_adjoint_close_to_fp64():
    trees = [random_tree(300, seed=91)]
    steps = 200
    m64, _ = _model(trees, precision="f64")
    target = _target(m64, steps, np.random.default_rng(3))
    r64 = loss_and_gradients(m64, steps, target, checkpoint_every=100)
    m32, _ = _model(trees, precision="f32")
    r32 = loss_and_gradients(m32, steps, target, checkpoint_every=100)
    assert r32[0] == pytest.approx(r64[0], rel=1e-3)
    for x32, x64 in zip(r32[1:4], r64[1:4]):
        assert np.linalg.norm(x32 - x64) <= 1e-2 * np.linalg.norm(x64)
    assert r32[4] == pytest.approx(r64[4], rel=1e-2)
    m64.close(); m32.close()


def test_autograd_function_wraps_the_adjoint():
    tree = random_tree(80, seed=5)
    m, _ = _model([tree])
    k = m._instance_count("hh")
    target = np.full((100, 1), -65.0)
    gna = torch.full((k,), 0.12, dtype=torch.float64, requires_grad=True)
    gk = torch.full((k,), 0.036, dtype=torch.float64, requires_grad=True)
    gl = torch.full((k,), 0.0003, dtype=torch.float64, requires_grad=True)
    ra = torch.tensor(100.0, dtype=torch.float64, requires_grad=True)
    L = trace_loss(m, gna, gk, gl, ra, 100, target, checkpoint_every=25)
    (3.0 * L).backward()
    ref = loss_and_gradients(m, 100, target, checkpoint_every=25)
    assert L.item() == pytest.approx(ref[0], rel=1e-12)
    assert np.allclose(gna.grad.numpy(), 3.0 * ref[1], rtol=1e-10, atol=0)
    assert ra.grad.item() == pytest.approx(3.0 * ref[4], rel=1e-10)
    m.close()


def test_adjoint_refuses_a_lumped_propagator():
    """The reverse sweep takes P^T from detailed balance, which lumped pruning breaks."""
    m = nw.RxD_Model(time_step=DT, temperature=CELSIUS, precision="f64", propagator_tolerance=1e-6,
                     propagator_lump=True, mechanisms=[nw.HH.configure(**HH_KW)])
    nr = m.add_tree(random_tree(60, seed=2))
    m.insert_everywhere("hh")
    nr.root.inject_current(0.3, 1e6)
    m._sync()
    with pytest.raises(NeuwonError, match="lumped"):
        loss_and_gradients(m, 20, np.full((20, 1), -65.0), checkpoint_every=10)
    m.close()
