"""Gradients of a soma-voltage trace loss, behind torch.autograd.Function.

The reference has no differentiation.  ``trace_loss`` runs the model forward on
the GPU for ``steps`` steps from its initial state and returns
    loss = mean over steps s and neurons j of (V_soma(j) after step s - target[s, j])^2
(V_soma = the voltage of each neuron's AP-detector segment, its soma by default),
differentiable with respect to the per-segment HH densities gnabar, gkbar,
glbar (S/cm2, one per HH instance in registration order) and the cytoplasmic
resistivity Ra (ohm cm).  The gradients come from the hand-written adjoint
kernels (nw_adjoint_forward / nw_adjoint_backward): checkpoints every
``checkpoint_every`` steps, recompute, transposed-propagator products and gate
Jacobians.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _forward(model, steps, target, checkpoint_every):
    t = np.ascontiguousarray(np.asarray(target, dtype=np.float64))
    if t.shape != (steps, len(model._neuron_root)):
        raise ValueError(f"target must have shape (steps, neurons) = ({steps}, {len(model._neuron_root)})")
    loss = ctypes.c_double()
    model._ctx.call("nw_adjoint_forward", int(steps), int(checkpoint_every), _lib.ptr(t), ctypes.byref(loss))
    model.input_hook.ticks += 2 * int(steps)
    model.advance_hook.ticks += int(steps)
    return loss.value


def _backward(model):
    m = model._instance_count("hh")
    g = [np.empty(m) for _ in range(3)]
    gra = ctypes.c_double()
    model._ctx.call("nw_adjoint_backward", float(model.cytoplasmic_resistance),
                    _lib.ptr(g[0]), _lib.ptr(g[1]), _lib.ptr(g[2]), ctypes.byref(gra))
    return g[0], g[1], g[2], gra.value


def loss_and_gradients(model, steps, target, checkpoint_every=100):
    """Loss from the initial state and d loss / d (densities S/cm2, Ra) as numpy arrays."""
    model.reset_state()
    loss = _forward(model, steps, target, checkpoint_every)
    gna, gk, gl, gra = _backward(model)
    scale = model.hh_density_scale()
    return loss, gna * scale, gk * scale, gl * scale, gra


class _TraceLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, gnabar, gkbar, glbar, ra, model, steps, target, checkpoint_every):
        model.set_cytoplasmic_resistance(float(ra))
        model.set_hh_densities(gnabar.detach().cpu().numpy(), gkbar.detach().cpu().numpy(),
                               glbar.detach().cpu().numpy())
        model.reset_state()
        loss = _forward(model, steps, target, checkpoint_every)
        ctx.model = model
        ctx.device, ctx.dtype = gnabar.device, gnabar.dtype
        return torch.tensor(loss, dtype=torch.float64, device=gnabar.device)

    @staticmethod
    def backward(ctx, grad):
        model = ctx.model
        gna, gk, gl, gra = _backward(model)
        scale = model.hh_density_scale()
        as_t = lambda a: torch.as_tensor(a, dtype=ctx.dtype, device=ctx.device)
        g = grad.to(ctx.dtype)
        return (g * as_t(gna * scale), g * as_t(gk * scale), g * as_t(gl * scale),
                g * torch.tensor(gra, dtype=ctx.dtype, device=ctx.device), None, None, None, None)


def trace_loss(model, gnabar, gkbar, glbar, ra, steps, target, checkpoint_every=100):
    """Differentiable loss; see the module docstring.  gnabar/gkbar/glbar: tensors with
    one density per HH instance (S/cm2); ra: scalar tensor (ohm cm)."""
    return _TraceLoss.apply(gnabar, gkbar, glbar, ra, model, int(steps), target, int(checkpoint_every))


def central_differences(build, trees, steps, target, params, ra=100.0, h_rel=1e-4, amps=None):
    """FP64 central differences of the trace loss for a list of parameters, without
    running the whole model per parameter: a per-segment density touches one neuron
    only, and the loss is a sum over neurons, so each (neuron, +h / -h) pair runs as
    two copies of that neuron inside one FP64 model, and the difference of their
    loss terms is the whole loss's difference.  Ra touches every neuron: two FP64
    runs of the whole model.

    build(trees, precision, ra, amps) -> RxD_Model with one HH instance per segment
    (registration order = segment order) and a soma clamp per neuron;
    params: list of ("gna" | "gk" | "gl", neuron, local segment) or ("ra",);
    target: (steps, neurons) soma voltages.  Returns the derivatives (S/cm2 or
    ohm cm units, matching loss_and_gradients) in the order of params."""
    from .workloads import HH_PARAMS
    n_neurons = len(trees)
    amps = list(amps) if amps is not None else [None] * n_neurons
    base = {"gna": HH_PARAMS["gnabar"], "gk": HH_PARAMS["gkbar"], "gl": HH_PARAMS["glbar"]}
    out = [None] * len(params)
    dens_idx = [k for k, p in enumerate(params) if p[0] != "ra"]
    if dens_idx:
        copies, cols, dens = [], [], []
        for k in dens_idx:
            kind, j, local = params[k]
            for sign in (1.0, -1.0):
                copies.append(trees[j])
                cols.append(j)
                d = {g: np.full(len(trees[j]), v) for g, v in base.items()}
                d[kind][local] += sign * h_rel * base[kind]
                dens.append(d)
        m = build(copies, "f64", ra, [amps[j] for j in cols])
        m.set_hh_densities(*(np.concatenate([d[g] for d in dens]) for g in ("gna", "gk", "gl")))
        m.reset_state()
        roots = np.asarray(m._neuron_root, dtype=np.int64)
        m._ctx.call("nw_probes_set", len(roots), _lib.ptr(roots), int(steps))
        m._ctx.advance(int(steps))
        v = np.empty((steps, len(roots)))
        got = ctypes.c_int64()
        m._ctx.call("nw_probes_read", _lib.ptr(v), 1, int(steps), ctypes.byref(got))
        m.close()
        terms = ((v - np.asarray(target)[:, cols]) ** 2).sum(axis=0) / (steps * n_neurons)
        for q, k in enumerate(dens_idx):
            h = h_rel * base[params[k][0]]
            out[k] = (terms[2 * q] - terms[2 * q + 1]) / (2 * h)
    for k, p in enumerate(params):
        if p[0] != "ra":
            continue
        losses = []
        for sign in (1.0, -1.0):
            m = build(trees, "f64", ra + sign * h_rel * ra, amps)
            m.reset_state()
            roots = np.asarray(m._neuron_root, dtype=np.int64)
            m._ctx.call("nw_probes_set", len(roots), _lib.ptr(roots), int(steps))
            m._ctx.advance(int(steps))
            v = np.empty((steps, len(roots)))
            got = ctypes.c_int64()
            m._ctx.call("nw_probes_read", _lib.ptr(v), 1, int(steps), ctypes.byref(got))
            m.close()
            losses.append(((v - np.asarray(target)) ** 2).mean())
        out[k] = (losses[0] - losses[1]) / (2 * h_rel * ra)
    return out
