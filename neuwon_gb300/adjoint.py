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
