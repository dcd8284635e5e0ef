"""Plain FP64 PyTorch statement of the same step, for checking the adjoint with autograd.

Dense propagator torch.linalg.matrix_exp(A(Ra)) (differentiable in Ra), HH as in
nmodl_library/artificial/hh.mod with the exact gate update, current clamps on the
half-step clock, the staggered order of neuwon/rxd/rxd_model.py:63-80 and the
soma-trace loss of neuwon_gb300.adjoint.
"""
import numpy as np
import torch

from oracle.reference_step import coefficient_coo


def _vtrap(x, y):
    r = x / y
    small = torch.abs(r) < 1e-6
    safe = torch.where(small, torch.ones_like(x), x)
    return torch.where(small, y * (1 - r / 2), safe / torch.expm1(safe / y))


def _gates(v, q10):
    am = 0.1 * _vtrap(-(v + 40), 10.0); bm = 4 * torch.exp(-(v + 65) / 18)
    ah = 0.07 * torch.exp(-(v + 65) / 20); bh = 1 / (torch.exp(-(v + 35) / 10) + 1)
    an = 0.01 * _vtrap(-(v + 55), 10.0); bn = 0.125 * torch.exp(-(v + 65) / 80)
    return (am, bm), (ah, bh), (an, bn)


def trace_loss(parent, R0, C, area, ra0, gnabar, gkbar, glbar, ra, *, dt, celsius, steps, clamps,
               det, target, ena, ek, el, v_init=-70.0):
    """clamps: [(segment, amps, first_tick, num_ticks)]; det: detector segment per neuron."""
    n = len(parent)
    h = 0.5 * dt
    dst, src, coef = coefficient_coo(parent, R0, C, h)
    A0 = np.zeros((n, n))
    np.add.at(A0, (dst, src), coef)
    A = torch.from_numpy(A0) * (ra0 / ra)
    P = torch.linalg.matrix_exp(A)
    C_t = torch.from_numpy(np.asarray(C, dtype=np.float64))
    kI = h / C_t
    kG = h * 1e-3 / C_t
    scale = torch.from_numpy(np.asarray(area, dtype=np.float64)) * 1e-8
    cna, ck, cl = gnabar * scale, gkbar * scale, glbar * scale
    q10 = 3.0 ** ((celsius - 6.3) / 10.0)
    v0 = torch.full((n,), float(v_init), dtype=torch.float64)
    (am, bm), (ah, bh), (an, bn) = _gates(v0, q10)
    m, hg, ng = am / (am + bm), ah / (ah + bh), an / (an + bn)
    V = v0
    target = torch.as_tensor(np.asarray(target, dtype=np.float64))
    det = torch.as_tensor(np.asarray(det, dtype=np.int64))
    loss = torch.zeros((), dtype=torch.float64)
    tick, gv = 0, False
    for s in range(steps):
        for half in (0, 1):
            tick += 1
            I = torch.zeros(n, dtype=torch.float64)
            for (seg, amps, first, count) in clamps:
                if first <= tick < first + count:
                    I = I + torch.nn.functional.one_hot(torch.tensor(seg), n).double() * amps
            if gv:
                gna = cna * m * m * m * hg
                gk = ck * ng * ng * ng * ng
                G = (gna + gk) + cl
                GE = (gna * ena + gk * ek) + cl * el
                E = GE / G
            else:
                G = torch.zeros(n, dtype=torch.float64)
                E = torch.zeros(n, dtype=torch.float64)
            alpha = torch.exp(-kG * G)
            x = E - (E - V) * alpha + kI * I
            V = P @ x
            if half == 0:
                (am, bm), (ah, bh), (an, bn) = _gates(V, q10)
                dtq = dt * q10
                minf, hinf, ninf = am / (am + bm), ah / (ah + bh), an / (an + bn)
                m = minf + (m - minf) * torch.exp(-dtq * (am + bm))
                hg = hinf + (hg - hinf) * torch.exp(-dtq * (ah + bh))
                ng = ninf + (ng - ninf) * torch.exp(-dtq * (an + bn))
                gv = True
        loss = loss + ((V[det] - target[s]) ** 2).sum()
    return loss / (steps * len(det))
