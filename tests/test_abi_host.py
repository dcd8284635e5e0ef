"""CPU tests: the C-ABI library builds, loads and exports every declared symbol;
host-side logic (morphology, geometry, sorting, clamps, NMODL front end,
contour-integral exponential) behaves.  No kernel is launched."""
import ctypes
import math
import os
import re

import numpy as np
import pytest
import scipy.linalg

import neuwon_gb300 as nw
from neuwon_gb300 import _lib
from neuwon_gb300.build import LIB, build
from neuwon_gb300.morphology import geometry, neuron_sizes, passive_electric, random_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "neuwon_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(nw_\w+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    build()
    lib = ctypes.CDLL(LIB)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(_lib.EXPORTS)


def test_every_option_name_is_documented_in_the_header():
    """nw_set_option / nw_get_option accept exactly the names the header documents."""
    src = open(os.path.join(ROOT, "neuwon_gb300", "csrc", "nw_api.cu")).read()
    names = set(re.findall(r'nm == "([a-z0-9_]+)"', src))
    header = open(HEADER).read()
    assert len(names) > 30
    assert sorted(n for n in names if f'"{n}"' not in header) == []


def test_version_call_needs_no_gpu():
    lib = _lib.load()
    assert lib.nw_version() >= 100


def test_context_creation_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.NeuwonError):
        _lib.Context(0, "f32")


def test_random_tree_is_seeded_and_binary():
    a = random_tree(3000, seed=4)
    b = random_tree(3000, seed=4)
    assert np.array_equal(a.parent, b.parent) and np.array_equal(a.coordinates, b.coordinates)
    counts = np.bincount(a.parent[1:], minlength=3000)
    assert counts[0] <= 4 and counts[1:].max() <= 2
    assert np.all(a.parent[1:] < np.arange(1, 3000))
    d = a.diameter[1:]
    assert d.max() <= 2.0 + 1e-12 and d.min() >= 0.5 - 1e-12
    L = np.linalg.norm(a.coordinates[1:] - a.coordinates[a.parent[1:]], axis=1)
    soma_child = a.parent[1:] == 0
    assert np.all((L[~soma_child] >= 5) & (L[~soma_child] <= 15))


def test_neuron_sizes_log_uniform():
    s = neuron_sizes(1024, seed=0)
    assert s.min() >= 500 and s.max() <= 20000
    assert 3.5e6 < s.sum() < 6.5e6


def test_capacitance_uses_creation_area():
    """A parent's capacitance does not see children attached later (segment.py:36-37)."""
    t = random_tree(50, seed=1)
    g = geometry(t)
    R, C = passive_electric(g)
    leaf = np.bincount(t.parent[1:], minlength=50) == 0
    np.testing.assert_allclose(C[leaf], 1e-14 * g["surface_area"][leaf])
    assert np.any(np.abs(C[~leaf][1:] - 1e-14 * g["surface_area"][~leaf][1:]) > 0)


def test_model_sorts_segments_by_neuron_stably():
    m = nw.RxD_Model()
    a = m.Neuron([0, 0, 0], 10)
    b = m.Neuron([50, 0, 0], 10)
    s1 = a.root.add_segment([12, 0, 0], 1)
    s2 = b.root.add_segment([62, 0, 0], 1)
    s3 = s1.add_segment([20, 0, 0], 1)
    order = np.argsort(m._seg_neuron[:m._n], kind="stable")        # Database.sort
    assert list(order) == [0, 2, 4, 1, 3]
    assert s3.parent == s1 and s1.children == [s3]
    dev = nw.morphology.device_order(m._parent[:m._n], m._seg_neuron[:m._n], 2)
    assert list(dev) == [0, 2, 4, 1, 3]                             # a chain: the same


def test_device_order_is_neuron_sort_refined_by_preorder():
    """Neurons stay contiguous in Database.sort's order; within a neuron every
    subtree occupies consecutive positions (depth-first, children in creation order)."""
    rng = np.random.default_rng(0)
    for trial in range(30):
        N = int(rng.integers(1, 5))
        parent, nid = [-1] * N, list(range(N))
        for k in range(int(rng.integers(1, 150))):
            j = int(rng.integers(0, N))
            cand = [i for i in range(len(parent)) if nid[i] == j]
            parent.append(int(rng.choice(cand)))
            nid.append(j)
        parent, nid = np.array(parent), np.array(nid)
        order = nw.morphology.device_order(parent, nid, N)
        stable = np.argsort(nid, kind="stable")
        assert np.array_equal(nid[order], nid[stable])              # same neuron blocks
        children = [[] for _ in parent]
        for i, p in enumerate(parent):
            if p >= 0:
                children[p].append(i)
        expect = []
        for j in range(N):
            st = [j]
            while st:
                u = st.pop()
                expect.append(u)
                st.extend(reversed(children[u]))
        assert np.array_equal(order, expect)


def test_inject_current_schedules_half_step_ticks():
    m = nw.RxD_Model(time_step=0.1)
    r = m.Neuron([0, 0, 0], 10).root
    r.inject_current(0.2, 1.0)
    seg, amps, first, count = m._clamps[-1]
    assert (seg, first, count) == (0, 1, 20) and amps == 0.2 * 1e-9   # electric.py:120


def test_nmodl_front_end_reads_hh_parameters(tmp_path):
    mod = tmp_path / "hh.mod"
    mod.write_text("NEURON { SUFFIX hh USEION na WRITE gna, ena }\n"
                   "PARAMETER {\n gnabar = .12 (S/cm2) <0,1e9>\n gkbar = .036 (S/cm2)\n"
                   " glbar = .0003 (S/cm2)\n ena = +60 (mV)\n ek = -88 (mV)\n el = -54.3 (mV)\n}\n")
    cls = nw.NMODL(str(mod))
    assert issubclass(cls, nw.HH)
    assert (cls.gnabar, cls.ek, cls.el) == (0.12, -88.0, -54.3)
    bad = tmp_path / "pas.mod"
    bad.write_text("NEURON { SUFFIX pas NONSPECIFIC_CURRENT i }\n")       # no density parameter
    with pytest.raises(NotImplementedError):
        nw.NMODL(str(bad))
    ode = tmp_path / "ode.mod"
    ode.write_text("NEURON { SUFFIX ode NONSPECIFIC_CURRENT i }\nPARAMETER { g = 1 (S/cm2) }\nSTATE { x }\n"
                   "BREAKPOINT { SOLVE d METHOD cnexp  g = g*x }\nDERIVATIVE d { x' = -x }\n")
    with pytest.raises(NotImplementedError, match="DERIVATIVE"):
        nw.NMODL(str(ode))


def test_user_python_mechanisms_are_rejected():
    class Foo(nw.Mechanism):
        @classmethod
        def get_name(cls):
            return "foo"
    with pytest.raises(NotImplementedError):
        nw.RxD_Model(mechanisms=[Foo])


def _tree_matrix(t, h_ms):
    R, C = passive_electric(geometry(t))
    n = len(t)
    A = np.zeros((n, n))
    h = h_ms * 1e-3
    for c in range(1, n):
        p = t.parent[c]
        A[p, c] += h / (R[c] * C[p]); A[c, c] -= h / (R[c] * C[c])
        A[c, p] += h / (R[c] * C[c]); A[p, p] -= h / (R[c] * C[p])
    return A


def test_contour_exponential_method_matches_scipy():
    """The device build's mathematics (parabolic contour, N = 32), restated densely."""
    t = random_tree(150, seed=9)
    for h_ms in (0.0125, 0.05, 0.5):
        A = _tree_matrix(t, h_ms)
        P = scipy.linalg.expm(A)
        N = 32
        th = -np.pi + (np.arange(N) + 0.5) * 2 * np.pi / N
        th = th[th > 0]
        z = N * (0.1309 - 0.1194 * th ** 2 + 0.25j * th)
        zp = N * (-0.2388 * th + 0.25j)
        Q = sum((np.exp(zk) * zpk * np.linalg.inv(zk * np.eye(len(t)) - A)).imag for zk, zpk in zip(z, zp))
        Q *= 2.0 / N
        assert np.abs(Q - P).max() < 2e-14


def test_tree_resolvent_by_edge_pivots_matches_dense_inverse():
    """Row i of (zI - A)^{-1} as products of directed-edge ratios (device algorithm, in numpy)."""
    t = random_tree(40, seed=2)
    R, C = passive_electric(geometry(t))
    n = len(t)
    h = 0.05e-3
    A = _tree_matrix(t, 0.05)
    z = 3.0 + 2.0j
    apc = lambda c: h / (R[c] * C[t.parent[c]])
    acp = lambda c: h / (R[c] * C[c])
    M_diag = z - np.diag(A)
    down = M_diag.astype(complex).copy()
    for c in range(n - 1, 0, -1):
        down[t.parent[c]] -= apc(c) * acp(c) / down[c]
    T = np.zeros(n, complex); up = np.zeros(n, complex)
    T[0] = down[0]
    for c in range(1, n):
        up[c] = T[t.parent[c]] + apc(c) * acp(c) / down[c]
        T[c] = down[c] - apc(c) * acp(c) / up[c]
    G = np.linalg.inv(z * np.eye(n) - A)
    children = {i: [c for c in range(1, n) if t.parent[c] == i] for i in range(n)}
    for i in (0, 7, 23, 39):
        row = np.zeros(n, complex)
        stack = [(i, -1, 1.0 / T[i])]
        while stack:
            cur, frm, y = stack.pop()
            row[cur] = y
            p = t.parent[cur]
            if p >= 0 and p != frm:
                stack.append((p, cur, acp(cur) / up[cur] * y))
            for c in children[cur]:
                if c != frm:
                    stack.append((c, cur, apc(c) / down[c] * y))
        np.testing.assert_allclose(row, G[i], rtol=1e-12, atol=1e-15)
