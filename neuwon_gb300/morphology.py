"""Seeded synthetic neuron morphologies and the reference's geometry rules.

The geometry functions restate, as vectorised numpy over whole trees, the
per-segment rules of the reference:

* ``neuwon/rxd/neuron/geometry.py:75-155`` -- length, primary flag, secondary
  length, surface area (end caps on leaves, attachment disks of lateral
  children subtracted), cross-sectional area and volume;
* ``neuwon/rxd/neuron/electric.py:49-54`` -- axial resistance
  ``Ra*1e4*length/xarea`` (ohm) and capacitance ``Cm*1e-14*area`` (F).

One quirk is kept on purpose: the reference computes a segment's capacitance
once, when the segment is created (``segment.py:36-37``), while its surface
area is recomputed every time a child is attached (``geometry.py:91``).  So
capacitance uses the *creation-time* area (the segment as a leaf, with its
end cap and no children), and mechanism magnitudes use the area at insertion
time, which for mechanisms inserted after the tree is grown is the final area.

The tree recipe (used for every workload of this package):

* segment 0 is the soma, a sphere of diameter ``soma_diameter`` at the origin;
* every further segment is a cylinder of length U(5, 15) um.  With
  probability ``p_branch`` it attaches to a uniformly chosen node that can take
  a lateral branch (a cylinder with exactly one child, or the soma while it has
  fewer than ``max_soma_children`` children); otherwise it extends a uniformly
  chosen leaf.  Cylinders never get more than two children.
* directions are isotropic random unit vectors; children of the soma start on
  its surface, so their secondary length is the drawn length;
* diameters taper linearly with path distance from the soma surface, from
  ``d_proximal`` to ``d_distal`` at the farthest tip.
"""
import math
import numpy as np

EPSILON = float(np.finfo(np.float64).eps)  # neuwon/database/dtypes.py:4
NULL = -1


class Tree:
    """One neuron's morphology in creation order (parents precede children)."""
    __slots__ = ("parent", "coordinates", "diameter")

    def __init__(self, parent, coordinates, diameter):
        self.parent = np.asarray(parent, dtype=np.int64)
        self.coordinates = np.asarray(coordinates, dtype=np.float64).reshape(-1, 3)
        self.diameter = np.asarray(diameter, dtype=np.float64)
        n = len(self.parent)
        assert self.coordinates.shape == (n, 3) and self.diameter.shape == (n,)
        idx = np.arange(n)
        nonroot = self.parent >= 0
        if np.any(self.parent[nonroot] >= idx[nonroot]):
            raise ValueError("parents must be created before their children")

    def __len__(self):
        return len(self.parent)


def random_tree(num_segments, seed, *, p_branch=0.1, soma_diameter=20.0,
                d_proximal=2.0, d_distal=0.5, length_range=(5.0, 15.0),
                max_soma_children=4):
    """Grow one seeded random binary tree of ``num_segments`` segments."""
    n = int(num_segments)
    if n < 1:
        raise ValueError("a neuron needs at least its soma")
    rng = np.random.default_rng(seed)
    u_choice = rng.random(n)
    u_pick = rng.random(n)
    lengths = rng.uniform(length_range[0], length_range[1], n)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)

    parent = np.full(n, NULL, dtype=np.int64)
    nchild = np.zeros(n, dtype=np.int64)
    # Swap-remove sets: leaves, and nodes that can take a lateral branch.
    leaves = np.empty(n, dtype=np.int64); leaf_pos = np.full(n, -1, np.int64); n_leaves = 0
    branch = np.empty(n, dtype=np.int64); branch_pos = np.full(n, -1, np.int64); n_branch = 0

    def add(arr, pos, cnt, x):
        arr[cnt] = x; pos[x] = cnt
        return cnt + 1

    def remove(arr, pos, cnt, x):
        k = pos[x]
        last = arr[cnt - 1]
        arr[k] = last; pos[last] = k; pos[x] = -1
        return cnt - 1

    n_leaves = add(leaves, leaf_pos, n_leaves, 0)
    n_branch = add(branch, branch_pos, n_branch, 0)
    for i in range(1, n):
        if u_choice[i] < p_branch and n_branch > 0:
            p = int(branch[min(int(u_pick[i] * n_branch), n_branch - 1)])
        else:
            p = int(leaves[min(int(u_pick[i] * n_leaves), n_leaves - 1)])
        parent[i] = p
        nchild[p] += 1
        if leaf_pos[p] >= 0:
            n_leaves = remove(leaves, leaf_pos, n_leaves, p)
        if p == 0:
            if nchild[0] >= max_soma_children and branch_pos[0] >= 0:
                n_branch = remove(branch, branch_pos, n_branch, 0)
        elif nchild[p] == 1:
            n_branch = add(branch, branch_pos, n_branch, p)
        elif branch_pos[p] >= 0:
            n_branch = remove(branch, branch_pos, n_branch, p)
        n_leaves = add(leaves, leaf_pos, n_leaves, i)

    # Path distance from the soma surface, then the linear taper.
    path = np.zeros(n)
    for i in range(1, n):
        path[i] = path[parent[i]] + lengths[i]
    far = path.max() if n > 1 else 1.0
    diameter = d_proximal - (d_proximal - d_distal) * path / far
    diameter[0] = soma_diameter
    coords = np.zeros((n, 3))
    r_soma = 0.5 * soma_diameter
    for i in range(1, n):
        p = parent[i]
        step = lengths[i] + (r_soma if p == 0 else 0.0)
        coords[i] = coords[p] + step * dirs[i]
    return Tree(parent, coords, diameter)


def neuron_sizes(num_neurons, seed, lo=500, hi=20000):
    """Log-uniform segment counts in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), num_neurons))).astype(np.int64)


def geometry(tree):
    """Reference geometry of a whole tree (neuwon/rxd/neuron/geometry.py:75-155).

    Returns a dict of float64 arrays: length, primary (bool), secondary_length,
    surface_area (final, with all children attached), creation_area (the
    segment alone as a leaf, which is what its capacitance sees),
    cross_sectional_area, volume.
    """
    parent, xyz, d = tree.parent, tree.coordinates, tree.diameter
    n = len(parent)
    root = parent < 0
    pidx = np.where(root, 0, parent)
    delta = xyz - xyz[pidx]
    length = np.where(root, (2.0 / 3.0) * d, np.sqrt(np.einsum("ij,ij->i", delta, delta)))
    # First child (lowest index) of a cylinder is its primary extension.
    first_child = np.full(n, n, dtype=np.int64)
    child_idx = np.nonzero(~root)[0]
    np.minimum.at(first_child, parent[child_idx], child_idx)
    parent_is_sphere = root[pidx]
    primary = (~root) & (~parent_is_sphere) & (first_child[pidx] == np.arange(n))
    parent_radius = 0.5 * d[pidx]
    enveloped = length < parent_radius + EPSILON
    secondary = np.where(primary | root | enveloped, length, length - parent_radius)
    nchild = np.bincount(parent[child_idx], minlength=n)
    disk = 0.25 * np.pi * (d ** 2)
    sphere = np.pi * (d ** 2)
    cyl = np.pi * d * secondary
    leaf_area = cyl + disk
    area = np.where(root, sphere, np.where(nchild == 0, leaf_area, cyl))
    lateral = child_idx[~primary[child_idx]]
    if len(lateral):
        attach = 0.25 * np.pi * (np.minimum(d[parent[lateral]], d[lateral]) ** 2)
        np.subtract.at(area, parent[lateral], attach)
    creation_area = np.where(root, sphere, leaf_area)
    volume = np.where(root, (4.0 / 3.0) * np.pi * (0.5 * d) ** 3, disk * secondary)
    return dict(length=length, primary=primary, secondary_length=secondary,
                surface_area=area, creation_area=creation_area,
                cross_sectional_area=disk, volume=volume)


def passive_electric(geom, cytoplasmic_resistance=100.0, membrane_capacitance=1.0):
    """Axial resistance (ohm) and capacitance (F); neuwon/rxd/neuron/electric.py:49-54."""
    Ra = cytoplasmic_resistance * 1e4   # ohm-cm -> ohm-um
    Cm = membrane_capacitance * 1e-14   # uF/cm^2 -> F/um^2
    R = Ra * geom["length"] / geom["cross_sectional_area"]
    C = Cm * geom["creation_area"]
    return R, C


def device_order(parent, seg_neuron, num_neurons):
    """Order of the segments on the device: neurons contiguous in neuron order (the
    stable sort by neuron of ``Database.sort``, database.py:189-222) and, within a
    neuron, depth-first preorder with children in creation order.  Preorder puts
    every subtree on consecutive indices, so a propagator row's columns form a few
    runs of neighbours (shared-memory and cache locality).  Vectorised: depths and
    path sums by pointer doubling, subtree sizes level by level.  Returns order
    (device position -> creation index)."""
    parent = np.asarray(parent, dtype=np.int64)
    seg_neuron = np.asarray(seg_neuron, dtype=np.int64)
    n = len(parent)
    if n == 0:
        return np.empty(0, np.int64)
    has_p = parent >= 0

    def path_sum(val):
        """sum of val over the node and its ancestors (roots included)."""
        acc = val.astype(np.int64).copy()
        anc = np.where(has_p, parent, -1)
        while True:
            m = anc >= 0
            if not m.any():
                return acc
            idx = np.nonzero(m)[0]
            a = anc[idx]
            acc[idx] += acc[a]
            anc[idx] = anc[a]

    depth = path_sum(has_p.astype(np.int64))
    size = np.ones(n, np.int64)
    by_depth = np.argsort(-depth, kind="stable")
    d_sorted = depth[by_depth]
    bounds = np.flatnonzero(np.diff(d_sorted)) + 1
    for grp in np.split(by_depth, bounds):
        grp = grp[has_p[grp]]
        if len(grp):
            np.add.at(size, parent[grp], size[grp])
    # Exclusive prefix of earlier siblings' subtree sizes (children in creation order).
    kids = np.flatnonzero(has_p)
    kids = kids[np.lexsort((kids, parent[kids]))]
    csum = np.cumsum(size[kids])
    first = np.r_[True, parent[kids][1:] != parent[kids][:-1]]
    group_start = np.maximum.accumulate(np.where(first, np.arange(len(kids)), 0))
    before = np.where(first, 0, csum - size[kids] - (csum[group_start] - size[kids[group_start]]))
    val = np.zeros(n, np.int64)
    val[kids] = 1 + before
    local = path_sum(val)
    counts = np.bincount(seg_neuron, minlength=num_neurons)
    start = np.concatenate([[0], np.cumsum(counts)])[:-1]
    pos = start[seg_neuron] + local
    order = np.empty(n, np.int64)
    order[pos] = np.arange(n)
    return order
