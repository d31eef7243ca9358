"""The device tree (skf_morton_keys, a stable device sort, then
skf_tree_build: refinement, 2:1 balance and neighbour tables from the sorted
keys) against the host build: every level array, the point order and the
neighbour tables are identical, on the golden point sets, on degenerate sets
(coincident points down to the finest level, points on a line, a single
point) and on 4e6 points in 32 Gaussian clusters (the learned-rank
workload)."""
import time

import numpy as np
import pytest

from golden_util import build_cases, load_build

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.nlevels == b.nlevels and a.nboxes == b.nboxes
    assert np.array_equal(a.c0, b.c0) and a.L0 == b.L0
    assert np.array_equal(a._perm, b._perm)
    assert np.array_equal(a._skeys, b._skeys)
    for name in ("_Lc", "_Lk", "_Ls", "_Le", "_Lleaf"):
        for la, lb in zip(getattr(a, name), getattr(b, name)):
            assert np.array_equal(la, lb), name
    for name in ("_children", "_parent", "_colleagues", "_coarse", "_box_center", "_box_length", "_leaves",
                 "level_sep", "_box_coords", "_box_start", "_box_end", "_is_leaf", "_box_level"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
        assert getattr(a, name).dtype == getattr(b, name).dtype, name


def _device_tree(points, leaf):
    from skelfmm_gb300 import tree as T

    saved = T.DEVICE_FRONT_END_MIN_POINTS
    T.DEVICE_FRONT_END_MIN_POINTS = 1
    try:
        return T.BalancedTree(points, leaf, device="cuda")
    finally:
        T.DEVICE_FRONT_END_MIN_POINTS = saved


@pytest.mark.parametrize("name", build_cases())
def test_device_front_end_gives_the_host_tree_on_golden_points(name):
    from skelfmm_gb300.tree import BalancedTree

    from skelfmm_gb300 import tree as T

    d = load_build(name)
    # (the golden sets are smaller than the device threshold)
    b = _device_tree(d["points"], int(d["leaf_size"]))
    _same(BalancedTree(d["points"], int(d["leaf_size"])), b)


def _degenerate_sets():
    rng = np.random.default_rng(11)
    out = []
    for ndim in (2, 3):
        p = rng.random((3000, ndim))
        p[100:400] = p[7]  # 300 coincident points: split down to the finest level
        out.append((f"coincident_{ndim}d", p, 16))
        t = rng.random(5000)
        line = np.stack([t] + [t * 1e-9] * (ndim - 1), axis=1)
        out.append((f"line_{ndim}d", line, 8))
        out.append((f"single_{ndim}d", rng.random((1, ndim)), 4))
        g = np.concatenate((rng.random((2000, ndim)) * 1e-4, rng.random((2000, ndim))))
        out.append((f"dense_corner_{ndim}d", g, 10))
    return out


@pytest.mark.parametrize("case", _degenerate_sets(), ids=lambda c: c[0])
def test_device_tree_on_degenerate_sets(case):
    from skelfmm_gb300.tree import BalancedTree

    _, pts, leaf = case
    a = BalancedTree(pts, leaf)
    b = _device_tree(pts, leaf)
    _same(a, b)
    if pts.shape[0] > 1 and "coincident" in case[0]:
        assert a.nlevels == a._depth + 1


def test_device_front_end_on_4e6_clustered_points():
    from skelfmm_gb300.tree import BalancedTree, get_point_dist

    pts = get_point_dist(4_000_000, "gaussian_clusters", rng=np.random.default_rng(0))
    # coincident points (ties in the finest cell) keep their input order
    pts[1000:1010] = pts[5]
    BalancedTree(pts[:200000], 256, device="cuda")  # first use of the kernels
    t0 = time.perf_counter()
    a = BalancedTree(pts, 256)
    t1 = time.perf_counter()
    b = BalancedTree(pts, 256, device="cuda")
    t2 = time.perf_counter()
    _same(a, b)
    print(f"host tree {t1 - t0:.3f} s, device front end {t2 - t1:.3f} s")


def _lists_cases():
    out = [(n, None) for n in build_cases()]
    out += [(c[0], c) for c in _degenerate_sets() if not c[0].startswith("single")]
    return out


@pytest.mark.parametrize("case", _lists_cases(), ids=lambda c: c[0])
def test_device_lists_equal_host_lists_at_every_root_level(case):
    """skf_lists_count / skf_lists_fill against the numpy lists on the same
    tree, for every possible root level."""
    import torch

    from skelfmm_gb300.recursive_skel import RecursiveSkeletonization

    name, deg = case
    if deg is None:
        d = load_build(name)
        pts, leaf = d["points"], int(d["leaf_size"])
    else:
        _, pts, leaf = deg
    tree = _device_tree(pts, leaf)
    # only the tree and the root level enter the lists (no skeletonization,
    # so leaves of coincident points above leaf_size are allowed here)
    fmm = RecursiveSkeletonization.__new__(RecursiveSkeletonization)
    fmm.tree, fmm.nboxes, fmm.ndim, fmm.device = tree, tree.nboxes, tree.ndim, torch.device("cuda")
    for root in range(tree.nlevels):
        fmm.root_level = root
        fmm.root_boxes = np.hstack((tree.get_leaves_above(root), tree.get_boxes_level(root))).astype(np.int64)
        h = fmm._lists_host()
        g = fmm._lists_device()
        for a, b in zip(h, g):
            assert a.dtype == b.dtype and np.array_equal(a, b), (name, root)


@pytest.mark.parametrize("bits", [60, 40, 9])
def test_sort_keys_is_a_stable_sort(bits):
    """skf_sort_keys against numpy's stable argsort, on keys with many ties
    and keys using only the low ``bits`` bits."""
    import torch

    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(bits)
    n = 300_001
    keys = rng.integers(0, 1 << bits, n, dtype=np.uint64)
    keys[::7] = keys[3]  # ties
    k = torch.from_numpy(keys.view(np.int64)).cuda()
    ko = torch.empty_like(k)
    perm = torch.empty(n, dtype=torch.int64, device="cuda")
    _lib.check(_lib.load().skf_sort_keys(n, _lib.ptr(k), _lib.ptr(ko), _lib.ptr(perm), bits,
                                         torch.cuda.current_stream().cuda_stream), "skf_sort_keys")
    ref = np.argsort(keys, kind="stable")
    assert np.array_equal(perm.cpu().numpy(), ref)
    assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[ref])
