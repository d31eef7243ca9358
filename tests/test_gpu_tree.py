"""The tree's device front end (skf_morton_keys and a stable device sort)
against the host build: every level array, the point order and the
neighbour tables are identical, on the golden point sets and on 4e6 points
in 32 Gaussian clusters (the learned-rank workload)."""
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
    for name in ("_children", "_parent", "_colleagues", "_coarse", "_box_center", "_box_length", "_leaves"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name


@pytest.mark.parametrize("name", build_cases())
def test_device_front_end_gives_the_host_tree_on_golden_points(name):
    from skelfmm_gb300.tree import BalancedTree

    from skelfmm_gb300 import tree as T

    d = load_build(name)
    saved = T.DEVICE_FRONT_END_MIN_POINTS
    T.DEVICE_FRONT_END_MIN_POINTS = 1  # the golden sets are smaller than the threshold
    try:
        b = BalancedTree(d["points"], int(d["leaf_size"]), device="cuda")
    finally:
        T.DEVICE_FRONT_END_MIN_POINTS = saved
    _same(BalancedTree(d["points"], int(d["leaf_size"])), b)


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
