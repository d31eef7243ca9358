"""The build's level bookkeeping on the library's host threads
(skf_level_candidates, skf_level_reorder) against the numpy formulation, on
host trees with random ranks and pivot orders standing in for the IDs
(no device work): candidates of every level of 2D and 3D adaptive trees,
and the skeleton-first reorder with its candidate -> position map."""
import numpy as np
import pytest


def _fake_build(points, leaf):
    from skelfmm_gb300.recursive_skel import RecursiveSkeletonization
    from skelfmm_gb300.tree import BalancedTree

    tree = BalancedTree(points, leaf)
    f = RecursiveSkeletonization.__new__(RecursiveSkeletonization)
    f.tree, f.N, f.nlevels = tree, tree.N, tree.nlevels
    for name in ("_ids", "_off", "_cand_src", "_final_pos"):
        setattr(f, name, [None] * tree.nlevels)
    f.bs_list = np.zeros(tree.nboxes, np.int64)
    f.rank_list = np.zeros(tree.nboxes, np.int64)
    return f


def _reorder_numpy(off, perm, ids):
    bs = np.diff(off)
    src = np.repeat(off[:-1], bs) + perm.astype(np.int64)
    fp = np.empty(ids.shape[0], dtype=np.int64)
    fp[src] = np.arange(ids.shape[0], dtype=np.int64)
    return ids[src], fp


@pytest.mark.parametrize("case", [("cube", 3, 30000, 32), ("gaussian_clusters", 3, 60000, 64),
                                  ("curvy_annulus", 2, 40000, 50), ("square", 2, 20000, 16)])
def test_native_level_bookkeeping_equals_numpy(case):
    import ctypes

    from skelfmm_gb300 import _lib
    from skelfmm_gb300.tree import get_point_dist

    name, _, n, leaf = case
    pts = get_point_dist(n, name, rng=np.random.default_rng(n))
    f = _fake_build(pts, leaf)
    tree = f.tree
    rng = np.random.default_rng(7)
    lib = _lib.load()
    for lev in range(tree.nlevels - 1, 0, -1):
        f._level_candidates_numpy(lev)
        ref = (f._ids[lev].copy(), f._off[lev].copy(), f._cand_src[lev].copy(), f.bs_list.copy())
        f._level_candidates(lev)
        assert np.array_equal(f._ids[lev], ref[0]) and np.array_equal(f._off[lev], ref[1])
        assert np.array_equal(f._cand_src[lev], ref[2]) and np.array_equal(f.bs_list, ref[3])
        # stand-in ID: random ranks and box-local pivot orders
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        off = f._off[lev]
        bs = np.diff(off)
        f.rank_list[ls:le] = np.minimum(bs, rng.integers(1, 40, le - ls))
        perm = (np.concatenate([rng.permutation(b) for b in bs]) if bs.size else np.zeros(0)).astype(np.int32)
        want_ids, want_fp = _reorder_numpy(off, perm, f._ids[lev])
        got_ids = np.empty_like(f._ids[lev])
        got_fp = np.empty(f._ids[lev].shape[0], dtype=np.int64)
        _lib.check(lib.skf_level_reorder(le - ls, _lib.ptr(off), _lib.ptr(perm), _lib.ptr(f._ids[lev]),
                                         _lib.ptr(got_ids), _lib.ptr(got_fp)), "skf_level_reorder")
        assert np.array_equal(got_ids, want_ids) and np.array_equal(got_fp, want_fp)
        f._ids[lev] = got_ids
    # a pivot order outside its box is rejected
    off = np.array([0, 2, 3], dtype=np.int64)
    bad = np.array([0, 2, 0], dtype=np.int32)
    ids = np.arange(3, dtype=np.int64)
    out, fp = np.empty(3, np.int64), np.empty(3, np.int64)
    assert lib.skf_level_reorder(2, _lib.ptr(off), _lib.ptr(bad), _lib.ptr(ids), _lib.ptr(out),
                                 _lib.ptr(fp)) == _lib.SKF_ERR_ARG
    total = ctypes.c_int64()
    assert lib.skf_level_candidates(1, None, None, None, None, 8, 0, None, None, None, None, 1, None, None, None,
                                    ctypes.byref(total)) == _lib.SKF_ERR_ARG


@pytest.mark.parametrize("case", [("gaussian_clusters", 60000, 64), ("curvy_annulus", 40000, 50)])
def test_native_parent_slots_and_gather_equal_numpy(case):
    """skf_parent_slots and skf_gather_i64 against numpy on a stand-in build
    (random ranks and pivot orders) skeletonized down to level 2."""
    from skelfmm_gb300 import _lib
    from skelfmm_gb300.tree import get_point_dist

    name, n, leaf = case
    f = _fake_build(get_point_dist(n, name, rng=np.random.default_rng(n)), leaf)
    tree = f.tree
    rng = np.random.default_rng(3)
    f.root_level = 2
    for lev in range(tree.nlevels - 1, f.root_level, -1):
        f._level_candidates(lev)
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        off = f._off[lev]
        bs = np.diff(off)
        f.rank_list[ls:le] = np.minimum(bs, rng.integers(1, 30, le - ls))
        perm = np.concatenate([rng.permutation(b) for b in bs]) if bs.size else np.zeros(0, np.int64)
        src = np.repeat(off[:-1], bs) + perm
        fp = np.empty(src.shape[0], dtype=np.int64)
        fp[src] = np.arange(src.shape[0])
        f._ids[lev] = f._ids[lev][src]
        f._final_pos[lev] = fp
    for lev in range(f.root_level, -1, -1):
        f._level_candidates(lev)
    # entry bases per level as the ragged build lays them out
    ebase = np.zeros(tree.nlevels + 1, dtype=np.int64)
    for lev in range(tree.nlevels):
        ebase[lev + 1] = ebase[lev] + (0 if f._off[lev] is None else int(f._off[lev][-1]))
    E = int(ebase[-1])
    assert np.array_equal(f._parent_slots(ebase, E), f._parent_slots_numpy(ebase, E))
    idx = rng.integers(0, E, 100000)
    src = rng.integers(-5, 5, E)
    out = np.empty(idx.shape[0], dtype=np.int64)
    _lib.check(_lib.load().skf_gather_i64(idx.shape[0], _lib.ptr(idx), _lib.ptr(src), E, _lib.ptr(out)), "gather")
    assert np.array_equal(out, src[idx])
    idx[7] = E
    assert _lib.load().skf_gather_i64(idx.shape[0], _lib.ptr(idx), _lib.ptr(src), E, _lib.ptr(out)) == _lib.SKF_ERR_ARG
