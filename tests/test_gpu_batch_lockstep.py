"""Lockstep build of many instances: the IDs of one level of every instance
run in one ``skf_skel_boxes_multi`` launch (each box with its own tree's
proxy surface).  The result matches the instances built one after another
(same ranks up to pivot ties of the differently scheduled FP64 QR), and the
applies agree with the FP64 direct sum; covered for a point kernel, a
geometry kernel, and a complex kernel whose proxy counts differ between
instances (boxes of several launches per level)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _build_pair(pts, op, param=0.0, geometries=None, tol=1e-6, leaf=128):
    from skelfmm_gb300.batch import SkelFMMBatch

    kw = dict(tol=tol, leaf_size=leaf, param=param, geometries=geometries, precision="fp64", tune=False)
    a = SkelFMMBatch(pts, op, lockstep=True, **kw)
    b = SkelFMMBatch(pts, op, lockstep=False, **kw)
    return a, b


def _compare(a, b, xs, tol_apply):
    ra, rb = a.ragged.box_rank.astype(np.int64), b.ragged.box_rank.astype(np.int64)
    assert ra.shape == rb.shape
    assert np.array_equal(a.ragged.box_level, b.ragged.box_level)
    same = np.mean(ra == rb)
    assert same >= 0.97, same
    assert np.abs(ra - rb).max() <= 2
    ya, yb = a.apply(xs), b.apply(xs)
    for y1, y2 in zip(ya, yb):
        assert np.abs(y1 - y2).max() <= tol_apply * np.abs(y2).max()
    errs = a.relerr(xs, ya, ncheck=200)
    assert errs.max() < 1e-5, errs
    torch.cuda.synchronize()


def test_lockstep_laplace2d_uneven():
    from skelfmm_gb300 import operators
    from skelfmm_gb300.tree import get_point_dist

    rng = np.random.default_rng(3)
    sizes = (1500, 6000, 2500, 20000, 900, 12000)
    pts = [get_point_dist(n, "curvy_annulus", rng=rng) for n in sizes]
    xs = [np.random.RandomState(i + 1).randn(n) for i, n in enumerate(sizes)]
    a, b = _build_pair(pts, operators.LAPLACE_2D)
    # every instance skeletonized to the same root as alone
    for fa, fb in zip(a.instance_ragged, b.instance_ragged):
        assert fa.root_level == fb.root_level and fa.nlevels == fb.nlevels
    _compare(a, b, xs, 1e-5)


def test_lockstep_double_layer_sphere():
    from skelfmm_gb300 import operators
    from skelfmm_gb300.tree import get_point_dist

    rng = np.random.default_rng(4)
    sizes = (8000, 3000, 15000)
    pts, geoms = [], []
    for i, n in enumerate(sizes):
        p = get_point_dist(n, "sphere_surface", rng=rng)
        pts.append(p * (1.0 + 0.5 * i) + i)
        geoms.append(p.copy())
    xs = [np.random.RandomState(i + 7).randn(n) for i, n in enumerate(sizes)]
    a, b = _build_pair(pts, operators.LAPLACE_DOUBLE_LAYER_3D, geometries=geoms, leaf=200)
    _compare(a, b, xs, 1e-5)


def test_lockstep_helmholtz2d_mixed_proxy_counts():
    from skelfmm_gb300 import operators
    from skelfmm_gb300.recursive_skel import nproxy_levels
    from skelfmm_gb300.tree import BalancedTree, get_point_dist

    rng = np.random.default_rng(5)
    sizes = (4000, 9000, 2500)
    scales = (1.0, 2.0, 0.5)
    pts = [get_point_dist(n, "curvy_annulus", rng=rng) * s for n, s in zip(sizes, scales)]
    kappa = 10.0
    # the instances' proxy counts differ at equal levels
    counts = [tuple(nproxy_levels(2, 1e-6, kappa, BalancedTree(p, 128).L0, 4)) for p in pts]
    assert len(set(counts)) > 1
    xs = [np.random.RandomState(i + 11).randn(n) + 1j * np.random.RandomState(i + 12).randn(n)
          for i, n in enumerate(sizes)]
    a, b = _build_pair(pts, operators.HELMHOLTZ_2D, param=kappa)
    _compare(a, b, xs, 1e-5)


def test_lockstep_rejects_mixed_operators():
    from skelfmm_gb300 import operators
    from skelfmm_gb300.batch import skel_trees_lockstep
    from skelfmm_gb300.recursive_skel import RecursiveSkeletonization
    from skelfmm_gb300.tree import BalancedTree, get_point_dist

    rng = np.random.default_rng(6)
    p = get_point_dist(3000, "curvy_annulus", rng=rng)
    f1 = RecursiveSkeletonization(BalancedTree(p, 128), operators.LAPLACE_2D, 0.0, 1e-6)
    f2 = RecursiveSkeletonization(BalancedTree(p, 128), operators.HELMHOLTZ_2D, 5.0, 1e-6)
    with pytest.raises(ValueError):
        skel_trees_lockstep([f1, f2], 500)
