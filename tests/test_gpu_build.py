"""GPU build (proxy matrices + pivoted-QR IDs on the device) vs the CPU
oracle's restatement of the reference build (skelfmm/recursive_skel.py,
skelfmm/util.py:13-51,87-124), and the full SkelFMM pipeline vs an FP64
direct sum."""
import numpy as np
import pytest

from golden_util import OPNAME, load_build, relinf
from oracle import skel_oracle as O

pytestmark = pytest.mark.gpu

CASES = ["lap2d_square", "lap2d_annulus", "lap3d_cube", "lap3d_sphere", "helm2d_square",
         "helm3d_sphere", "lapdl3d_sphere", "helmadl3d_sphere", "lap3d_c2params", "helm3d_sphere_k5",
         "lapdl3d_sphere_1e6", "helmdl3d_sphere_1e6"]


def _both(name):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.recursive_skel import RecursiveSkeletonization
    from skelfmm_gb300.tree import BalancedTree

    d = load_build(name)
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    geom = d.get("geometry")
    g = RecursiveSkeletonization(tree, operators.BY_NAME[str(d["operator"])], float(d["kappa"]),
                                 float(d["tol"]), geometry=geom).skel_tree(int(d["npoints_max"]))
    o = O.OracleBuild(tree, O.OPERATORS[OPNAME[str(d["operator"])]], float(d["kappa"]), float(d["tol"]),
                      geometry=geom).skel_tree(int(d["npoints_max"]))
    return d, tree, g, o


@pytest.mark.parametrize("name", CASES)
def test_gpu_ids_match_oracle(name):
    d, tree, g, o = _both(name)
    assert g.root_level == o.root_level
    # ranks: identical except where an |R_kk| sits within rounding of the cutoff
    diff = np.abs(g.rank_list - o.rank_list)
    assert diff.max() <= 1
    assert np.count_nonzero(diff) <= max(1, tree.nboxes // 50)
    same = 0
    for b in range(tree.nboxes):
        if o.proj[b] is None or g.rank_list[b] != o.rank_list[b]:
            continue
        r = int(o.rank_list[b])
        if r == 0:
            continue
        if np.array_equal(np.sort(g.pid[b][:r]), np.sort(o.pid[b][:r])):
            same += 1
            if np.array_equal(g.pid[b][:r], o.pid[b][:r]) and g.proj[b].size:
                # same skeleton order and redundant order: T agrees
                red_same = np.array_equal(g.pid[b][r:], o.pid[b][r:])
                if red_same:
                    assert relinf(g.proj[b], o.proj[b]) < 1e-6
    ncmp = sum(1 for b in range(tree.nboxes) if o.proj[b] is not None and o.rank_list[b] > 0)
    assert same >= 0.9 * ncmp


@pytest.mark.parametrize("name", CASES)
def test_gpu_build_apply_accuracy(name):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    d = load_build(name)
    op = operators.BY_NAME[str(d["operator"])]
    f = SkelFMM(d["points"], op, geometry=d.get("geometry"), tol=float(d["tol"]),
                leaf_size=int(d["leaf_size"]), param=float(d["kappa"]), npoints_max=int(d["npoints_max"]))
    y = f.apply(d["x"])
    # the reference's own error on the same targets bounds what the method gives
    err_ref = relinf(d["y_batched"][d["dense_idx"]], d["y_dense"])
    err = relinf(y[d["dense_idx"]], d["y_dense"])
    assert err < max(10 * err_ref, 10 * float(d["tol"]), 1e-12)
    fm = SkelFMM(d["points"], op, geometry=d.get("geometry"), tol=float(d["tol"]),
                 leaf_size=int(d["leaf_size"]), param=float(d["kappa"]), npoints_max=int(d["npoints_max"]),
                 precision="mixed")
    ym = fm.apply(d["x"])
    slack = 2e-6
    assert relinf(ym[d["dense_idx"]], d["y_dense"]) < err + slack


def test_skelfmm_api_contract(capsys):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    rng = np.random.default_rng(0)
    xx = rng.random((1200, 2))
    f = SkelFMM(xx, operators.LAPLACE_2D, tol=1e-5, leaf_size=20, defer_build=True)
    assert f.build_time_seconds == 0.0 and f.rank_max == 0
    q = np.random.RandomState(0).randn(1200)
    y = f.apply(q)
    assert "Building SkelFMM on first matvec" in capsys.readouterr().out
    assert y.shape == (1200,) and f.build_time_seconds > 0 and f.rank_max > 0
    assert f.relerr_fmm_apply_check(q, ncheck=200) < 1e-4
    bm = f.benchmark_matvec(nrepeat=2, warmup=1)
    assert bm["min_seconds"] > 0
    with pytest.raises(ValueError):
        f.apply(np.zeros((3, 3)))
    with pytest.raises(TypeError):
        SkelFMM(xx, "laplace", defer_build=True)
    custom = operators.PointKernelOperator("toy", 2, operators.laplace_2d)
    with pytest.raises(NotImplementedError):
        SkelFMM(xx, custom, tol=1e-5, leaf_size=20)
    # direct sum on the GPU agrees with the dense numpy kernel
    idx = np.arange(0, 1200, 7)
    dense = operators.LAPLACE_2D.numpy_matrix(xx[idx], xx) @ q
    assert relinf(f.direct_apply(q, idx), dense) < 1e-12


def test_clustered_build_with_large_boxes():
    """Clustered points give a few boxes of ~1,000+ candidates per level; the
    build factors those on thread-block clusters.  The FP64 apply still meets
    the tolerance against the direct sum, and ranks stay within one of a
    rebuild (same tree, same IDs: the build is deterministic)."""
    import torch

    from skelfmm_gb300 import _lib, operators
    from skelfmm_gb300.skel_fmm import SkelFMM, direct_sum
    from skelfmm_gb300.tree import get_point_dist

    pts = get_point_dist(300_000, "gaussian_clusters", rng=np.random.default_rng(0))
    f = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=256, keep_host_fmm=True)
    g = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=256, keep_host_fmm=True)
    assert np.array_equal(f.fmm.rank_list, g.fmm.rank_list)
    bs = np.array([0 if p is None else p.shape[0] for p in f.fmm.pid])
    assert bs.max() >= 800  # large boxes present
    x = np.random.RandomState(1).randn(pts.shape[0])
    y = f.apply(x)
    idx = np.random.default_rng(0).choice(pts.shape[0], 500, replace=False)
    yd = direct_sum(operators.LAPLACE_3D, pts, x, idx)
    assert relinf(y[idx], yd) < 1e-6
    torch.cuda.synchronize()
