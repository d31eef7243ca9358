"""Multi-instance batching on the GPU: uneven curvy-annulus 2D Laplace
instances concatenated into one plan, applied in one pass per phase (and
from a captured CUDA graph), agree with each instance applied alone and with
the FP64 direct sum."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = (1500, 6000, 2500, 20000, 900)


@pytest.fixture(scope="module")
def instances():
    from skelfmm_gb300.tree import get_point_dist

    rng = np.random.default_rng(0)
    pts = [get_point_dist(n, "curvy_annulus", rng=rng) for n in SIZES]
    xs = [np.random.RandomState(i + 1).randn(n) for i, n in enumerate(SIZES)]
    return pts, xs


def test_batch_fp64_matches_single_instances(instances):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.batch import SkelFMMBatch
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts, xs = instances
    b = SkelFMMBatch(pts, operators.LAPLACE_2D, tol=1e-6, leaf_size=128, precision="fp64", tune=False,
                     lockstep=False)
    ys = b.apply(xs)
    for p, x, y in zip(pts, xs, ys):
        y1 = SkelFMM(p, operators.LAPLACE_2D, tol=1e-6, leaf_size=128).apply(x)
        assert np.abs(y - y1).max() <= 1e-12 * np.abs(y1).max()
    errs = b.relerr(xs, ys, ncheck=300)
    assert errs.max() < 1e-5, errs


def test_batch_mixed_graph_autotuned(instances):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.batch import SkelFMMBatch

    pts, xs = instances
    b = SkelFMMBatch(pts, operators.LAPLACE_2D, tol=1e-6, leaf_size=128, precision="mixed", tune=True)
    assert b.tuning and b.plan.tuned in b.tuning
    ys = b.apply(xs)
    errs = b.relerr(xs, ys, ncheck=300)
    assert errs.max() < 1e-5, errs
    # the same apply replayed from a CUDA graph gives the same numbers
    b.capture()
    ys_g = b.apply(xs)
    for y, yg in zip(ys, ys_g):
        assert np.array_equal(y, yg)
    # new charges through the captured graph
    xs2 = [np.random.RandomState(100 + i).randn(n).astype(np.float32) for i, n in enumerate(SIZES)]
    ys2 = b.apply(xs2)
    assert b.relerr(xs2, ys2, ncheck=200).max() < 1e-5


def test_batch_rejects_wrong_length(instances):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.batch import SkelFMMBatch

    pts, xs = instances
    b = SkelFMMBatch(pts[:2], operators.LAPLACE_2D, tol=1e-6, leaf_size=128, tune=False)
    with pytest.raises(ValueError):
        b.apply([xs[0]])
    torch.cuda.synchronize()
