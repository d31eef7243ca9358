"""Saved builds replayed on the GPU and the captured CUDA graph of a built
operator: load-then-apply is bitwise equal to the saved operator's apply, a
build made by the CPU oracle and saved in the framework's format matches
the oracle's apply to 1e-12, and graph replays equal eager applies bitwise."""
import os

import numpy as np
import pytest

from golden_util import GOLDEN, relinf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_load_then_apply_is_bitwise_equal(precision, tmp_path):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts = np.random.default_rng(3).random((20000, 3))
    x = np.random.RandomState(4).randn(pts.shape[0])
    f = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=100, precision=precision)
    y = f.apply(x)
    path = os.path.join(tmp_path, "op.npz")
    f.save(path)
    g = SkelFMM.load(path)
    assert g.precision == precision and g.rank_max == f.rank_max
    if getattr(f.plan, "tuned", None):
        # the mixed apply's scheme is chosen by timing: use the saved one's
        from skelfmm_gb300 import _lib

        sym, shape = f.plan.tuned
        g.plan.set_option(_lib.OPT_SYMMETRIC, sym)
        g.plan.set_option(_lib.OPT_SYM_SHAPE if sym else _lib.OPT_PACKED_SHAPE, shape)
    assert np.array_equal(g.apply(x), y)


def test_cpu_oracle_build_replays_on_the_gpu():
    from skelfmm_gb300.plan import load_ragged
    from skelfmm_gb300.skel_fmm import SkelFMM

    path = os.path.join(GOLDEN, "saved_oracle_lap3d_sphere.npz")
    _, extra = load_ragged(path)
    f = SkelFMM.load(path)
    y = f.apply(extra["x"])
    assert relinf(y, extra["y_oracle"]) < 1e-12
    fm = SkelFMM.load(path, precision="mixed")
    assert relinf(fm.apply(extra["x"]), extra["y_oracle"]) < 2e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_eager_apply(precision):
    import torch

    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts = np.random.default_rng(5).random((30000, 3))
    x = np.random.RandomState(6).randn(pts.shape[0])
    f = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=120, precision=precision)
    y_eager = f.apply(x)
    f.capture()
    y1 = f.apply(x)
    y2 = f.apply(x)
    assert np.array_equal(y1, y_eager) and np.array_equal(y2, y_eager)
    xt = torch.from_numpy(x).cuda()
    assert np.array_equal(f.apply_device(xt).cpu().numpy(), y_eager)
    g = SkelFMM(pts, operators.HELMHOLTZ_3D, tol=1e-5, leaf_size=120, param=3.0, precision=precision,
                cuda_graph=True)
    xc = x + 1j * np.random.RandomState(7).randn(pts.shape[0])
    yg = g.apply(xc)
    g._graph = None
    assert np.array_equal(g.apply(xc), yg)
