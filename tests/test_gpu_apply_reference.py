"""GPU apply given the reference's own build (import path) vs the reference's
apply (SkelFMMBatched.matvec, FP64, skelfmm/batched_fmm.py:539-564)."""
import numpy as np
import pytest

from golden_util import build_cases, load_build, relinf

pytestmark = pytest.mark.gpu


def _plan(name):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.plan import Plan, ragged_from_reference
    from skelfmm_gb300.tree import BalancedTree

    d = load_build(name)
    op = operators.BY_NAME[str(d["operator"])]
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    return d, Plan(ragged_from_reference(tree, d, op, float(d["kappa"])))


@pytest.mark.parametrize("name", build_cases())
def test_fp64_apply_matches_reference(name):
    import torch
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    x = d["x"]
    xt = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    yt = torch.empty_like(xt)
    plan.apply_device(xt, yt, _lib.PREC_FP64, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    y = yt.cpu().numpy()
    # torch's bessel_j0/y0 in the reference vs CUDA's j0/y0 differ near 1e-10
    tol = 1e-9 if str(d["operator"]) == "HELMHOLTZ_2D" else 1e-12
    assert relinf(y, d["y_batched"]) < tol


@pytest.mark.parametrize("name", build_cases())
def test_mixed_apply_meets_tolerance(name):
    import torch
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    y = np.empty_like(d["x"])
    plan.apply_host(np.ascontiguousarray(d["x"]), y, _lib.PREC_MIXED)
    # mixed = FP32 kernel evaluation on top of the FMM's own approximation;
    # the same bound for every operator (the double layers' (x-y).n, which
    # cancels to ~r^2 on a surface, is formed from FP32 pairs to FP32
    # rounding of the result)
    tol = 2e-6
    err_fmm = relinf(d["y_batched"][d["dense_idx"]], d["y_dense"])
    assert relinf(y, d["y_batched"]) < tol
    assert relinf(y[d["dense_idx"]], d["y_dense"]) < err_fmm + tol


def test_host_and_device_apply_agree():
    import torch
    from skelfmm_gb300 import _lib

    d, plan = _plan("lap3d_cube")
    x = np.ascontiguousarray(d["x"])
    y_host = np.empty_like(x)
    plan.apply_host(x, y_host, _lib.PREC_FP64)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    plan.apply_device(xt, yt, _lib.PREC_FP64)
    torch.cuda.synchronize()
    assert np.array_equal(yt.cpu().numpy(), y_host)
    # deterministic: no atomics, repeated applies are bitwise identical
    y2 = np.empty_like(x)
    plan.apply_host(x, y2, _lib.PREC_FP64)
    assert np.array_equal(y2, y_host)


@pytest.mark.parametrize("name", ["lap2d_square", "lap2d_annulus", "lap3d_cube", "lap3d_sphere", "helm3d_sphere"])
def test_packed_and_scalar_mixed_kernels_agree(name):
    """The packed FP32x2 kernels (Laplace, Helmholtz 3D) and the scalar FP32
    kernel perform the same per-pair arithmetic; only the summation grouping
    differs."""
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    x = np.ascontiguousarray(d["x"])
    y_packed = np.empty_like(x)
    plan.apply_host(x, y_packed, _lib.PREC_MIXED)
    plan.set_option(1, 1)
    y_scalar = np.empty_like(x)
    plan.apply_host(x, y_scalar, _lib.PREC_MIXED)
    plan.set_option(1, 0)
    assert relinf(y_packed, y_scalar) < 1e-6
    assert relinf(y_packed, d["y_batched"]) < 2e-6


@pytest.mark.parametrize("name", ["lap2d_square", "lap2d_annulus", "lap3d_cube", "lap3d_sphere", "helm3d_sphere"])
def test_symmetric_translations_agree(name):
    """Evaluating each kernel block once for both directions (symmetric path)
    gives the same apply as evaluating every direction separately."""
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    x = np.ascontiguousarray(d["x"])
    assert plan.info.npairs_evaluated_mixed < plan.info.npairs_fused
    y_sym = np.empty_like(x)
    plan.apply_host(x, y_sym, _lib.PREC_MIXED)
    plan.set_option(3, 0)
    y_dir = np.empty_like(x)
    plan.apply_host(x, y_dir, _lib.PREC_MIXED)
    plan.set_option(3, 1)
    assert relinf(y_sym, y_dir) < 1e-6
    assert relinf(y_sym, d["y_batched"]) < 2e-6
    y2 = np.empty_like(x)
    plan.apply_host(x, y2, _lib.PREC_MIXED)
    assert np.array_equal(y2, y_sym)  # deterministic


@pytest.mark.parametrize("name", ["lap3d_cube", "lap3d_c2params", "lap2d_annulus", "helm3d_sphere"])
def test_symmetric_tile_shapes_agree(name):
    """Every tile shape of the symmetric kernel (sources per tile, blocks per
    SM, and the source-split kernel on a grid or a persistent queue) gives the
    same apply up to the order of the partial sums; each is deterministic."""
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    x = np.ascontiguousarray(d["x"])
    ys = []
    for shape in range(6):
        plan.set_option(_lib.OPT_SYM_SHAPE, shape)
        y = np.empty_like(x)
        plan.apply_host(x, y, _lib.PREC_MIXED)
        ys.append(y)
        y2 = np.empty_like(x)
        plan.apply_host(x, y2, _lib.PREC_MIXED)
        assert np.array_equal(y2, y)
    plan.set_option(_lib.OPT_SYM_SHAPE, 0)
    for y in ys[1:]:
        assert relinf(y, ys[0]) < 1e-6
    assert relinf(ys[0], d["y_batched"]) < 2e-6



@pytest.mark.parametrize("name", ["lap3d_cube", "lap2d_annulus", "lap2d_square", "helm3d_sphere", "helm2d_square"])
def test_packed_block_shapes_agree(name):
    """Every block shape of the per-direction packed kernel (4, 2 or 1 warps
    on 256-row items, 1 warp on 64-row items) gives the same apply up to the
    order of the sums, within 2e-6 of the reference's apply."""
    from skelfmm_gb300 import _lib

    d, plan = _plan(name)
    x = np.ascontiguousarray(d["x"])
    plan.set_option(_lib.OPT_SYMMETRIC, 0)
    ys = []
    for shape in range(4):
        plan.set_option(_lib.OPT_PACKED_SHAPE, shape)
        y = np.empty_like(x)
        plan.apply_host(x, y, _lib.PREC_MIXED)
        ys.append(y)
        y2 = np.empty_like(x)
        plan.apply_host(x, y2, _lib.PREC_MIXED)
        assert np.array_equal(y2, y)
    plan.set_option(_lib.OPT_PACKED_SHAPE, 0)
    plan.set_option(_lib.OPT_SYMMETRIC, 1)
    for y in ys[1:]:
        assert relinf(y, ys[0]) < 1e-6
    for y in ys:
        assert relinf(y, d["y_batched"]) < 2e-6

