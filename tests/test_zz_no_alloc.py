"""The no-allocation entry point skf_skel_boxes_noalloc against skf_skel_boxes.

skf_skel_boxes_noalloc serves callers that may not allocate device memory on
the build path (for example, a process whose own pool owns the GPU's memory):
it runs the same proxy-ID kernel with its workspace in a fixed device array
inside the library.  This file is named to be collected last, so a run that
stops at its first failure has already run every other test; it also passes
on its own in a fresh process (the first call sets the array up).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _level(points, leaf_size):
    """Boxes of the deepest level of a tree: ragged points, centres, side length."""
    from skelfmm_gb300.tree import BalancedTree

    tree = BalancedTree(points, leaf_size)
    boxes = tree.get_boxes_level(tree.nlevels - 1)
    xs = [points[tree.get_box_inds(b)] for b in boxes]
    return xs, tree.get_boxes_centers(boxes), tree.get_box_length(boxes[0])


def _prepared(xs, centers, length, cplx):
    """Device buffers of one call, as the two argument groups around
    (nproxy, tol): (off, x, geom, centers, length) and (rank, perm, t_off,
    t_out, stream); the tensors stay referenced by the returned tuple."""
    import torch

    from skelfmm_gb300 import _lib

    bs = np.array([x.shape[0] for x in xs], dtype=np.int64)
    off = np.zeros(len(xs) + 1, dtype=np.int64)
    np.cumsum(bs, out=off[1:])
    cap = bs * bs // 4 + bs
    t_off = np.zeros(len(xs), dtype=np.int64)
    np.cumsum(cap[:-1], out=t_off[1:])
    dev = torch.device("cuda")
    keep = [torch.from_numpy(np.ascontiguousarray(np.concatenate(xs))).to(dev),
            torch.from_numpy(np.ascontiguousarray(centers)).to(dev), torch.from_numpy(off).to(dev),
            torch.from_numpy(t_off).to(dev), torch.zeros(len(xs), dtype=torch.int32, device=dev),
            torch.zeros(int(off[-1]), dtype=torch.int32, device=dev),
            torch.zeros(int(cap.sum()), dtype=torch.complex128 if cplx else torch.float64, device=dev)]
    x_t, c_t, off_t, t_off_t, rank, perm, t_buf = keep
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ((_lib.ptr(off_t), _lib.ptr(x_t), None, _lib.ptr(c_t), float(length)),
            (_lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t), _lib.ptr(t_buf), stream), keep)


def _call(fname, op, kappa, tol, nproxy, xs, centers, length, cplx):
    import torch

    from skelfmm_gb300 import _lib

    a0, a1, keep = _prepared(xs, centers, length, cplx)
    rank, perm, t_buf = keep[4], keep[5], keep[6]
    rank.fill_(-1)
    perm.fill_(-1)
    status = getattr(_lib.load(), fname)(op, float(kappa), len(xs), *a0, int(nproxy), float(tol), *a1)
    _lib.check(status, fname)
    torch.cuda.synchronize()
    bs = np.array([x.shape[0] for x in xs], dtype=np.int64)
    t_off = keep[3].cpu().numpy()
    rank_h = rank.cpu().numpy()
    t_h = t_buf.cpu().numpy()
    blocks = [t_h[t_off[i]: t_off[i] + rank_h[i] * (bs[i] - rank_h[i])] for i in range(len(xs))]
    return rank_h, perm.cpu().numpy(), blocks


def _compare(op, kappa, tol, nproxy, xs, centers, length, cplx):
    ref = _call("skf_skel_boxes", op, kappa, tol, nproxy, xs, centers, length, cplx)
    got = _call("skf_skel_boxes_noalloc", op, kappa, tol, nproxy, xs, centers, length, cplx)
    assert np.array_equal(got[0], ref[0])
    assert np.all(ref[0] > 0)
    assert np.array_equal(got[1], ref[1])
    for a, b in zip(got[2], ref[2]):
        # the ID tests' tolerance; same kernel and inputs, so in practice identical
        assert np.allclose(a, b, rtol=1e-10, atol=1e-10 * max(1.0, float(np.abs(b).max(initial=0.0))))


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    rng = np.random.default_rng(11)
    # call 1: 3D Laplace, leaf level of a uniform cube (64 boxes of ~94 points)
    xs3, c3, l3 = _level(rng.random((6000, 3)), 200)
    _compare(1, 0.0, 1e-6, 400, xs3, c3, l3, False)
    # call 2 right after: 2D Helmholtz (complex), different sizes; the array
    # still holds call 1's proxy matrices and must not leak into the result
    xs2, c2, l2 = _level(rng.random((3000, 2)), 60)
    _compare(2, 3.0, 1e-6, 60, xs2, c2, l2, True)


def _grid_boxes(rng, nside, npts):
    """nside^2 square boxes of side 1/nside, npts random points in each."""
    h = 1.0 / nside
    ij = np.stack(np.meshgrid(np.arange(nside), np.arange(nside), indexing="ij"), -1).reshape(-1, 2)
    centers = (ij + 0.5) * h
    xs = [c + (rng.random((npts, 2)) - 0.5) * h for c in centers]
    return xs, centers, h


def test_noalloc_runs_levels_larger_than_one_batch():
    """5,184 boxes: more than the 4,096 per-batch offset slots, so the level
    runs as two batches that reuse the array (the second batch's offsets start
    past the first's boxes)."""
    rng = np.random.default_rng(21)
    xs, c, h = _grid_boxes(rng, 72, 12)
    assert len(xs) > 4096
    _compare(0, 0.0, 1e-6, 60, xs, c, h, False)


def test_noalloc_allocates_no_device_memory():
    """Free device memory (cudaMemGetInfo) is the same before and after a
    call, once the library's pooled workspaces are returned; the call also
    leaves torch's allocator untouched."""
    import torch

    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(4)
    xs, c, h = _grid_boxes(rng, 40, 30)
    _call("skf_skel_boxes_noalloc", 0, 0.0, 1e-6, 60, xs, c, h, False)  # set-up call
    args = _prepared(xs, c, h, False)
    torch.cuda.synchronize()
    _lib.check(_lib.load().skf_trim_workspace(), "skf_trim_workspace")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    torch_reserved0 = torch.cuda.memory_reserved()
    status = _lib.load().skf_skel_boxes_noalloc(0, 0.0, len(xs), *args[0], 60, 1e-6, *args[1])
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert status == _lib.SKF_OK
    assert free1 == free0
    assert torch.cuda.memory_reserved() == torch_reserved0


def test_noalloc_reports_non_finite_points():
    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(8)
    xs, c, h = _grid_boxes(rng, 6, 20)
    xs[5][3, 0] = np.nan
    with pytest.raises(_lib.SkfError) as err:
        _call("skf_skel_boxes_noalloc", 0, 0.0, 1e-6, 60, xs, c, h, False)
    assert err.value.status == _lib.SKF_ERR_ID


def test_noalloc_rejects_boxes_beyond_the_scratch():
    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(3)
    # one 3D box of 15,000 points: 600 proxies x 15,000 x 8 B = 72 MB > 64 MiB
    x = rng.random((15000, 3)) * 0.1
    with pytest.raises(_lib.SkfError) as err:
        _call("skf_skel_boxes_noalloc", 1, 0.0, 1e-6, 512, [x], np.array([[0.05, 0.05, 0.05]]), 0.1, False)
    assert err.value.status == _lib.SKF_ERR_SCRATCH
    assert "scratch" in str(err.value)
