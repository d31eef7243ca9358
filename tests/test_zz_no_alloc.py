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


def _call(fname, op, kappa, tol, nproxy, xs, centers, length, cplx):
    import torch

    from skelfmm_gb300 import _lib

    bs = np.array([x.shape[0] for x in xs], dtype=np.int64)
    off = np.zeros(len(xs) + 1, dtype=np.int64)
    np.cumsum(bs, out=off[1:])
    cap = bs * bs // 4 + bs
    t_off = np.zeros(len(xs), dtype=np.int64)
    np.cumsum(cap[:-1], out=t_off[1:])
    dev = torch.device("cuda")
    x_t = torch.from_numpy(np.ascontiguousarray(np.concatenate(xs))).to(dev)
    c_t = torch.from_numpy(np.ascontiguousarray(centers)).to(dev)
    off_t = torch.from_numpy(off).to(dev)
    t_off_t = torch.from_numpy(t_off).to(dev)
    rank = torch.full((len(xs),), -1, dtype=torch.int32, device=dev)
    perm = torch.full((int(off[-1]),), -1, dtype=torch.int32, device=dev)
    t_buf = torch.zeros(int(cap.sum()), dtype=torch.complex128 if cplx else torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    status = getattr(_lib.load(), fname)(
        op, float(kappa), len(xs), _lib.ptr(off_t), _lib.ptr(x_t), None, _lib.ptr(c_t), float(length),
        int(nproxy), float(tol), _lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t), _lib.ptr(t_buf),
        ctypes.c_void_p(stream))
    _lib.check(status, fname)
    torch.cuda.synchronize()
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


def test_noalloc_rejects_boxes_beyond_the_scratch():
    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(3)
    # one 3D box of 15,000 points: 600 proxies x 15,000 x 8 B = 72 MB > 64 MiB
    x = rng.random((15000, 3)) * 0.1
    with pytest.raises(_lib.SkfError) as err:
        _call("skf_skel_boxes_noalloc", 1, 0.0, 1e-6, 512, [x], np.array([[0.05, 0.05, 0.05]]), 0.1, False)
    assert err.value.status == _lib.SKF_ERR_SCRATCH
    assert "scratch" in str(err.value)
