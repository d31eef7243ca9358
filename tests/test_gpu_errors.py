"""Error paths of the device entry points, injected on the host: a NaN point
in a level's boxes makes its proxy matrix non-finite and skf_skel_boxes
returns SKF_ERR_ID (RuntimeError in Python); the library stays usable."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _skel_boxes(xs, centers, length, op=1, tol=1e-6, nproxy=400):
    import torch

    from skelfmm_gb300 import _lib

    bs = np.array([x.shape[0] for x in xs], dtype=np.int64)
    off = np.zeros(len(xs) + 1, dtype=np.int64)
    np.cumsum(bs, out=off[1:])
    t_off = np.zeros(len(xs), dtype=np.int64)
    np.cumsum((bs * bs)[:-1], out=t_off[1:])
    dev = torch.device("cuda")
    x_t = torch.from_numpy(np.ascontiguousarray(np.concatenate(xs))).to(dev)
    c_t = torch.from_numpy(np.ascontiguousarray(centers)).to(dev)
    off_t = torch.from_numpy(off).to(dev)
    t_off_t = torch.from_numpy(t_off).to(dev)
    rank = torch.zeros(len(xs), dtype=torch.int32, device=dev)
    perm = torch.zeros(int(off[-1]), dtype=torch.int32, device=dev)
    t_buf = torch.zeros(int((bs * bs).sum()), dtype=torch.float64, device=dev)
    st = _lib.load().skf_skel_boxes(op, 0.0, len(xs), _lib.ptr(off_t), _lib.ptr(x_t), None, _lib.ptr(c_t),
                                    float(length), nproxy, float(tol), _lib.ptr(rank), _lib.ptr(perm),
                                    _lib.ptr(t_off_t), _lib.ptr(t_buf),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, rank.cpu().numpy()


def _boxes(rng, nbox=6, n=120):
    centers = rng.random((nbox, 3))
    xs = [c + (rng.random((n, 3)) - 0.5) * 0.1 for c in centers]
    return xs, centers, 0.1


def test_nan_point_gives_err_id_and_the_library_stays_usable():
    from skelfmm_gb300 import _lib

    rng = np.random.default_rng(5)
    xs, centers, length = _boxes(rng)
    st, good = _skel_boxes(xs, centers, length)
    assert st == _lib.SKF_OK and np.all(good > 0)
    bad = [x.copy() for x in xs]
    bad[3][17, 2] = np.nan
    st, _ = _skel_boxes(bad, centers, length)
    assert st == _lib.SKF_ERR_ID
    assert b"non-finite" in _lib.load().skf_status_string(st)
    with pytest.raises(RuntimeError):
        _lib.check(st, "skf_skel_boxes")
    st, again = _skel_boxes(xs, centers, length)
    assert st == _lib.SKF_OK and np.array_equal(again, good)


def test_max_bs_and_max_rank_are_reported_and_do_not_cap_ranks():
    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts = np.random.default_rng(2).random((6000, 3))
    a = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=100, keep_host_fmm=True)
    b = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=100, keep_host_fmm=True, max_bs=300, max_rank=5)
    assert a.fmm.max_rank == 75 and a.fmm.max_bs == 800
    assert b.fmm.max_rank == 5 and b.fmm.max_bs == 300
    assert np.array_equal(a.fmm.rank_list, b.fmm.rank_list)
    assert b.rank_max > 5
