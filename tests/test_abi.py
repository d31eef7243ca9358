"""The C ABI library (libskf.so) loads and exports every function that
include/skf.h declares; argument validation answers without a GPU (no compute
calls are made here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from skelfmm_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.load()


def declared_functions():
    text = open(os.path.join(REPO, "include", "skf.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(skf_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_the_header():
    from skelfmm_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_strings_and_version(lib):
    from skelfmm_gb300 import _lib

    assert lib.skf_version() >= 1
    assert lib.skf_status_string(_lib.SKF_OK) == b"ok"
    assert b"argument" in lib.skf_status_string(_lib.SKF_ERR_ARG)
    assert b"scratch" in lib.skf_status_string(_lib.SKF_ERR_SCRATCH)


def test_invalid_arguments_are_rejected_before_any_device_work(lib):
    from skelfmm_gb300 import _lib

    h = ctypes.c_void_p()
    assert lib.skf_plan_create(None, ctypes.byref(h)) == _lib.SKF_ERR_ARG
    d = _lib.PlanDesc()
    d.op = 99
    assert lib.skf_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SKF_ERR_ARG
    d.op = 1
    d.ndim = 2  # 3D operator with 2D points
    assert lib.skf_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SKF_ERR_ARG
    assert lib.skf_plan_apply(None, None, None, 0, None) == _lib.SKF_ERR_ARG
    assert lib.skf_plan_set_option(None, 1, 1) == _lib.SKF_ERR_ARG
    # bad operator / precision / empty batch on the kernel and build entry points
    assert lib.skf_kernel_apply(42, 0.0, 1, 1, 1, None, None, None, None, None, None, None, None, None, 0,
                                None) == _lib.SKF_ERR_ARG
    assert lib.skf_kernel_apply(1, 0.0, 0, 0, 0, None, None, None, None, None, None, None, None, None, 0,
                                None) == _lib.SKF_OK
    assert lib.skf_skel_boxes(1, 0.0, 1, None, None, None, None, 0.5, 0, 1e-6, None, None, None, None,
                              None) == _lib.SKF_ERR_ARG
    assert lib.skf_skel_boxes_noalloc(1, 0.0, 0, None, None, None, None, 0.5, 400, 1e-6, None, None, None, None,
                                      None) == _lib.SKF_OK
    # several trees in one launch: bad operator, missing per-box lengths, empty
    assert lib.skf_skel_boxes_multi(42, 0.0, 1, None, None, None, None, None, 400, 1e-6, None, None, None, None,
                                    None) == _lib.SKF_ERR_ARG
    assert lib.skf_skel_boxes_multi(1, 0.0, 1, None, None, None, None, None, 400, 1e-6, None, None, None, None,
                                    None) == _lib.SKF_ERR_ARG
    assert lib.skf_skel_boxes_multi(1, 0.0, 0, None, None, None, None, None, 400, 1e-6, None, None, None, None,
                                    None) == _lib.SKF_OK
    # tree: dimension, depth (ndim x depth <= 63), leaf size, keys, output handle
    t = ctypes.c_void_p()
    for args in ((4, 10, 1, 20), (3, 10, 1, 22), (2, 10, 1, 0), (3, 0, 1, 20)):
        nd, n, key, depth = args
        assert lib.skf_tree_build(nd, n, ctypes.c_void_p(8) if key else None, depth, 16, ctypes.byref(t),
                                  None) == _lib.SKF_ERR_ARG
    assert lib.skf_tree_build(3, 10, None, 20, 16, ctypes.byref(t), None) == _lib.SKF_ERR_ARG
    assert lib.skf_tree_build(3, 10, ctypes.c_void_p(8), 20, 0, ctypes.byref(t), None) == _lib.SKF_ERR_ARG
    assert lib.skf_tree_build(3, 10, ctypes.c_void_p(8), 20, 16, None, None) == _lib.SKF_ERR_ARG
    assert lib.skf_tree_query(None, None, None) == _lib.SKF_ERR_ARG
    assert lib.skf_tree_export(None, *([None] * 11)) == _lib.SKF_ERR_ARG
    lib.skf_tree_destroy(None)
    # lists: dimension, root level, missing tables; sort: bit count, empty input
    total = ctypes.c_int64()
    assert lib.skf_lists_count(4, 10, None, None, None, None, 0, None, 0, None, ctypes.byref(total),
                               None) == _lib.SKF_ERR_ARG
    assert lib.skf_lists_count(3, 10, None, None, None, None, -1, None, 0, None, ctypes.byref(total),
                               None) == _lib.SKF_ERR_ARG
    assert lib.skf_lists_fill(3, 10, None, None, None, None, 0, None, 0, None, None, None, None) == _lib.SKF_ERR_ARG
    assert lib.skf_sort_keys(10, None, None, None, 0, None) == _lib.SKF_ERR_ARG
    assert lib.skf_sort_keys(10, None, None, None, 65, None) == _lib.SKF_ERR_ARG
    assert lib.skf_sort_keys(0, None, None, None, 60, None) == _lib.SKF_OK
    assert lib.skf_morton_keys(3, 10, None, None, 1.0, 22, None, None, None) == _lib.SKF_ERR_ARG


def test_errors_map_to_python_exceptions():
    from skelfmm_gb300 import _lib

    with pytest.raises(ValueError):
        _lib.check(_lib.SKF_ERR_ARG, "x")
    with pytest.raises(_lib.SkfError) as e:
        _lib.check(_lib.SKF_ERR_SCRATCH, "x")
    assert e.value.status == _lib.SKF_ERR_SCRATCH


def test_non_finite_coordinates_are_rejected_by_plan_create(lib):
    """A NaN coordinate in the ragged description: SKF_ERR_ARG before any
    device allocation (the host validation runs first)."""
    import numpy as np

    from skelfmm_gb300 import _lib

    xyz = np.array([[0.1, 0.2, 0.3], [np.nan, 0.5, 0.5]])
    keep = dict(level=np.zeros(1, np.int32), off=np.array([0, 2], np.int64), rank=np.zeros(1, np.int32),
                pslot=np.full(2, -1, np.int64), pe=np.arange(2, dtype=np.int64), pp=np.arange(2, dtype=np.int64),
                toff=np.full(1, -1, np.int64), t=np.zeros(1), loff=np.array([0, 1], np.int64),
                lsrc=np.zeros(1, np.int32), lkind=np.full(1, 3, np.int8), xyz=xyz)
    d = _lib.PlanDesc()
    d.op, d.ndim, d.kappa, d.npoints = 1, 3, 0.0, 2
    d.nboxes, d.nlevels, d.root_level = 1, 1, 0
    d.box_level, d.box_off, d.box_rank = (keep[k].ctypes.data for k in ("level", "off", "rank"))
    d.entry_xyz, d.entry_pslot = keep["xyz"].ctypes.data, keep["pslot"].ctypes.data
    d.nperm, d.perm_entry, d.perm_point = 2, keep["pe"].ctypes.data, keep["pp"].ctypes.data
    d.t_off, d.t_data, d.t_len = keep["toff"].ctypes.data, keep["t"].ctypes.data, 1
    d.list_off, d.list_src, d.list_kind = (keep[k].ctypes.data for k in ("loff", "lsrc", "lkind"))
    h = ctypes.c_void_p()
    assert lib.skf_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SKF_ERR_ARG
    assert not h.value


def test_python_api_rejects_non_finite_inputs():
    """A NaN point, normal or charge is refused on the host with ValueError
    (no build or device work starts)."""
    import numpy as np

    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts = np.random.default_rng(0).random((500, 3))
    bad = pts.copy()
    bad[7, 1] = np.nan
    with pytest.raises(ValueError):
        SkelFMM(bad, operators.LAPLACE_3D, tol=1e-6, leaf_size=64, defer_build=True)
    geom = pts / np.linalg.norm(pts, axis=1, keepdims=True)
    geom[3, 0] = np.inf
    with pytest.raises(ValueError):
        SkelFMM(pts, operators.LAPLACE_DOUBLE_LAYER_3D, geometry=geom, tol=1e-6, leaf_size=64, defer_build=True)
    f = SkelFMM(pts, operators.LAPLACE_3D, tol=1e-6, leaf_size=64, defer_build=True)
    f._is_built = True  # the charge check precedes any device work
    q = np.ones(500)
    q[11] = np.nan
    with pytest.raises(ValueError):
        f.apply(q)


def test_max_bs_and_max_rank_must_be_integers():
    """max_bs / max_rank are accepted (they pre-size the reference's padded
    storage and never cap a rank); non-integers are refused."""
    import numpy as np

    from skelfmm_gb300 import operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    pts = np.random.default_rng(0).random((500, 2))
    with pytest.raises(ValueError):
        SkelFMM(pts, operators.LAPLACE_2D, leaf_size=64, max_bs=10.5, max_rank=3, defer_build=True)
    SkelFMM(pts, operators.LAPLACE_2D, leaf_size=64, max_bs=100, max_rank=3, defer_build=True)
