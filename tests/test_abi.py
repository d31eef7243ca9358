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


def test_errors_map_to_python_exceptions():
    from skelfmm_gb300 import _lib

    with pytest.raises(ValueError):
        _lib.check(_lib.SKF_ERR_ARG, "x")
    with pytest.raises(_lib.SkfError) as e:
        _lib.check(_lib.SKF_ERR_SCRATCH, "x")
    assert e.value.status == _lib.SKF_ERR_SCRATCH
