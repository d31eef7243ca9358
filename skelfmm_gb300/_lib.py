"""ctypes binding of the C ABI in ``include/skf.h`` (``libskf.so``).

The library is built in-tree by ``skelfmm_gb300._build``; there is no CPU
fallback: if the library is missing or cannot be loaded, every call that needs
it raises.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libskf.so")

SKF_OK = 0
SKF_ERR_ARG = 1
SKF_ERR_OOM = 2
SKF_ERR_CUDA = 3
SKF_ERR_UNSUPPORTED = 4
SKF_ERR_ID = 5
SKF_ERR_SCRATCH = 7

PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_T32 = 2

OPT_SCALAR_MIXED, OPT_PACKED_SHAPE, OPT_SYMMETRIC, OPT_SYM_SHAPE = 1, 2, 3, 4
KIND_COLLEAGUE = 0
KIND_COARSE_UP = 1
KIND_COARSE_DOWN = 2
KIND_ROOT = 3

_p = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double
_f32 = ctypes.c_float


class PlanDesc(ctypes.Structure):
    _fields_ = [
        ("op", _i32), ("ndim", _i32), ("kappa", _f64), ("npoints", _i64),
        ("nboxes", _i32), ("nlevels", _i32), ("root_level", _i32),
        ("box_level", _p), ("box_off", _p), ("box_rank", _p),
        ("entry_xyz", _p), ("entry_geom", _p), ("entry_pslot", _p),
        ("nperm", _i64), ("perm_entry", _p), ("perm_point", _p),
        ("t_off", _p), ("t_data", _p), ("t_len", _i64),
        ("list_off", _p), ("list_src", _p), ("list_kind", _p), ("t_on_device", _i32),
        ("entries_on_device", _i32),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("nentries", _i64), ("npairs_fused", _i64), ("t_scalars", _i64),
        ("device_bytes", _i64), ("nwork", _i32), ("is_complex", _i32),
        ("npairs_evaluated_mixed", _i64), ("launches_fp64", _i32), ("launches_mixed", _i32),
        ("rows_256_over_64", _f64),
    ]


# exported symbol -> (restype, argtypes); every symbol include/skf.h declares
SIGNATURES = {
    "skf_version": (_i32, []),
    "skf_status_string": (ctypes.c_char_p, [_i32]),
    "skf_plan_create": (_i32, [ctypes.POINTER(PlanDesc), ctypes.POINTER(_p)]),
    "skf_plan_destroy": (_i32, [_p]),
    "skf_plan_query": (_i32, [_p, ctypes.POINTER(PlanInfo)]),
    "skf_plan_apply": (_i32, [_p, _p, _p, _i32, _p]),
    "skf_plan_apply_host": (_i32, [_p, _p, _p, _i32, _p]),
    "skf_plan_set_option": (_i32, [_p, _i32, _i64]),
    "skf_plan_time_translations": (_i32, [_p, _i32, _i32, _p, ctypes.POINTER(ctypes.c_float)]),
    "skf_kernel_apply": (_i32, [_i32, _f64, _i32, _i32, _i32, _p, _p, _p, _p, _p, _p, _p, _p, _p, _i32, _p]),
    "skf_skel_boxes": (_i32, [_i32, _f64, _i32, _p, _p, _p, _p, _f64, _i32, _f64, _p, _p, _p, _p, _p]),
    "skf_skel_boxes_noalloc": (_i32, [_i32, _f64, _i32, _p, _p, _p, _p, _f64, _i32, _f64, _p, _p, _p, _p, _p]),
    "skf_proxy_rows": (_i32, [_i32, _i32, ctypes.POINTER(_i32)]),
    "skf_skel_boxes_randomized": (_i32, [_i32, _f64, _i32, _p, _p, _p, _p, _f64, _i32, _f64, _p, _i32, _i32,
                                         ctypes.c_uint64, _i32, _f64, _f64, _p, _p, _p, _p, _p, _p, _p]),
    "skf_copy_segments": (_i32, [_i64, _p, _p, _p, _p, _p, _i32, _p]),
    "skf_box_moments": (_i32, [_i32, _i32, _p, _p, _p, _f64, _p, _p]),
    "skf_morton_keys": (_i32, [_i32, _i64, _p, _p, _f64, _i32, _p, _p, _p]),
    "skf_sort_keys": (_i32, [_i64, _p, _p, _p, _i32, _p]),
    "skf_level_candidates": (_i32, [_i64, _p, _p, _p, _p, _i32, _i64, _p, _p, _p, _p, _i64, _p, _p, _p, _p]),
    "skf_level_reorder": (_i32, [_i64, _p, _p, _p, _p, _p]),
    "skf_parent_slots": (_i32, [_i32, _p, _p, _p, _p, _p, _i64, _p]),
    "skf_gather_i64": (_i32, [_i64, _p, _p, _i64, _p]),
    "skf_tree_build": (_i32, [_i32, _i64, _p, _i32, _i64, _p, _p]),
    "skf_tree_query": (_i32, [_p, _p, _p]),
    "skf_tree_export": (_i32, [_p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "skf_tree_destroy": (None, [_p]),
    "skf_lists_count": (_i32, [_i32, _i64, _p, _p, _p, _p, _i32, _p, _i64, _p, _p, _p]),
    "skf_lists_fill": (_i32, [_i32, _i64, _p, _p, _p, _p, _i32, _p, _i64, _p, _p, _p, _p]),
    "skf_skel_boxes_multi": (_i32, [_i32, _f64, _i32, _p, _p, _p, _p, _p, _i32, _f64, _p, _p, _p, _p, _p]),
    "skf_trim_workspace": (_i32, []),
    "skf_mlp_num_params": (_i64, [_i32]),
    "skf_mlp_scratch_floats": (_i64, [_i32, _i64]),
    "skf_mlp_bf16": (_i32, [_p, _p, _i64, _p]),
    "skf_mlp_predict": (_i32, [_i32, _p, _p, _i64, _p, _p]),
    "skf_mlp_train_step": (_i32, [_i32, _p, _p, _p, _p, _i64, _p, _p, _p, _p, _i32, _f32, _f32, _f32, _f32,
                                  _i32, _p, _p]),
}

_lib = None


class SkfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def load(path=None):
    """Load ``libskf.so`` (once).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python -m skelfmm_gb300._build)"
        )
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status, what=""):
    if status == SKF_OK:
        return
    msg = load().skf_status_string(status).decode()
    text = f"{what}: {msg}" if what else msg
    if status == SKF_ERR_ARG:
        raise ValueError(text)
    raise SkfError(status, text)


def ptr(a):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)
