"""Device plan of a built skeletonization (ragged CSR layout) and its apply.

``RaggedBuild`` is the host-side description the C ABI consumes
(``skf_plan_desc`` in ``include/skf.h``); ``Plan`` owns the device copy.
``ragged_from_reference`` converts a build in the reference's padded layout
(``RecursiveSkeletonization`` after ``setup_lists``,
skelfmm/recursive_skel.py:106-120, 515-539, 622-780) — the data
``SkelFMMBatched.build_from_copy`` (skelfmm/batched_fmm.py:92-174) copies to
the device — into that description.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .operators import cuda_op_id, is_complex_op


@dataclass
class RaggedBuild:
    op: int
    ndim: int
    kappa: float
    npoints: int
    nlevels: int
    root_level: int
    box_level: np.ndarray   # int32 [nb]
    box_off: np.ndarray     # int64 [nb+1]
    box_rank: np.ndarray    # int32 [nb]
    entry_xyz: np.ndarray   # f64 [E, ndim] (numpy, or a CUDA tensor)
    entry_geom: np.ndarray | None  # f64 [E, 3] (numpy, or a CUDA tensor)
    entry_pslot: np.ndarray  # int64 [E]
    perm_entry: np.ndarray   # int64 [N]
    perm_point: np.ndarray   # int64 [N]
    t_off: np.ndarray        # int64 [nb]
    t_data: np.ndarray       # f64 or c128, flat
    list_off: np.ndarray     # int64 [nb+1]
    list_src: np.ndarray     # int32 [L]
    list_kind: np.ndarray    # int8 [L]

    @property
    def nboxes(self):
        return int(self.box_level.shape[0])

    @property
    def nentries(self):
        return int(self.box_off[-1])


def lists_to_csr(nboxes, pairs_by_kind):
    """Group (target, source) pair arrays of each kind by target box."""
    tgt, src, kind = [], [], []
    for k, pairs in pairs_by_kind:
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        tgt.append(pairs[:, 0])
        src.append(pairs[:, 1])
        kind.append(np.full(pairs.shape[0], k, dtype=np.int8))
    tgt = np.concatenate(tgt) if tgt else np.zeros(0, np.int64)
    src = np.concatenate(src) if src else np.zeros(0, np.int64)
    kind = np.concatenate(kind) if kind else np.zeros(0, np.int8)
    order = np.argsort(tgt, kind="stable")
    counts = np.bincount(tgt, minlength=nboxes)
    off = np.zeros(nboxes + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return off, src[order].astype(np.int32), kind[order].astype(np.int8)


def ragged_from_reference(tree, fmm, operator, kappa=0.0):
    """Ragged description of a build held in the reference's padded layout.

    ``fmm`` exposes the attributes of a reference ``RecursiveSkeletonization``
    after ``setup_lists`` (a live object, or a mapping of the same arrays).
    """
    get = (lambda k: fmm[k]) if isinstance(fmm, dict) else (lambda k: getattr(fmm, k))
    nb = tree.nboxes
    bs = np.asarray(get("bs_list"), dtype=np.int64)
    rk = np.asarray(get("rank_list"), dtype=np.int64)
    XX = np.asarray(get("XX_list"))
    max_bs = XX.shape[1]
    min_rank = int(get("min_rank"))
    root_level = int(get("root_level"))
    levels = tree.get_boxes_levels().astype(np.int32)
    off = np.zeros(nb + 1, dtype=np.int64)
    np.cumsum(bs, out=off[1:])
    E = int(off[-1])
    # padded index box*max_bs + k  ->  entry index off[box] + k
    def pad_to_entry(p):
        p = np.asarray(p, dtype=np.int64)
        return off[p // max_bs] + p % max_bs

    mask = np.arange(max_bs)[None, :] < bs[:, None]
    entry_xyz = XX[mask]
    entry_geom = None
    geom_list = None
    try:
        geom_list = get("geom_list")
    except (KeyError, AttributeError):
        geom_list = None
    if geom_list is not None:
        entry_geom = np.asarray(geom_list)[mask]
    pslot = np.full(E, -1, dtype=np.int64)
    pslot[pad_to_entry(get("child_skel_inds"))] = pad_to_entry(get("box_skel_inds"))
    perm_entry = pad_to_entry(get("short_vec_inds"))
    perm_point = np.asarray(get("long_vec_inds"), dtype=np.int64)

    cplx = is_complex_op(operator)
    proj = np.asarray(get("proj_list"))
    projt = np.asarray(get("proj_list_tree"))
    tree_boxes = np.asarray(get("tree_boxes"), dtype=np.int64)
    leaf = tree.are_leaves(np.arange(nb))
    t_off = np.full(nb, -1, dtype=np.int64)
    blocks = []
    acc = 0
    for b in range(nb):
        r, s = int(rk[b]), int(bs[b])
        if r <= 0 or levels[b] <= root_level:
            continue
        if leaf[b]:
            T = proj[b, :r, r - min_rank: s - min_rank]
        else:
            T = projt[int(np.searchsorted(tree_boxes, b)), :r, r - min_rank: s - min_rank]
        t_off[b] = acc
        blocks.append(np.ascontiguousarray(T).ravel())
        acc += r * (s - r)
    dt = np.complex128 if cplx else np.float64
    t_data = np.concatenate(blocks).astype(dt) if blocks else np.zeros(1, dt)

    coll = np.vstack((np.asarray(get("leaf_uskel_from_qskel_list")).reshape(-1, 2),
                      np.asarray(get("tree_uskel_from_qskel_list")).reshape(-1, 2)))
    list_off, list_src, list_kind = lists_to_csr(nb, [
        (_lib.KIND_COLLEAGUE, coll),
        (_lib.KIND_COARSE_UP, get("uskel_from_q_list")),
        (_lib.KIND_COARSE_DOWN, get("u_from_qskel_list")),
        (_lib.KIND_ROOT, get("u_from_q_list")),
    ])
    return RaggedBuild(
        op=cuda_op_id(operator), ndim=tree.ndim, kappa=float(kappa), npoints=int(tree.N),
        nlevels=int(tree.nlevels), root_level=root_level, box_level=levels, box_off=off,
        box_rank=rk.astype(np.int32), entry_xyz=np.ascontiguousarray(entry_xyz, dtype=np.float64),
        entry_geom=None if entry_geom is None else np.ascontiguousarray(entry_geom, dtype=np.float64),
        entry_pslot=pslot, perm_entry=perm_entry, perm_point=perm_point, t_off=t_off,
        t_data=t_data, list_off=list_off, list_src=list_src, list_kind=list_kind,
    )


# ------------------------------------------------------------------ saved builds
# A built operator on disk: the ragged description (the arrays skf_plan_create
# takes) in one numpy .npz archive, with a format tag, a version and the
# scalar type of T.  Loading it and creating a plan gives the same apply, bit
# for bit, as the plan it was saved from; a build made anywhere (the GPU
# build, a CPU build in the reference's layout through ragged_from_reference)
# can be saved and replayed on the GPU later.
FORMAT_TAG = "skelfmm_gb300.ragged_build"
FORMAT_VERSION = 1
_ARRAYS = ("box_level", "box_off", "box_rank", "entry_xyz", "entry_pslot", "perm_entry", "perm_point", "t_off",
           "t_data", "list_off", "list_src", "list_kind")
_DTYPES = {"box_level": np.int32, "box_off": np.int64, "box_rank": np.int32, "entry_xyz": np.float64,
           "entry_pslot": np.int64, "perm_entry": np.int64, "perm_point": np.int64, "t_off": np.int64,
           "list_off": np.int64, "list_src": np.int32, "list_kind": np.int8}


def host_array(a):
    """``a`` as a numpy array (device tensors copied to the host)."""
    return a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a


def save_ragged(rb: RaggedBuild, path, extra=None):
    """Write ``rb`` (T and entries copied to the host if they are on the
    device) to ``path`` (.npz).  ``extra``: further named arrays stored
    beside it."""
    t = np.asarray(host_array(rb.t_data))
    out = {"format": np.array(FORMAT_TAG), "version": np.array(FORMAT_VERSION),
           "t_dtype": np.array(str(t.dtype)),
           "scalars": np.array([rb.op, rb.ndim, rb.npoints, rb.nlevels, rb.root_level], dtype=np.int64),
           "kappa": np.array(rb.kappa, dtype=np.float64)}
    for k in _ARRAYS:
        out[k] = t if k == "t_data" else np.ascontiguousarray(host_array(getattr(rb, k)), dtype=_DTYPES[k])
    if rb.entry_geom is not None:
        out["entry_geom"] = np.ascontiguousarray(host_array(rb.entry_geom), dtype=np.float64)
    for k, v in (extra or {}).items():
        out["extra/" + k] = np.asarray(v)
    with open(path, "wb") as f:
        np.savez(f, **out)


def load_ragged(path):
    """(RaggedBuild, extra) from a file written by save_ragged; ValueError
    for another format, a newer version or inconsistent arrays."""
    with np.load(path, allow_pickle=False) as d:
        if "format" not in d.files or str(d["format"]) != FORMAT_TAG:
            raise ValueError(f"{path}: not a saved skelfmm_gb300 build")
        if int(d["version"]) > FORMAT_VERSION:
            raise ValueError(f"{path}: format version {int(d['version'])} is newer than {FORMAT_VERSION}")
        op, ndim, npoints, nlevels, root_level = (int(v) for v in d["scalars"])
        arrs = {k: d[k] for k in _ARRAYS}
        if str(arrs["t_data"].dtype) != str(d["t_dtype"]) or \
                arrs["t_data"].dtype != (np.complex128 if is_complex_op(op) else np.float64):
            raise ValueError(f"{path}: T blocks have the wrong scalar type for the operator")
        geom = d["entry_geom"] if "entry_geom" in d.files else None
        extra = {k[6:]: d[k] for k in d.files if k.startswith("extra/")}
        kappa = float(d["kappa"])
    nb = arrs["box_level"].shape[0]
    if arrs["box_off"].shape[0] != nb + 1 or arrs["list_off"].shape[0] != nb + 1 or \
            arrs["entry_xyz"].shape[0] != int(arrs["box_off"][-1]):
        raise ValueError(f"{path}: inconsistent array sizes")
    rb = RaggedBuild(op=op, ndim=ndim, kappa=kappa, npoints=npoints, nlevels=nlevels, root_level=root_level,
                     entry_geom=geom, **arrs)
    return rb, extra


# translation kernel variants (operator, precision, symmetric, shape) that
# have run in this process: their first launch carries the module load
_WARMED = set()


class Plan:
    """A built operator resident on the device (owns an ``skf_plan``)."""

    def __init__(self, rb: RaggedBuild):
        lib = _lib.load()
        self.rb = rb
        self.op = rb.op
        self.npoints = rb.npoints
        self.is_complex = is_complex_op(rb.op)
        keep = {}

        def arr(name, a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep[name] = a
            return a.ctypes.data

        d = _lib.PlanDesc()
        d.op = rb.op
        d.ndim = rb.ndim
        d.kappa = rb.kappa
        d.npoints = rb.npoints
        d.nboxes = rb.nboxes
        d.nlevels = rb.nlevels
        d.root_level = rb.root_level
        d.box_level = arr("box_level", rb.box_level, np.int32)
        d.box_off = arr("box_off", rb.box_off, np.int64)
        d.box_rank = arr("box_rank", rb.box_rank, np.int32)
        if isinstance(rb.entry_xyz, torch.Tensor):
            # entries already on the device (a build's own gather): used in place
            def dev(name, a):
                if a is None:
                    return None
                if not a.is_cuda or a.dtype != torch.float64:
                    raise ValueError(f"device {name} must be a CUDA float64 tensor")
                a = a.contiguous()
                keep[name] = a
                return a.data_ptr()

            if rb.entry_geom is not None and not isinstance(rb.entry_geom, torch.Tensor):
                raise ValueError("entry_geom must live where entry_xyz does")
            d.entry_xyz = dev("entry_xyz", rb.entry_xyz)
            d.entry_geom = dev("entry_geom", rb.entry_geom)
            d.entries_on_device = 1
        else:
            d.entry_xyz = arr("entry_xyz", rb.entry_xyz, np.float64)
            d.entry_geom = None if rb.entry_geom is None else arr("entry_geom", rb.entry_geom, np.float64)
            d.entries_on_device = 0
        d.entry_pslot = arr("entry_pslot", rb.entry_pslot, np.int64)
        d.nperm = int(rb.perm_entry.shape[0])
        d.perm_entry = arr("perm_entry", rb.perm_entry, np.int64)
        d.perm_point = arr("perm_point", rb.perm_point, np.int64)
        d.t_off = arr("t_off", rb.t_off, np.int64)
        if isinstance(rb.t_data, torch.Tensor):
            # T blocks already on the device: copied device to device
            tdt = torch.complex128 if self.is_complex else torch.float64
            if not rb.t_data.is_cuda or rb.t_data.dtype != tdt or not rb.t_data.is_contiguous():
                raise ValueError("device t_data must be a contiguous CUDA tensor of the operator's dtype")
            keep["t_data"] = rb.t_data
            d.t_data = rb.t_data.data_ptr()
            d.t_on_device = 1
        else:
            tdt = np.complex128 if self.is_complex else np.float64
            d.t_data = arr("t_data", rb.t_data, tdt)
            d.t_on_device = 0
        d.t_len = int(rb.t_data.shape[0])
        d.list_off = arr("list_off", rb.list_off, np.int64)
        d.list_src = arr("list_src", rb.list_src, np.int32)
        d.list_kind = arr("list_kind", rb.list_kind, np.int8)
        h = ctypes.c_void_p()
        _lib.check(lib.skf_plan_create(ctypes.byref(d), ctypes.byref(h)), "skf_plan_create")
        self._h = h
        info = _lib.PlanInfo()
        _lib.check(lib.skf_plan_query(h, ctypes.byref(info)), "skf_plan_query")
        self.info = info

    @property
    def handle(self):
        return self._h

    def save(self, path):
        """Write the plan's build to ``path`` (see save_ragged)."""
        save_ragged(self.rb, path)

    @classmethod
    def load(cls, path):
        """A plan on the current device from a file written by ``save``."""
        rb, _ = load_ragged(path)
        return cls(rb)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().skf_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply_device(self, x, y, precision=_lib.PREC_FP64, stream=None):
        """y = A x for device tensors (float64 / complex128, length N)."""
        _lib.check(_lib.load().skf_plan_apply(self._h, _lib.ptr(x), _lib.ptr(y), int(precision),
                                              None if stream is None else ctypes.c_void_p(stream)),
                   "skf_plan_apply")

    def apply_host(self, x, y, precision=_lib.PREC_FP64, stream=None):
        """y = A x for host arrays; copies in and out, synchronises."""
        _lib.check(_lib.load().skf_plan_apply_host(self._h, _lib.ptr(x), _lib.ptr(y), int(precision),
                                                   None if stream is None else ctypes.c_void_p(stream)),
                   "skf_plan_apply_host")

    def set_option(self, option, value):
        _lib.check(_lib.load().skf_plan_set_option(self._h, int(option), int(value)), "skf_plan_set_option")

    def autotune(self, precision=_lib.PREC_MIXED, reps=3, exhaustive=False):
        """Time translation schemes this plan supports and keep the fastest.

        Candidates: for real operators the source-split symmetric kernel
        (when the lists are symmetric) and the per-direction packed kernel's
        4-warp shape (256-row items) and 1-warp shape (64-row items); for
        Helmholtz 3D the block-barrier symmetric kernel's 64 and 32-source
        tiles and the packed kernel's 4-warp, 2-warp and 1-warp/64-row
        shapes; with ``exhaustive`` every shape of both kernels.  Each
        candidate is timed once, then the two fastest ``reps`` times unless
        the fastest leads by more than 15 %.  The 64-row shape is a candidate
        only where its items evaluate at least 20 % fewer rows.  Returns
        {(symmetric, shape): ms}; the choice is kept in ``self.tuned``."""
        self.set_option(_lib.OPT_SYMMETRIC, 1)
        info = self._query()
        sym_ok = info.npairs_evaluated_mixed < info.npairs_fused
        if exhaustive:
            # shapes 4 and 5: the source-split Laplace kernel (grid, persistent queue)
            sym_shapes, dir_shapes = (range(4) if self.is_complex else range(6)), range(4)
        else:
            sym_shapes, dir_shapes = ((0, 2), (0, 2, 3)) if self.is_complex else ((4,), (0, 3))
        if not exhaustive and 3 in dir_shapes and self._row_gain_64() < 1.25:
            # 64-row items evaluate too few rows less than 256-row items to pay
            dir_shapes = tuple(sh for sh in dir_shapes if sh != 3)
        cands = ([(1, sh) for sh in sym_shapes] if sym_ok else []) + [(0, sh) for sh in dir_shapes]

        def select(sym, shape):
            self.set_option(_lib.OPT_SYMMETRIC, sym)
            self.set_option(_lib.OPT_SYM_SHAPE if sym else _lib.OPT_PACKED_SHAPE, shape)

        gain64 = self._row_gain_64() if (0, 3) in cands else 1.0
        results = {}
        for sym, shape in cands:
            if (sym, shape) == (0, 3) and (0, 0) in results and results:
                # 64-row items cut the 256-row shape's evaluated rows by
                # gain64 at most, so they cannot beat a candidate already
                # faster than the 256-row time / gain64
                if min(results.values()) < results[(0, 0)] / gain64:
                    continue
            select(sym, shape)
            key = (int(self.op), int(precision), sym, shape)
            if key not in _WARMED:
                # first launch of this kernel variant in the process (module load)
                self.time_translations(precision, reps=1)
                _WARMED.add(key)
            results[(sym, shape)] = self.time_translations(precision, reps=1)
        top = sorted(results, key=results.get)[:2]
        clear = len(top) < 2 or results[top[1]] > 1.15 * results[top[0]]
        for cand in ([] if clear else top):
            if results[cand] < 20.0:
                # long launches keep the single timing: their spread is well
                # below the differences between schemes
                select(*cand)
                results[cand] = self.time_translations(precision, reps=reps)
        best = min(results, key=results.get)
        select(*best)
        self.info = self._query()
        self.tuned = best
        return results

    def _row_gain_64(self):
        """Rows a per-direction translation evaluates with 256-row work items
        over those with 64-row items (each target box's rows padded to the
        item, weighted by the entries of its list's sources; computed at plan
        creation)."""
        return float(self._query().rows_256_over_64)

    def _query(self):
        info = _lib.PlanInfo()
        _lib.check(_lib.load().skf_plan_query(self._h, ctypes.byref(info)), "skf_plan_query")
        return info

    def time_translations(self, precision, reps=5, stream=None):
        ms = ctypes.c_float()
        _lib.check(_lib.load().skf_plan_time_translations(self._h, int(precision), int(reps),
                                                          None if stream is None else ctypes.c_void_p(stream),
                                                          ctypes.byref(ms)), "skf_plan_time_translations")
        return float(ms.value)
