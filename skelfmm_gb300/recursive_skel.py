"""Strong recursive skeletonization: host orchestration of the GPU build.

Mirrors ``RecursiveSkeletonization`` (skelfmm/recursive_skel.py:12-780): the
level loop, skeleton bookkeeping and translation lists run on the host
(integer work on box ids), while the proxy-surface kernel matrices and the
interpolative decompositions of every box of a level run on the GPU in one
``skf_skel_boxes`` call.  The result is a ragged build (``RaggedBuild``) ready
for ``Plan``.
"""

from __future__ import annotations

import ctypes
from time import perf_counter

import numpy as np
import torch

from . import _lib
from .operators import _require_operator, cuda_op_id, is_complex_op
from .plan import RaggedBuild, lists_to_csr


def nproxy_levels(ndim, tol, kappa, L0, nlevels):
    """Proxy counts per level (skelfmm/recursive_skel.py:72-85)."""
    ndigits = int(-np.log10(tol / 100))
    out = np.zeros(nlevels, dtype=int)
    for lev in range(nlevels):
        box_length = L0 * 2 ** (-lev)
        if ndim == 2:
            nproxy = int(ndigits * 10) + int(4 * kappa * box_length)
        else:
            nproxy = np.max(np.array([int(ndigits ** 2 * 8), 400]))
            nproxy += 2 * kappa * box_length * np.max(np.array([5, ndigits - 1])) + (10 if kappa > 0 else 0)
        out[lev] = nproxy
    return out


def _concat_ranges(starts, lens):
    """Concatenation of the integer ranges [starts[i], starts[i] + lens[i])."""
    lens = np.asarray(lens, dtype=np.int64)
    total = int(lens.sum())
    if total == 0:
        return np.zeros(0, dtype=np.int64)
    before = np.cumsum(lens) - lens
    return np.arange(total, dtype=np.int64) + np.repeat(np.asarray(starts, dtype=np.int64) - before, lens)


class _BoxView:
    """``view[b]`` -> per-box slice of level-flat storage (read only)."""

    def __init__(self, nboxes, getter):
        self._n = nboxes
        self._get = getter

    def __len__(self):
        return self._n

    def __getitem__(self, b):
        return self._get(int(b))

    def __iter__(self):
        return (self._get(b) for b in range(self._n))


class RecursiveSkeletonization:
    """Build of the skeletonized tree for one operator (GPU IDs).

    Storage is level-flat: ``_ids[lev]`` holds the point ids of every box of
    level ``lev`` back to back (box ``b`` at ``_off[lev][b - level_sep[lev]]``),
    in skeleton-first order once the level is skeletonized; the T blocks of a
    level stay on the device in ``_tdev[lev]`` (row-major r x (bs - r) per
    box at ``_toff[lev]``).
    """

    def __init__(self, tree, operator, kappa, tol, max_bs=-1, max_rank=-1, geometry=None, device=None):
        self.N = tree.N
        self.tree = tree
        self.nlevels = tree.nlevels
        self.nboxes = tree.nboxes
        self.kappa = float(kappa)
        self.operator = _require_operator(operator)
        self.op_id = cuda_op_id(self.operator)
        self.ndim = tree.ndim
        self.tol = tol
        self.geometry = None if geometry is None else np.ascontiguousarray(geometry, dtype=np.float64)
        if self.operator.ndim > 0 and self.operator.ndim != self.ndim:
            raise ValueError("Operator dimensionality does not match the tree dimensionality")
        if self.operator.requires_geometry and self.geometry is None:
            raise ValueError("Geometry is required for this operator")
        if self.geometry is not None and self.geometry.shape[0] != self.N:
            raise ValueError("Geometry must be aligned with tree.XX")
        self.device = torch.device("cuda") if device is None else torch.device(device)
        if self.device.type != "cuda":
            raise RuntimeError("the skeletonization build runs on a CUDA device")

        self.nproxy_level = nproxy_levels(self.ndim, tol, self.kappa, tree.L0, self.nlevels)
        self.max_bs_leaf = tree.leaf_size
        # max_bs / max_rank size the reference's padded storage before the
        # build (skelfmm/recursive_skel.py:87-94); it grows that storage when a
        # box needs more (:230-247, :285-307), so they never cap a rank.  The
        # ragged layout here has no padded storage: both are validated and
        # kept as the reference computes them, and do not change the build.
        for name, v in (("max_bs", max_bs), ("max_rank", max_rank)):
            if int(v) != v:
                raise ValueError(f"{name} must be an integer")
        if max_bs > 0 and max_rank > 0:
            self.max_rank = int(max_rank)
            self.max_bs = max(int(max_bs), int(self.max_bs_leaf))
        else:
            self.max_rank = int(self.max_bs_leaf * 0.75)
            self.max_bs = int((2 ** self.ndim) * self.max_bs_leaf)
        self.max_rank_leaf = self.max_rank
        if np.any(tree.get_box_npoints(tree.get_leaves()) > self.max_bs_leaf):
            raise ValueError("Leaf block size exceeds maximum allowed")
        self.bs_list = np.zeros(self.nboxes, dtype=np.int64)
        self.rank_list = np.zeros(self.nboxes, dtype=np.int64)
        leaves = tree.get_leaves()
        self.bs_list[leaves] = tree.get_box_npoints(leaves)
        nl = self.nlevels
        self._ids = [None] * nl
        self._off = [None] * nl
        self._cand_src = [None] * nl   # candidate -> child-level entry (or -1)
        self._final_pos = [None] * nl  # candidate -> entry position after the ID
        self._tdev = [None] * nl
        self._toff = [None] * nl
        self.root_level = max(0, nl - 1)
        self.level_times = {}
        self.level_stats = {}
        self._resid_by_lev = {}
        self._status_by_lev = {}  # per box: 0 pivoted QR, 10 * rounds + 1 kept, + 2 rejected
        self._sketch_by_lev = {}  # per box: sketch rank tried (0: none)
        # optional callable(fmm, lev, boxes, x_lev, off) -> predicted ranks (int64,
        # -1 = no prediction): enables the sampled (randomized) IDs
        self.rank_predictor = None
        self.oversample = 10   # sketch rows beyond the predicted rank
        self.rho = 16          # nonzeros per sketch row
        self.nchk = 16         # proxy rows of the residual check
        self.sketch_factor = 0.5  # rank rule on the sketch: |R_kk| <= factor * tol * |R_00|
        self.resid_factor = 2.0  # keep the randomized ID when its residual on checked rows <= factor * tol
        self.seed = 12345
        self._XX_dev = torch.from_numpy(np.ascontiguousarray(tree.XX)).to(self.device)
        self._geom_dev = None
        if self.geometry is not None:
            self._geom_dev = torch.from_numpy(self.geometry).to(self.device)
        self.pid = _BoxView(self.nboxes, self._box_ids)
        self.proj = _BoxView(self.nboxes, self._box_proj)

    @property
    def rank_max(self):
        pos = self.rank_list[self.rank_list > 0]
        return int(pos.max()) if pos.size else 0

    # ------------------------------------------------------------ views
    def _box_ids(self, b):
        lev = int(self.tree._box_level[b])
        if self._ids[lev] is None:
            if self.tree.is_leaf(b):
                return np.asarray(self.tree.get_box_inds(b), dtype=np.int64)
            return None
        i = b - int(self.tree.level_sep[lev])
        o = self._off[lev]
        return self._ids[lev][o[i]:o[i + 1]]

    def _box_proj(self, b):
        lev = int(self.tree._box_level[b])
        if self._tdev[lev] is None:
            return None
        i = b - int(self.tree.level_sep[lev])
        r, s = int(self.rank_list[b]), int(self.bs_list[b])
        t0 = int(self._toff[lev][i])
        return self._tdev[lev][t0:t0 + r * (s - r)].cpu().numpy().reshape(r, s - r)

    # ------------------------------------------------------------ levels
    def _level_candidates(self, lev):
        """Entries of every box at ``lev`` before its ID: the points of a
        leaf, else the skeletons of its children in child order
        (recursive_skel.py:209-262); on the host threads of the library
        (``skf_level_candidates``), the same arrays as
        ``_level_candidates_numpy``."""
        tree = self.tree
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        nbl = le - ls
        lib = _lib.load()
        child = lev + 1 < self.nlevels and self._ids[lev + 1] is not None
        leaf = np.ascontiguousarray(tree._is_leaf[ls:le], dtype=np.uint8)
        start = np.ascontiguousarray(tree._box_start[ls:le], dtype=np.int64)
        end = np.ascontiguousarray(tree._box_end[ls:le], dtype=np.int64)
        ch = np.ascontiguousarray(tree._children[ls:le], dtype=np.int64)
        rank = np.ascontiguousarray(self.rank_list, dtype=np.int64)
        perm = np.ascontiguousarray(tree._perm, dtype=np.int64)
        coff = np.ascontiguousarray(self._off[lev + 1], dtype=np.int64) if child else None
        cids = np.ascontiguousarray(self._ids[lev + 1], dtype=np.int64) if child else None
        cfirst = int(tree.level_sep[lev + 1]) if child else 0
        off = np.empty(nbl + 1, dtype=np.int64)
        total = ctypes.c_int64()
        args = (nbl, _lib.ptr(leaf), _lib.ptr(start), _lib.ptr(end), _lib.ptr(ch), int(ch.shape[1]), cfirst,
                _lib.ptr(coff), _lib.ptr(cids), _lib.ptr(rank), _lib.ptr(perm), int(self.N), _lib.ptr(off))
        _lib.check(lib.skf_level_candidates(*args, None, None, ctypes.byref(total)), "skf_level_candidates")
        ids = np.empty(int(total.value), dtype=np.int64)
        cand = np.empty(int(total.value), dtype=np.int64)
        _lib.check(lib.skf_level_candidates(*args, _lib.ptr(ids), _lib.ptr(cand), ctypes.byref(total)),
                   "skf_level_candidates")
        self._ids[lev] = ids
        self._off[lev] = off
        self._cand_src[lev] = cand
        self._final_pos[lev] = None
        self.bs_list[ls:le] = np.diff(off)

    def _level_candidates_numpy(self, lev):
        """``_level_candidates`` with numpy (the arrays it is checked
        against)."""
        tree = self.tree
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        boxes = np.arange(ls, le, dtype=np.int64)
        leaf = tree._is_leaf[boxes]
        lb = boxes[leaf]
        seg_box = [lb]
        seg_start = [tree._box_start[lb]]
        seg_len = [tree._box_end[lb] - tree._box_start[lb]]
        seg_child = [np.full(lb.shape[0], -1, dtype=np.int64)]
        if lev + 1 < self.nlevels and self._ids[lev + 1] is not None:
            nlb = boxes[~leaf]
            ch = tree._children[nlb]
            mask = ch >= 0
            cb = np.repeat(nlb, ch.shape[1]).reshape(ch.shape)[mask]
            cc = ch[mask]
            cl = cc - int(tree.level_sep[lev + 1])
            seg_box.append(cb)
            seg_start.append(self.N + self._off[lev + 1][cl])
            seg_len.append(self.rank_list[cc])
            seg_child.append(cc)
        sb = np.concatenate(seg_box)
        order = np.argsort(sb, kind="stable")
        sb = sb[order]
        st = np.concatenate(seg_start)[order]
        sl = np.concatenate(seg_len)[order].astype(np.int64)
        # idx addresses [point order | child level's ids]: gather from each
        # part directly instead of concatenating them
        idx = _concat_ranges(st, sl)
        from_child = idx >= self.N
        ids = np.empty(idx.shape[0], dtype=np.int64)
        pm = ~from_child
        ids[pm] = tree._perm[idx[pm]]
        if lev + 1 < self.nlevels and self._ids[lev + 1] is not None:
            ids[from_child] = self._ids[lev + 1][idx[from_child] - self.N]
        bs = np.bincount(sb - ls, weights=sl, minlength=le - ls).astype(np.int64)
        off = np.zeros(le - ls + 1, dtype=np.int64)
        np.cumsum(bs, out=off[1:])
        self._ids[lev] = ids
        self._off[lev] = off
        self._cand_src[lev] = np.where(from_child, idx - self.N, -1)
        self._final_pos[lev] = None
        self.bs_list[ls:le] = bs

    def _leaf_level_entries(self, lev):
        """Entries of a level above the root: leaves hold their points."""
        self._level_candidates(lev)

    def _level_inputs(self, lev):
        """Device inputs of the IDs of every box at ``lev``: entry offsets,
        gathered coordinates (and geometry), box centers, the T buffer and
        its per-box offsets (capacity bs^2/4 + bs per box)."""
        tree = self.tree
        dev = self.device
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        off = self._off[lev]
        bs = np.diff(off)
        ids_t = torch.from_numpy(self._ids[lev]).to(dev)
        x = self._XX_dev.index_select(0, ids_t).contiguous()
        g = None
        if self._geom_dev is not None:
            g = self._geom_dev.index_select(0, ids_t).contiguous()
        cap = (bs * bs) // 4 + bs
        t_off = np.zeros(le - ls, dtype=np.int64)
        np.cumsum(cap[:-1], out=t_off[1:])
        return {"lev": lev, "nbl": le - ls, "off": off, "bs": bs, "x": x, "g": g,
                "centers": np.ascontiguousarray(tree._box_center[ls:le]), "length": float(tree.L0 * 0.5 ** lev),
                "nproxy": int(self.nproxy_level[lev]), "cap": cap, "t_off": t_off}

    def _skel_level(self, lev):
        """Proxy IDs of every box at ``lev`` on the GPU in one call.  With a
        rank predictor, every box whose predicted rank is below its size
        first tries the randomized ID at that rank (sparse-sign sketch of
        predicted rank + oversampling rows), kept when its residual on
        held-out rows of the proxy matrix is within tol, else the full
        pivoted-QR ID (decided per box inside the kernel)."""
        tree = self.tree
        dev = self.device
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        inp = self._level_inputs(lev)
        nbl, off, bs, x, g = inp["nbl"], inp["off"], inp["bs"], inp["x"], inp["g"]
        t_off = inp["t_off"]
        centers = torch.from_numpy(inp["centers"]).to(dev)
        tdt = torch.complex128 if is_complex_op(self.op_id) else torch.float64
        t_buf = torch.zeros(max(int(inp["cap"].sum()), 1), dtype=tdt, device=dev)
        rank = torch.zeros(nbl, dtype=torch.int32, device=dev)
        perm = torch.zeros(max(int(off[-1]), 1), dtype=torch.int32, device=dev)
        off_t = torch.from_numpy(off).to(dev)
        t_off_t = torch.from_numpy(t_off).to(dev)
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        lib = _lib.load()
        length = inp["length"]
        mrows = self._mrows(lev)
        stats = {"boxes": nbl, "rows_full": int(mrows)}
        pred = None
        if self.rank_predictor is not None and self.tol < 1:
            t0 = perf_counter()
            pred = np.asarray(self.rank_predictor(self, lev, np.arange(ls, le), x, off), dtype=np.int64)
            stats["predict_s"] = perf_counter() - t0
        if pred is None:
            _lib.check(lib.skf_skel_boxes(
                self.op_id, self.kappa, nbl, _lib.ptr(off_t), _lib.ptr(x), _lib.ptr(g), _lib.ptr(centers), length,
                int(self.nproxy_level[lev]), float(self.tol), _lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t),
                _lib.ptr(t_buf), stream), "skf_skel_boxes")
            stats.update(randomized=0, kept=0, fallback=0)
        else:
            kpred = np.where((pred > 0) & (bs > 0), np.minimum(pred, bs), 0).astype(np.int32)
            kpred_t = torch.from_numpy(kpred).to(dev)
            resid = torch.empty(nbl, dtype=torch.float64, device=dev)
            status = torch.empty(nbl, dtype=torch.int8, device=dev)
            _lib.check(lib.skf_skel_boxes_randomized(
                self.op_id, self.kappa, nbl, _lib.ptr(off_t), _lib.ptr(x), _lib.ptr(g), _lib.ptr(centers), length,
                int(self.nproxy_level[lev]), float(self.tol), _lib.ptr(kpred_t), int(self.oversample), int(self.rho),
                int(self.seed + lev), int(self.nchk), float(self.sketch_factor * self.tol),
                float(self.resid_factor * self.tol), _lib.ptr(resid),
                _lib.ptr(status), _lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t), _lib.ptr(t_buf), stream),
                "skf_skel_boxes_randomized")
            st = status.cpu().numpy()
            self._last_resid = resid.cpu().numpy()
            self._resid_by_lev[lev] = self._last_resid
            self._status_by_lev[lev] = st
            self._sketch_by_lev[lev] = kpred
            rounds = st // 10
            stats.update(randomized=int(np.count_nonzero(st > 0)), kept=int(np.count_nonzero(st % 10 == 1)),
                         fallback=int(np.count_nonzero(st % 10 == 2)), sketch_rounds=int(rounds.sum()),
                         sketch_rows=int(np.sum(np.where(st > 0, (kpred + self.oversample) * (2 ** rounds - 1), 0))))
            self._last_pred = pred
            self._last_status = st
        self.level_stats[lev] = stats
        self._level_finish(inp, rank.cpu().numpy(), perm.cpu().numpy()[: int(off[-1])], t_buf)

    def _level_finish(self, inp, rank_h, perm_h, t_buf):
        """Skeleton-first entry order, ranks and compacted T blocks of level
        ``inp["lev"]`` from the IDs' ranks, box-local pivot orders and the T
        buffer (laid out at ``inp["t_off"]``)."""
        lev, off, bs, t_off = inp["lev"], inp["off"], inp["bs"], inp["t_off"]
        nbl = inp["nbl"]
        ls, le = int(self.tree.level_sep[lev]), int(self.tree.level_sep[lev + 1])
        dev = self.device
        cplx = is_complex_op(self.op_id)
        rank_h = np.asarray(rank_h).astype(np.int64)
        perm_h = np.ascontiguousarray(perm_h, dtype=np.int32)
        ids = np.ascontiguousarray(self._ids[lev], dtype=np.int64)
        # skeleton-first ids, candidate -> final position (host threads)
        new_ids = np.empty_like(ids)
        fp = np.empty(ids.shape[0], dtype=np.int64)
        _lib.check(_lib.load().skf_level_reorder(nbl, _lib.ptr(np.ascontiguousarray(off, dtype=np.int64)),
                                                 _lib.ptr(perm_h), _lib.ptr(ids), _lib.ptr(new_ids), _lib.ptr(fp)),
                   "skf_level_reorder")
        self._ids[lev] = new_ids
        self._final_pos[lev] = fp
        self.rank_list[ls:le] = rank_h
        # compact the T blocks
        tl = rank_h * (bs - rank_h)
        toff = np.zeros(nbl + 1, dtype=np.int64)
        np.cumsum(tl, out=toff[1:])
        tc = torch.empty(max(int(toff[-1]), 1), dtype=t_buf.dtype, device=dev)
        nz = np.flatnonzero(tl > 0)
        if nz.size:
            so = torch.from_numpy(t_off[nz]).to(dev)
            do = torch.from_numpy(toff[:-1][nz]).to(dev)
            ln = torch.from_numpy(tl[nz]).to(dev)
            stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            _lib.check(_lib.load().skf_copy_segments(int(nz.size), _lib.ptr(so), _lib.ptr(do), _lib.ptr(ln),
                                                     _lib.ptr(t_buf), _lib.ptr(tc), 16 if cplx else 8, stream),
                       "skf_copy_segments")
        self._tdev[lev] = tc
        self._toff[lev] = toff[:-1]

    def _mrows(self, lev):
        out = ctypes.c_int32()
        _lib.check(_lib.load().skf_proxy_rows(self.op_id, int(self.nproxy_level[lev]), ctypes.byref(out)),
                   "skf_proxy_rows")
        return int(out.value)

    def skel_tree(self, npoints_max, p=None, verbose=False):
        """Level loop of recursive_skel.py:326-502 with GPU IDs per level.

        ``p`` (the reference's process pool) is accepted and ignored.
        """
        tree = self.tree
        self.root_level = max(0, tree.nlevels - 1)
        for lev in range(tree.nlevels - 1, 0, -1):
            if self._is_root_level(lev, npoints_max, verbose):
                break
            t0 = perf_counter()
            self._skel_level(lev)
            torch.cuda.synchronize(self.device)
            self.level_times[lev] = perf_counter() - t0
            if verbose:
                print("\t Level %2d ids: %5.3f s" % (lev, self.level_times[lev]))
        _lib.check(_lib.load().skf_trim_workspace(), "skf_trim_workspace")
        self._entries_above_root()
        return self

    def _is_root_level(self, lev, npoints_max, verbose=False):
        """Candidates of ``lev``; True (and ``root_level = lev``) when the
        level loop stops there: level 2, or few enough points left
        (recursive_skel.py:370-385)."""
        tree = self.tree
        self._level_candidates(lev)
        npoints_lev = int(np.sum(self.bs_list[tree.get_boxes_level(lev)]) +
                          np.sum(self.bs_list[tree.get_leaves_above(lev)]))
        if verbose:
            print("\t Level %2d has %6d npoints" % (lev, npoints_lev))
        if lev == 2 or npoints_lev <= npoints_max:
            self.root_level = lev
            return True
        return False

    def _entries_above_root(self):
        if self.tree.nlevels == 1:
            self._level_candidates(0)
        for lev in range(self.root_level - 1, -1, -1):
            self._leaf_level_entries(lev)

    def _parent_slots(self, ebase, nentries):
        """Parent slots: skeleton entry i of child c sits at candidate
        position t of its parent, which the parent's ID moved to
        ``_final_pos`` (``skf_parent_slots`` on the library's host threads;
        the same array as ``_parent_slots_numpy``)."""
        levs = [lev for lev in range(self.root_level, self.nlevels - 1) if self._cand_src[lev] is not None]
        keep = [(np.ascontiguousarray(self._cand_src[lev], dtype=np.int64),
                 None if self._final_pos[lev] is None else np.ascontiguousarray(self._final_pos[lev], dtype=np.int64))
                for lev in levs]
        ptrs = ctypes.c_void_p * max(len(levs), 1)
        cs_p = ptrs(*[k[0].ctypes.data for k in keep])
        fp_p = ptrs(*[None if k[1] is None else k[1].ctypes.data for k in keep])
        ncand = np.array([k[0].shape[0] for k in keep] or [0], dtype=np.int64)
        bchild = np.array([ebase[lev + 1] for lev in levs] or [0], dtype=np.int64)
        bparent = np.array([ebase[lev] for lev in levs] or [0], dtype=np.int64)
        pslot = np.empty(nentries, dtype=np.int64)
        _lib.check(_lib.load().skf_parent_slots(len(levs), cs_p, fp_p, _lib.ptr(ncand), _lib.ptr(bchild),
                                                _lib.ptr(bparent), nentries, _lib.ptr(pslot)), "skf_parent_slots")
        return pslot

    def _parent_slots_numpy(self, ebase, nentries):
        pslot = np.full(nentries, -1, dtype=np.int64)
        for lev in range(self.root_level, self.nlevels - 1):
            cs = self._cand_src[lev]
            if cs is None:
                continue
            t = np.flatnonzero(cs >= 0)
            fpos = t if self._final_pos[lev] is None else self._final_pos[lev][t]
            pslot[ebase[lev + 1] + cs[t]] = ebase[lev] + fpos
        return pslot

    def _lists_host(self):
        """The translation lists in CSR by target box, with numpy (the same
        lists as ``_lists_device``)."""
        tree = self.tree
        below = tree.get_boxes_levels() > self.root_level
        boxes_below = np.flatnonzero(below)
        col = tree.get_boxes_colleague_neigh_fullvec(boxes_below)
        t = np.repeat(boxes_below, col.shape[1])
        s = col.ravel()
        coll = np.stack((t[s >= 0], s[s >= 0]), 1)
        crs = tree.get_boxes_coarse_neigh_fullvec(boxes_below)
        t = np.repeat(boxes_below, crs.shape[1])
        s = crs.ravel()
        up = np.stack((t[s >= 0], s[s >= 0]), 1)
        rb = self.root_boxes
        root = np.stack((np.repeat(rb, rb.shape[0]), np.tile(rb, rb.shape[0])), 1)
        return lists_to_csr(self.nboxes, [
            (_lib.KIND_COLLEAGUE, coll), (_lib.KIND_COARSE_UP, up),
            (_lib.KIND_COARSE_DOWN, up[:, ::-1]), (_lib.KIND_ROOT, root)])

    def _lists_device(self):
        """The translation lists in CSR by target box, built on the device
        from the tree's neighbour tables (skf_lists_count / skf_lists_fill)."""
        tree = self.tree
        dev = self.device
        lib = _lib.load()

        def up(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int64)).to(dev)

        dt = getattr(tree, "_dev_tables", None)
        tdev = None if dt is None else dt["colleagues"].device
        if tdev is not None and tdev.type == dev.type and (dev.index is None or tdev.index == dev.index):
            # the device tree's own tables
            col, crs, ch, lev = dt["colleagues"], dt["coarse"], dt["children"], dt["level"]
        else:
            col, crs, ch, lev = up(tree._colleagues), up(tree._coarse), up(tree._children), up(tree._box_level)
        rb = up(self.root_boxes)
        nb = self.nboxes
        off = torch.empty(nb + 1, dtype=torch.int64, device=dev)
        total = ctypes.c_int64()
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        args = (self.ndim, nb, _lib.ptr(col), _lib.ptr(crs), _lib.ptr(ch), _lib.ptr(lev), int(self.root_level),
                _lib.ptr(rb), int(rb.shape[0]))
        _lib.check(lib.skf_lists_count(*args, _lib.ptr(off), ctypes.byref(total), stream), "skf_lists_count")
        n = int(total.value)
        src = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        kind = torch.empty(max(n, 1), dtype=torch.int8, device=dev)
        _lib.check(lib.skf_lists_fill(*args, _lib.ptr(off), _lib.ptr(src), _lib.ptr(kind), stream), "skf_lists_fill")
        return off.cpu().numpy(), src[:n].cpu().numpy(), kind[:n].cpu().numpy()

    def setup_lists(self, verbose=False):
        """Translation lists (recursive_skel.py:622-712, on the device) and
        index maps (recursive_skel.py:714-780), built directly in ragged
        form."""
        tree = self.tree
        nb = self.nboxes
        leaf_mask = tree._is_leaf
        root_boxes = np.hstack((tree.get_leaves_above(self.root_level),
                                tree.get_boxes_level(self.root_level))).astype(np.int64)
        self.root_boxes = root_boxes
        leaves = tree.get_leaves()
        # leaves at the root level or below (the sorted leaves minus those above)
        self.skel_leaves = leaves[tree._box_level[leaves] > self.root_level]
        self.list_off, self.list_src, self.list_kind = self._lists_device()

        # entries: levels in order, boxes in order (levels above the root:
        # leaves only)
        bs = np.zeros(nb, dtype=np.int64)
        ids_all, ebase = [], np.zeros(self.nlevels + 1, dtype=np.int64)
        for lev in range(self.nlevels):
            ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
            if self._ids[lev] is None:
                ebase[lev + 1] = ebase[lev]
                continue
            bl = np.diff(self._off[lev])
            if lev < self.root_level:
                bl = np.where(leaf_mask[ls:le], bl, 0)
                keep = np.repeat(leaf_mask[ls:le], np.diff(self._off[lev]))
                ids_all.append(self._ids[lev][keep])
            else:
                ids_all.append(self._ids[lev])
            bs[ls:le] = bl
            ebase[lev + 1] = ebase[lev] + int(bl.sum())
        self.bs_list = bs
        off = np.zeros(nb + 1, dtype=np.int64)
        np.cumsum(bs, out=off[1:])
        self.box_off = off
        ids = np.concatenate(ids_all) if ids_all else np.zeros(0, np.int64)
        self.entry_pid = ids
        pslot = self._parent_slots(ebase, int(off[-1]))
        self.entry_pslot = pslot
        # the entries of the leaves, in box order
        self.perm_entry = _concat_ranges(off[:-1][leaves], bs[leaves])
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        self.perm_point = np.empty(self.perm_entry.shape[0], dtype=np.int64)
        _lib.check(_lib.load().skf_gather_i64(self.perm_entry.shape[0], _lib.ptr(self.perm_entry), _lib.ptr(ids),
                                              ids.shape[0], _lib.ptr(self.perm_point)), "skf_gather_i64")
        # T blocks: device buffers of the skeletonized levels, back to back
        cplx = is_complex_op(self.op_id)
        t_off = np.full(nb, -1, dtype=np.int64)
        parts, acc = [], 0
        for lev in range(self.root_level + 1, self.nlevels):
            if self._tdev[lev] is None:
                continue
            ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
            r = self.rank_list[ls:le]
            has = r > 0
            t_off[ls:le] = np.where(has, self._toff[lev] + acc, -1)
            used = int((r * (np.diff(self._off[lev]) - r)).sum())
            parts.append(self._tdev[lev][:used] if used else self._tdev[lev][:0])
            acc += used
        dt = torch.complex128 if cplx else torch.float64
        self.t_off = t_off
        self.t_data = torch.cat(parts) if acc else torch.zeros(1, dtype=dt, device=self.device)
        if verbose:
            print("\t root level %d, %d root boxes, %d entries" % (self.root_level, root_boxes.shape[0], off[-1]))

    def _gather_xyz(self, pid):
        """Coordinates of the points ``pid`` (device float64 [len, ndim]),
        gathered from the build's device copy."""
        idx = torch.from_numpy(np.ascontiguousarray(pid, dtype=np.int64)).to(self.device)
        return self._XX_dev.index_select(0, idx)

    def ragged(self):
        """The build as a ``RaggedBuild``; T and the entries' coordinates
        (and normals) stay on the device."""
        geom = None
        if self._geom_dev is not None:
            idx = torch.from_numpy(np.ascontiguousarray(self.entry_pid, dtype=np.int64)).to(self.device)
            geom = self._geom_dev.index_select(0, idx)
        return RaggedBuild(
            op=self.op_id, ndim=self.ndim, kappa=self.kappa, npoints=int(self.N), nlevels=int(self.nlevels),
            root_level=int(self.root_level), box_level=self.tree.get_boxes_levels().astype(np.int32),
            box_off=self.box_off, box_rank=self.rank_list.astype(np.int32),
            entry_xyz=self._gather_xyz(self.entry_pid), entry_geom=geom,
            entry_pslot=self.entry_pslot, perm_entry=self.perm_entry, perm_point=self.perm_point,
            t_off=self.t_off, t_data=self.t_data, list_off=self.list_off, list_src=self.list_src,
            list_kind=self.list_kind,
        )
