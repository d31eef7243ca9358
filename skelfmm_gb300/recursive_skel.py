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


class RecursiveSkeletonization:
    """Build of the skeletonized tree for one operator (GPU IDs)."""

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

        leaves = tree.get_leaves()
        self.nproxy_level = nproxy_levels(self.ndim, tol, self.kappa, tree.L0, self.nlevels)
        self.max_bs_leaf = tree.leaf_size
        self.bs_list = np.zeros(self.nboxes, dtype=np.int64)
        self.rank_list = np.zeros(self.nboxes, dtype=np.int64)
        self.pid = [None] * self.nboxes
        self.proj = [None] * self.nboxes  # host copies of T (rank x (bs-rank))
        for leaf in leaves:
            inds = tree.get_box_inds(leaf)
            if inds.shape[0] > self.max_bs_leaf:
                raise ValueError("Leaf block size exceeds maximum allowed")
            self.pid[leaf] = np.asarray(inds, dtype=np.int64)
            self.bs_list[leaf] = inds.shape[0]
        self.root_level = max(0, self.nlevels - 1)
        self.level_times = {}
        self._XX_dev = torch.from_numpy(np.ascontiguousarray(tree.XX)).to(self.device)

    @property
    def rank_max(self):
        pos = self.rank_list[self.rank_list > 0]
        return int(pos.max()) if pos.size else 0

    def _update_lev_skel(self, lev):
        """Parent candidate set = children's skeletons (recursive_skel.py:209-262)."""
        for box in self.tree.get_boxes_level(lev):
            if self.tree.is_leaf(box):
                continue
            parts = [self.pid[c][: self.rank_list[c]] for c in self.tree.get_box_children(box)]
            self.pid[box] = np.concatenate(parts) if parts else np.zeros(0, np.int64)
            self.bs_list[box] = self.pid[box].shape[0]

    def _skel_level(self, lev):
        """Proxy IDs of every box at ``lev`` in one GPU call."""
        tree = self.tree
        boxes = tree.get_boxes_level(lev)
        bs = self.bs_list[boxes]
        off = np.zeros(boxes.shape[0] + 1, dtype=np.int64)
        np.cumsum(bs, out=off[1:])
        ids = np.concatenate([self.pid[b] for b in boxes]) if off[-1] > 0 else np.zeros(0, np.int64)
        dev = self.device
        ids_t = torch.from_numpy(ids).to(dev)
        x = self._XX_dev.index_select(0, ids_t).contiguous()
        g = None
        if self.geometry is not None:
            g = torch.from_numpy(self.geometry).to(dev).index_select(0, ids_t).contiguous()
        centers = torch.from_numpy(np.ascontiguousarray(tree.get_boxes_centers(boxes))).to(dev)
        cplx = is_complex_op(self.op_id)
        cap = (bs * bs) // 4 + bs
        t_off = np.zeros(boxes.shape[0], dtype=np.int64)
        np.cumsum(cap[:-1], out=t_off[1:])
        t_len = int(cap.sum())
        t_buf = torch.zeros(max(t_len, 1), dtype=torch.complex128 if cplx else torch.float64, device=dev)
        rank = torch.zeros(boxes.shape[0], dtype=torch.int32, device=dev)
        perm = torch.zeros(max(int(off[-1]), 1), dtype=torch.int32, device=dev)
        off_t = torch.from_numpy(off).to(dev)
        t_off_t = torch.from_numpy(t_off).to(dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(_lib.load().skf_skel_boxes(
            self.op_id, self.kappa, int(boxes.shape[0]), _lib.ptr(off_t), _lib.ptr(x), _lib.ptr(g),
            _lib.ptr(centers), float(tree.get_box_length(boxes[0])), int(self.nproxy_level[lev]),
            float(self.tol), _lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t), _lib.ptr(t_buf),
            ctypes.c_void_p(stream)), "skf_skel_boxes")
        rank_h = rank.cpu().numpy().astype(np.int64)
        perm_h = perm.cpu().numpy().astype(np.int64)
        t_h = t_buf.cpu().numpy()
        for i, b in enumerate(boxes):
            r, s = int(rank_h[i]), int(bs[i])
            p = perm_h[off[i]: off[i + 1]]
            self.rank_list[b] = r
            self.pid[b] = self.pid[b][p]
            self.proj[b] = t_h[t_off[i]: t_off[i] + r * (s - r)].reshape(r, s - r)

    def skel_tree(self, npoints_max, p=None, verbose=False):
        """Level loop of recursive_skel.py:326-502 with GPU IDs per level.

        ``p`` (the reference's process pool) is accepted and ignored.
        """
        tree = self.tree
        self.root_level = max(0, tree.nlevels - 1)
        for lev in range(tree.nlevels - 1, 0, -1):
            self._update_lev_skel(lev)
            boxes_lev = tree.get_boxes_level(lev)
            active = np.hstack((tree.get_leaves_above(lev), boxes_lev)).astype(np.int64)
            npoints_lev = int(np.sum(self.bs_list[active]))
            if verbose:
                print("\t Level %2d has %6d npoints" % (lev, npoints_lev))
            if lev == 2 or npoints_lev <= npoints_max:
                self.root_level = lev
                break
            t0 = perf_counter()
            self._skel_level(lev)
            torch.cuda.synchronize(self.device)
            self.level_times[lev] = perf_counter() - t0
            if verbose:
                print("\t Level %2d ids: %5.3f s" % (lev, self.level_times[lev]))
        return self

    def setup_lists(self, verbose=False):
        """Translation lists (recursive_skel.py:622-712) and index maps
        (recursive_skel.py:714-780), built directly in ragged form."""
        tree = self.tree
        nb = self.nboxes
        levels = tree.get_boxes_levels()
        leaf_mask = tree.are_leaves(np.arange(nb))
        below = levels > self.root_level
        boxes_below = np.flatnonzero(below)
        col = tree.get_boxes_colleague_neigh_fullvec(boxes_below)
        t = np.repeat(boxes_below, col.shape[1])
        s = col.ravel()
        coll = np.stack((t[s >= 0], s[s >= 0]), 1)
        crs = tree.get_boxes_coarse_neigh_fullvec(boxes_below)
        t = np.repeat(boxes_below, crs.shape[1])
        s = crs.ravel()
        up = np.stack((t[s >= 0], s[s >= 0]), 1)
        root_boxes = np.hstack((tree.get_leaves_above(self.root_level),
                                tree.get_boxes_level(self.root_level))).astype(np.int64)
        root = np.stack((np.repeat(root_boxes, root_boxes.shape[0]),
                         np.tile(root_boxes, root_boxes.shape[0])), 1)
        self.root_boxes = root_boxes
        self.skel_leaves = np.setdiff1d(tree.get_leaves(), tree.get_leaves_above(self.root_level + 1))
        self.colleague_pairs = coll
        self.coarse_up_pairs = up
        self.list_off, self.list_src, self.list_kind = lists_to_csr(nb, [
            (_lib.KIND_COLLEAGUE, coll), (_lib.KIND_COARSE_UP, up),
            (_lib.KIND_COARSE_DOWN, up[:, ::-1]), (_lib.KIND_ROOT, root)])

        # entries and offsets
        bs = np.array([0 if p is None else p.shape[0] for p in self.pid], dtype=np.int64)
        self.bs_list = bs
        off = np.zeros(nb + 1, dtype=np.int64)
        np.cumsum(bs, out=off[1:])
        self.box_off = off
        ids = np.concatenate([self.pid[b] for b in range(nb) if bs[b] > 0])
        self.entry_pid = ids
        # parent slots of skeleton entries
        pslot = np.full(int(off[-1]), -1, dtype=np.int64)
        for lev in range(self.root_level, self.nlevels):
            for box in tree.get_boxes_level(lev):
                if leaf_mask[box]:
                    continue
                kids = tree.get_box_children(box)
                rk = self.rank_list[kids]
                if lev == self.root_level:
                    pos = np.arange(int(rk.sum()))
                else:
                    cand = np.concatenate([self.pid[c][: self.rank_list[c]] for c in kids])
                    order = np.argsort(self.pid[box])
                    pos = order[np.searchsorted(self.pid[box], cand, sorter=order)]
                acc = 0
                for c, r in zip(kids, rk):
                    pslot[off[c]: off[c] + r] = off[box] + pos[acc: acc + r]
                    acc += r
        self.entry_pslot = pslot
        leaves = tree.get_leaves()
        self.perm_entry = np.concatenate([np.arange(off[b], off[b + 1]) for b in leaves])
        self.perm_point = np.concatenate([self.pid[b] for b in leaves])
        # T blocks
        cplx = is_complex_op(self.op_id)
        t_off = np.full(nb, -1, dtype=np.int64)
        blocks = []
        acc = 0
        for b in range(nb):
            r = int(self.rank_list[b])
            if r <= 0 or levels[b] <= self.root_level or self.proj[b] is None:
                continue
            t_off[b] = acc
            blocks.append(self.proj[b].ravel())
            acc += self.proj[b].size
        dt = np.complex128 if cplx else np.float64
        self.t_off = t_off
        self.t_data = np.concatenate(blocks).astype(dt) if blocks else np.zeros(1, dt)
        if verbose:
            print("\t root level %d, %d root boxes, %d entries" % (self.root_level, root_boxes.shape[0], off[-1]))

    def ragged(self):
        geom = None if self.geometry is None else self.geometry[self.entry_pid]
        return RaggedBuild(
            op=self.op_id, ndim=self.ndim, kappa=self.kappa, npoints=int(self.N), nlevels=int(self.nlevels),
            root_level=int(self.root_level), box_level=self.tree.get_boxes_levels().astype(np.int32),
            box_off=self.box_off, box_rank=self.rank_list.astype(np.int32),
            entry_xyz=np.ascontiguousarray(self.tree.XX[self.entry_pid]), entry_geom=geom,
            entry_pslot=self.entry_pslot, perm_entry=self.perm_entry, perm_point=self.perm_point,
            t_off=self.t_off, t_data=self.t_data, list_off=self.list_off, list_src=self.list_src,
            list_kind=self.list_kind,
        )
