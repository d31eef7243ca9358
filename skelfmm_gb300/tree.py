"""Adaptive 2:1-balanced quadtree / octree and the point-cloud helpers around it.

The reference takes its tree from the external ``simpletree`` package
(``pyproject.toml:22``), which is not vendored.  This module is the framework's
own tree with the interface the reference calls:

* ``BalancedTree(points, leaf_size)`` (called at ``skelfmm/skel_fmm.py:150``),
  with the accessors used in ``skelfmm/recursive_skel.py:54-76,142-166,217-220,
  358-360,377,643-653,692-699,728-731,746-753`` and ``skelfmm/batched_fmm.py:11-20,146``;
* ``get_cube_surface`` / ``get_sphere_surface`` (proxy surfaces,
  ``skelfmm/util.py:72-78``);
* ``findin_sorted`` (``skelfmm/recursive_skel.py:7,315,569``);
* ``get_point_dist`` (the demo point clouds the reference tests draw from).

Tree definition (the contract the skeletonization relies on):

* The root box is the bounding square/cube of the points: centre ``c0`` is the
  midpoint of the per-axis extremes and side ``L0`` the largest extent.
* A box is split when it holds more than ``leaf_size`` points.  Children that
  would be empty are not created, so every leaf holds at least one point.
* 2:1 balance: no leaf at level ``k`` touches (shares a face, edge or corner
  with) any box at level ``k+2`` or finer.  Leaves that violate this are split
  until no violation is left.
* Boxes are numbered level by level; inside a level they follow Morton order.
  Children rows list the existing children in Morton order, padded with -1.
* Colleague rows hold the same-level boxes whose index offsets lie in
  ``{-1,0,1}^d`` (self included), in lexicographic offset order, padded with -1.
* Coarse-neighbour rows of a box at level ``l`` hold the leaves at level
  ``l-1`` that touch it, padded with -1.
"""

from __future__ import annotations

import itertools

import numpy as np

_MAX_DEPTH = {2: 30, 3: 20}
# with a CUDA device given, clouds of at least this many points build their
# tree there (faster from a few thousand points on; the trees are identical)
DEVICE_FRONT_END_MIN_POINTS = 1


def _spread_bits(v: np.ndarray, ndim: int, nbits: int) -> np.ndarray:
    """Put bit b of ``v`` at bit b*ndim (the standard shift-and-mask bit
    interleave; 2D up to 32 bits, 3D up to 21 bits)."""
    x = v.astype(np.uint64) & np.uint64((1 << nbits) - 1 if nbits < 64 else ~0)
    if ndim == 2:
        steps = ((16, 0x0000FFFF0000FFFF), (8, 0x00FF00FF00FF00FF), (4, 0x0F0F0F0F0F0F0F0F),
                 (2, 0x3333333333333333), (1, 0x5555555555555555))
    elif ndim == 3:
        steps = ((32, 0x001F00000000FFFF), (16, 0x001F0000FF0000FF), (8, 0x100F00F00F00F00F),
                 (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249))
    else:
        out = np.zeros(v.shape, dtype=np.uint64)
        one = np.uint64(1)
        for bit in range(nbits):
            out |= ((x >> np.uint64(bit)) & one) << np.uint64(bit * ndim)
        return out
    for sh, mask in steps:
        x = (x | (x << np.uint64(sh))) & np.uint64(mask)
    return x


def morton_encode(coords: np.ndarray, nbits: int) -> np.ndarray:
    """Interleave the bits of integer coordinates ``coords[n, d]``.

    Axis 0 takes the most significant bit of every ``d``-bit group.
    """
    coords = np.asarray(coords)
    ndim = coords.shape[1]
    code = np.zeros(coords.shape[0], dtype=np.uint64)
    for d in range(ndim):
        code |= _spread_bits(coords[:, d].astype(np.uint64), ndim, nbits) << np.uint64(ndim - 1 - d)
    return code


def findin_sorted(arr, val):
    """Index of ``val`` in the sorted array ``arr``, or -1 when absent."""
    arr = np.asarray(arr)
    ind = int(np.searchsorted(arr, val))
    if ind < arr.shape[0] and arr[ind] == val:
        return ind
    return -1


class BalancedTree:
    """Adaptive, 2:1-balanced tree over ``points[N, d]`` (d = 2 or 3)."""

    def __init__(self, points, leaf_size, device=None):
        """``device``: a CUDA device (torch.device or string) to build the
        tree there for clouds of DEVICE_FRONT_END_MIN_POINTS or more: the
        points' integer cells and Morton keys in a CUDA kernel, the stable
        key sort on the device, then the box levels, the 2:1 balance and the
        neighbour tables from the sorted keys (skf_tree_build).  The tree is
        identical to the host build."""
        XX = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
        if XX.ndim != 2 or XX.shape[1] not in (2, 3):
            raise ValueError("points must have shape (N, 2) or (N, 3)")
        if XX.shape[0] == 0:
            raise ValueError("points must not be empty")
        if int(leaf_size) < 1:
            raise ValueError("leaf_size must be positive")
        self.XX = XX
        self.N, self.ndim = XX.shape
        self.leaf_size = int(leaf_size)
        ndim = self.ndim

        D = _MAX_DEPTH[ndim]
        self._depth = D
        if (device is not None and str(device).startswith("cuda") and self.N >= DEVICE_FRONT_END_MIN_POINTS
                and self.N < 2 ** 31):  # the device sort indexes points with 32-bit counts
            skeys = self._front_end_device(XX, device)
            self._box_levels_device(skeys)
            self._set_geometry()
            return
        else:
            lo = XX.min(axis=0)
            hi = XX.max(axis=0)
            self.c0 = 0.5 * (lo + hi)
            ext = float(np.max(hi - lo))
            self.L0 = ext if ext > 0 else 1.0
            corner = self.c0 - 0.5 * self.L0
            # (x - corner) / L0 * 2^D, floored and clipped to [0, 2^D - 1], in place
            scaled = XX - corner[None, :]
            scaled /= self.L0
            scaled *= float(1 << D)
            np.floor(scaled, out=scaled)
            np.minimum(scaled, float((1 << D) - 1), out=scaled)
            np.maximum(scaled, 0.0, out=scaled)
            q = scaled.astype(np.int64)
            del scaled
            keys = morton_encode(q, D)
            # stable argsort: an unstable sort, then input order restored among
            # equal keys (points sharing a finest cell; rare)
            perm = np.argsort(keys)
            skeys = keys[perm]
            tie = np.flatnonzero(skeys[1:] == skeys[:-1])
            if tie.size:
                pos = np.unique(np.concatenate((tie, tie + 1)))
                perm[pos] = perm[pos][np.lexsort((perm[pos], skeys[pos]))]
            self._perm = perm
            self._skeys = skeys
            self._q = q  # integer coordinates in input order (box corners via _perm)

        # per level (sorted by Morton code): coords, codes, point ranges, leaf flags
        self._Lc = [np.zeros((1, ndim), dtype=np.int64)]
        self._Lk = [np.zeros(1, dtype=np.uint64)]
        self._Ls = [np.zeros(1, dtype=np.int64)]
        self._Le = [np.full(1, self.N, dtype=np.int64)]
        self._Lleaf = [np.ones(1, dtype=bool)]

        # adaptive refinement, level by level
        lev = 0
        while lev < D:
            split = np.flatnonzero(self._Lleaf[lev] & (self._Le[lev] - self._Ls[lev] > self.leaf_size))
            if split.size == 0:
                break
            self._split_boxes(lev, split)
            lev += 1

        # 2:1 balance
        self._balance()

        self._finalize()

    # ------------------------------------------------------------------ build
    def _front_end_device(self, XX, device):
        """Root box, integer cells, keys and the stable key order computed on
        ``device``: skf_morton_keys (the same FP64 steps as the host path)
        and a stable device radix sort (skf_sort_keys; ties keep the input
        order).  Returns the sorted keys (device)."""
        import torch

        from . import _lib

        dev = torch.device(device)
        x = torch.from_numpy(XX).to(dev)
        lo, hi = torch.aminmax(x, dim=0)
        lo, hi = lo.cpu().numpy(), hi.cpu().numpy()
        self.c0 = 0.5 * (lo + hi)
        ext = float(np.max(hi - lo))
        self.L0 = ext if ext > 0 else 1.0
        corner = self.c0 - 0.5 * self.L0
        n, ndim = XX.shape
        ct = torch.from_numpy(np.ascontiguousarray(corner)).to(dev)
        keys = torch.empty(n, dtype=torch.int64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        lib = _lib.load()
        _lib.check(lib.skf_morton_keys(ndim, n, _lib.ptr(x), _lib.ptr(ct), float(self.L0), self._depth,
                                       _lib.ptr(keys), None, stream), "skf_morton_keys")
        skeys = torch.empty_like(keys)
        perm = torch.empty(n, dtype=torch.int64, device=dev)
        _lib.check(lib.skf_sort_keys(n, _lib.ptr(keys), _lib.ptr(skeys), _lib.ptr(perm), ndim * self._depth, stream),
                   "skf_sort_keys")
        self._perm = perm.cpu().numpy()
        self._skeys = skeys.cpu().numpy().view(np.uint64)
        return skeys

    def _box_levels_device(self, skeys):
        """Refinement, 2:1 balance and the neighbour tables on the device
        (skf_tree_build over the sorted keys), copied into the host arrays
        the host build fills."""
        import ctypes

        import torch

        from . import _lib

        lib = _lib.load()
        ndim = self.ndim
        h = ctypes.c_void_p()
        stream = torch.cuda.current_stream(skeys.device).cuda_stream
        _lib.check(lib.skf_tree_build(ndim, self.N, _lib.ptr(skeys), self._depth, self.leaf_size, ctypes.byref(h),
                                      stream), "skf_tree_build")
        try:
            nlev, nb = ctypes.c_int32(), ctypes.c_int64()
            _lib.check(lib.skf_tree_query(h, ctypes.byref(nlev), ctypes.byref(nb)), "skf_tree_query")
            nlev, nb = int(nlev.value), int(nb.value)
            nc, nq = 1 << ndim, 3 ** ndim
            level_sep = np.zeros(nlev + 1, dtype=np.int64)
            code = np.empty(nb, dtype=np.uint64)
            coords = np.empty((nb, ndim), dtype=np.int64)
            start = np.empty(nb, dtype=np.int64)
            end = np.empty(nb, dtype=np.int64)
            leaf = np.empty(nb, dtype=np.uint8)
            parent = np.empty(nb, dtype=np.int64)
            children = np.empty((nb, nc), dtype=np.int64)
            colleagues = np.empty((nb, nq), dtype=np.int64)
            coarse = np.empty((nb, nc), dtype=np.int64)
            _lib.check(lib.skf_tree_export(h, *(_lib.ptr(a) for a in (
                level_sep, code, coords, start, end, leaf, parent, children, colleagues, coarse)), stream),
                "skf_tree_export")
            # the neighbour tables also stay on the device for the lists
            dev = skeys.device
            dch = torch.empty((nb, nc), dtype=torch.int64, device=dev)
            dco = torch.empty((nb, nq), dtype=torch.int64, device=dev)
            dcr = torch.empty((nb, nc), dtype=torch.int64, device=dev)
            _lib.check(lib.skf_tree_export(h, None, None, None, None, None, None, None, _lib.ptr(dch), _lib.ptr(dco),
                                           _lib.ptr(dcr), stream), "skf_tree_export")
        finally:
            lib.skf_tree_destroy(h)
        self._dev_tables = {"children": dch, "colleagues": dco, "coarse": dcr,
                            "level": torch.repeat_interleave(torch.arange(nlev, dtype=torch.int64, device=dev),
                                                             torch.from_numpy(np.diff(level_sep)).to(dev))}
        leaf = leaf.astype(bool)
        sl = [slice(int(level_sep[l]), int(level_sep[l + 1])) for l in range(nlev)]
        self._Lc = [coords[s] for s in sl]
        self._Lk = [code[s] for s in sl]
        self._Ls = [start[s] for s in sl]
        self._Le = [end[s] for s in sl]
        self._Lleaf = [leaf[s] for s in sl]
        self.nlevels = nlev
        self.level_sep = level_sep
        self.nboxes = nb
        self._box_coords = coords
        self._box_start = start
        self._box_end = end
        self._is_leaf = leaf
        self._box_level = np.repeat(np.arange(nlev, dtype=np.int64), np.diff(level_sep))
        self._leaves = np.flatnonzero(leaf).astype(np.int64)
        self.nleaves = int(self._leaves.shape[0])
        self._children = children
        self._parent = parent
        self._colleagues = colleagues
        self._coarse = coarse

    def _lookup(self, lev, coords):
        """Index within level ``lev`` of the boxes at integer ``coords``, -1 if absent."""
        n = self._Lk[lev].shape[0]
        nmax = (1 << lev) - 1
        valid = np.all((coords >= 0) & (coords <= nmax), axis=1)
        codes = morton_encode(np.where(valid[:, None], coords, 0), lev)
        pos = np.searchsorted(self._Lk[lev], codes)
        posc = np.minimum(pos, max(n - 1, 0))
        found = valid & (pos < n) & (self._Lk[lev][posc] == codes)
        return np.where(found, posc, -1)

    def _split_boxes(self, lev, sel):
        """Split the leaves ``sel`` (indices within level ``lev``): their
        non-empty children join level ``lev + 1``."""
        D = self._depth
        if lev + 1 > D or sel.size == 0:
            return
        starts = self._Ls[lev][sel]
        ends = self._Le[lev][sel]
        lens = ends - starts
        shift = np.uint64(self.ndim * (D - lev - 1))
        if sel.size == self._Ls[lev].shape[0] and int(lens.sum()) == self.N:
            # every box of the level splits: the points in order, child
            # boundaries where the child code changes
            ck = self._skeys >> shift
            brk = np.flatnonzero(ck[1:] != ck[:-1]) + 1
            first = np.concatenate(([0], brk)).astype(np.int64)
            cs = first
            ce = np.concatenate((brk, [self.N])).astype(np.int64)
        else:
            # concatenated point ranges [start, end) of the boxes
            before = np.cumsum(lens) - lens
            idx = np.arange(int(lens.sum()), dtype=np.int64) + np.repeat(starts - before, lens)
            ck = self._skeys[idx] >> shift
            brk = np.flatnonzero((ck[1:] != ck[:-1]) | (idx[1:] != idx[:-1] + 1)) + 1
            first = np.concatenate(([0], brk))
            cs = idx[first]
            ce = np.concatenate((idx[brk - 1] + 1, [idx[-1] + 1]))
        coords = (self._q[self._perm[cs]] >> (D - lev - 1)).astype(np.int64)
        codes = ck[first]
        self._Lleaf[lev][sel] = False
        if len(self._Lk) <= lev + 1:
            self._Lc.append(coords)
            self._Lk.append(codes)
            self._Ls.append(cs.astype(np.int64))
            self._Le.append(ce.astype(np.int64))
            self._Lleaf.append(np.ones(cs.shape[0], dtype=bool))
            return
        k = np.concatenate((self._Lk[lev + 1], codes))
        order = np.argsort(k, kind="stable")
        self._Lk[lev + 1] = k[order]
        self._Lc[lev + 1] = np.concatenate((self._Lc[lev + 1], coords))[order]
        self._Ls[lev + 1] = np.concatenate((self._Ls[lev + 1], cs))[order]
        self._Le[lev + 1] = np.concatenate((self._Le[lev + 1], ce))[order]
        self._Lleaf[lev + 1] = np.concatenate((self._Lleaf[lev + 1], np.ones(cs.shape[0], dtype=bool)))[order]

    def _balance(self):
        """Split every leaf at level l-2 that touches a box at level l, until
        none is left."""
        ndim = self.ndim
        combos = np.array(list(itertools.product((0, 1), repeat=ndim)), dtype=np.int64)
        changed = True
        while changed:
            changed = False
            for lev in range(len(self._Lk) - 1, 1, -1):
                C = self._Lc[lev]
                if C.shape[0] == 0:
                    continue
                nmax = (1 << (lev - 2)) - 1
                g0 = np.maximum(0, -((4 - C) // 4))  # ceil((b-4)/4)
                g1 = np.minimum(nmax, (C + 1) // 4)
                G = (g0[:, None, :] + combos[None, :, :]).reshape(-1, ndim)
                ok = np.all(G <= np.repeat(g1, combos.shape[0], axis=0), axis=1)
                codes = np.unique(morton_encode(G[ok], lev - 2))
                Lk = self._Lk[lev - 2]
                pos = np.minimum(np.searchsorted(Lk, codes), Lk.shape[0] - 1)
                pos = pos[Lk[pos] == codes]
                marks = np.unique(pos[self._Lleaf[lev - 2][pos]])
                if marks.size:
                    self._split_boxes(lev - 2, marks)
                    changed = True

    def _finalize(self):
        ndim = self.ndim
        nlev = len(self._Lk)
        while nlev > 0 and self._Lk[nlev - 1].shape[0] == 0:
            nlev -= 1
        for name in ("_Lc", "_Lk", "_Ls", "_Le", "_Lleaf"):
            setattr(self, name, getattr(self, name)[:nlev])
        self.nlevels = nlev

        level_sep = np.zeros(nlev + 1, dtype=np.int64)
        for lev in range(nlev):
            level_sep[lev + 1] = level_sep[lev] + self._Lk[lev].shape[0]
        self.level_sep = level_sep
        self.nboxes = int(level_sep[-1])
        self._box_coords = np.concatenate(self._Lc, axis=0)
        self._box_start = np.concatenate(self._Ls)
        self._box_end = np.concatenate(self._Le)
        self._is_leaf = np.concatenate(self._Lleaf)
        self._box_level = np.concatenate([np.full(self._Lk[l].shape[0], l, dtype=np.int64) for l in range(nlev)])
        self._leaves = np.flatnonzero(self._is_leaf).astype(np.int64)
        self.nleaves = int(self._leaves.shape[0])

        nb = self.nboxes
        nchild = 1 << ndim
        children = np.full((nb, nchild), -1, dtype=np.int64)
        parent = np.full(nb, -1, dtype=np.int64)
        for lev in range(1, nlev):
            base = level_sep[lev]
            n = self._Lk[lev].shape[0]
            pl = self._lookup(lev - 1, self._Lc[lev] >> 1)
            pg = pl + level_sep[lev - 1]
            parent[base:base + n] = pg
            # siblings are contiguous in Morton order
            firsts = np.concatenate(([0], np.flatnonzero(pg[1:] != pg[:-1]) + 1))
            slot = np.arange(n) - np.repeat(firsts, np.diff(np.concatenate((firsts, [n]))))
            children[pg, slot] = base + np.arange(n)
        self._children = children
        self._parent = parent

        # colleagues: offsets in {-1,0,1}^d, lexicographic
        offsets = np.array(list(itertools.product((-1, 0, 1), repeat=ndim)), dtype=np.int64)
        colleagues = np.full((nb, offsets.shape[0]), -1, dtype=np.int64)
        coarse = np.full((nb, nchild), -1, dtype=np.int64)
        pair = np.array(list(itertools.product((0, 1), repeat=ndim)), dtype=np.int64)
        for lev in range(nlev):
            base = level_sep[lev]
            C = self._Lc[lev]
            n = C.shape[0]
            for k in range(offsets.shape[0]):
                pos = self._lookup(lev, C + offsets[k][None, :])
                colleagues[base:base + n, k] = np.where(pos >= 0, pos + base, -1)
            if lev == 0:
                continue
            # coarse neighbours: leaves one level up touching the box, parent excluded
            nmax_up = (1 << (lev - 1)) - 1
            g0 = np.maximum(0, -((2 - C) // 2))  # ceil((x-2)/2)
            g1 = np.minimum(nmax_up, (C + 1) // 2)
            par = C >> 1
            found = np.full((n, pair.shape[0]), -1, dtype=np.int64)
            for t in range(pair.shape[0]):
                G = g0 + pair[t][None, :]
                ok = np.all(G <= g1, axis=1) & ~np.all(G == par, axis=1)
                pos = self._lookup(lev - 1, np.where(ok[:, None], G, -1))
                gpos = pos + level_sep[lev - 1]
                keep = (pos >= 0) & self._is_leaf[np.where(pos >= 0, gpos, 0)]
                found[:, t] = np.where(keep, gpos, -1)
            # compact each row, keeping the enumeration order
            order = np.argsort(found < 0, axis=1, kind="stable")
            coarse[base:base + n] = np.take_along_axis(found, order, axis=1)
        self._colleagues = colleagues
        self._coarse = coarse
        self._set_geometry()

    def _set_geometry(self):
        lengths = self.L0 * np.power(0.5, self._box_level.astype(np.float64))
        corner = self.c0 - 0.5 * self.L0
        self._box_length = lengths
        self._box_center = corner[None, :] + (self._box_coords.astype(np.float64) + 0.5) * lengths[:, None]

    # ------------------------------------------------------------- accessors
    def get_leaves(self):
        return self._leaves.copy()

    def get_boxes_level(self, lev):
        return np.arange(self.level_sep[lev], self.level_sep[lev + 1], dtype=np.int64)

    def get_box_inds(self, box):
        return self._perm[self._box_start[box]:self._box_end[box]]

    def get_box_npoints(self, boxes=None):
        if boxes is None:
            return self._box_end - self._box_start
        boxes = np.asarray(boxes)
        return self._box_end[boxes] - self._box_start[boxes]

    def is_leaf(self, box):
        return bool(self._is_leaf[box])

    def are_leaves(self, boxes):
        return self._is_leaf[np.asarray(boxes, dtype=np.int64)]

    def get_box_children(self, box):
        row = self._children[box]
        return row[row >= 0]

    def get_boxes_children_fullvec(self, boxes):
        return self._children[np.asarray(boxes, dtype=np.int64)]

    def get_box_parent(self, box):
        return int(self._parent[box])

    def get_box_length(self, box):
        return float(self._box_length[box])

    def get_box_center(self, box):
        return self._box_center[box].copy()

    def get_boxes_centers(self, boxes):
        return self._box_center[np.asarray(boxes, dtype=np.int64)]

    def get_box_level(self, box):
        return int(self._box_level[box])

    def get_boxes_levels(self, boxes=None):
        if boxes is None:
            return self._box_level.copy()
        return self._box_level[np.asarray(boxes, dtype=np.int64)]

    def get_leaves_above(self, lev):
        leaves = self._leaves
        return leaves[self._box_level[leaves] < lev]

    def get_box_colleague_neigh(self, box):
        row = self._colleagues[box]
        return row[row >= 0]

    def get_boxes_colleague_neigh_fullvec(self, boxes):
        return self._colleagues[np.asarray(boxes, dtype=np.int64)]

    def get_box_coarse_neigh(self, box):
        row = self._coarse[box]
        return row[row >= 0]

    def get_boxes_coarse_neigh_fullvec(self, boxes):
        return self._coarse[np.asarray(boxes, dtype=np.int64)]

    def get_box_coords(self, boxes=None):
        if boxes is None:
            return self._box_coords.copy()
        return self._box_coords[np.asarray(boxes, dtype=np.int64)]


# ---------------------------------------------------------------- geometry
def get_cube_surface(center, length, nproxy):
    """Proxy points on the boundary of the square/cube of side ``length``.

    2D: ``4*ceil(nproxy/4)`` points, equispaced along the perimeter.
    3D: ``6*n*n`` points with ``n = ceil(sqrt(nproxy/6))``, at the cell
    centres of an ``n x n`` grid on each face.
    """
    center = np.asarray(center, dtype=np.float64)
    h = 0.5 * float(length)
    ndim = center.shape[0]
    if ndim == 2:
        n = max(1, int(np.ceil(nproxy / 4.0)))
        t = -h + float(length) * np.arange(n, dtype=np.float64) / n
        pts = np.concatenate(
            (
                np.stack((t, np.full(n, -h)), axis=1),
                np.stack((np.full(n, h), t), axis=1),
                np.stack((-t, np.full(n, h)), axis=1),
                np.stack((np.full(n, -h), -t), axis=1),
            ),
            axis=0,
        )
        return pts + center[None, :]
    n = max(1, int(np.ceil(np.sqrt(nproxy / 6.0))))
    s = -h + float(length) * (np.arange(n, dtype=np.float64) + 0.5) / n
    a, b = np.meshgrid(s, s, indexing="ij")
    a = a.ravel()
    b = b.ravel()
    full = np.full(a.shape[0], h)
    faces = []
    for axis in range(3):
        others = [d for d in range(3) if d != axis]
        for sign in (-1.0, 1.0):
            f = np.empty((a.shape[0], 3))
            f[:, axis] = sign * full
            f[:, others[0]] = a
            f[:, others[1]] = b
            faces.append(f)
    return np.concatenate(faces, axis=0) + center[None, :]


def get_sphere_surface(center, length, npoints):
    """``npoints`` proxy points on the circle/sphere of diameter ``length``.

    2D: equispaced angles.  3D: Fibonacci (golden-angle) spiral.
    """
    center = np.asarray(center, dtype=np.float64)
    r = 0.5 * float(length)
    n = max(1, int(npoints))
    if center.shape[0] == 2:
        th = 2.0 * np.pi * np.arange(n, dtype=np.float64) / n
        return center[None, :] + r * np.stack((np.cos(th), np.sin(th)), axis=1)
    k = np.arange(n, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * k / n
    rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.pi * (3.0 - np.sqrt(5.0)) * k
    pts = np.stack((rho * np.cos(phi), rho * np.sin(phi), z), axis=1)
    return center[None, :] + r * pts


POINT_GEOMETRIES = (
    "square",
    "cube",
    "circle_surface",
    "cube_surface",
    "sphere_surface",
    "annulus",
    "curvy_annulus",
    "gaussian_clusters",
)


def get_point_dist(N, name, rng=None):
    """Demo point clouds.  Draws from ``rng`` (a numpy Generator) when given,
    else from numpy's global random state."""
    N = int(N)
    if rng is None:
        rand = np.random.rand
        randn = np.random.randn
    else:
        rand = lambda *s: rng.random(s)  # noqa: E731
        randn = lambda *s: rng.standard_normal(s)  # noqa: E731
    if name == "square":
        return rand(N, 2)
    if name == "cube":
        return rand(N, 3)
    if name == "circle_surface":
        th = 2 * np.pi * rand(N)
        return np.stack((np.cos(th), np.sin(th)), axis=1)
    if name == "sphere_surface":
        g = randn(N, 3)
        return g / np.linalg.norm(g, axis=1, keepdims=True)
    if name == "cube_surface":
        pts = rand(N, 3)
        face = np.floor(rand(N) * 6).astype(np.int64)
        axis = face // 2
        pts[np.arange(N), axis] = (face % 2).astype(np.float64)
        return pts
    if name in ("annulus", "curvy_annulus"):
        rho = 0.5 + 0.5 * rand(N)
        th = 2 * np.pi * rand(N)
        r = rho * (1 + 0.25 * np.cos(6 * th)) if name == "curvy_annulus" else rho
        return np.stack((r * np.cos(th), r * np.sin(th)), axis=1)
    if name == "gaussian_clusters":
        # 32 isotropic Gaussian clusters, centres uniform in the unit cube,
        # standard deviations log-uniform in [1e-3, 5e-2]
        centres = rand(32, 3)
        sigma = np.exp(np.log(1e-3) + (np.log(5e-2) - np.log(1e-3)) * rand(32))
        which = np.minimum((rand(N) * 32).astype(np.int64), 31)
        return centres[which] + sigma[which, None] * randn(N, 3)
    raise ValueError(f"Unknown geometry {name!r}. Available: {', '.join(POINT_GEOMETRIES)}")
