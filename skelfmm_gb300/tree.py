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


def _spread_bits(v: np.ndarray, ndim: int, nbits: int) -> np.ndarray:
    out = np.zeros(v.shape, dtype=np.uint64)
    one = np.uint64(1)
    for b in range(nbits):
        out |= ((v >> np.uint64(b)) & one) << np.uint64(b * ndim)
    return out


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

    def __init__(self, points, leaf_size):
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

        lo = XX.min(axis=0)
        hi = XX.max(axis=0)
        self.c0 = 0.5 * (lo + hi)
        ext = float(np.max(hi - lo))
        self.L0 = ext if ext > 0 else 1.0

        D = _MAX_DEPTH[ndim]
        self._depth = D
        corner = self.c0 - 0.5 * self.L0
        scaled = (XX - corner[None, :]) / self.L0 * float(1 << D)
        q = np.clip(np.floor(scaled), 0, (1 << D) - 1).astype(np.int64)
        keys = morton_encode(q, D)
        perm = np.argsort(keys, kind="stable")
        self._perm = perm
        self._skeys = keys[perm]
        self._sq = q[perm]

        # per level: dict coords-tuple -> [start, end, is_leaf]
        levels = [{(0,) * ndim: [0, self.N, True]}]
        self._levels = levels

        # adaptive refinement
        lev = 0
        while lev < D:
            to_split = [c for c, rec in levels[lev].items() if rec[1] - rec[0] > self.leaf_size]
            if not to_split:
                break
            for c in to_split:
                self._split(lev, c)
            lev += 1

        # 2:1 balance
        self._balance()

        self._finalize()

    # ------------------------------------------------------------------ build
    def _split(self, lev, coords):
        rec = self._levels[lev][coords]
        if not rec[2]:
            return
        start, end = rec[0], rec[1]
        D = self._depth
        ndim = self.ndim
        if lev + 1 > D:
            return
        if len(self._levels) <= lev + 1:
            self._levels.append({})
        shift = np.uint64(ndim * (D - lev - 1))
        ck = self._skeys[start:end] >> shift
        brk = np.flatnonzero(ck[1:] != ck[:-1]) + 1
        starts = np.concatenate(([0], brk)) + start
        ends = np.concatenate((brk, [end - start])) + start
        child_level = self._levels[lev + 1]
        for s, e in zip(starts.tolist(), ends.tolist()):
            cc = tuple((self._sq[s] >> (D - lev - 1)).tolist())
            child_level[cc] = [s, e, True]
        rec[2] = False

    def _balance(self):
        ndim = self.ndim
        changed = True
        while changed:
            changed = False
            for lev in range(len(self._levels) - 1, 1, -1):
                coarse = self._levels[lev - 2]
                nmax = (1 << (lev - 2)) - 1
                marks = set()
                for c in self._levels[lev].keys():
                    ranges = []
                    for b in c:
                        g0 = max(0, -((4 - b) // 4))  # ceil((b-4)/4)
                        g1 = min(nmax, (b + 1) // 4)
                        ranges.append(range(g0, g1 + 1))
                    for g in itertools.product(*ranges):
                        rec = coarse.get(g)
                        if rec is not None and rec[2]:
                            marks.add(g)
                for g in marks:
                    self._split(lev - 2, g)
                    changed = True

    def _finalize(self):
        ndim = self.ndim
        D = self._depth
        nlev = len(self._levels)
        while nlev > 0 and not self._levels[nlev - 1]:
            nlev -= 1
        self._levels = self._levels[:nlev]
        self.nlevels = nlev

        coords_all, start_all, end_all, leaf_all, level_all = [], [], [], [], []
        level_sep = np.zeros(nlev + 1, dtype=np.int64)
        index_of = []
        for lev in range(nlev):
            items = list(self._levels[lev].items())
            cs = np.array([k for k, _ in items], dtype=np.int64).reshape(-1, ndim)
            codes = morton_encode(cs, max(lev, 1))
            order = np.argsort(codes, kind="stable")
            cs = cs[order]
            recs = [items[i][1] for i in order.tolist()]
            base = level_sep[lev]
            level_sep[lev + 1] = base + len(recs)
            index_of.append({tuple(cs[i].tolist()): base + i for i in range(len(recs))})
            coords_all.append(cs)
            start_all.append([r[0] for r in recs])
            end_all.append([r[1] for r in recs])
            leaf_all.append([r[2] for r in recs])
            level_all.append(np.full(len(recs), lev, dtype=np.int64))

        self.level_sep = level_sep
        self.nboxes = int(level_sep[-1])
        self._box_coords = np.concatenate(coords_all, axis=0)
        self._box_start = np.concatenate([np.asarray(s, dtype=np.int64) for s in start_all])
        self._box_end = np.concatenate([np.asarray(s, dtype=np.int64) for s in end_all])
        self._is_leaf = np.concatenate([np.asarray(s, dtype=bool) for s in leaf_all])
        self._box_level = np.concatenate(level_all)
        self._leaves = np.flatnonzero(self._is_leaf).astype(np.int64)
        self.nleaves = int(self._leaves.shape[0])

        nb = self.nboxes
        nchild = 1 << ndim
        children = np.full((nb, nchild), -1, dtype=np.int64)
        parent = np.full(nb, -1, dtype=np.int64)
        for lev in range(1, nlev):
            pidx = index_of[lev - 1]
            kids = {}
            for c, b in index_of[lev].items():
                p = pidx[tuple(x >> 1 for x in c)]
                parent[b] = p
                kids.setdefault(p, []).append(b)
            for p, bl in kids.items():
                bl.sort()
                children[p, : len(bl)] = bl
        self._children = children
        self._parent = parent

        # colleagues: offsets in {-1,0,1}^d, lexicographic
        offsets = list(itertools.product((-1, 0, 1), repeat=ndim))
        ncol = len(offsets)
        colleagues = np.full((nb, ncol), -1, dtype=np.int64)
        coarse = np.full((nb, nchild), -1, dtype=np.int64)
        for lev in range(nlev):
            idx = index_of[lev]
            nmax = (1 << lev) - 1
            up = index_of[lev - 1] if lev > 0 else None
            nmax_up = (1 << (lev - 1)) - 1 if lev > 0 else -1
            for c, b in idx.items():
                for k, off in enumerate(offsets):
                    n = tuple(ci + oi for ci, oi in zip(c, off))
                    if min(n) < 0 or max(n) > nmax:
                        continue
                    nbx = idx.get(n)
                    if nbx is not None:
                        colleagues[b, k] = nbx
                if up is None:
                    continue
                ranges = []
                for x in c:
                    g0 = max(0, -((2 - x) // 2))  # ceil((x-2)/2)
                    g1 = min(nmax_up, (x + 1) // 2)
                    ranges.append(range(g0, g1 + 1))
                acc = 0
                par = tuple(x >> 1 for x in c)
                for g in itertools.product(*ranges):
                    if g == par:
                        continue
                    nbx = up.get(g)
                    if nbx is not None and self._is_leaf[nbx]:
                        coarse[b, acc] = nbx
                        acc += 1
        self._colleagues = colleagues
        self._coarse = coarse

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
    raise ValueError(f"Unknown geometry {name!r}. Available: {', '.join(POINT_GEOMETRIES)}")
