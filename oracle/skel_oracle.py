"""CPU oracle for the strong-recursive-skeletonization build and apply.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the framework's
product code never imports it.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` use it.

It restates, in numpy/scipy, the algorithm of the reference implementation
(annayesy/skelFMM), keeping the reference's data layout so its arrays can be
compared one-to-one with the reference's own (see ``tests/golden/``):

* dense kernels ................. ``skelfmm/util.py:128-377``
* proxy matrix + pivoted-QR ID .. ``skelfmm/util.py:13-51, 72-124, 404-437``
* skeletonization build ......... ``skelfmm/recursive_skel.py:19-122, 142-166,
                                   209-324, 326-502, 504-539``
* translation lists, index maps . ``skelfmm/recursive_skel.py:622-780``
* apply ......................... ``skelfmm/batched_fmm.py:382-564`` (FP64 CPU)

The tree is an input (any object with the ``simpletree`` accessors); proxy
surfaces follow the framework's tree definition (restated below so the oracle
does not import product code).  The oracle is pinned against the reference's
own outputs by ``tests/test_oracle_golden.py``.
"""

from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
from scipy.linalg import qr, solve_triangular
from scipy.special import j0, y0

FOUR_PI_INV = 1.0 / (4.0 * np.pi)


# --------------------------------------------------------------- kernels
def _dist(XX, YY):
    diff = XX[:, None, :] - YY[None, :, :]
    d2 = np.einsum("ijk,ijk->ij", diff, diff)
    return diff, d2


def laplace_2d(XX, YY, param=0.0, not_self=False, **_):
    """log|x-y|; coincident pairs give 0 (util.py:128-149)."""
    _, d2 = _dist(XX, YY)
    r = np.sqrt(d2)
    if not not_self:
        r = np.where(d2 == 0, 1.0, r)
    return np.log(r)


def laplace_3d(XX, YY, param=0.0, not_self=False, **_):
    """1/|x-y|; coincident pairs give 0 (util.py:151-174)."""
    _, d2 = _dist(XX, YY)
    r = np.sqrt(d2)
    with np.errstate(divide="ignore"):
        out = 1.0 / r
    if not not_self:
        out[d2 == 0] = 0.0
    return out


def helmholtz_2d(XX, YY, param=0.0, not_self=False, **_):
    """J0(kr) + i Y0(kr); coincident pairs give 0 (util.py:176-202)."""
    _, d2 = _dist(XX, YY)
    r = np.sqrt(d2)
    zero = d2 == 0
    if not not_self:
        r = np.where(zero, 1.0, r)
    kr = param * r
    out = j0(kr) + 1j * y0(kr)
    if not not_self:
        out[zero] = 0.0
    return out


def helmholtz_3d(XX, YY, param=0.0, not_self=False, **_):
    """exp(i k r)/r; coincident pairs give 0 (util.py:204-232)."""
    _, d2 = _dist(XX, YY)
    r = np.sqrt(d2)
    zero = d2 == 0
    rr = np.where(zero, np.inf, r)
    out = np.exp(1j * param * r) / rr
    out[zero] = 0.0
    return out


def _dl_parts(XX, YY, geom, side):
    diff, d2 = _dist(XX, YY)
    d2 = np.where(d2 == 0, 1.0, d2)
    if side == "source":
        rotn = np.einsum("ijk,jk->ij", diff, geom)
    else:
        rotn = np.einsum("ijk,ik->ij", diff, geom)
    return rotn, d2


def laplace_3d_double_layer(XX, YY, param=0.0, src_geom=None, **_):
    """-(1/4pi) (x-y).n_y / r^3 (util.py:234-265)."""
    rotn, d2 = _dl_parts(XX, YY, src_geom, "source")
    return -FOUR_PI_INV * rotn / (d2 * np.sqrt(d2))


def laplace_3d_adjoint_double_layer(XX, YY, param=0.0, trg_geom=None, **_):
    """+(1/4pi) (x-y).n_x / r^3 (util.py:267-298)."""
    rotn, d2 = _dl_parts(XX, YY, trg_geom, "target")
    return FOUR_PI_INV * rotn / (d2 * np.sqrt(d2))


def helmholtz_3d_double_layer(XX, YY, param=0.0, src_geom=None, **_):
    """(1/4pi) (x-y).n_y e^{ikr}(ikr-1)/r^3 (util.py:301-338)."""
    rotn, d2 = _dl_parts(XX, YY, src_geom, "source")
    r = np.sqrt(d2)
    kr = param * r
    return FOUR_PI_INV * rotn * np.exp(1j * kr) * (1j * kr - 1.0) / (d2 * r)


def helmholtz_3d_adjoint_double_layer(XX, YY, param=0.0, trg_geom=None, **_):
    """-(1/4pi) (x-y).n_x e^{ikr}(ikr-1)/r^3 (util.py:341-377)."""
    rotn, d2 = _dl_parts(XX, YY, trg_geom, "target")
    r = np.sqrt(d2)
    kr = param * r
    return -FOUR_PI_INV * rotn * np.exp(1j * kr) * (1j * kr - 1.0) / (d2 * r)


class OracleOperator:
    """Restatement of the operator metadata (operators.py:17-216)."""

    def __init__(self, name, ndim, func, proxy_surface, geometry_side, is_symmetric, is_complex):
        self.name = name
        self.ndim = ndim
        self.func = func
        self.proxy_surface = proxy_surface
        self.geometry_side = geometry_side
        self.is_symmetric = is_symmetric
        self.is_complex = is_complex

    @property
    def requires_geometry(self):
        return self.geometry_side is not None

    def matrix(self, x_trg, x_src, geom_trg=None, geom_src=None, param=0.0, not_self=False):
        kw = {}
        if self.geometry_side == "source":
            kw["src_geom"] = geom_src
        elif self.geometry_side == "target":
            kw["trg_geom"] = geom_trg
        return self.func(x_trg, x_src, param=param, not_self=not_self, **kw)


OPERATORS = {
    "laplace_2d": OracleOperator("laplace_2d", 2, laplace_2d, "cube", None, True, False),
    "laplace_3d": OracleOperator("laplace_3d", 3, laplace_3d, "cube", None, True, False),
    "helmholtz_2d": OracleOperator("helmholtz_2d", 2, helmholtz_2d, "cube", None, True, True),
    "helmholtz_3d": OracleOperator("helmholtz_3d", 3, helmholtz_3d, "cube", None, True, True),
    "laplace_double_layer_3d": OracleOperator(
        "laplace_double_layer_3d", 3, laplace_3d_double_layer, "sphere", "source", False, False),
    "laplace_adjoint_double_layer_3d": OracleOperator(
        "laplace_adjoint_double_layer_3d", 3, laplace_3d_adjoint_double_layer, "sphere", "target", False, False),
    "helmholtz_double_layer_3d": OracleOperator(
        "helmholtz_double_layer_3d", 3, helmholtz_3d_double_layer, "sphere", "source", False, True),
    "helmholtz_adjoint_double_layer_3d": OracleOperator(
        "helmholtz_adjoint_double_layer_3d", 3, helmholtz_3d_adjoint_double_layer, "sphere", "target", False, True),
}


# --------------------------------------------------------------- proxy surfaces
def cube_surface(center, length, nproxy):
    """Proxy points on the square/cube boundary (framework tree definition)."""
    center = np.asarray(center, dtype=np.float64)
    h = 0.5 * float(length)
    if center.shape[0] == 2:
        n = max(1, int(np.ceil(nproxy / 4.0)))
        t = -h + float(length) * np.arange(n, dtype=np.float64) / n
        pts = np.concatenate((np.stack((t, np.full(n, -h)), 1), np.stack((np.full(n, h), t), 1),
                              np.stack((-t, np.full(n, h)), 1), np.stack((np.full(n, -h), -t), 1)), 0)
        return pts + center[None, :]
    n = max(1, int(np.ceil(np.sqrt(nproxy / 6.0))))
    s = -h + float(length) * (np.arange(n, dtype=np.float64) + 0.5) / n
    a, b = np.meshgrid(s, s, indexing="ij")
    a, b = a.ravel(), b.ravel()
    out = []
    for axis in range(3):
        o = [d for d in range(3) if d != axis]
        for sign in (-1.0, 1.0):
            f = np.empty((a.shape[0], 3))
            f[:, axis] = sign * h
            f[:, o[0]] = a
            f[:, o[1]] = b
            out.append(f)
    return np.concatenate(out, 0) + center[None, :]


def sphere_surface(center, length, npoints):
    """Proxy points on the circle/sphere of diameter ``length``."""
    center = np.asarray(center, dtype=np.float64)
    r = 0.5 * float(length)
    n = max(1, int(npoints))
    if center.shape[0] == 2:
        th = 2.0 * np.pi * np.arange(n, dtype=np.float64) / n
        return center[None, :] + r * np.stack((np.cos(th), np.sin(th)), 1)
    k = np.arange(n, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * k / n
    rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.pi * (3.0 - np.sqrt(5.0)) * k
    return center[None, :] + r * np.stack((rho * np.cos(phi), rho * np.sin(phi), z), 1)


def proxy_points(op, center, box_length, nproxy):
    """util.py:72-78: proxy surface of side 2.95 * box length."""
    L = 2.95 * box_length
    if op.proxy_surface == "cube":
        return cube_surface(center, L, nproxy)
    return sphere_surface(center, L, nproxy)


def stacked_proxy_matrix(op, x_box, center, box_length, nproxy, geom=None, param=0.0):
    """util.py:87-124."""
    xp = proxy_points(op, center, box_length, nproxy)
    if op.is_symmetric and geom is None:
        K_BP = op.matrix(x_box, xp, param=param, not_self=True)
        return np.vstack((K_BP.T, K_BP.T))
    normals = None
    if op.proxy_surface == "sphere":
        normals = xp - np.asarray(center)[None, :]
        normals = normals / np.linalg.norm(normals, axis=1, keepdims=True)
    src_geom = normals if op.geometry_side == "source" else None
    trg_geom = normals if op.geometry_side == "target" else None
    K_BP = op.matrix(x_box, xp, geom_trg=geom, geom_src=src_geom, param=param, not_self=True)
    K_PB = op.matrix(xp, x_box, geom_trg=trg_geom, geom_src=geom, param=param, not_self=True)
    return np.vstack((K_PB, K_BP.T))


def pivoted_qr_id(K, rank_or_eps):
    """util.py:13-51: column ID from LAPACK pivoted QR."""
    ncols = K.shape[1]
    R, piv = qr(K, mode="r", pivoting=True, overwrite_a=True, check_finite=False)
    R = np.asarray(R)[:ncols, :]
    if rank_or_eps < 1:
        d = np.abs(np.diag(R))
        rank = 0 if (d.size == 0 or d[0] == 0) else int(np.count_nonzero(d > rank_or_eps * d[0]))
    else:
        rank = int(rank_or_eps)
    rank = max(0, min(rank, ncols))
    idx = np.asarray(piv, dtype=np.int64)
    if rank == 0 or rank == ncols:
        proj = np.zeros((rank, ncols - rank), dtype=K.dtype)
    else:
        proj = solve_triangular(R[:rank, :rank], R[:rank, rank:], lower=False, check_finite=False)
    return rank, idx, proj


def skel_box(op, kappa, x_box, center, box_length, tol, nproxy, geom=None):
    """util.py:404-437."""
    K = stacked_proxy_matrix(op, x_box, center, box_length, nproxy, geom=geom, param=kappa)
    return pivoted_qr_id(K, tol)


def _skel_task(args):
    """Pool worker: one box's proxy ID (util.py:381-402), single-threaded BLAS."""
    opname, kappa, xb, c, len_l, tol, nproxy, gb = args
    try:
        from threadpoolctl import threadpool_limits
    except ImportError:  # pragma: no cover
        return skel_box(OPERATORS[opname], kappa, xb, c, len_l, tol, nproxy, geom=gb)
    with threadpool_limits(limits=1):
        return skel_box(OPERATORS[opname], kappa, xb, c, len_l, tol, nproxy, geom=gb)


def translation_sample(op_name, kappa, entry_xyz, entry_geom, box_off, box_rank, list_off, list_src,
                       list_kind, q, qh, boxes, nthreads=None):
    """Dense CPU translations (FP64, kernel blocks materialised as the
    reference's batched path does, batched_fmm.py:180-302) into the target
    boxes ``boxes`` of a ragged build.  Returns (u, uh, pair evaluations)
    per box; used to time the reference algorithm on a bounded sample."""
    op = OPERATORS[op_name]

    def one(U):
        oU, eU = int(box_off[U]), int(box_off[U + 1])
        rU = int(box_rank[U])
        XU = entry_xyz[oU:eU]
        GU = None if entry_geom is None else entry_geom[oU:eU]
        au = np.zeros(eU - oU, q.dtype)
        ah = np.zeros(eU - oU, q.dtype)
        npairs = 0
        for l in range(int(list_off[U]), int(list_off[U + 1])):
            s, kind = int(list_src[l]), int(list_kind[l])
            oS, eS = int(box_off[s]), int(box_off[s + 1])
            rS = int(box_rank[s])
            GS = None if entry_geom is None else entry_geom[oS:eS]
            K = op.matrix(XU, entry_xyz[oS:eS], geom_trg=GU, geom_src=GS, param=kappa)
            if U == s:
                np.fill_diagonal(K, 0.0)
            npairs += K.size
            au += K @ q[oS:eS]
            if kind == 0:
                ah[:rU] -= K[:rU, :rS] @ qh[oS:oS + rS]
            elif kind == 1:
                ah[:rU] -= K[:rU] @ q[oS:eS]
            elif kind == 2:
                au -= K[:, :rS] @ qh[oS:oS + rS]
        return au, ah, npairs

    with ThreadPoolExecutor(nthreads or max(1, os.cpu_count() or 1)) as ex:
        return list(ex.map(one, list(boxes)))


def nproxy_levels(ndim, tol, kappa, L0, nlevels):
    """recursive_skel.py:72-85."""
    ndigits = int(-np.log10(tol / 100))
    out = np.zeros(nlevels, dtype=int)
    for lev in range(nlevels):
        box_length = L0 * 2 ** (-lev)
        if ndim == 2:
            nproxy = int(ndigits * 10)
            nproxy += int(4 * kappa * box_length)
        else:
            nproxy = np.max(np.array([int(ndigits ** 2 * 8), 400]))
            nproxy += 2 * kappa * box_length * np.max(np.array([5, ndigits - 1])) + (10 if kappa > 0 else 0)
        out[lev] = nproxy
    return out


# --------------------------------------------------------------- build
class OracleBuild:
    """Restatement of ``RecursiveSkeletonization`` (recursive_skel.py), with the
    reference's padded storage layout.  Additionally tracks, per box, the
    original point index of every entry (``pid_list``)."""

    def __init__(self, tree, op, kappa, tol, geometry=None):
        self.tree = tree
        self.op = op
        self.kappa = float(kappa)
        self.tol = tol
        self.N = tree.N
        self.ndim = tree.ndim
        self.nlevels = tree.nlevels
        self.nboxes = tree.nboxes
        self.geometry = geometry
        if op.ndim != self.ndim:
            raise ValueError("Operator dimensionality does not match the tree dimensionality")
        if op.requires_geometry and geometry is None:
            raise ValueError("Geometry is required for this operator")

        leaves = tree.get_leaves()
        tb, sep = [], [0]
        for lev in range(self.nlevels):
            b = tree.get_boxes_level(lev)
            t = np.setdiff1d(b, leaves)
            tb.append(t)
            sep.append(sep[-1] + t.shape[0])
        self.tree_boxes = np.concatenate(tb).astype(int) if tb else np.zeros(0, int)
        self.tree_lev_sep = np.array(sep, dtype=int)
        self.nproxy_level = nproxy_levels(self.ndim, tol, self.kappa, tree.L0, self.nlevels)

        self.max_bs_leaf = tree.leaf_size
        self.bs_list = np.zeros(self.nboxes, dtype=int)
        self.rank_list = np.zeros(self.nboxes, dtype=int)
        self.pid = [None] * self.nboxes   # original point ids, current order
        self.proj = [None] * self.nboxes  # T = R11^{-1} R12, shape (rank, bs-rank)
        for leaf in leaves:
            inds = tree.get_box_inds(leaf).copy()
            if inds.shape[0] > self.max_bs_leaf:
                raise ValueError("Leaf block size exceeds maximum allowed")
            self.pid[leaf] = inds
            self.bs_list[leaf] = inds.shape[0]

    def _update_lev_skel(self, lev):
        """recursive_skel.py:209-262 (storage growth omitted: layout only)."""
        for box in self.tree.get_boxes_level(lev):
            if self.tree.is_leaf(box):
                continue
            parts = [self.pid[c][: self.rank_list[c]] for c in self.tree.get_box_children(box)]
            self.pid[box] = np.concatenate(parts) if parts else np.zeros(0, int)
            self.bs_list[box] = self.pid[box].shape[0]

    def skel_tree(self, npoints_max, pool=None):
        """recursive_skel.py:326-502.  ``pool``: an optional process pool
        (``multiprocessing`` spawn context, as the reference's ``p="auto"``)
        that takes the boxes of a level; otherwise serial."""
        tree = self.tree
        self.root_level = max(0, tree.nlevels - 1)
        for lev in range(tree.nlevels - 1, 0, -1):
            self._update_lev_skel(lev)
            boxes_lev = tree.get_boxes_level(lev)
            active = np.hstack((tree.get_leaves_above(lev), boxes_lev)).astype(int)
            if lev == 2 or np.sum(self.bs_list[active]) <= npoints_max:
                self.root_level = lev
                break
            len_l = tree.get_box_length(boxes_lev[0])
            centers = tree.get_boxes_centers(boxes_lev)
            nproxy = int(self.nproxy_level[lev])
            tasks = []
            for box, c in zip(boxes_lev, centers):
                ids = self.pid[box]
                gb = None if self.geometry is None else self.geometry[ids]
                tasks.append((self.op.name, self.kappa, tree.XX[ids], c, len_l, self.tol, nproxy, gb))
            if pool is None:
                results = map(_skel_task, tasks)
            else:
                results = pool.imap(_skel_task, tasks, chunksize=max(1, len(tasks) // 64))
            for box, (rank, idx, proj) in zip(boxes_lev, results):
                self.rank_list[box] = rank
                self.pid[box] = self.pid[box][idx]
                self.proj[box] = proj
        self._finish()
        return self

    def _finish(self):
        """prune_skel (recursive_skel.py:515-539) + lists + index maps."""
        tree = self.tree
        leaves = tree.get_leaves()
        self.max_bs = int(np.max(self.bs_list))
        self.max_rank = int(np.max(self.rank_list))
        pos = self.rank_list[self.rank_list > 0]
        self.min_rank = int(np.min(pos)) if pos.size else 0
        self.max_bs_leaf = int(np.max(self.bs_list[leaves]))
        self.max_rank_leaf = int(np.max(self.rank_list[leaves]))
        self._parallel_lists()
        self._precompute_inds()

    # padded views in the reference's layout (recursive_skel.py:106-120, 533-539)
    def XX_list(self):
        out = np.zeros((self.nboxes, self.max_bs, self.ndim))
        for b in range(self.nboxes):
            if self.pid[b] is not None and self.bs_list[b] > 0:
                out[b, : self.bs_list[b]] = self.tree.XX[self.pid[b]]
        return out

    def proj_lists(self):
        dt = np.complex128 if self.op.is_complex else np.float64
        leaves = set(self.tree.get_leaves().tolist())
        pl = np.zeros((self.nboxes, self.max_rank_leaf, max(self.max_bs_leaf - self.min_rank, 0)), dt)
        pt = np.zeros((self.tree_boxes.shape[0], self.max_rank, max(self.max_bs - self.min_rank, 0)), dt)
        for b in range(self.nboxes):
            P = self.proj[b]
            if P is None:
                continue
            r, bs = self.rank_list[b], self.bs_list[b]
            if b in leaves:
                pl[b, :r, r - self.min_rank: bs - self.min_rank] = P
            else:
                i = int(np.searchsorted(self.tree_boxes, b))
                pt[i, :r, r - self.min_rank: bs - self.min_rank] = P
        return pl, pt

    def _parallel_lists(self):
        """recursive_skel.py:622-712."""
        tree = self.tree
        leaf_mask = tree.are_leaves(np.arange(tree.nboxes))
        leaf_coll, tree_coll, coarse_up = [], [], []
        for lev in range(self.root_level + 1, self.nlevels):
            boxes = tree.get_boxes_level(lev)
            crow = tree.get_boxes_colleague_neigh_fullvec(boxes)
            krow = tree.get_boxes_coarse_neigh_fullvec(boxes)
            for box, coll, coarse in zip(boxes, crow, krow):
                coll = coll[coll >= 0]
                if coll.size:
                    if leaf_mask[box]:
                        m = leaf_mask[coll]
                        leaf_coll += [(box, c) for c in coll[m]]
                        tree_coll += [(box, c) for c in coll[~m]]
                    else:
                        tree_coll += [(box, c) for c in coll]
                coarse = coarse[coarse >= 0]
                coarse_up += [(box, c) for c in coarse]
        as2 = lambda L: np.array(L, dtype=int).reshape(-1, 2)  # noqa: E731
        self.leaf_uskel_from_qskel_list = as2(leaf_coll)
        self.tree_uskel_from_qskel_list = as2(tree_coll)
        self.uskel_from_q_list = as2(coarse_up)
        self.u_from_qskel_list = self.uskel_from_q_list[:, ::-1].copy()
        lev_boxes = tree.get_boxes_level(self.root_level)
        self.root_boxes = np.hstack((tree.get_leaves_above(self.root_level), lev_boxes)).astype(int)
        self.skel_leaves = np.setdiff1d(tree.get_leaves(), tree.get_leaves_above(self.root_level + 1))
        rb = self.root_boxes
        self.u_from_q_list = np.stack((np.repeat(rb, rb.shape[0]), np.tile(rb, rb.shape[0])), 1)

    def _precompute_inds(self):
        """recursive_skel.py:714-780."""
        tree = self.tree
        mb = self.max_bs
        short, long_ = [], []
        for leaf in tree.get_leaves():
            bs = int(self.bs_list[leaf])
            short.append(np.arange(bs) + leaf * mb)
            long_.append(self.pid[leaf])
        self.short_vec_inds = np.concatenate(short).astype(int)
        self.long_vec_inds = np.concatenate(long_).astype(int)

        leaf_mask = tree.are_leaves(np.arange(self.nboxes))
        off = np.zeros(self.nlevels + 1, dtype=int)
        bsk, csk = [], []
        acc_total = 0
        for lev in range(self.root_level, self.nlevels):
            boxes = tree.get_boxes_level(lev)
            tboxes = boxes[~leaf_mask[boxes]]
            for box, row in zip(tboxes, tree.get_boxes_children_fullvec(tboxes)):
                bs = int(self.bs_list[box])
                cand = np.concatenate([self.pid[c][: self.rank_list[c]] for c in row if c >= 0])
                # position of candidate k in the box's permuted order
                order = np.empty(bs, dtype=int)
                if lev == self.root_level:
                    order[:] = np.arange(bs)
                else:
                    pos = {int(p): i for i, p in enumerate(self.pid[box].tolist())}
                    order[:] = [pos[int(p)] for p in cand.tolist()]
                acc = 0
                for c in row:
                    if c < 0:
                        continue
                    rc = int(self.rank_list[c])
                    bsk.append(order[acc: acc + rc] + box * mb)
                    csk.append(np.arange(rc) + c * mb)
                    acc += rc
                    acc_total += rc
            off[lev + 1] = acc_total
        self.box_skel_inds = np.concatenate(bsk).astype(int) if bsk else np.zeros(0, int)
        self.child_skel_inds = np.concatenate(csk).astype(int) if csk else np.zeros(0, int)
        self.inds_lev_offset = off


# --------------------------------------------------------------- apply
class OracleApply:
    """FP64 CPU apply restating ``SkelFMMBatched.matvec`` (batched_fmm.py:382-564).

    Kernel blocks are materialised per target box over all of its source boxes
    (the same work the reference does in pair chunks); ``nthreads`` host threads
    share the target boxes.
    """

    def __init__(self, build: OracleBuild, nthreads=None):
        self.b = build
        self.nthreads = nthreads or max(1, os.cpu_count() or 1)
        b = build
        self.leaf_mask = b.tree.are_leaves(np.arange(b.nboxes))
        self.dtype = np.complex128 if b.op.is_complex else np.float64
        self.X = [None if p is None else b.tree.XX[p] for p in b.pid]
        self.G = [None if (p is None or b.geometry is None) else b.geometry[p] for p in b.pid]
        # per target box: list of (source box, kind); kinds: 0 colleague, 1 coarse-up,
        # 2 coarse-down, 3 root dense
        work = {}
        for u, q in np.vstack((b.leaf_uskel_from_qskel_list, b.tree_uskel_from_qskel_list)):
            work.setdefault(int(u), []).append((int(q), 0))
        for u, q in b.uskel_from_q_list:
            work.setdefault(int(u), []).append((int(q), 1))
        for u, q in b.u_from_qskel_list:
            work.setdefault(int(u), []).append((int(q), 2))
        for u, q in b.u_from_q_list:
            work.setdefault(int(u), []).append((int(q), 3))
        self.work = work

    def _K(self, u, q, ru=None, rq=None):
        b = self.b
        XU = self.X[u] if ru is None else self.X[u][:ru]
        XQ = self.X[q] if rq is None else self.X[q][:rq]
        GU = None if self.G[u] is None else (self.G[u] if ru is None else self.G[u][:ru])
        GQ = None if self.G[q] is None else (self.G[q] if rq is None else self.G[q][:rq])
        K = b.op.matrix(XU, XQ, geom_trg=GU, geom_src=GQ, param=b.kappa, not_self=False)
        if u == q:
            n = min(K.shape)
            K[np.arange(n), np.arange(n)] = 0.0
        return K

    def upward(self, x):
        b = self.b
        q = [np.zeros(int(s), self.dtype) for s in b.bs_list]
        for leaf in b.tree.get_leaves():
            q[leaf][:] = x[b.pid[leaf]]
        qh = [v.copy() for v in q]
        for lev in range(b.nlevels - 1, b.root_level, -1):
            boxes = b.tree.get_boxes_level(lev)
            for box in boxes:
                r = int(b.rank_list[box])
                qh[box] = q[box].copy()
                if b.proj[box] is not None and r > 0:
                    qh[box][:r] = q[box][:r] + b.proj[box] @ q[box][r:]
            # children skeletons -> parent entries (addto_skel_lev, upward)
            for box in b.tree.get_boxes_level(lev - 1):
                if self.leaf_mask[box]:
                    continue
                parts = [qh[c][: b.rank_list[c]] for c in b.tree.get_box_children(box)]
                cand = np.concatenate(parts)
                order = self._order(box, lev - 1)
                q[box][order] = cand
        return q, qh

    def _order(self, box, lev):
        b = self.b
        if not hasattr(self, "_orders"):
            self._orders = {}
        if box not in self._orders:
            cand = np.concatenate([b.pid[c][: b.rank_list[c]] for c in b.tree.get_box_children(box)])
            if lev == b.root_level:
                self._orders[box] = np.arange(cand.shape[0])
            else:
                pos = {int(p): i for i, p in enumerate(b.pid[box].tolist())}
                self._orders[box] = np.array([pos[int(p)] for p in cand.tolist()], dtype=int)
        return self._orders[box]

    def translate_box(self, u, q, qh):
        """All translations into target box u (addto_uvec + subtract_from_uskel)."""
        b = self.b
        bu, ru = int(b.bs_list[u]), int(b.rank_list[u])
        acc_u = np.zeros(bu, self.dtype)
        acc_h = np.zeros(bu, self.dtype)
        for s, kind in self.work.get(u, ()):
            rs = int(b.rank_list[s])
            K = self._K(u, s)
            acc_u += K @ q[s]
            if kind == 0:
                acc_h[:ru] -= K[:ru, :rs] @ qh[s][:rs]
            elif kind == 1:
                acc_h[:ru] -= K[:ru] @ q[s]
            elif kind == 2:
                acc_u -= K[:, :rs] @ qh[s][:rs]
        return acc_u, acc_h

    def work_items(self):
        """Every kernel block of one apply as (target, source, kind, evaluations)."""
        b = self.b
        return [(u, s, kind, int(b.bs_list[u]) * int(b.bs_list[s]))
                for u, lst in self.work.items() for s, kind in lst]

    def translate_items(self, items, q, qh):
        """The kernel blocks ``items`` (target, source, kind, ...) of one apply
        with translate_box's arithmetic, spread over the host threads; returns
        the kernel evaluations done.  Used to time a bounded sample of the
        apply (the products are computed and dropped)."""
        b = self.b

        def one(it):
            u, s, kind = int(it[0]), int(it[1]), int(it[2])
            ru, rs = int(b.rank_list[u]), int(b.rank_list[s])
            K = self._K(u, s)
            acc_u = K @ q[s]
            if kind == 0:
                acc_h = -(K[:ru, :rs] @ qh[s][:rs])
            elif kind == 1:
                acc_h = -(K[:ru] @ q[s])
            elif kind == 2:
                acc_u = acc_u - K[:, :rs] @ qh[s][:rs]
                acc_h = None
            else:
                acc_h = None
            del acc_u, acc_h
            return K.size

        with ThreadPoolExecutor(self.nthreads) as ex:
            return int(sum(ex.map(one, list(items))))

    def translations(self, q, qh, boxes=None):
        b = self.b
        boxes = list(self.work.keys()) if boxes is None else list(boxes)
        u = [np.zeros(int(s), self.dtype) for s in b.bs_list]
        uh = [np.zeros(int(s), self.dtype) for s in b.bs_list]
        with ThreadPoolExecutor(self.nthreads) as ex:
            for box, (a, h) in zip(boxes, ex.map(lambda t: self.translate_box(t, q, qh), boxes)):
                u[box] = a
                uh[box] = h
        return u, uh

    def downward(self, u, uh, x_shape):
        b = self.b
        for lev in range(b.root_level, b.nlevels):
            boxes = b.tree.get_boxes_level(lev)
            if lev > b.root_level:
                for box in b.tree.get_boxes_level(lev - 1):
                    if self.leaf_mask[box]:
                        continue
                    order = self._order(box, lev - 1)
                    vals = u[box][order]
                    acc = 0
                    for c in b.tree.get_box_children(box):
                        rc = int(b.rank_list[c])
                        uh[c][:rc] += vals[acc: acc + rc]
                        acc += rc
            for box in boxes:
                r = int(b.rank_list[box])
                if lev > b.root_level and r > 0 and b.proj[box] is not None:
                    u[box][:r] += uh[box][:r]
                    u[box][r:] += b.proj[box].T @ uh[box][:r]
        y = np.zeros(x_shape, self.dtype)
        for leaf in b.tree.get_leaves():
            y[b.pid[leaf]] = u[leaf]
        return y

    def matvec(self, x):
        x = np.asarray(x)
        x = x.astype(self.dtype) if self.b.op.is_complex or not np.iscomplexobj(x) else x
        q, qh = self.upward(x)
        u, uh = self.translations(q, qh)
        return self.downward(u, uh, x.shape)


def dense_apply(op, points, x, idx, geometry=None, kappa=0.0):
    """FP64 direct sum on targets ``idx`` (skel_fmm.py:218-257)."""
    gs = geometry if op.geometry_side == "source" else None
    gt = geometry[idx] if op.geometry_side == "target" else None
    out = []
    for s in range(0, len(idx), 256):
        t = idx[s: s + 256]
        gtt = None if gt is None else gt[s: s + 256]
        out.append(op.matrix(points[t], points, geom_trg=gtt, geom_src=gs, param=kappa) @ x)
    return np.concatenate(out)
