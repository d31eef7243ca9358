"""Many independent FMM instances applied as one operator.

Instances (uneven sizes, adaptive trees, different skeleton ranks) are built
separately and then concatenated into a single ragged plan: boxes, entries,
interaction lists and interpolation blocks of all instances live in one CSR
layout, so one apply runs every phase (permute, upward T per level, the
translations of all levels, downward T^T, permute) for all instances with a
single launch per phase.  Levels are aligned at each instance's root level.
The apply can be captured once into a CUDA graph and replayed.

An autotuner picks, per plan, the translation scheme (symmetric or
per-direction) and the packed kernel's block shape by timing them.
"""

from __future__ import annotations

import ctypes
from time import perf_counter

import numpy as np
import torch

from . import _lib
from .operators import is_complex_op
from .plan import Plan, RaggedBuild
from .recursive_skel import RecursiveSkeletonization
from .skel_fmm import direct_sum
from .tree import BalancedTree


def concat_ragged(rbs):
    """One ragged build holding every instance; instance i's points occupy
    rows [starts[i], starts[i+1]) of the concatenated input vector."""
    op = rbs[0].op
    if any(rb.op != op or rb.ndim != rbs[0].ndim or rb.kappa != rbs[0].kappa for rb in rbs):
        raise ValueError("instances must share the operator, dimension and kappa")
    R = max(rb.root_level for rb in rbs)
    nlev = max(rb.nlevels - rb.root_level for rb in rbs) + R
    box_level, box_rank, box_off = [], [], [np.zeros(1, np.int64)]
    xyz, geom, pslot, pe, pp, t_off, t_data = [], [], [], [], [], [], []
    list_off, list_src, list_kind = [np.zeros(1, np.int64)], [], []
    eoff = boff = poff = toff = loff = 0
    starts = [0]
    for rb in rbs:
        nb = rb.nboxes
        box_level.append(np.maximum(rb.box_level.astype(np.int64) - rb.root_level + R, 0).astype(np.int32))
        box_rank.append(rb.box_rank)
        box_off.append(rb.box_off[1:] + eoff)
        xyz.append(rb.entry_xyz)
        if rb.entry_geom is not None:
            geom.append(rb.entry_geom)
        pslot.append(np.where(rb.entry_pslot >= 0, rb.entry_pslot + eoff, -1))
        pe.append(rb.perm_entry + eoff)
        pp.append(rb.perm_point + poff)
        t_off.append(np.where(rb.t_off >= 0, rb.t_off + toff, -1))
        t_data.append(rb.t_data)
        list_off.append(rb.list_off[1:] + loff)
        list_src.append(rb.list_src.astype(np.int64) + boff)
        list_kind.append(rb.list_kind)
        eoff += rb.nentries
        boff += nb
        poff += rb.npoints
        toff += int(rb.t_data.shape[0])
        loff += int(rb.list_off[-1])
        starts.append(poff)
    def cat(parts):
        # device parts stay on the device
        if not any(isinstance(a, torch.Tensor) for a in parts):
            return np.concatenate(parts)
        dev = next(a.device for a in parts if isinstance(a, torch.Tensor))
        return torch.cat([a if isinstance(a, torch.Tensor) else torch.from_numpy(np.asarray(a)).to(dev)
                          for a in parts])

    out = RaggedBuild(
        op=op, ndim=rbs[0].ndim, kappa=rbs[0].kappa, npoints=int(poff), nlevels=int(nlev), root_level=int(R),
        box_level=np.concatenate(box_level), box_off=np.concatenate(box_off), box_rank=np.concatenate(box_rank),
        entry_xyz=cat(xyz), entry_geom=cat(geom) if geom else None,
        entry_pslot=np.concatenate(pslot), perm_entry=np.concatenate(pe), perm_point=np.concatenate(pp),
        t_off=np.concatenate(t_off), t_data=None, list_off=np.concatenate(list_off),
        list_src=np.concatenate(list_src).astype(np.int32), list_kind=np.concatenate(list_kind),
    )
    out.t_data = cat(t_data)
    return out, np.asarray(starts, dtype=np.int64)


def skel_trees_lockstep(fmms, npoints_max):
    """``skel_tree(npoints_max)`` of every instance, level by level in step:
    step k skeletonizes level nlevels_i - 1 - k of each instance i still
    below its root, all of them (grouped by proxy count) in one
    ``skf_skel_boxes_multi`` launch, each box with its own tree's proxy
    surface.  The IDs are those of the per-instance level loop
    (skelfmm/recursive_skel.py:370-498 per instance); only the launches are
    shared.  Instances with a rank predictor are not supported."""
    if not fmms:
        return fmms
    if any(f.rank_predictor is not None for f in fmms):
        raise ValueError("the lockstep build runs the pivoted-QR IDs only")
    f0 = fmms[0]
    if any(f.op_id != f0.op_id or f.kappa != f0.kappa or f.tol != f0.tol or f.device != f0.device for f in fmms):
        raise ValueError("instances must share the operator, kappa, tolerance and device")
    dev = f0.device
    lib = _lib.load()
    tdt = torch.complex128 if is_complex_op(f0.op_id) else torch.float64
    lev = {}
    for i, f in enumerate(fmms):
        f.root_level = max(0, f.tree.nlevels - 1)
        if f.tree.nlevels - 1 >= 1:
            lev[i] = f.tree.nlevels - 1
    while lev:
        groups = {}
        for i in list(lev):
            f, lv = fmms[i], lev[i]
            if f._is_root_level(lv, npoints_max):
                del lev[i]
                continue
            inp = f._level_inputs(lv)
            groups.setdefault(inp["nproxy"], []).append((i, inp))
        for nproxy, members in groups.items():
            nb = [m[1]["nbl"] for m in members]
            ne = [int(m[1]["off"][-1]) for m in members]
            nt = [int(m[1]["cap"].sum()) for m in members]
            b0 = np.concatenate(([0], np.cumsum(nb)))
            e0 = np.concatenate(([0], np.cumsum(ne)))
            t0 = np.concatenate(([0], np.cumsum(nt)))
            off = np.concatenate([[0]] + [m[1]["off"][1:] + e0[k] for k, m in enumerate(members)]).astype(np.int64)
            t_off = np.concatenate([m[1]["t_off"] + t0[k] for k, m in enumerate(members)]).astype(np.int64)
            lens = np.concatenate([np.full(m[1]["nbl"], m[1]["length"]) for m in members])
            centers = np.concatenate([m[1]["centers"] for m in members])
            x = torch.cat([m[1]["x"] for m in members])
            g = torch.cat([m[1]["g"] for m in members]) if members[0][1]["g"] is not None else None
            t_buf = torch.zeros(max(int(t0[-1]), 1), dtype=tdt, device=dev)
            rank = torch.zeros(int(b0[-1]), dtype=torch.int32, device=dev)
            perm = torch.zeros(max(int(e0[-1]), 1), dtype=torch.int32, device=dev)
            off_t = torch.from_numpy(off).to(dev)
            t_off_t = torch.from_numpy(t_off).to(dev)
            lens_t = torch.from_numpy(lens).to(dev)
            cen_t = torch.from_numpy(np.ascontiguousarray(centers)).to(dev)
            stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            _lib.check(lib.skf_skel_boxes_multi(
                f0.op_id, f0.kappa, int(b0[-1]), _lib.ptr(off_t), _lib.ptr(x), _lib.ptr(g), _lib.ptr(cen_t),
                _lib.ptr(lens_t), int(nproxy), float(f0.tol), _lib.ptr(rank), _lib.ptr(perm), _lib.ptr(t_off_t),
                _lib.ptr(t_buf), stream), "skf_skel_boxes_multi")
            rank_h = rank.cpu().numpy()
            perm_h = perm.cpu().numpy()
            for k, (i, inp) in enumerate(members):
                f = fmms[i]
                f.level_stats[inp["lev"]] = {"boxes": inp["nbl"], "randomized": 0, "kept": 0, "fallback": 0,
                                             "launch_boxes": int(b0[-1])}
                f._level_finish(inp, rank_h[b0[k]:b0[k + 1]], perm_h[e0[k]:e0[k + 1]],
                                t_buf[int(t0[k]):int(t0[k + 1])])
                lev[i] -= 1
                if lev[i] < 1:
                    del lev[i]
    _lib.check(lib.skf_trim_workspace(), "skf_trim_workspace")
    for f in fmms:
        f._entries_above_root()
    return fmms


def autotune(plan: Plan, precision=_lib.PREC_MIXED, reps=3):
    """Time the translation schemes this plan supports and keep the fastest
    (``Plan.autotune``).  Returns {setting: ms}."""
    return plan.autotune(precision, reps)


class SkelFMMBatch:
    """Independent instances (points_i, same operator) applied together.

    ``apply(xs)`` takes a list of charge vectors (or one concatenated vector)
    and returns the list of potentials.  The instances' IDs run level by
    level in step, one launch per level for all of them (``lockstep=False``:
    one instance after another).  ``capture()`` records the device
    apply into a CUDA graph for the given precision; later applies replay it.
    """

    def __init__(self, point_sets, operator, tol=1e-6, leaf_size=128, param=0.0, geometries=None,
                 npoints_max=500, precision="mixed", tune=True, lockstep=True):
        self.operator = operator
        self.param = param
        self.precision = precision
        self.point_sets = [np.asarray(p, dtype=np.float64) for p in point_sets]
        self.geometries = geometries
        self.sizes = [int(p.shape[0]) for p in point_sets]
        ph = {}
        t = perf_counter()

        def lap(name):
            nonlocal t
            torch.cuda.synchronize()
            now = perf_counter()
            ph[name] = now - t
            t = now

        trees = [BalancedTree(pts, leaf_size, device="cuda") for pts in self.point_sets]
        lap("trees")
        fmms = [RecursiveSkeletonization(tree, operator, param, tol,
                                         geometry=None if geometries is None else geometries[i])
                for i, tree in enumerate(trees)]
        if lockstep:
            skel_trees_lockstep(fmms, npoints_max)
        else:
            for fmm in fmms:
                fmm.skel_tree(npoints_max=npoints_max)
        lap("ids")
        rbs = []
        for fmm in fmms:
            fmm.setup_lists()
            rbs.append(fmm.ragged())
        self.instance_ragged = rbs
        self.ragged, self.starts = concat_ragged(rbs)
        lap("lists")
        self.plan = Plan(self.ragged)
        lap("plan")
        self.N = int(self.starts[-1])
        self.cplx = is_complex_op(operator)
        self._prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
        self.tuning = autotune(self.plan, self._prec) if (tune and self._prec != _lib.PREC_FP64) else None
        lap("autotune")
        # build phases (s): device trees, lockstep IDs, lists + concatenation,
        # plan creation, autotuning
        self.build_phases_seconds = ph
        dt = torch.complex128 if self.cplx else torch.float64
        self._x = torch.zeros(self.N, dtype=dt, device="cuda")
        self._y = torch.zeros(self.N, dtype=dt, device="cuda")
        self._graph = None

    def capture(self):
        """Record one device apply (on the internal buffers) into a CUDA graph."""
        self.plan.apply_device(self._x, self._y, self._prec)  # warm-up outside capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        with torch.cuda.graph(g, stream=s):
            self.plan.apply_device(self._x, self._y, self._prec, torch.cuda.current_stream().cuda_stream)
        self._graph = g
        return g

    def apply_device(self, x=None):
        """Apply to the concatenated device vector ``x`` (or the internal buffer)."""
        if x is not None:
            self._x.copy_(x)
        if self._graph is not None:
            self._graph.replay()
        else:
            self.plan.apply_device(self._x, self._y, self._prec,
                                   torch.cuda.current_stream().cuda_stream)
        return self._y

    def apply(self, xs):
        """Potentials of every instance; ``xs`` is a list of per-instance charge
        vectors (float32/float64/complex) or one concatenated vector."""
        x = np.concatenate([np.asarray(v) for v in xs]) if isinstance(xs, (list, tuple)) else np.asarray(xs)
        if x.shape[0] != self.N:
            raise ValueError("charge vectors must match the instances' sizes")
        self._x.copy_(torch.from_numpy(np.ascontiguousarray(x, dtype=np.complex128 if self.cplx else np.float64)))
        y = self.apply_device().cpu().numpy()
        return [y[self.starts[i]:self.starts[i + 1]] for i in range(len(self.sizes))]

    def direct_apply(self, i, x, indices):
        """FP64 direct sum of instance ``i`` at ``indices`` (its own points)."""
        return direct_sum(self.operator, self.point_sets[i], x, indices, param=self.param,
                          geometry=None if self.geometries is None else self.geometries[i])

    def relerr(self, xs, ys, ncheck=200, seed=0):
        """Per-instance relative l-inf error of ``ys`` against the FP64 direct
        sum on ``ncheck`` sampled targets of each instance."""
        rng = np.random.default_rng(seed)
        errs = []
        for i, (x, y) in enumerate(zip(xs, ys)):
            idx = rng.choice(self.sizes[i], size=min(ncheck, self.sizes[i]), replace=False)
            yd = self.direct_apply(i, np.asarray(x, dtype=np.complex128 if self.cplx else np.float64), idx)
            errs.append(float(np.abs(y[idx] - yd).max() / max(np.abs(yd).max(), 1e-300)))
        return np.asarray(errs)
