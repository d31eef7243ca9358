"""Public fast-apply object (drop-in for ``skelfmm.SkelFMM``, skelfmm/skel_fmm.py:55-282).

Same constructor arguments, ``build()``, ``apply(x)``, ``matvec``,
``relerr_fmm_apply_check`` and ``benchmark_matvec``.  The build runs the
proxy IDs on the GPU; the apply runs entirely on the GPU:

* ``use_single_precision=False`` (default) -> the plain FP64 apply;
* ``use_single_precision=True`` -> the mixed apply (FP32 kernel evaluation
  with FP64 accumulation, FP32 interpolation matrices).

``precision="fp64"|"mixed"`` selects the same explicitly.
"""

from __future__ import annotations

import contextlib
import io
from time import perf_counter

import numpy as np
import torch

from . import _lib
from .operators import _require_operator, cuda_op_id, is_complex_op
from .plan import Plan, load_ragged, save_ragged
from .recursive_skel import RecursiveSkeletonization
from .tree import BalancedTree


def warmup_cuda_fmm_apply(apply, x):
    """Run one apply so later timings exclude first-call costs (skel_fmm.py:38-52)."""
    device = getattr(apply, "device", None)
    if not (isinstance(device, torch.device) and device.type == "cuda"):
        return False
    apply.apply(x)
    torch.cuda.synchronize(device)
    return True


def direct_sum(operator, points, x, indices, *, param=0.0, geometry=None, device=None):
    """FP64 direct sum ``(K x)[indices]`` over all ``points`` on the GPU.

    The kernel is evaluated on the fly (``skf_kernel_apply``); a coincident
    pair contributes 0, as in the dense kernels.
    """
    from .kernels import batched_kernel_apply

    dev = torch.device("cuda") if device is None else device
    points = np.asarray(points, dtype=np.float64)
    idx = np.asarray(indices, dtype=np.int64)
    cplx = is_complex_op(operator)
    n = points.shape[0]
    # sources split into chunks, one batched "pair" per chunk, so the sum
    # spreads over the whole GPU; partial sums are added in FP64
    nchunk = max(1, min(1024, n // 4096))
    csz = -(-n // nchunk)
    pad = nchunk * csz - n
    pts = np.concatenate((points, np.zeros((pad, points.shape[1]))))
    xv = np.concatenate((np.asarray(x, dtype=np.complex128 if cplx else np.float64),
                         np.zeros(pad, dtype=np.complex128 if cplx else np.float64)))
    src = torch.from_numpy(pts.reshape(nchunk, csz, -1)).to(dev)
    xq = torch.from_numpy(xv.reshape(nchunk, csz, 1)).to(dev)
    ncnt = torch.full((nchunk,), csz, dtype=torch.int32, device=dev)
    ncnt[-1] = csz - pad
    gs = None
    if operator.geometry_side == "source":
        g = np.concatenate((geometry, np.zeros((pad, 3))))
        gs = torch.from_numpy(np.ascontiguousarray(g, dtype=np.float64).reshape(nchunk, csz, 3)).to(dev)
    out = []
    for s in range(0, idx.shape[0], 2048):
        t = idx[s: s + 2048]
        trg = torch.from_numpy(np.ascontiguousarray(points[t])).to(dev).unsqueeze(0).expand(nchunk, -1, -1)
        gtt = None
        if operator.geometry_side == "target":
            gtt = torch.from_numpy(np.ascontiguousarray(geometry[t], dtype=np.float64)).to(dev)
            gtt = gtt.unsqueeze(0).expand(nchunk, -1, -1)
        part = batched_kernel_apply(cuda_op_id(operator), xq, trg, src, param=param, geom_trg=gtt,
                                    geom_src=gs, n=ncnt)
        out.append(part.sum(dim=0)[:, 0].cpu().numpy())
    return np.concatenate(out)


class SkelFMM:
    """Build and apply a fast operator on one GPU."""

    def __init__(self, points, operator, geometry=None, tol=1e-5, rank_or_tol=None, leaf_size=200,
                 use_single_precision=False, param=0.0, quiet=True, keep_host_fmm=False, defer_build=False,
                 npoints_max=500, p="auto", max_bs=-1, max_rank=-1, precision=None, learned_rank=False,
                 cuda_graph=False, autotune=True):
        self.points = np.asarray(points, dtype=np.float64)
        if self.points.ndim != 2 or not np.all(np.isfinite(self.points)):
            raise ValueError("points must be a finite [N, ndim] array")
        if geometry is not None and not np.all(np.isfinite(np.asarray(geometry, dtype=np.float64))):
            raise ValueError("geometry must be finite")
        # learned_rank: False (pivoted-QR IDs, as the reference), True (packaged
        # rank network), a path to weights, or a RankMLP
        self.learned_rank = learned_rank
        self.operator = _require_operator(operator)
        self.geometry = geometry
        self.param = param
        self.rank_or_tol = tol if rank_or_tol is None else rank_or_tol
        self.leaf_size = leaf_size
        self.tree = None
        self.nlevels = 0
        self.nboxes = 0
        self.nleaves = 0
        self._quiet = quiet
        self._keep_host_fmm = keep_host_fmm
        self._use_single_precision = use_single_precision
        if precision is None:
            precision = "mixed" if use_single_precision else "fp64"
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self._build_npoints_max = npoints_max
        self._build_p = p
        for name, v in (("max_bs", max_bs), ("max_rank", max_rank)):
            if int(v) != v:
                raise ValueError(f"{name} must be an integer")
        # pre-sizes of the reference's padded storage (never a rank cap there);
        # passed to RecursiveSkeletonization, which reports them
        self._max_bs_limit = int(max_bs)
        self._max_rank_limit = int(max_rank)
        self._is_built = False
        self._lazy_build_notice_printed = False

        self.fmm = None
        self.plan = None
        self.batched = None
        # cuda_graph: record one apply of the built operator into a CUDA graph
        # (capture()); applies then replay it on static device buffers
        self._cuda_graph = bool(cuda_graph)
        # autotune: time the translation schemes after the build and keep the
        # fastest (mixed precision); False keeps the plan's default scheme
        self._autotune = bool(autotune)
        self._graph = None
        self._gx = self._gy = None
        self.device = torch.device("cuda") if torch.cuda.is_available() else None
        self.kernel_backend = "cuda-sm103a"
        self.tree_time_seconds = 0.0
        self.skel_time_seconds = 0.0
        self.setup_time_seconds = 0.0
        self.build_time_seconds = 0.0
        self.rank_max = 0
        self.host_build_storage_bytes = 0
        self.host_storage_bytes = 0
        self.device_storage_bytes = 0
        self.total_storage_bytes = 0
        self.nbytes = 0
        if not defer_build:
            self.build()

    @property
    def _prec_code(self):
        return _lib.PREC_MIXED if self.precision == "mixed" else _lib.PREC_FP64

    def _synchronize(self):
        if isinstance(self.device, torch.device) and self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def build(self, *, npoints_max=None, p=None, verbose=False):
        if self._is_built:
            return self
        if self.device is None:
            raise RuntimeError("SkelFMM needs a CUDA device (there is no CPU path)")
        cuda_op_id(self.operator)  # rejects operators without a CUDA kernel
        if npoints_max is None:
            npoints_max = self._build_npoints_max
        t_build = perf_counter()
        ctx = contextlib.ExitStack()
        with ctx as stack:
            if self._quiet:
                stack.enter_context(contextlib.redirect_stdout(io.StringIO()))
                stack.enter_context(contextlib.redirect_stderr(io.StringIO()))
            t0 = perf_counter()
            self.tree = BalancedTree(self.points, leaf_size=self.leaf_size, device=self.device)
            self.tree_time_seconds = perf_counter() - t0
            self.nlevels = self.tree.nlevels
            self.nboxes = self.tree.nboxes
            self.nleaves = self.tree.nleaves
            fmm = RecursiveSkeletonization(self.tree, self.operator, kappa=self.param, tol=self.rank_or_tol,
                                           max_bs=self._max_bs_limit, max_rank=self._max_rank_limit,
                                           geometry=self.geometry, device=self.device)
            if self.learned_rank is not False and self.learned_rank is not None:
                from .rank_model import DEFAULT_WEIGHTS, LearnedRankPredictor, RankMLP

                lr = self.learned_rank
                model = lr if isinstance(lr, RankMLP) else RankMLP.load(DEFAULT_WEIGHTS if lr is True else lr)
                fmm.rank_predictor = LearnedRankPredictor(model)
            t0 = perf_counter()
            fmm.skel_tree(npoints_max=npoints_max, verbose=verbose)
            self.skel_time_seconds = perf_counter() - t0
            t0 = perf_counter()
            fmm.setup_lists(verbose=verbose)
            t1 = perf_counter()
            self.plan = Plan(fmm.ragged())
            torch.cuda.synchronize(self.device)
            t2 = perf_counter()
            self.tuning = None
            if self._prec_code != _lib.PREC_FP64 and self._autotune:
                # translation scheme and tile shape for this plan, by timing them
                self.tuning = self.plan.autotune(self._prec_code, reps=2)
            torch.cuda.synchronize(self.device)
            t3 = perf_counter()
            self.setup_time_seconds = t3 - t0
            # setup split: lists and index maps, plan creation, autotuning
            self.setup_phases_seconds = {"lists": t1 - t0, "plan": t2 - t1, "autotune": t3 - t2}
        self.build_time_seconds = perf_counter() - t_build
        self.rank_max = fmm.rank_max
        self.fmm = fmm if self._keep_host_fmm else None
        self.device_storage_bytes = int(self.plan.info.device_bytes)
        self.host_build_storage_bytes = int(sum(a.nbytes for a in fmm._ids if a is not None))
        self.host_storage_bytes = self.host_build_storage_bytes if self._keep_host_fmm else 0
        self.total_storage_bytes = self.host_storage_bytes + self.device_storage_bytes
        self.nbytes = self.total_storage_bytes
        self._is_built = True
        if self._cuda_graph:
            self.capture()
        return self

    def capture(self):
        """Record one device apply of the built operator into a CUDA graph.

        The graph works on two device vectors owned by this object; ``apply``
        and ``apply_device`` then copy the charges in, replay the graph (one
        launch of the whole apply: permutation, upward passes, translations,
        partial sums, downward passes) and copy the potentials out.  The
        replay performs the same kernels on the same data as the eager apply,
        so its results are bitwise equal."""
        self._ensure_built()
        dt = torch.complex128 if is_complex_op(self.operator) else torch.float64
        n = self.points.shape[0]
        self._gx = torch.zeros(n, dtype=dt, device=self.device)
        self._gy = torch.zeros(n, dtype=dt, device=self.device)
        # first launches (kernel attributes, module loading) outside the capture
        self.plan.apply_device(self._gx, self._gy, self._prec_code, torch.cuda.current_stream(self.device).cuda_stream)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=torch.cuda.Stream(self.device)):
            self.plan.apply_device(self._gx, self._gy, self._prec_code, torch.cuda.current_stream().cuda_stream)
        self._graph = g
        return g

    def save(self, path):
        """Write the built operator to ``path`` (.npz): its ragged build and
        the points, operator, parameter, tolerance and leaf size, so that
        ``SkelFMM.load`` can apply it without building again."""
        self._ensure_built()
        extra = {"points": self.points, "operator": np.array(self.operator.name),
                 "param": np.array(float(self.param)), "tol": np.array(float(self.rank_or_tol)),
                 "leaf_size": np.array(int(self.leaf_size)), "precision": np.array(self.precision)}
        if self.geometry is not None:
            extra["geometry"] = np.asarray(self.geometry, dtype=np.float64)
        save_ragged(self.plan.rb, path, extra)

    @classmethod
    def load(cls, path, *, precision=None, cuda_graph=False):
        """A built operator from a file written by ``save`` (or by
        ``plan.save_ragged`` with the same extra fields), on the current
        device; ``precision`` overrides the saved one."""
        from .operators import BY_NAME

        rb, extra = load_ragged(path)
        op = BY_NAME[str(extra["operator"])]
        geom = extra.get("geometry")
        obj = cls(extra["points"], op, geometry=geom, tol=float(extra["tol"]), leaf_size=int(extra["leaf_size"]),
                  param=float(extra["param"]), precision=precision or str(extra["precision"]), defer_build=True,
                  cuda_graph=cuda_graph)
        if cuda_op_id(op) != rb.op or rb.npoints != obj.points.shape[0]:
            raise ValueError(f"{path}: build and stored operator or points disagree")
        t0 = perf_counter()
        obj.plan = Plan(rb)
        obj.tuning = obj.plan.autotune(obj._prec_code, reps=2) if obj._prec_code != _lib.PREC_FP64 else None
        obj.nlevels, obj.nboxes = rb.nlevels, rb.nboxes
        obj.rank_max = int(np.max(rb.box_rank)) if rb.nboxes else 0
        obj.device_storage_bytes = int(obj.plan.info.device_bytes)
        obj.total_storage_bytes = obj.nbytes = obj.device_storage_bytes
        obj.setup_time_seconds = obj.build_time_seconds = perf_counter() - t0
        obj._is_built = True
        if cuda_graph:
            obj.capture()
        return obj

    def _ensure_built(self, *, announce=False):
        if getattr(self, "_is_built", True):
            return
        if announce and not self._lazy_build_notice_printed:
            print("\tBuilding SkelFMM on first matvec; subsequent matvecs will be fast.")
            self._lazy_build_notice_printed = True
        self.build()

    def apply(self, x):
        self._ensure_built(announce=True)
        x_np = np.asarray(x)
        if x_np.ndim != 1:
            raise ValueError("apply expects a 1D vector")
        if x_np.shape[0] != self.points.shape[0]:
            raise ValueError("Source vector length must match the number of points")
        if not np.all(np.isfinite(x_np)):
            # one non-finite charge reaches every output through the far field
            raise ValueError("apply expects finite charges")
        cplx = is_complex_op(self.operator)
        if np.iscomplexobj(x_np) and not cplx:
            re = self.apply(np.ascontiguousarray(x_np.real))
            im = self.apply(np.ascontiguousarray(x_np.imag))
            return re + 1j * im
        dt = np.complex128 if cplx else np.float64
        xin = np.ascontiguousarray(x_np, dtype=dt)
        if self._graph is not None:
            self._gx.copy_(torch.from_numpy(xin))
            self._graph.replay()
            y = self._gy.cpu().numpy()
        else:
            y = np.empty_like(xin)
            self.plan.apply_host(xin, y, self._prec_code)
        if not cplx and self._use_single_precision:
            return y.astype(np.float32)
        if cplx and self._use_single_precision:
            return y.astype(np.complex64)
        return y

    def matvec(self, x):
        return self.apply(x)

    def apply_device(self, x, y=None):
        """y = A x for CUDA tensors (no host copies)."""
        self._ensure_built()
        cplx = is_complex_op(self.operator)
        dt = torch.complex128 if cplx else torch.float64
        x = x.to(dtype=dt).contiguous()
        if y is None:
            y = torch.empty_like(x)
        if self._graph is not None:
            self._gx.copy_(x)
            self._graph.replay()
            y.copy_(self._gy)
            return y
        self.plan.apply_device(x, y, self._prec_code, torch.cuda.current_stream(x.device).cuda_stream)
        return y

    def direct_apply(self, x, indices):
        """FP64 direct sum ``(K x)[indices]`` on the GPU (kernel evaluated on the fly)."""
        return direct_sum(self.operator, self.points, x, indices, param=self.param, geometry=self.geometry,
                          device=self.device)

    def relerr_fmm_apply_check(self, x, *, ncheck=64, seed=0, indices=None):
        """||y_dense - y_fmm||_inf / ||y_dense||_inf on a subset of targets (skel_fmm.py:218-257).

        The dense reference is an FP64 direct sum evaluated on the GPU.
        """
        self._ensure_built()
        x = np.asarray(x)
        if x.ndim != 1:
            raise ValueError("relerr_fmm_apply_check expects a 1D source vector")
        if x.shape[0] != self.points.shape[0]:
            raise ValueError("Source vector length must match the number of points")
        if indices is None:
            rng = np.random.default_rng(seed)
            indices = rng.choice(self.points.shape[0], size=min(int(ncheck), self.points.shape[0]), replace=False)
        else:
            indices = np.asarray(indices, dtype=int)
        y_fast = self.apply(x)
        y_true = self.direct_apply(x, indices)
        denom = max(np.linalg.norm(y_true, ord=np.inf), 1e-30)
        return np.linalg.norm(y_true - y_fast[indices], ord=np.inf) / denom

    def benchmark_matvec(self, *, nrepeat=3, warmup=1, seed=0):
        self._ensure_built()
        x = np.random.RandomState(seed).randn(self.points.shape[0])
        warmup_cuda_fmm_apply(self, x)
        for _ in range(max(warmup, 0)):
            self.apply(x)
            self._synchronize()
        times = []
        for _ in range(max(nrepeat, 1)):
            self._synchronize()
            t0 = perf_counter()
            self.apply(x)
            self._synchronize()
            times.append(perf_counter() - t0)
        return {
            "times_seconds": tuple(times),
            "avg_seconds": float(np.mean(times)),
            "min_seconds": float(np.min(times)),
            "max_seconds": float(np.max(times)),
        }
