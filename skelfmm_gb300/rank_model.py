"""Learned skeleton ranks: box features, the BF16 rank network and the
predictor that drives the randomized (row-sampled) IDs of the build.

No counterpart in the reference, whose build always runs the column-pivoted
QR ID of the full proxy matrix (skelfmm/util.py:13-51).  Here a 3-layer
perceptron (width 128, BF16, trained and evaluated by the library's own CUDA
kernels ``skf_mlp_*``) predicts the log rank ratio log2((rank + 1) / (bs + 1))
of every box (bs = the points its ID factors) from cheap geometric features;
the build then computes a randomized ID at the predicted rank from a sketch
of ``predicted rank + oversampling`` rows of the proxy matrix, checks it on
rows of the full matrix, and falls back to the full pivoted-QR ID for the
boxes whose check misses the tolerance (``RecursiveSkeletonization``).
The pivoted-QR builds are both the training labels and the measure of the
predictor's error.
"""

from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np
import torch

from . import _lib
from .operators import is_complex_op

NFEAT = 22
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rank_mlp.npz")


def level_features(fmm, lev, x_lev=None, off=None):
    """Features [nboxes_at_lev, NFEAT] (float32) of every box of ``lev`` from
    its candidate points (the points its ID factors):

    0 level, 1 log2(candidates + 1), 2 log2(proxy rows), 3 colleagues,
    4 children, 5 leaf flag, 6-8 mean offset from the centre / width,
    9-14 second central moments / width^2 (xx yy zz xy xz yz), 15 log10 tol,
    16 kappa * width, 17 3D flag, 18 complex-kernel flag, 19 geometry-kernel
    flag, 20 log2(points under the box + 1), 21 coarse neighbours.
    Offsets and moments come from the library's ``skf_box_moments`` kernel
    over ``x_lev`` (the level's candidate coordinates on the device, in
    ``off`` segments; gathered from the build's device copy when None).
    """
    tree = fmm.tree
    ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
    nbl = le - ls
    if off is None:
        off = fmm._off[lev]
    bs = np.diff(off).astype(np.int64)
    d = tree.ndim
    w = float(tree.L0 * 0.5 ** lev)
    m9 = box_moments(fmm, lev, x_lev, off)
    s1 = m9[:, :d]
    mom = m9[:, 3:9]
    F = np.zeros((nbl, NFEAT), dtype=np.float64)
    boxes = np.arange(ls, le)
    F[:, 0] = lev
    F[:, 1] = np.log2(bs + 1.0)
    F[:, 2] = np.log2(max(fmm._mrows(lev), 1))
    F[:, 3] = (tree._colleagues[boxes] >= 0).sum(1)
    F[:, 4] = (tree._children[boxes] >= 0).sum(1)
    F[:, 5] = tree._is_leaf[boxes]
    F[:, 6:6 + d] = s1
    F[:, 9:15] = mom
    F[:, 15] = np.log10(fmm.tol) if fmm.tol < 1 else 0.0
    F[:, 16] = fmm.kappa * w
    F[:, 17] = d == 3
    F[:, 18] = is_complex_op(fmm.op_id)
    F[:, 19] = fmm.op_id >= 4
    F[:, 20] = np.log2(tree.get_box_npoints(boxes) + 1.0)
    F[:, 21] = (tree._coarse[boxes] >= 0).sum(1)
    return F.astype(np.float32)


def box_moments(fmm, lev, x_lev, off):
    """[nboxes_at_lev, 9] float64 from ``skf_box_moments``: mean offset of
    each box's candidate points from its centre and their second central
    moments (xx yy zz xy xz yz), in units of the box width."""
    tree = fmm.tree
    ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
    nbl = le - ls
    dev = fmm.device
    if x_lev is None:
        ids_t = torch.from_numpy(np.ascontiguousarray(fmm._ids[lev], dtype=np.int64)).to(dev)
        x_lev = fmm._XX_dev.index_select(0, ids_t)
    x_lev = x_lev.contiguous()
    off_t = torch.from_numpy(np.ascontiguousarray(off, dtype=np.int64)).to(dev)
    cen = torch.from_numpy(np.ascontiguousarray(tree._box_center[ls:le], dtype=np.float64)).to(dev)
    out = torch.empty((max(nbl, 1), 9), dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(_lib.load().skf_box_moments(nbl, tree.ndim, _lib.ptr(off_t), _lib.ptr(x_lev), _lib.ptr(cen),
                                           float(tree.L0 * 0.5 ** lev), _lib.ptr(out), stream), "skf_box_moments")
    return out[:nbl].cpu().numpy()


def rank_target(rank, bs):
    """Training target of a box: log2((rank + 1) / (bs + 1)) <= 0."""
    return (np.log2(np.asarray(rank, np.float64) + 1.0) - np.log2(np.asarray(bs, np.float64) + 1.0)).astype(np.float32)


def rank_from_target(y, bs):
    """Inverse of ``rank_target`` (rounded, clipped to [0, bs])."""
    bs = np.asarray(bs, np.float64)
    r = np.rint((bs + 1.0) * np.exp2(np.minimum(np.asarray(y, np.float64), 0.0)) - 1.0)
    return np.clip(r, 0, bs).astype(np.int64)


def build_training_set(fmm):
    """(features, rank target, bs) of every skeletonized box of a finished
    pivoted-QR build."""
    Xs, ys, bss = [], [], []
    tree = fmm.tree
    for lev in range(fmm.root_level + 1, fmm.nlevels):
        if fmm._ids[lev] is None:
            continue
        F = level_features(fmm, lev)
        ls, le = int(tree.level_sep[lev]), int(tree.level_sep[lev + 1])
        bs = np.diff(fmm._off[lev])
        keep = bs > 0
        Xs.append(F[keep])
        ys.append(rank_target(fmm.rank_list[ls:le][keep], bs[keep]))
        bss.append(bs[keep])
    if not Xs:
        return np.zeros((0, NFEAT), np.float32), np.zeros(0, np.float32), np.zeros(0, np.int64)
    return np.concatenate(Xs), np.concatenate(ys), np.concatenate(bss)


class RankMLP:
    """The rank network on the device: FP32 master parameters, a BF16
    mirror, Adam state, and the feature normalisation (mean / std)."""

    def __init__(self, nin=NFEAT, seed=0, device="cuda"):
        lib = _lib.load()
        self.nin = int(nin)
        self.P = int(lib.skf_mlp_num_params(self.nin))
        if self.P <= 0:
            raise ValueError("unsupported number of input features")
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        H = 128
        parts = [torch.randn(H, self.nin, generator=g) * (2.0 / self.nin) ** 0.5, torch.zeros(H),
                 torch.randn(H, H, generator=g) * (2.0 / H) ** 0.5, torch.zeros(H),
                 torch.randn(H, generator=g) * (1.0 / H) ** 0.5, torch.zeros(1)]
        self.theta = torch.cat([p.reshape(-1) for p in parts]).float().to(self.device)
        self.theta16 = torch.empty(self.P, dtype=torch.bfloat16, device=self.device)
        self._sync16()
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        self.step = 0
        self.mu = np.zeros(self.nin, np.float32)
        self.sd = np.ones(self.nin, np.float32)
        self.y_mu = 0.0

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _sync16(self):
        _lib.check(_lib.load().skf_mlp_bf16(_lib.ptr(self.theta), _lib.ptr(self.theta16), self.P, self._stream()),
                   "skf_mlp_bf16")

    def set_parameters(self, theta):
        self.theta = torch.as_tensor(np.asarray(theta, np.float32)).to(self.device).contiguous()
        self._sync16()

    def _inputs(self, X):
        Xn = (np.asarray(X, np.float32) - self.mu) / self.sd
        x = torch.from_numpy(np.ascontiguousarray(Xn, dtype=np.float32)).to(self.device)
        x16 = torch.empty(x.shape, dtype=torch.bfloat16, device=self.device)
        _lib.check(_lib.load().skf_mlp_bf16(_lib.ptr(x), _lib.ptr(x16), x.numel(), self._stream()), "skf_mlp_bf16")
        return x16

    def predict(self, X):
        """Network output (the rank target) for feature rows X."""
        X = np.asarray(X, np.float32)
        if X.shape[0] == 0:
            return np.zeros(0, np.float32)
        x16 = self._inputs(X)
        y = torch.empty(X.shape[0], dtype=torch.float32, device=self.device)
        _lib.check(_lib.load().skf_mlp_predict(self.nin, _lib.ptr(self.theta16), _lib.ptr(x16), X.shape[0],
                                               _lib.ptr(y), self._stream()), "skf_mlp_predict")
        return y.cpu().numpy() + self.y_mu

    def _step(self, x16, t, lr, apply):
        lib = _lib.load()
        n = int(t.shape[0])
        scratch = torch.empty(int(lib.skf_mlp_scratch_floats(self.nin, n)), dtype=torch.float32, device=self.device)
        grad = torch.empty(self.P, dtype=torch.float32, device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        if apply:
            self.step += 1
        _lib.check(lib.skf_mlp_train_step(self.nin, _lib.ptr(self.theta), _lib.ptr(self.theta16), _lib.ptr(x16),
                                          _lib.ptr(t), n, _lib.ptr(scratch), _lib.ptr(grad), _lib.ptr(self.m),
                                          _lib.ptr(self.v), max(self.step, 1), float(lr), 0.9, 0.999, 1e-8,
                                          1 if apply else 0, _lib.ptr(loss), self._stream()), "skf_mlp_train_step")
        return grad, loss

    def gradient(self, X, y):
        """(loss, gradient) of the mean squared error at the current BF16
        parameters, without an update (normalised inputs X, targets y)."""
        x16 = self._inputs(X)
        t = torch.from_numpy(np.asarray(y, np.float32) - self.y_mu).to(self.device)
        g, loss = self._step(x16, t, 0.0, False)
        return float(loss.item()), g.cpu().numpy()

    def fit(self, X, y, steps=4000, batch=4096, lr=2e-3, lr_min=1e-4, seed=0, normalise=True, log_every=0):
        """Minibatch Adam on the mean squared error of the rank target, with a
        cosine learning-rate decay.  Returns the loss history."""
        X = np.asarray(X, np.float32)
        y = np.asarray(y, np.float32)
        if normalise:
            self.mu = X.mean(0)
            self.sd = X.std(0)
            self.sd[self.sd < 1e-6] = 1.0
            self.y_mu = float(y.mean())
        x16 = self._inputs(X)
        t = torch.from_numpy(y - self.y_mu).to(self.device)
        n = X.shape[0]
        g = torch.Generator(device=self.device).manual_seed(seed)
        hist = []
        for s in range(steps):
            lr_s = lr_min + 0.5 * (lr - lr_min) * (1 + np.cos(np.pi * s / max(steps, 1)))
            if batch >= n:
                xb, tb = x16, t
            else:
                idx = torch.randint(0, n, (batch,), device=self.device, generator=g)
                xb = x16.index_select(0, idx).contiguous()
                tb = t.index_select(0, idx).contiguous()
            _, loss = self._step(xb, tb, lr_s, True)
            if log_every and (s % log_every == 0 or s == steps - 1):
                hist.append((s, float(loss.item())))
        return hist

    def save(self, path, **meta):
        np.savez(path, theta=self.theta.cpu().numpy(), mu=self.mu, sd=self.sd, y_mu=np.float32(self.y_mu),
                 nin=np.int32(self.nin), **meta)

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device="cuda"):
        d = np.load(path)
        m = cls(nin=int(d["nin"]), device=device)
        m.set_parameters(d["theta"])
        m.mu = d["mu"].astype(np.float32)
        m.sd = d["sd"].astype(np.float32)
        m.y_mu = float(d["y_mu"])
        return m


class CalibratedRankPredictor:
    """Callable for ``RecursiveSkeletonization.rank_predictor`` that turns a
    per-box estimate y of the rank target (``estimate``) into sketch ranks.

    The build runs from the finest level to the root, so the ranks of level
    l + 1 are known when level l is predicted (kept randomized IDs report
    their sketch rank, the others their pivoted-QR rank; boxes left at full
    rank are not used).  Their error e =
    actual - y is fitted as a + b y by least squares, and level l's estimate
    becomes y + max(0, a + b y + q), q the ``calibrate`` quantile of the fit's
    residuals: this follows an estimate that drifts, level by level and with
    the box size, on a point distribution it was not fitted to.  Boxes of
    ``big_box`` candidates or more take the ``calibrate_big`` quantile: a
    rejected large box pays the full pivoted-QR ID on top of its sketch,
    while a few more sketch rows cost little.  The predicted rank is then
    ``margin`` above the corrected estimate, capped at the box size."""

    def __init__(self, margin=16, calibrate=0.9, calibrate_big=0.995, big_box=256):
        self.margin = int(margin)
        self.calibrate = calibrate
        self.calibrate_big = calibrate_big
        self.big_box = int(big_box)
        self.shifts = {}
        self._prev = None

    def estimate(self, fmm, lev, boxes, x_lev, off):
        raise NotImplementedError

    def _correction(self, fmm, lev):
        """(a, b, q, q_big) fitted on level lev + 1 of the same build, else
        None."""
        p = self._prev
        if not self.calibrate or p is None or p[0]() is not fmm or p[1] != lev + 1:
            return None
        _, _, boxes, y, bs = p
        rank = fmm.rank_list[boxes]
        keep = (bs > 0) & (rank < bs)  # full-rank boxes say nothing of the estimate
        if np.count_nonzero(keep) < 2:
            return None
        yk = y[keep]
        err = rank_target(rank[keep], bs[keep]) - yk
        A = np.stack([np.ones_like(yk), yk], 1)
        coef = np.linalg.lstsq(A, err, rcond=None)[0]
        res = err - A @ coef
        q = float(np.quantile(res, self.calibrate))
        q_big = float(np.quantile(res, max(self.calibrate, self.calibrate_big)))
        return float(coef[0]), float(coef[1]), q, q_big

    def __call__(self, fmm, lev, boxes, x_lev, off):
        bs = np.diff(off)
        y = np.asarray(self.estimate(fmm, lev, boxes, x_lev, off), np.float64)
        fit = self._correction(fmm, lev)
        if fit is None:
            shift = np.zeros_like(y)
        else:
            q = np.where(bs >= self.big_box, fit[3], fit[2])
            shift = np.maximum(fit[0] + fit[1] * y + q, 0.0)
        self.shifts[lev] = float(shift.mean()) if shift.size else 0.0
        self._prev = (weakref.ref(fmm), lev, np.asarray(boxes), y, bs)
        k = rank_from_target(y + shift, bs) + self.margin
        return np.clip(k, 1, np.maximum(bs, 1))


class LearnedRankPredictor(CalibratedRankPredictor):
    """The rank network's estimate (``RankMLP`` on ``level_features``),
    calibrated level by level.  It sets the sketch size of every box."""

    def __init__(self, model: RankMLP, margin=16, calibrate=0.9, calibrate_big=0.995, big_box=256):
        super().__init__(margin, calibrate, calibrate_big, big_box)
        self.model = model

    def estimate(self, fmm, lev, boxes, x_lev, off):
        return self.model.predict(level_features(fmm, lev, x_lev, off))
