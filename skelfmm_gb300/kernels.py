"""GPU kernel-block products: the reference's ``kernel_apply`` seam
(skelfmm/batched_fmm.py:21-44, 180-217; skelfmm/operators.py:69-89) on the
C ABI's ``skf_kernel_apply``.  Device tensors only."""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .operators import _COMPLEX_IDS


def _dev(t, dtype):
    if t is None:
        return None
    t = torch.as_tensor(t)
    if t.device.type != "cuda":
        raise ValueError("skelfmm_gb300 kernels need CUDA tensors (there is no CPU path)")
    return t.to(dtype).contiguous()


def batched_kernel_apply(op_id, q, x_trg, x_src, *, param=0.0, geom_trg=None, geom_src=None,
                         self_interaction=False, precision=_lib.PREC_FP64, m=None, n=None):
    """``out[b] = K(x_trg[b], x_src[b]) @ q[b]``; shapes [b,m,d], [b,n,d], [b,n,1].

    ``self_interaction`` (bool or per-pair bool tensor) zeroes the diagonal.
    ``m``/``n`` (int32 tensors) give per-pair valid lengths (default: full).
    """
    cplx = op_id in _COMPLEX_IDS
    x_trg = _dev(x_trg, torch.float64)
    x_src = _dev(x_src, torch.float64)
    B, M, _ = x_trg.shape
    Nn = x_src.shape[1]
    qd = torch.complex128 if cplx else torch.float64
    q = _dev(q, qd)
    if q.dim() == 3:
        if q.shape[-1] != 1:
            raise ValueError("q must have a single right-hand side")
        q = q[..., 0]
    q = q.contiguous()
    gt = _dev(geom_trg, torch.float64)
    gs = _dev(geom_src, torch.float64)
    dev = x_trg.device
    mm = torch.full((B,), M, dtype=torch.int32, device=dev) if m is None else _dev(m, torch.int32)
    nn = torch.full((B,), Nn, dtype=torch.int32, device=dev) if n is None else _dev(n, torch.int32)
    if isinstance(self_interaction, (bool, np.bool_)):
        sf = torch.full((B,), 1 if self_interaction else 0, dtype=torch.int8, device=dev)
    else:
        sf = _dev(self_interaction, torch.int8)
    out = torch.zeros((B, M), dtype=qd, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(_lib.load().skf_kernel_apply(
        int(op_id), float(param), int(B), int(M), int(Nn), _lib.ptr(mm), _lib.ptr(nn), _lib.ptr(x_trg),
        _lib.ptr(x_src), _lib.ptr(gt), _lib.ptr(gs), _lib.ptr(q), _lib.ptr(sf), _lib.ptr(out),
        int(precision), stream), "skf_kernel_apply")
    return out.unsqueeze(-1)
