"""Kernel operator objects (drop-in for ``skelfmm.operators``).

Mirrors ``KernelOperator`` / ``PointKernelOperator`` /
``GeometryAwareKernelOperator`` and the eight built-ins of
skelfmm/operators.py:17-227.  Each built-in carries the id of its CUDA
kernel (``cuda_id``, the ``SKF_*`` operator ids of include/skf.h):

* ``numpy_matrix`` evaluates a dense FP64 block on the host (the reference's
  dense kernels, skelfmm/util.py:128-377), as the reference API does;
* ``torch_apply`` evaluates batched blocks ``K(x_trg, x_src) @ q`` on the
  GPU through ``skf_kernel_apply`` (the reference's batched torch kernels,
  skelfmm/util_batched.py:240-656); there is no CPU path;
* ``keops_apply`` returns None (PyKeOps is not used).

An operator without a CUDA kernel id cannot be built or applied: the build
raises ``NotImplementedError``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.special import j0, y0

FOUR_PI_INV = 1.0 / (4.0 * np.pi)

SKF_LAPLACE_2D = 0
SKF_LAPLACE_3D = 1
SKF_HELMHOLTZ_2D = 2
SKF_HELMHOLTZ_3D = 3
SKF_LAPLACE_DOUBLE_LAYER_3D = 4
SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D = 5
SKF_HELMHOLTZ_DOUBLE_LAYER_3D = 6
SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D = 7
_COMPLEX_IDS = {SKF_HELMHOLTZ_2D, SKF_HELMHOLTZ_3D, SKF_HELMHOLTZ_DOUBLE_LAYER_3D,
                SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D}


# ------------------------------------------------------------- dense numpy kernels
def _pairwise(XX, YY):
    diff = XX[:, None, :] - YY[None, :, :]
    return diff, np.einsum("ijk,ijk->ij", diff, diff)


def laplace_2d(XX, YY, param=0, assume_not_self_interaction=False):
    assert param == 0, "Parameter must be 0 for Laplace kernel"
    _, d2 = _pairwise(XX, YY)
    r = np.sqrt(d2)
    if not assume_not_self_interaction:
        r[d2 == 0] = 1.0
    return np.log(r)


def laplace_3d(XX, YY, param=0, assume_not_self_interaction=False):
    assert param == 0, "Parameter must be 0 for Laplace kernel"
    _, d2 = _pairwise(XX, YY)
    r = np.sqrt(d2)
    if not assume_not_self_interaction:
        r[d2 == 0] = np.inf
    return 1.0 / r


def helmholtz_2d(XX, YY, param, assume_not_self_interaction=False):
    _, d2 = _pairwise(XX, YY)
    r = np.sqrt(d2)
    zero = d2 == 0
    if not assume_not_self_interaction:
        r[zero] = 1.0
    out = j0(param * r) + 1j * y0(param * r)
    if not assume_not_self_interaction:
        out[zero] = 0
    return out


def helmholtz_3d(XX, YY, param, assume_not_self_interaction=False):
    _, d2 = _pairwise(XX, YY)
    r = np.sqrt(d2)
    zero = d2 == 0
    out = np.exp(1j * param * r)
    rr = r.copy()
    if not assume_not_self_interaction:
        rr[zero] = np.inf
    out = out / rr
    if not assume_not_self_interaction:
        out[zero] = 0
    return out


def _dl(XX, YY, geom, side):
    diff, d2 = _pairwise(XX, YY)
    d2 = np.where(d2 == 0, 1.0, d2)
    rotn = np.einsum("ijk,jk->ij", diff, geom) if side == "source" else np.einsum("ijk,ik->ij", diff, geom)
    return rotn, d2


def laplace_3d_double_layer(XX, YY, param=0, src_geom=None, assume_not_self_interaction=False):
    if src_geom is None:
        raise ValueError("src_geom is required for the Laplace double-layer kernel")
    rotn, d2 = _dl(XX, YY, src_geom, "source")
    return -FOUR_PI_INV * rotn / (d2 * np.sqrt(d2))


def laplace_3d_adjoint_double_layer(XX, YY, param=0, trg_geom=None, assume_not_self_interaction=False):
    if trg_geom is None:
        raise ValueError("trg_geom is required for the Laplace adjoint double-layer kernel")
    rotn, d2 = _dl(XX, YY, trg_geom, "target")
    return FOUR_PI_INV * rotn / (d2 * np.sqrt(d2))


def helmholtz_3d_double_layer(XX, YY, param, src_geom=None, assume_not_self_interaction=False):
    if src_geom is None:
        raise ValueError("src_geom is required for the Helmholtz double-layer kernel")
    rotn, d2 = _dl(XX, YY, src_geom, "source")
    r = np.sqrt(d2)
    kr = param * r
    return FOUR_PI_INV * rotn * np.exp(1j * kr) * (1j * kr - 1.0) / (d2 * r)


def helmholtz_3d_adjoint_double_layer(XX, YY, param, trg_geom=None, assume_not_self_interaction=False):
    if trg_geom is None:
        raise ValueError("trg_geom is required for the Helmholtz adjoint double-layer kernel")
    rotn, d2 = _dl(XX, YY, trg_geom, "target")
    r = np.sqrt(d2)
    kr = param * r
    return -FOUR_PI_INV * rotn * np.exp(1j * kr) * (1j * kr - 1.0) / (d2 * r)


# ------------------------------------------------------------- operator objects
@dataclass
class KernelOperator:
    """Stateless kernel/operator interface (skelfmm/operators.py:17-108)."""

    name: str = "custom"
    ndim: int = -1
    numpy_func: object = None
    torch_func: object = None
    keops_func: object = None
    proxy_surface: str = "cube"
    geometry_side: str | None = None
    is_symmetric: bool = False
    cuda_id: int = -1

    def __post_init__(self):
        if self.geometry_side not in {None, "source", "target"}:
            raise ValueError("geometry_side must be None, 'source', or 'target'")

    @property
    def requires_geometry(self):
        return self.geometry_side is not None

    @property
    def has_keops(self):
        return self.keops_func is not None

    @property
    def has_cuda(self):
        return self.cuda_id >= 0

    def _geom_kwargs(self, geom_trg=None, geom_src=None):
        if self.geometry_side == "source":
            return {"src_geom": geom_src}
        if self.geometry_side == "target":
            return {"trg_geom": geom_trg}
        return {}

    def numpy_matrix(self, x_trg, x_src, *, geom_trg=None, geom_src=None, param=0.0,
                     assume_not_self_interaction=False):
        if self.numpy_func is None:
            raise NotImplementedError
        return self.numpy_func(x_trg, x_src, param=param,
                               assume_not_self_interaction=assume_not_self_interaction,
                               **self._geom_kwargs(geom_trg, geom_src))

    def torch_apply(self, q, x_trg, x_src, *, geom_trg=None, geom_src=None, param=0.0,
                    self_interaction=False):
        """Batched ``K(x_trg[b], x_src[b]) @ q[b]`` on the GPU ([b,m,d],[b,n,d],[b,n,1])."""
        if self.torch_func is not None:
            return self.torch_func(q, x_trg, x_src, param, self_interaction,
                                   **self._geom_kwargs(geom_trg, geom_src))
        if not self.has_cuda:
            raise NotImplementedError
        from .kernels import batched_kernel_apply

        return batched_kernel_apply(self.cuda_id, q, x_trg, x_src, param=param,
                                    geom_trg=geom_trg, geom_src=geom_src,
                                    self_interaction=self_interaction)

    def keops_apply(self, q, x_trg, x_src, *, geom_trg=None, geom_src=None, param=0.0,
                    self_interaction=False):
        if self.keops_func is None:
            return None
        kw = self._geom_kwargs(geom_trg, geom_src)
        if param == 0.0:
            return self.keops_func(q, x_trg, x_src, self_interaction, **kw)
        return self.keops_func(q, x_trg, x_src, param, self_interaction, **kw)


class PointKernelOperator(KernelOperator):
    """Point kernels without extra geometry (skelfmm/operators.py:111-132)."""

    def __init__(self, name, ndim, numpy_func, torch_func=None, keops_func=None, proxy_surface="cube",
                 is_symmetric=True, cuda_id=-1):
        super().__init__(name=name, ndim=ndim, numpy_func=numpy_func, torch_func=torch_func,
                         keops_func=keops_func, proxy_surface=proxy_surface, is_symmetric=is_symmetric,
                         cuda_id=cuda_id)


class GeometryAwareKernelOperator(KernelOperator):
    """Kernels with one aligned source or target geometry (skelfmm/operators.py:135-156)."""

    def __init__(self, name, ndim, numpy_func, torch_func=None, keops_func=None, *, geometry_side,
                 cuda_id=-1):
        super().__init__(name=name, ndim=ndim, numpy_func=numpy_func, torch_func=torch_func,
                         keops_func=keops_func, proxy_surface="sphere", geometry_side=geometry_side,
                         cuda_id=cuda_id)


LAPLACE_2D = PointKernelOperator("laplace_2d", 2, laplace_2d, cuda_id=SKF_LAPLACE_2D)
LAPLACE_3D = PointKernelOperator("laplace_3d", 3, laplace_3d, cuda_id=SKF_LAPLACE_3D)
HELMHOLTZ_2D = PointKernelOperator("helmholtz_2d", 2, helmholtz_2d, cuda_id=SKF_HELMHOLTZ_2D)
HELMHOLTZ_3D = PointKernelOperator("helmholtz_3d", 3, helmholtz_3d, cuda_id=SKF_HELMHOLTZ_3D)
LAPLACE_DOUBLE_LAYER_3D = GeometryAwareKernelOperator(
    "laplace_double_layer_3d", 3, laplace_3d_double_layer, geometry_side="source",
    cuda_id=SKF_LAPLACE_DOUBLE_LAYER_3D)
LAPLACE_ADJOINT_DOUBLE_LAYER_3D = GeometryAwareKernelOperator(
    "laplace_adjoint_double_layer_3d", 3, laplace_3d_adjoint_double_layer, geometry_side="target",
    cuda_id=SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D)
HELMHOLTZ_DOUBLE_LAYER_3D = GeometryAwareKernelOperator(
    "helmholtz_double_layer_3d", 3, helmholtz_3d_double_layer, geometry_side="source",
    cuda_id=SKF_HELMHOLTZ_DOUBLE_LAYER_3D)
HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D = GeometryAwareKernelOperator(
    "helmholtz_adjoint_double_layer_3d", 3, helmholtz_3d_adjoint_double_layer, geometry_side="target",
    cuda_id=SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D)

BUILTINS = (LAPLACE_2D, LAPLACE_3D, HELMHOLTZ_2D, HELMHOLTZ_3D, LAPLACE_DOUBLE_LAYER_3D,
            LAPLACE_ADJOINT_DOUBLE_LAYER_3D, HELMHOLTZ_DOUBLE_LAYER_3D, HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D)
BY_NAME = {op.name: op for op in BUILTINS}
BY_NAME.update({
    "LAPLACE_2D": LAPLACE_2D, "LAPLACE_3D": LAPLACE_3D, "HELMHOLTZ_2D": HELMHOLTZ_2D,
    "HELMHOLTZ_3D": HELMHOLTZ_3D, "LAPLACE_DOUBLE_LAYER_3D": LAPLACE_DOUBLE_LAYER_3D,
    "LAPLACE_ADJOINT_DOUBLE_LAYER_3D": LAPLACE_ADJOINT_DOUBLE_LAYER_3D,
    "HELMHOLTZ_DOUBLE_LAYER_3D": HELMHOLTZ_DOUBLE_LAYER_3D,
    "HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D": HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D,
})


def _require_operator(operator):
    """Validate that an explicit ``KernelOperator`` was provided (operators.py:220-227)."""
    if not isinstance(operator, KernelOperator):
        raise TypeError(
            "Expected a KernelOperator instance. "
            "Use objects from skelfmm_gb300.operators such as operators.LAPLACE_3D."
        )
    return operator


def cuda_op_id(op):
    if isinstance(op, (int, np.integer)):
        return int(op)
    op = _require_operator(op)
    if not op.has_cuda:
        raise NotImplementedError(f"operator {op.name!r} has no CUDA kernel in this framework")
    return int(op.cuda_id)


def is_complex_op(op):
    return cuda_op_id(op) in _COMPLEX_IDS
