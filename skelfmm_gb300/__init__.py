"""GB300-native strong-recursive-skeletonization FMM (drop-in for skelfmm).

Public surface mirrors ``skelfmm/__init__.py``: ``SkelFMM``,
``RecursiveSkeletonization``, ``operators`` and ``warmup_cuda_fmm_apply``;
``Plan`` is the device-resident apply (the role of ``SkelFMMBatched``);
``SkelFMMBatch`` applies many independent instances as one operator and
``RankMLP`` is the rank network of the learned-rank build.
"""

from . import operators  # noqa: F401
from .tree import BalancedTree  # noqa: F401

__all__ = ["SkelFMM", "RecursiveSkeletonization", "Plan", "SkelFMMBatch", "RankMLP", "operators",
           "warmup_cuda_fmm_apply", "BalancedTree"]


def __getattr__(name):
    if name in ("SkelFMM", "warmup_cuda_fmm_apply"):
        from . import skel_fmm

        return getattr(skel_fmm, name)
    if name == "RecursiveSkeletonization":
        from .recursive_skel import RecursiveSkeletonization

        return RecursiveSkeletonization
    if name in ("Plan", "SkelFMMBatched"):
        from .plan import Plan

        return Plan
    if name == "SkelFMMBatch":
        from .batch import SkelFMMBatch

        return SkelFMMBatch
    if name == "RankMLP":
        from .rank_model import RankMLP

        return RankMLP
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
