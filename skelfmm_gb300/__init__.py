"""GB300-native strong-recursive-skeletonization FMM (drop-in for skelfmm)."""

from . import operators  # noqa: F401
from .tree import BalancedTree  # noqa: F401

__all__ = ["operators", "BalancedTree"]
