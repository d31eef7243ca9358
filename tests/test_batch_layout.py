"""Concatenating independent builds into one ragged plan (multi-instance
batching) keeps every instance's apply unchanged — checked on the host with
the numpy model of the device apply."""
import numpy as np

from golden_util import load_build, relinf
from ragged_ref import ragged_apply
from skelfmm_gb300 import operators
from skelfmm_gb300.batch import concat_ragged
from skelfmm_gb300.plan import ragged_from_reference
from skelfmm_gb300.tree import BalancedTree


def _rb(name):
    d = load_build(name)
    op = operators.BY_NAME[str(d["operator"])]
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    return d, ragged_from_reference(tree, d, op, float(d["kappa"]))


def test_concatenated_plan_reproduces_each_instance():
    (d1, r1), (d2, r2) = _rb("lap2d_square"), _rb("lap2d_annulus")
    cat, starts = concat_ragged([r1, r2])
    assert cat.npoints == r1.npoints + r2.npoints
    assert list(starts) == [0, r1.npoints, r1.npoints + r2.npoints]
    assert cat.nentries == r1.nentries + r2.nentries
    # every instance keeps its root level aligned to the common one
    assert cat.root_level == max(r1.root_level, r2.root_level)
    y = ragged_apply(cat, np.concatenate((d1["x"], d2["x"])))
    assert relinf(y[: r1.npoints], d1["y_batched"]) < 1e-12
    assert relinf(y[r1.npoints:], d2["y_batched"]) < 1e-12


def test_concat_rejects_mixed_operators():
    import pytest

    (_, r1), (_, r2) = _rb("lap2d_square"), _rb("lap3d_cube")
    with pytest.raises(ValueError):
        concat_ragged([r1, r2])
