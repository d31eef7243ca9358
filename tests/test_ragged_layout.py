"""Host-side checks of the ragged plan layout (no GPU): the reference's padded
build converted by ``ragged_from_reference`` and executed by a numpy model of
the device apply reproduces the reference's apply."""
import numpy as np
import pytest

from golden_util import build_cases, load_build, relinf
from ragged_ref import ragged_apply
from skelfmm_gb300 import operators
from skelfmm_gb300.plan import ragged_from_reference
from skelfmm_gb300.tree import BalancedTree


def ragged_for(name):
    d = load_build(name)
    op = operators.BY_NAME[str(d["operator"])]
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    return d, ragged_from_reference(tree, d, op, float(d["kappa"]))


@pytest.mark.parametrize("name", build_cases())
def test_ragged_model_matches_reference_apply(name):
    d, rb = ragged_for(name)
    assert rb.nentries == int(d["bs_list"].sum())
    assert np.array_equal(np.sort(rb.perm_point), np.arange(rb.npoints))
    y = ragged_apply(rb, d["x"])
    tol = 1e-9 if str(d["operator"]) == "HELMHOLTZ_2D" else 1e-12
    assert relinf(y, d["y_batched"]) < tol


@pytest.mark.parametrize("name", build_cases())
def test_ragged_lists_cover_reference_pairs(name):
    d, rb = ragged_for(name)
    n = sum(len(d[k]) for k in ("leaf_uskel_from_qskel_list", "tree_uskel_from_qskel_list",
                                "uskel_from_q_list", "u_from_qskel_list", "u_from_q_list"))
    assert rb.list_off[-1] == n
    # every skeleton entry below the root has a distinct parent slot
    ps = rb.entry_pslot[rb.entry_pslot >= 0]
    assert np.unique(ps).shape == ps.shape
