"""Saved builds (skelfmm_gb300.plan.save_ragged / load_ragged, the format of
Plan.save and SkelFMM.save): a round trip keeps every array, bad files are
refused, and the committed CPU-oracle build (tests/golden/make_saved_build.py)
is what the oracle builds today.  The GPU replay is in test_gpu_saved_graph.py."""
import os

import numpy as np
import pytest

from golden_util import GOLDEN, load_build

ARRAYS = ("box_level", "box_off", "box_rank", "entry_xyz", "entry_pslot", "perm_entry", "perm_point", "t_off",
          "t_data", "list_off", "list_src", "list_kind")


def _rb(name):
    from skelfmm_gb300 import operators
    from skelfmm_gb300.plan import ragged_from_reference
    from skelfmm_gb300.tree import BalancedTree

    d = load_build(name)
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    return ragged_from_reference(tree, d, operators.BY_NAME[str(d["operator"])], float(d["kappa"]))


@pytest.mark.parametrize("name", ["lap3d_sphere", "helm3d_sphere", "lapdl3d_sphere"])
def test_round_trip_keeps_every_array(name, tmp_path):
    from skelfmm_gb300.plan import load_ragged, save_ragged

    rb = _rb(name)
    path = os.path.join(tmp_path, "b.npz")
    save_ragged(rb, path, {"note": np.array("x")})
    rb2, extra = load_ragged(path)
    for k in ARRAYS:
        a, b = getattr(rb, k), getattr(rb2, k)
        assert a.dtype == b.dtype or k != "t_data"
        assert np.array_equal(np.asarray(a), b), k
    assert (rb.entry_geom is None) == (rb2.entry_geom is None)
    if rb.entry_geom is not None:
        assert np.array_equal(rb.entry_geom, rb2.entry_geom)
    for k in ("op", "ndim", "kappa", "npoints", "nlevels", "root_level"):
        assert getattr(rb, k) == getattr(rb2, k), k
    assert str(extra["note"]) == "x"


def test_bad_files_are_refused(tmp_path):
    from skelfmm_gb300.plan import FORMAT_VERSION, load_ragged, save_ragged

    other = os.path.join(tmp_path, "other.npz")
    np.savez(other, a=np.zeros(3))
    with pytest.raises(ValueError):
        load_ragged(other)
    rb = _rb("lap2d_square")
    path = os.path.join(tmp_path, "b.npz")
    save_ragged(rb, path)
    d = dict(np.load(path))
    d["version"] = np.array(FORMAT_VERSION + 1)
    newer = os.path.join(tmp_path, "newer.npz")
    np.savez(newer, **d)
    with pytest.raises(ValueError):
        load_ragged(newer)
    d["version"] = np.array(FORMAT_VERSION)
    d["t_data"] = d["t_data"].astype(np.complex128)
    d["t_dtype"] = np.array("complex128")
    wrong = os.path.join(tmp_path, "wrong.npz")
    np.savez(wrong, **d)
    with pytest.raises(ValueError):
        load_ragged(wrong)


def test_committed_oracle_build_is_reproduced():
    import sys

    sys.path.insert(0, GOLDEN)
    from make_saved_build import OUT, oracle_saved_build

    from skelfmm_gb300.plan import load_ragged

    rb, extra = oracle_saved_build()
    rb2, extra2 = load_ragged(OUT)
    for k in ARRAYS:
        if k == "t_data":
            assert np.allclose(rb.t_data, rb2.t_data, rtol=0, atol=1e-12 * np.abs(rb.t_data).max())
        else:
            assert np.array_equal(getattr(rb, k), getattr(rb2, k)), k
    assert np.array_equal(extra["x"], extra2["x"])
    assert np.allclose(extra["y_oracle"], extra2["y_oracle"], rtol=1e-13, atol=0)
