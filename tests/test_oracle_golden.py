"""Pin the CPU oracle against the reference's own outputs (tests/golden/).

The fixtures were produced by running the reference implementation
(skelfmm/recursive_skel.py, skelfmm/batched_fmm.py, skelfmm/util.py,
skelfmm/util_batched.py) on this framework's tree; see make_golden.py.
"""
import numpy as np
import pytest

from golden_util import OPNAME, build_cases, load_build, load_groups, relinf
from oracle import skel_oracle as O
from skelfmm_gb300.tree import BalancedTree

LIST_KEYS = [
    "leaf_uskel_from_qskel_list", "tree_uskel_from_qskel_list", "uskel_from_q_list",
    "u_from_qskel_list", "u_from_q_list", "root_boxes", "skel_leaves", "short_vec_inds",
    "long_vec_inds", "box_skel_inds", "child_skel_inds", "inds_lev_offset", "tree_boxes",
    "tree_lev_sep", "nproxy_level",
]


def _oracle_build(d):
    op = O.OPERATORS[OPNAME[str(d["operator"])]]
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    geom = d.get("geometry")
    b = O.OracleBuild(tree, op, float(d["kappa"]), float(d["tol"]), geometry=geom)
    return b.skel_tree(int(d["npoints_max"]))


def _redundant_order(mine, ref, r, bs):
    """Permutation p with mine[r + k] == ref[r + p[k]]: the entries past the
    rank, matched by their coordinates.  Their pivot order is decided by
    column norms at rounding level, so it can differ between two correct
    pivoted QRs (the oracle factors K once where the reference factors the
    stacked [K; K]); the skeleton rows [0, r) must agree exactly."""
    a, b = mine[r:bs], ref[r:bs]
    ia = np.lexsort(a.T[::-1])
    ib = np.lexsort(b.T[::-1])
    assert np.array_equal(a[ia], b[ib])
    p = np.empty(bs - r, dtype=np.int64)
    p[ia] = ib
    return p


@pytest.mark.parametrize("name", build_cases())
def test_oracle_build_matches_reference(name):
    d = load_build(name)
    b = _oracle_build(d)
    assert b.root_level == int(d["root_level"])
    assert np.array_equal(b.bs_list, d["bs_list"])
    assert np.array_equal(b.rank_list, d["rank_list"])
    assert b.min_rank == int(d["min_rank"]) and b.max_rank == int(d["max_rank"])
    X, R = b.XX_list(), d["XX_list"][:, : b.max_bs]
    pl, pt = b.proj_lists()
    ref_pl, ref_pt = d["proj_list"], d["proj_list_tree"]
    assert pl.shape == ref_pl.shape and pt.shape == ref_pt.shape
    tree_boxes = np.asarray(d["tree_boxes"])
    min_rank = int(d["min_rank"])
    reordered = 0
    for box in range(X.shape[0]):
        if np.array_equal(X[box], R[box]):
            continue
        r, bs = int(d["rank_list"][box]), int(d["bs_list"][box])
        assert np.array_equal(X[box, :r], R[box, :r])
        assert not X[box, bs:].any() and not R[box, bs:].any()
        p = _redundant_order(X[box], R[box], r, bs)
        # T's columns follow the redundant entries; align them the same way
        if box in tree_boxes:
            i = int(np.searchsorted(tree_boxes, box))
            mine_t, ref_t = pt[i], ref_pt[i]
        else:
            mine_t, ref_t = pl[box], ref_pl[box]
        cols = np.arange(r, bs) - min_rank
        mine_t[:r, cols] = mine_t[:r, cols[np.argsort(p)]]
        reordered += 1
    # every reordered box is a large one (redundant columns at rounding level)
    assert reordered <= max(2, X.shape[0] // 20)
    for mine, ref in ((pl, ref_pl), (pt, ref_pt)):
        scale = max(1.0, float(np.abs(ref).max()) if ref.size else 1.0)
        assert np.allclose(mine, ref, rtol=1e-9, atol=1e-9 * scale)
    # padded leaf slot -> point: equal except inside the reordered redundant
    # rows, where each side must hold the point its own XX_list shows there
    max_bs = X.shape[1]
    for k in LIST_KEYS:
        if k == "long_vec_inds" and reordered:
            mine_s, mine_p = np.asarray(b.short_vec_inds), np.asarray(b.long_vec_inds)
            ref_s, ref_p = d["short_vec_inds"], d["long_vec_inds"]
            assert np.array_equal(mine_s, ref_s)
            pts = d["points"]
            assert np.array_equal(pts[mine_p], X.reshape(-1, X.shape[2])[mine_s])
            assert np.array_equal(pts[ref_p], R.reshape(-1, R.shape[2])[ref_s])
            same = mine_p == ref_p
            box, slot = mine_s // max_bs, mine_s % max_bs
            assert np.all(same | (slot >= d["rank_list"][box]))
            continue
        if k == "box_skel_inds" and reordered:
            # child skeleton slot -> slot in the parent box: each side's parent
            # slot holds the child's point in its own XX_list
            child = np.asarray(b.child_skel_inds)
            assert np.array_equal(child, d["child_skel_inds"])
            mine_par, ref_par = np.asarray(b.box_skel_inds), d["box_skel_inds"]
            Xf, Rf = X.reshape(-1, X.shape[2]), R.reshape(-1, R.shape[2])
            assert np.array_equal(Xf[mine_par], Xf[child])
            assert np.array_equal(Rf[ref_par], Rf[child])
            box, slot = mine_par // max_bs, mine_par % max_bs
            assert np.all((mine_par == ref_par) | (slot >= d["rank_list"][box]))
            continue
        assert np.array_equal(np.asarray(getattr(b, k)), d[k]), k


@pytest.mark.parametrize("name", build_cases())
def test_oracle_apply_matches_reference(name):
    d = load_build(name)
    b = _oracle_build(d)
    y = O.OracleApply(b, nthreads=2).matvec(d["x"])
    # torch's bessel_j0/y0 (reference, helmholtz_2d) and scipy's differ near 1e-10
    tol = 1e-9 if str(d["operator"]) == "HELMHOLTZ_2D" else 1e-12
    assert relinf(y, d["y_batched"]) < tol
    if "y_serial" in d:
        assert relinf(y, d["y_serial"]) < 1e-12
    assert relinf(y[d["dense_idx"]], d["y_dense"]) < max(10 * float(d["tol"]), 1e-12)


def test_oracle_kernels_match_reference_blocks():
    groups = load_groups("kernels.npz")
    fn = {
        "laplace_2d": "laplace_2d", "laplace_3d": "laplace_3d", "helmholtz_2d": "helmholtz_2d",
        "helmholtz_3d": "helmholtz_3d", "laplace_3d_double_layer": "laplace_double_layer_3d",
        "laplace_3d_adjoint_double_layer": "laplace_adjoint_double_layer_3d",
        "helmholtz_3d_double_layer": "helmholtz_double_layer_3d",
        "helmholtz_3d_adjoint_double_layer": "helmholtz_adjoint_double_layer_3d",
    }
    assert len(groups) == 32
    for key, g in groups.items():
        kname, m, case = key.split("/")
        op = O.OPERATORS[fn[kname]]
        geom = g.get("geom")
        K = op.matrix(g["x"], g["y"], geom_trg=geom, geom_src=geom, param=float(g["kappa"]))
        if case == "self":
            np.fill_diagonal(K, 0.0)
        tol = 1e-9 if kname == "helmholtz_2d" else 1e-10
        assert relinf(K @ g["q"], g["out"]) < tol, key


def test_oracle_id_matches_reference():
    groups = load_groups("ids.npz")
    for opname, g in groups.items():
        op = O.OPERATORS[OPNAME[opname]]
        rank, idx, proj = O.skel_box(op, float(g["kappa"]), g["x"], g["center"], float(g["length"]),
                                     float(g["tol"]), int(g["nproxy"]), geom=g.get("geom"))
        assert rank == int(g["rank"])
        assert np.array_equal(idx, g["idx"])
        if proj.size:
            assert relinf(proj, g["proj"]) < 1e-8
