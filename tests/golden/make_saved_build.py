"""Write ``saved_oracle_lap3d_sphere.npz``: a build made on the CPU by the
oracle (the reference's pivoted-QR build restated in numpy/scipy), saved in
the framework's build format so a GPU run can replay it without building.

    python tests/golden/make_saved_build.py

The file also holds one seeded charge vector and the oracle's FP64 apply of
it (``extra/x``, ``extra/y_oracle``).  ``tests/test_saved_build.py`` checks
that this script reproduces the committed file's arrays exactly.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "saved_oracle_lap3d_sphere.npz")


def oracle_saved_build():
    """(RaggedBuild, extra) of the oracle build of 3D Laplace on 4,000 sphere
    points, tol 1e-6, leaf 60."""
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    from oracle import skel_oracle as O
    from skelfmm_gb300 import operators
    from skelfmm_gb300.plan import ragged_from_reference
    from skelfmm_gb300.tree import BalancedTree, get_point_dist

    rng = np.random.default_rng(31)
    pts = get_point_dist(4000, "sphere_surface", rng=rng)
    tol, leaf = 1e-6, 60
    tree = BalancedTree(pts, leaf)
    ob = O.OracleBuild(tree, O.OPERATORS["laplace_3d"], 0.0, tol).skel_tree(400)
    fmm = {k: getattr(ob, k) for k in (
        "bs_list", "rank_list", "min_rank", "root_level", "tree_boxes", "leaf_uskel_from_qskel_list",
        "tree_uskel_from_qskel_list", "uskel_from_q_list", "u_from_qskel_list", "u_from_q_list",
        "short_vec_inds", "long_vec_inds", "box_skel_inds", "child_skel_inds")}
    fmm["XX_list"] = ob.XX_list()
    fmm["proj_list"], fmm["proj_list_tree"] = ob.proj_lists()
    rb = ragged_from_reference(tree, fmm, operators.LAPLACE_3D, 0.0)
    x = rng.standard_normal(pts.shape[0])
    y = O.OracleApply(ob, nthreads=2).matvec(x)
    extra = {"points": pts, "operator": np.array("laplace_3d"), "param": np.array(0.0), "tol": np.array(tol),
             "leaf_size": np.array(leaf), "precision": np.array("fp64"), "x": x, "y_oracle": y}
    return rb, extra


if __name__ == "__main__":
    sys.path.insert(0, REPO)
    from skelfmm_gb300.plan import save_ragged

    rb, extra = oracle_saved_build()
    save_ragged(rb, OUT, extra)
    print(OUT, os.path.getsize(OUT), "bytes")
