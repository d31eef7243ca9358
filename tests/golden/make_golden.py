"""Generate the golden fixtures in this folder by running the reference
implementation (annayesy/skelFMM, pure Python) on small seeded inputs.

Run from the repository root with the path of a reference checkout
(optionally followed by the names of the build cases to regenerate):

    python tests/golden/make_golden.py <reference-checkout> [case ...]

The reference imports the external ``simpletree`` package, which is not
vendored; ``simpletree_shim/`` stands in for it with the framework's own tree,
so the fixtures pin everything downstream of the tree (proxy IDs, skeleton
bookkeeping, translation lists, index maps, apply) to the reference's code.

Each ``build_*.npz`` holds the inputs of one case, the reference's build
(``RecursiveSkeletonization`` after ``skel_tree`` + ``setup_lists``), the
reference's outputs for one seeded charge vector (``SkelFMMBatched.matvec`` on
CPU in FP64, and the serial ``RecursiveSkeletonization.matvec``), and a dense
FP64 direct sum on a subset of targets.  ``kernels.npz`` holds the batched
kernel-block products of ``skelfmm/util_batched.py`` on near-coincident point
sets; ``ids.npz`` holds proxy interpolative decompositions of single boxes
(``skelfmm/util.py:404-437``).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _setup_paths(reference_root):
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(HERE, "simpletree_shim"))
    sys.path.insert(0, reference_root)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", "")


CASES = [
    # name, operator, geometry, N, leaf, tol, kappa, npoints_max, seed
    ("lap2d_square", "LAPLACE_2D", "square", 1500, 40, 1e-6, 0.0, 150, 0),
    ("lap2d_annulus", "LAPLACE_2D", "curvy_annulus", 3000, 50, 1e-5, 0.0, 300, 1),
    ("lap3d_cube", "LAPLACE_3D", "cube", 8000, 30, 1e-3, 0.0, 500, 2),
    ("lap3d_sphere", "LAPLACE_3D", "sphere_surface", 3000, 40, 1e-5, 0.0, 400, 3),
    ("helm2d_square", "HELMHOLTZ_2D", "square", 1500, 40, 1e-5, 3.0, 150, 4),
    ("helm3d_sphere", "HELMHOLTZ_3D", "sphere_surface", 3000, 40, 1e-5, 2.0, 400, 5),
    ("lapdl3d_sphere", "LAPLACE_DOUBLE_LAYER_3D", "sphere_surface", 1500, 40, 1e-5, 0.0, 200, 6),
    ("lapadl3d_sphere", "LAPLACE_ADJOINT_DOUBLE_LAYER_3D", "sphere_surface", 1500, 40, 1e-5, 0.0, 200, 7),
    ("helmdl3d_sphere", "HELMHOLTZ_DOUBLE_LAYER_3D", "sphere_surface", 1500, 40, 1e-5, 2.0, 200, 8),
    ("helmadl3d_sphere", "HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D", "sphere_surface", 1500, 40, 1e-5, 2.0, 200, 9),
    # The benchmark's parameters (3D Laplace, tol 1e-6, leaf 400: 512 proxy
    # points): a sparse cube with two dense neighbouring level-3 boxes, so the
    # tree has a skeletonized level of parent boxes with 1,000+ entries.
    ("lap3d_c2params", "LAPLACE_3D", "cube_two_dense_boxes", 9202, 400, 1e-6, 0.0, 500, 10),
    # 3D Helmholtz on the sphere at tol 1e-6, leaf 400, kappa h_leaf = 1.25.
    ("helm3d_sphere_k5", "HELMHOLTZ_3D", "sphere_surface", 24000, 400, 1e-6, 5.0, 500, 11),
    # double layers at tol 1e-6
    ("lapdl3d_sphere_1e6", "LAPLACE_DOUBLE_LAYER_3D", "sphere_surface", 2000, 40, 1e-6, 0.0, 200, 12),
    ("helmdl3d_sphere_1e6", "HELMHOLTZ_DOUBLE_LAYER_3D", "sphere_surface", 2000, 40, 1e-6, 2.0, 200, 13),
]


def _points(geom_name, N, rng):
    from simpletree import get_point_dist

    if geom_name == "cube_two_dense_boxes":
        # two corners pin the root box to [0,1]^3; 3000 uniform points; 3100
        # points uniform in each of the level-3 boxes [3/8,1/2]^3 and
        # [1/2,5/8]x[3/8,1/2]^2 (8 leaves of ~390 points each)
        ncl = (N - 3002) // 2
        bg = rng.random((3000, 3))
        c1 = 0.377 + rng.random((ncl, 3)) * 0.121
        c2 = 0.377 + rng.random((N - 3002 - ncl, 3)) * 0.121
        c2[:, 0] += 0.125
        return np.vstack([np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]]), bg, c1, c2])
    return get_point_dist(N, geom_name, rng=rng)


def make_builds(only=()):
    import torch
    from skelfmm import RecursiveSkeletonization, SkelFMMBatched, operators
    from simpletree import BalancedTree

    for name, opname, geom_name, N, leaf, tol, kappa, npmax, seed in CASES:
        if only and name not in only:
            continue
        op = getattr(operators, opname)
        rng = np.random.default_rng(seed)
        pts = _points(geom_name, N, rng)
        geometry = None
        if op.requires_geometry:
            geometry = pts / np.linalg.norm(pts, axis=1, keepdims=True)
        tree = BalancedTree(pts, leaf_size=leaf)
        fmm = RecursiveSkeletonization(tree, op, kappa=kappa, tol=tol, geometry=geometry)
        fmm.skel_tree(npoints_max=npmax, p=None, verbose=False)
        fmm.setup_lists()
        batched = SkelFMMBatched(tree, op, kappa=kappa)
        batched.build_from_copy(fmm, use_single_precision=False)

        x = rng.standard_normal(N)
        if kappa > 0:
            x = x + 1j * rng.standard_normal(N)
        # The serial apply (recursive_skel.py:994-1017) keeps real skeleton
        # vectors, so it only runs for real kernels.
        y_serial = fmm.matvec(x.copy()) if kappa == 0 else None
        xt = torch.from_numpy(x)
        y_batched = batched.matvec(xt).cpu().numpy()

        idx = np.sort(rng.choice(N, size=min(200, N), replace=False))
        geom_src = geometry if op.geometry_side == "source" else None
        geom_trg = geometry[idx] if op.geometry_side == "target" else None
        y_dense = op.numpy_matrix(pts[idx], pts, geom_trg=geom_trg, geom_src=geom_src, param=kappa) @ x

        out = dict(
            name=name, operator=opname, geometry_name=geom_name, N=N, leaf_size=leaf, tol=tol,
            kappa=kappa, npoints_max=npmax, seed=seed,
            points=pts, x=x, y_batched=y_batched,
            dense_idx=idx, y_dense=y_dense,
            nlevels=tree.nlevels, nboxes=tree.nboxes, root_level=fmm.root_level,
            min_rank=fmm.min_rank, max_rank=fmm.max_rank, max_bs=fmm.max_bs,
            max_rank_leaf=fmm.max_rank_leaf, max_bs_leaf=fmm.max_bs_leaf,
            nproxy_level=fmm.nproxy_level,
            bs_list=fmm.bs_list, rank_list=fmm.rank_list, idx_list=fmm.idx_list,
            XX_list=fmm.XX_list, proj_list=fmm.proj_list, proj_list_tree=fmm.proj_list_tree,
            tree_boxes=fmm.tree_boxes, tree_lev_sep=fmm.tree_lev_sep,
            leaf_uskel_from_qskel_list=fmm.leaf_uskel_from_qskel_list,
            tree_uskel_from_qskel_list=fmm.tree_uskel_from_qskel_list,
            uskel_from_q_list=fmm.uskel_from_q_list, u_from_qskel_list=fmm.u_from_qskel_list,
            u_from_q_list=fmm.u_from_q_list, root_boxes=fmm.root_boxes, skel_leaves=fmm.skel_leaves,
            short_vec_inds=fmm.short_vec_inds, long_vec_inds=fmm.long_vec_inds,
            box_skel_inds=fmm.box_skel_inds, child_skel_inds=fmm.child_skel_inds,
            inds_lev_offset=fmm.inds_lev_offset,
        )
        if geometry is not None:
            out["geometry"] = geometry
            out["geom_list"] = fmm.geom_list
        if y_serial is not None:
            out["y_serial"] = y_serial
        np.savez_compressed(os.path.join(HERE, f"build_{name}.npz"), **out)
        ys = y_batched if y_serial is None else y_serial
        rel = np.linalg.norm(y_batched - ys, np.inf) / np.linalg.norm(ys, np.inf)
        err = np.linalg.norm(y_batched[idx] - y_dense, np.inf) / np.linalg.norm(y_dense, np.inf)
        print(f"{name}: N={N} levels={tree.nlevels} root={fmm.root_level} rank_max={fmm.rank_max} "
              f"batched-vs-serial={rel:.2e} vs-dense={err:.2e}")


def _clustered_points(ndim, npts):
    # Same construction as the reference's kernel tests (tests/test_batched.py:58-63).
    rng = np.random.default_rng(1234 + ndim + npts)
    base = rng.random((npts, ndim)) * 0.15
    offsets = np.linspace(1e-6, npts * 1e-6, npts, dtype=np.float64)[:, None]
    direction = np.arange(1, ndim + 1, dtype=np.float64)[None, :]
    return base + offsets * direction


def make_kernels():
    import torch
    from skelfmm import util_batched

    out = {}
    specs = [
        ("laplace_2d", 2, 0.0, False, None),
        ("laplace_3d", 3, 0.0, False, None),
        ("helmholtz_2d", 2, 3.0, True, None),
        ("helmholtz_3d", 3, 2.0, True, None),
        ("laplace_3d_double_layer", 3, 0.0, False, "src"),
        ("laplace_3d_adjoint_double_layer", 3, 0.0, False, "trg"),
        ("helmholtz_3d_double_layer", 3, 2.0, True, "src"),
        ("helmholtz_3d_adjoint_double_layer", 3, 2.0, True, "trg"),
    ]
    for fname, ndim, kappa, cplx, side in specs:
        for m in (6, 37):
            xx = _clustered_points(ndim, m)
            for case, yy, self_bool in (("near", xx + 5e-7, False), ("self", xx, True)):
                rng = np.random.default_rng(2024 + ndim + m)
                q = rng.random((m, 1))
                if cplx:
                    q = q + 1j * rng.random((m, 1))
                g = None
                if side is not None:
                    base = yy if side == "src" else xx
                    g = base / np.linalg.norm(base, axis=1, keepdims=True)
                kw = {}
                if side == "src":
                    kw["src_geom"] = torch.tensor(g).unsqueeze(0)
                elif side == "trg":
                    kw["trg_geom"] = torch.tensor(g).unsqueeze(0)
                qt = torch.tensor(q).unsqueeze(0)
                res = getattr(util_batched, fname)(
                    qt, torch.tensor(xx).unsqueeze(0), torch.tensor(yy).unsqueeze(0), kappa, self_bool, **kw
                )[0].numpy()
                key = f"{fname}/{m}/{case}"
                out[key + "/x"] = xx
                out[key + "/y"] = yy
                out[key + "/q"] = q
                out[key + "/out"] = res
                out[key + "/kappa"] = np.array(kappa)
                if g is not None:
                    out[key + "/geom"] = g
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **out)
    print("kernels:", len(out) // 5, "cases")


def make_ids():
    from skelfmm import operators, util

    out = {}
    specs = [
        ("LAPLACE_2D", 2, 0.0, 1e-6, 24, 30),
        ("LAPLACE_3D", 3, 0.0, 1e-6, 400, 250),
        ("HELMHOLTZ_3D", 3, 2.0, 1e-5, 420, 200),
        ("HELMHOLTZ_2D", 2, 8.0, 1e-5, 60, 40),
        ("LAPLACE_DOUBLE_LAYER_3D", 3, 0.0, 1e-5, 400, 150),
        ("HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D", 3, 2.0, 1e-5, 420, 150),
    ]
    for i, (opname, ndim, kappa, tol, nproxy, bs) in enumerate(specs):
        op = getattr(operators, opname)
        rng = np.random.default_rng(100 + i)
        center = rng.random(ndim)
        length = 0.25
        xb = center[None, :] + (rng.random((bs, ndim)) - 0.5) * length
        geom = None
        if op.requires_geometry:
            geom = rng.standard_normal((bs, ndim))
            geom /= np.linalg.norm(geom, axis=1, keepdims=True)
        rank, idx, proj = util.skel_box_helper(op, kappa, xb, center, length, tol, nproxy=nproxy, geom=geom)
        K = util.build_stacked_proxy_matrix(op, xb, center, length, nproxy, geom=geom, param=kappa)
        key = f"{opname}"
        out[key + "/x"] = xb
        out[key + "/center"] = center
        out[key + "/length"] = np.array(length)
        out[key + "/tol"] = np.array(tol)
        out[key + "/kappa"] = np.array(kappa)
        out[key + "/nproxy"] = np.array(nproxy)
        out[key + "/rank"] = np.array(rank)
        out[key + "/idx"] = idx
        out[key + "/proj"] = proj
        out[key + "/Kshape"] = np.array(K.shape)
        out[key + "/Knorm"] = np.array(np.linalg.norm(K))
        if geom is not None:
            out[key + "/geom"] = geom
        print(f"id {opname}: bs={bs} rank={rank} K={K.shape}")
    np.savez_compressed(os.path.join(HERE, "ids.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference-checkout> [case ...]")
    _setup_paths(sys.argv[1])
    only = tuple(sys.argv[2:])
    if not only:
        make_kernels()
        make_ids()
    make_builds(only)
