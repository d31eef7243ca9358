"""Train the rank network of the learned-rank build on pivoted-QR builds.

    python -m skelfmm_gb300.train_rank_model [--out PATH] [--small]

Runs the pivoted-QR GPU build on the three single-instance workloads the
framework is benchmarked on (2D Laplace N=1e5 tol 1e-5 leaf 200; 3D Laplace
N=1e6 uniform cube tol 1e-6 leaf 400; 3D Helmholtz kappa=25 N=2e6 unit sphere
tol 1e-6 leaf 400) and on scaled variants of them (other leaf sizes and
tolerances, the Laplace kernel on the sphere), collects (box features, log
rank ratio) of every skeletonized box, trains the network with the
library's BF16 kernels and writes the weights (default: the packaged
``rank_mlp.npz``).  Nothing from the clustered workload the learned build is
measured on enters training.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import operators
from .rank_model import DEFAULT_WEIGHTS, RankMLP, build_training_set, rank_from_target
from .recursive_skel import RecursiveSkeletonization
from .tree import BalancedTree, get_point_dist

# (name, operator, geometry, N, tol, leaf, kappa)
WORKLOADS = [
    ("laplace2d_square_1e5", operators.LAPLACE_2D, "square", 100_000, 1e-5, 200, 0.0),
    ("laplace3d_cube_1e6", operators.LAPLACE_3D, "cube", 1_000_000, 1e-6, 400, 0.0),
    ("helmholtz3d_sphere_2e6", operators.HELMHOLTZ_3D, "sphere_surface", 2_000_000, 1e-6, 400, 25.0),
    ("laplace2d_square_1e5_leaf64_tol1e-6", operators.LAPLACE_2D, "square", 100_000, 1e-6, 64, 0.0),
    ("laplace3d_cube_3e5_leaf128", operators.LAPLACE_3D, "cube", 300_000, 1e-6, 128, 0.0),
    ("laplace3d_cube_3e5_leaf256", operators.LAPLACE_3D, "cube", 300_000, 1e-6, 256, 0.0),
    ("laplace3d_cube_2e5_leaf256_tol1e-8", operators.LAPLACE_3D, "cube", 200_000, 1e-8, 256, 0.0),
    ("laplace3d_cube_2e5_leaf256_tol1e-4", operators.LAPLACE_3D, "cube", 200_000, 1e-4, 256, 0.0),
    ("laplace3d_sphere_5e5_leaf256", operators.LAPLACE_3D, "sphere_surface", 500_000, 1e-6, 256, 0.0),
    ("helmholtz3d_sphere_5e5_leaf256", operators.HELMHOLTZ_3D, "sphere_surface", 500_000, 1e-6, 256, 25.0),
    ("laplace3d_cube_3e5_leaf32", operators.LAPLACE_3D, "cube", 300_000, 1e-6, 32, 0.0),
    ("laplace3d_cube_3e5_leaf64", operators.LAPLACE_3D, "cube", 300_000, 1e-6, 64, 0.0),
    ("laplace3d_sphere_3e5_leaf32", operators.LAPLACE_3D, "sphere_surface", 300_000, 1e-6, 32, 0.0),
    ("laplace3d_sphere_3e5_leaf64", operators.LAPLACE_3D, "sphere_surface", 300_000, 1e-6, 64, 0.0),
    ("laplace2d_square_1e5_leaf32", operators.LAPLACE_2D, "square", 100_000, 1e-5, 32, 0.0),
    ("helmholtz3d_sphere_5e5_leaf64", operators.HELMHOLTZ_3D, "sphere_surface", 500_000, 1e-6, 64, 25.0),
]


def collect(workloads, scale=1.0, log=print):
    Xs, ys, bss, tags = [], [], [], []
    for i, (name, op, geo, N, tol, leaf, kappa) in enumerate(workloads):
        n = max(2000, int(N * scale))
        pts = get_point_dist(n, geo, rng=np.random.default_rng(i))
        t0 = time.perf_counter()
        tree = BalancedTree(pts, leaf)
        fmm = RecursiveSkeletonization(tree, op, kappa, tol).skel_tree(500)
        torch.cuda.synchronize()
        X, y, bs = build_training_set(fmm)
        log(f"{name}: N={n} boxes={X.shape[0]} build {time.perf_counter() - t0:.2f}s")
        Xs.append(X)
        ys.append(y)
        bss.append(bs)
        tags.append(np.full(X.shape[0], i, np.int32))
    return np.concatenate(Xs), np.concatenate(ys), np.concatenate(bss), np.concatenate(tags)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--small", action="store_true", help="10%% of every workload (quick check)")
    ap.add_argument("--steps", type=int, default=6000)
    args = ap.parse_args(argv)
    X, y, bs, tag = collect(WORKLOADS, scale=0.1 if args.small else 1.0)
    rng = np.random.default_rng(0)
    val = rng.random(X.shape[0]) < 0.1
    m = RankMLP()
    t0 = time.perf_counter()
    hist = m.fit(X[~val], y[~val], steps=args.steps, log_every=500)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    pv = m.predict(X[val])
    r_true = rank_from_target(y[val], bs[val])
    r_pred = rank_from_target(pv, bs[val])
    stats = {
        "samples": int(X.shape[0]), "train_s": round(t_train, 2), "history": hist,
        "val_mse_target": float(np.mean((pv - y[val]) ** 2)),
        "val_mae_rank": float(np.mean(np.abs(r_pred - r_true))),
        "val_under_frac": float(np.mean(r_pred < r_true)),
        "val_rel_err_median": float(np.median(np.abs(r_pred - r_true) / np.maximum(r_true, 1))),
        "workloads": [w[0] for w in WORKLOADS],
    }
    print(json.dumps(stats))
    m.save(args.out, stats=json.dumps(stats))


if __name__ == "__main__":
    main()
