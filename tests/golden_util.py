"""Helpers to load the golden fixtures produced by tests/golden/make_golden.py."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

OPNAME = {
    "LAPLACE_2D": "laplace_2d",
    "LAPLACE_3D": "laplace_3d",
    "HELMHOLTZ_2D": "helmholtz_2d",
    "HELMHOLTZ_3D": "helmholtz_3d",
    "LAPLACE_DOUBLE_LAYER_3D": "laplace_double_layer_3d",
    "LAPLACE_ADJOINT_DOUBLE_LAYER_3D": "laplace_adjoint_double_layer_3d",
    "HELMHOLTZ_DOUBLE_LAYER_3D": "helmholtz_double_layer_3d",
    "HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D": "helmholtz_adjoint_double_layer_3d",
}


def build_cases():
    return sorted(os.path.basename(f)[6:-4] for f in glob.glob(os.path.join(GOLDEN, "build_*.npz")))


def load_build(name):
    d = np.load(os.path.join(GOLDEN, f"build_{name}.npz"), allow_pickle=False)
    return {k: d[k] for k in d.files}


def load_groups(fname):
    d = np.load(os.path.join(GOLDEN, fname), allow_pickle=False)
    groups = {}
    for k in d.files:
        head, leaf = k.rsplit("/", 1)
        groups.setdefault(head, {})[leaf] = d[k]
    return groups


def relinf(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel(), np.inf) / max(np.linalg.norm(b.ravel(), np.inf), 1e-300))
