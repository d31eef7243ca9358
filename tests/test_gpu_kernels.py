"""GPU kernel blocks (skf_kernel_apply) vs the reference's batched torch
kernels (skelfmm/util_batched.py) on near-coincident and self point sets
(the case of tests/test_batched.py:201-237, xx and xx + 5e-7)."""
import numpy as np
import pytest

from golden_util import load_groups, relinf

pytestmark = pytest.mark.gpu

FN = {
    "laplace_2d": 0, "laplace_3d": 1, "helmholtz_2d": 2, "helmholtz_3d": 3,
    "laplace_3d_double_layer": 4, "laplace_3d_adjoint_double_layer": 5,
    "helmholtz_3d_double_layer": 6, "helmholtz_3d_adjoint_double_layer": 7,
}


@pytest.mark.parametrize("precision", [0, 1])
def test_kernel_blocks_match_reference(precision):
    import torch
    from skelfmm_gb300.kernels import batched_kernel_apply

    groups = load_groups("kernels.npz")
    for key, g in groups.items():
        kname, m, case = key.split("/")
        op = FN[kname]
        geom = g.get("geom")
        gt = gs = None
        if op in (4, 6):
            gs = torch.tensor(geom).unsqueeze(0).cuda()
        elif op in (5, 7):
            gt = torch.tensor(geom).unsqueeze(0).cuda()
        out = batched_kernel_apply(op, torch.tensor(g["q"]).unsqueeze(0).cuda(),
                                   torch.tensor(g["x"]).unsqueeze(0).cuda(),
                                   torch.tensor(g["y"]).unsqueeze(0).cuda(), param=float(g["kappa"]),
                                   geom_trg=gt, geom_src=gs, self_interaction=(case == "self"),
                                   precision=precision)[0].cpu().numpy()
        if precision == 0:
            tol = 1e-9 if kname == "helmholtz_2d" else 1e-10
        else:
            # double layers included: (x-y).n is formed to FP32 rounding of
            # the result (compensated dot product of FP32 pairs)
            tol = 2e-6
        assert relinf(out, g["out"]) < tol, (key, relinf(out, g["out"]))
