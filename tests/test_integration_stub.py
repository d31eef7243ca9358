"""The reference-side ctypes binding printed in INTEGRATION.md, executed as
written on the reference's own golden builds: its FP64 apply through
skf_plan_apply_host matches the reference's SkelFMMBatched.matvec
(skelfmm/batched_fmm.py:539-564) and its mixed apply meets the bound of the
framework's own tests."""
import os
import re
from types import SimpleNamespace

import pytest

from golden_util import load_build, relinf

HERE = os.path.dirname(os.path.abspath(__file__))
DOC = os.path.join(os.path.dirname(HERE), "INTEGRATION.md")


def _stub_source():
    text = open(DOC).read()
    m = re.search(r"<!-- stub:begin -->\s*```python\n(.*?)```\s*<!-- stub:end -->", text, re.S)
    assert m, "INTEGRATION.md has no marked stub block"
    return m.group(1)


def test_stub_block_compiles():
    compile(_stub_source(), "INTEGRATION.md:stub", "exec")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lap3d_c2params", "helm3d_sphere", "lapdl3d_sphere_1e6", "lap2d_annulus"])
def test_stub_apply_matches_reference(name, monkeypatch):
    from skelfmm_gb300 import _lib
    from skelfmm_gb300.tree import BalancedTree

    _lib.load()
    monkeypatch.setenv("SKF_LIB", _lib.LIB_PATH)
    ns = {}
    exec(compile(_stub_source(), "INTEGRATION.md:stub", "exec"), ns)
    d = load_build(name)
    tree = BalancedTree(d["points"], int(d["leaf_size"]))
    fmm = SimpleNamespace(**d)
    # the reference's operator names are the constants' names in lower case
    op = SimpleNamespace(name=str(d["operator"]).lower())
    g = ns["GB300Apply"](tree, fmm, op, float(d["kappa"]))
    y = g.matvec(d["x"])
    assert relinf(y, d["y_batched"]) < 1e-12
    ym = g.matvec(d["x"], single_precision=True)
    assert relinf(ym, d["y_batched"]) < 2e-6
