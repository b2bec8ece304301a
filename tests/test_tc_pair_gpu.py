"""The CTA-pair tensor-core M2L (tcgen05 cta_group::2, opt-in with IBIM_TC_PAIR=1) against the
default one-CTA kernel: the same 3xTF32 products, accumulated in other chunks (256 pairs per CTA
pair instead of 128 per CTA), so the mixed FMM outputs agree to FP32 summation order."""

import json
import os
import subprocess
import sys

import numpy as np
import pytest

import ibim
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
import numpy as np
sys.path[:0] = [{root!r}, {pkg!r}, {tests!r}]
import ibim
from conftest import load_golden
from test_oracle_golden import bie_densities, probe_vector
G = load_golden({case!r}); P = G["params"]; s = G["surface"]
ctx = ibim.Context(0)
t = ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], P["h"])
pl = t.plan({order}, P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED)
kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
out = pl.apply(ibim.KERNEL_BIE_FUSED, kp, bie_densities(s, P["h"], probe_vector(len(s))))
np.save({path!r}, out)
print(json.dumps(pl.stats()))
"""


@pytest.mark.parametrize("case,order", [("cavity", None), ("p1hje", None), ("synth30", 5), ("p1hje", 3), ("synth30", 6)])
def test_pair_kernel_matches_one_cta_kernel(ctx, golden, case, order, tmp_path):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    p = order or P["np"]
    path = str(tmp_path / "pair.npy")
    code = CHILD.format(root=ROOT, pkg=os.path.join(ROOT, "ibim-levelset_gb300"), tests=HERE, case=case,
                        order=p, path=path)
    env = dict(os.environ, IBIM_TC_PAIR="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert json.loads(r.stdout.strip().splitlines()[-1])["v_pairs"] > 0
    b = np.load(path)
    t = ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], P["h"])
    pl = t.plan(p, P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    a = pl.apply(ibim.KERNEL_BIE_FUSED, kp, bie_densities(s, P["h"], probe_vector(len(s))))
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 1e-6, (o, case)
