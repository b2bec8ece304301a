"""Operand forms of the mixed path's tensor-core M2L against each other, each in its own process
(the form is fixed per process by the environment): the CTA-pair kernel (tcgen05 cta_group::2,
IBIM_TC_PAIR=1, TF32 splits) and the one-CTA kernel with TF32 splits (IBIM_TC_FP16=0) compute the
same 3xTF32 products in other chunks, so they agree to FP32 summation order; the default scaled
FP16 splits carry as many bits (each form is 1e-6..3e-6 from the FP64 operator, the FP16 one
the closer)."""

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


def run_child(tmp_path, case, order, env_extra, tag):
    path = str(tmp_path / f"{tag}.npy")
    code = CHILD.format(root=ROOT, pkg=os.path.join(ROOT, "ibim-levelset_gb300"), tests=HERE, case=case,
                        order=order, path=path)
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert json.loads(r.stdout.strip().splitlines()[-1])["v_pairs"] > 0
    return np.load(path)


@pytest.mark.parametrize("case,order", [("cavity", None), ("p1hje", None), ("synth30", 5), ("p1hje", 3), ("synth30", 6)])
def test_pair_kernel_matches_one_cta_kernel(ctx, golden, case, order, tmp_path):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    p = order or P["np"]
    pair = run_child(tmp_path, case, p, {"IBIM_TC_PAIR": "1"}, "pair")
    tf32 = run_child(tmp_path, case, p, {"IBIM_TC_FP16": "0"}, "tf32")
    t = ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], P["h"])
    pl = t.plan(p, P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    fp16 = pl.apply(ibim.KERNEL_BIE_FUSED, kp, bie_densities(s, P["h"], probe_vector(len(s))))
    for o in range(4):
        assert np.abs(pair[o] - tf32[o]).max() / np.abs(tf32[o]).max() < 1e-6, (o, case)
        # each form is 1e-6..3e-6 (max-normalised) from the FP64 operator on these fixtures
        assert np.abs(fp16[o] - tf32[o]).max() / np.abs(tf32[o]).max() < 4e-6, (o, case)


@pytest.mark.parametrize("case,order", [("cavity", None), ("p1hje", None), ("synth30", 6), ("synth30", 3)])
@pytest.mark.parametrize("fp16,form", [("1", None), ("1", "P"), ("0", None), ("1", "6"), ("1", "7")])
def test_launch_forms_match_one_cta_of_four(ctx, golden, case, order, fp16, form, tmp_path):
    """Two CTAs of two row tiles per SM (IBIM_TC_RT=2), the persistent form (IBIM_TC_RT=P, FP16)
    and the FP16 CTA-pair forms (IBIM_TC_RT=6 and 7: 2-SM MMAs of M = 256 over chunks of up to
    256 pairs, odd row-tile counts included at orders 3 and 6) issue the same products per row
    tile in the same K order as one CTA of four (IBIM_TC_RT=4); only the order of the atomic adds
    into the locals differs."""
    G = golden(case)
    p = order or G["params"]["np"]
    env = {"IBIM_TC_FP16": fp16}
    if form is not None:
        env["IBIM_TC_RT"] = form
    got = run_child(tmp_path, case, p, env, "form")
    one = run_child(tmp_path, case, p, {"IBIM_TC_RT": "4", "IBIM_TC_FP16": fp16}, "one")
    for o in range(4):
        assert np.abs(got[o] - one[o]).max() / np.abs(one[o]).max() < 1e-6, (o, case)
