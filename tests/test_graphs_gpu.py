"""The mixed matvec replayed as a CUDA graph (the default) against direct launches
(IBIM_GRAPHS=0), each in its own process since the switch is read once: the same kernels on the
same staged data, so whole solves agree as closely as two mixed solves do (the FP32 atomic
accumulations' order varies from run to run: energies within 1e-6, the bound the mixed path's
other alone-against-batched checks use), with the same iteration counts, and the graph path
reports its kernels in the launch count."""

import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import json, sys
sys.path[:0] = [{root!r}, {pkg!r}, {tests!r}]
import ibim
from conftest import load_golden, config_for
G = load_golden({case!r}); P = G["params"]
ctx = ibim.Context(0)
cfg = config_for(P)
cfg.precision = ibim.PRECISION_MIXED
out = []
for _ in range(2):
    n0 = ibim.launch_count()
    r = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    out.append(dict(energy=r["energy"], iters=r["gmres_iters"], launches=ibim.launch_count() - n0))
print(json.dumps(out))
"""


def run(case, graphs):
    code = CHILD.format(root=ROOT, pkg=os.path.join(ROOT, "ibim-levelset_gb300"), tests=HERE, case=case)
    env = dict(os.environ, IBIM_GRAPHS=graphs)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("case", ["p1hje", "synth300"])
def test_graph_replay_matches_direct_launches(case):
    g, d = run(case, "1"), run(case, "0")
    for a, b in zip(g, d):
        assert a["iters"] == b["iters"]
        assert abs(a["energy"] - b["energy"]) <= 1e-6 * abs(b["energy"]), (a, b)
        # every kernel of a replayed graph is counted; the graph path adds no launches of its own
        assert abs(a["launches"] - b["launches"]) <= 0.02 * b["launches"], (a, b)
