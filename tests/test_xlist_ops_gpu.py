"""X-list interactions (a coarser source leaf's multipole to a node's local expansion,
bbfmm.h:556-560) applied as precomputed operators inside the batched M2L contraction, against the
on-the-fly X kernels (IBIM_X_ONTHEFLY): the same kernel values at the same Chebyshev node pairs,
summed in another order."""

import os

import numpy as np
import pytest

import ibim
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu


def plans(ctx, G, precision, targets=None):
    P = G["params"]
    s = G["surface"]
    t = ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], P["h"])
    os.environ["IBIM_X_ONTHEFLY"] = "1"
    try:
        fly = t.plan(P["np"], P["maxpoint"], P["maxlevel"], targets=targets, precision=precision)
    finally:
        del os.environ["IBIM_X_ONTHEFLY"]
    ops = t.plan(P["np"], P["maxpoint"], P["maxlevel"], targets=targets, precision=precision)
    return t, fly, ops


@pytest.mark.parametrize("case", ["synth30", "p1hje", "cavity"])
def test_x_operators_match_on_the_fly_fp64(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    _, fly, ops = plans(ctx, G, ibim.PRECISION_FP64)
    sf, so = fly.stats(), ops.stats()
    assert sf["x_pairs"] == so["x_pairs"] and sf["v_pairs"] == so["v_pairs"]
    assert so["operators"] > sf["operators"] or so["x_pairs"] == 0
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = fly.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = ops.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 1e-12, o


def test_x_operators_atom_targets(ctx, golden):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    _, fly, ops = plans(ctx, G, ibim.PRECISION_FP64, targets=G["centers"])
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = fly.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = ops.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    assert np.abs(a - b).max() / np.abs(a).max() < 1e-12


@pytest.mark.parametrize("precision", [ibim.PRECISION_MIXED, ibim.PRECISION_FP64_TC])
def test_x_operators_other_precisions(ctx, golden, precision):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    _, fly, ops = plans(ctx, G, precision)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = fly.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = ops.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    tol = 2e-5 if precision == ibim.PRECISION_MIXED else 1e-10
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < tol, o
