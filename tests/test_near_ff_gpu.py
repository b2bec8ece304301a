"""The FP64-class near field in float-float arithmetic (IBIM_PRECISION_FP64_TC) against the native
FP64 near field.

With the tree cut at level 1 every leaf is a neighbour of every other, so the FMM is its near
field alone and the two precisions differ only by the float-float evaluation (about 2^-44 per
pair).  Yukawa screening lengths from none (kappa = 0, the Laplace branch) to kappa = 40 (kappa r
beyond the exponential's table, where e^{-kappa r} is taken as zero) are covered, for the
plan's own points and for extra targets."""

import numpy as np
import pytest

import ibim
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu

TOL_NEAR = 2e-12  # max-normalised, per output field, near field alone
TOL_FULL = 1e-10  # with the far field (sliced M2L digits dominate)


def tube_of(ctx, G):
    s = G["surface"]
    return ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], G["params"]["h"])


def max_err(a, b):
    return max(np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() for o in range(a.shape[0]))


@pytest.mark.parametrize("case", ["born", "p1hje", "cavity"])
@pytest.mark.parametrize("kappa", [None, 0.0, 40.0])
def test_near_field_only(ctx, golden, case, kappa):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    a64 = t.plan(P["np"], P["maxpoint"], 1)
    aff = t.plan(P["np"], P["maxpoint"], 1, precision=ibim.PRECISION_FP64_TC)
    st = a64.stats()
    assert st["v_pairs"] == 0 and st["x_pairs"] == 0 and st["near_pairs"] > 0
    kp = ibim.kernel_params(P["kappa"] if kappa is None else kappa, P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = a64.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = aff.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    assert max_err(a, b) < TOL_NEAR


def test_near_field_extra_targets(ctx, golden):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    rng = np.random.default_rng(5)
    lo, hi = s[:, :3].min(0), s[:, :3].max(0)
    pts = lo + (hi - lo) * rng.random((3000, 3))
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    for maxlevel, tol in ((1, TOL_NEAR), (P["maxlevel"], TOL_FULL)):
        a = t.plan(P["np"], P["maxpoint"], maxlevel, targets=pts).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
        b = t.plan(P["np"], P["maxpoint"], maxlevel, targets=pts,
                   precision=ibim.PRECISION_FP64_TC).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
        assert max_err(a, b) < tol, maxlevel


def test_near_field_k3_scaled(ctx, golden):
    """The K3 factor 1/(4 pi) (k3_scaled) reaches the float-float kernel parameters."""
    G = golden("born")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"], k3_scaled=1)
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = t.plan(P["np"], P["maxpoint"], 1).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = t.plan(P["np"], P["maxpoint"], 1, precision=ibim.PRECISION_FP64_TC).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    assert max_err(a, b) < TOL_NEAR
