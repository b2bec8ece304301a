"""Mixed-precision path (FP32 FMM inside FP64 iterative refinement) against the FP64 path."""

import numpy as np
import pytest

import ibim
from conftest import config_for
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu


def tube_of(ctx, G):
    s = G["surface"]
    return ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], G["params"]["h"])


@pytest.mark.parametrize("case", ["synth30", "p1hje", "cavity"])
def test_mixed_fmm_close_to_fp64(ctx, golden, case):
    """FP32 near and far field: same approximation, FP32 rounding only (~1e-6 relative)."""
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    p64 = t.plan(P["np"], P["maxpoint"], P["maxlevel"])
    p32 = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = p64.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = p32.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 2e-5, o
    x = probe_vector(len(s))
    y64 = p64.matvec(kp, x)
    y32 = p32.matvec(kp, x)
    assert np.linalg.norm(y64 - y32) / np.linalg.norm(y64) < 1e-6


def test_mixed_atom_targets(ctx, golden):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = t.plan(P["np"], P["maxpoint"], P["maxlevel"], targets=G["centers"]).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = t.plan(P["np"], P["maxpoint"], P["maxlevel"], targets=G["centers"],
               precision=ibim.PRECISION_MIXED).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    assert np.abs(a - b).max() / np.abs(a).max() < 2e-5


@pytest.mark.parametrize("case", ["born", "synth30", "p1hje", "synth300"])
def test_mixed_energy_within_1e4_of_fp64(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    t = tube_of(ctx, G)
    r64 = t.electric(G["centers"], G["charges"], config_for(P, ibim.PRECISION_FP64))
    r32 = t.electric(G["centers"], G["charges"], config_for(P, ibim.PRECISION_MIXED))
    rel = abs(r32["energy"] - r64["energy"]) / abs(r64["energy"])
    assert rel < 1e-4, rel
    assert r32["gmres_status"] == 0
    assert r32["residual"] < P["tol"]
    assert r32["matvecs_fp64"] >= 1


def test_mixed_full_solve(ctx, golden):
    G = golden("synth30")
    P = G["params"]
    r64 = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(P, ibim.PRECISION_FP64))
    r32 = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(P, ibim.PRECISION_MIXED))
    assert abs(r32["energy"] - r64["energy"]) / abs(r64["energy"]) < 1e-4


@pytest.mark.parametrize("case", ["synth30", "cavity"])
def test_mixed_levelset_close_to_fp64(ctx, golden, case):
    """FP32 grid and WENO arithmetic: the interface region agrees with the FP64 grid to ~1e-5."""
    G = golden(case)
    P = G["params"]
    g64, s64 = ctx.levelset(G["centers"], G["radii"], config_for(P, ibim.PRECISION_FP64))
    g32, s32 = ctx.levelset(G["centers"], G["radii"], config_for(P, ibim.PRECISION_MIXED))
    a = g64.download()
    b = g32.download()
    near = np.abs(a) < (P["thickness"] + 2) * P["h"]
    assert np.abs(a - b)[near].max() < 1e-4
    t64 = g64.surface(P["thickness"])
    t32 = g32.surface(P["thickness"])
    assert abs(len(t64) - len(t32)) <= max(2, 0.002 * len(t64))
    assert abs(t64.inclusion - t32.inclusion) <= max(2, 0.01 * max(1, t64.inclusion))


@pytest.mark.parametrize("case", ["synth30", "p1hje"])
def test_mixed_rhs_close_to_fp64(ctx, golden, case):
    """FP32 load (electric.cpp:395-412) with compensated sums: ~1e-7 of the FP64 right-hand side."""
    G = golden(case)
    P = G["params"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    b64 = t.plan(P["np"], P["maxpoint"], P["maxlevel"]).rhs(kp, G["centers"], G["charges"])
    b32 = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED).rhs(kp, G["centers"],
                                                                                            G["charges"])
    n = len(b64) // 2
    for part in (slice(0, n), slice(n, 2 * n)):
        assert np.abs(b32[part] - b64[part]).max() <= 2e-6 * np.abs(b64[part]).max()


@pytest.mark.parametrize("order", [3, 6])
def test_mixed_fmm_other_orders(ctx, golden, order):
    """The tensor-core contraction at other operator sizes (4p^3 = 108: one row tile; 864: seven
    row tiles in two CTA row groups of 4 and 3)."""
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = t.plan(order, P["maxpoint"], P["maxlevel"]).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = t.plan(order, P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED).apply(ibim.KERNEL_BIE_FUSED, kp,
                                                                                          dens)
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 2e-5, o


def test_mixed_plan_follows_kernel_parameter_changes(ctx, golden):
    """The tensor-core operator images are keyed on the kernel parameters: a second kappa on the
    same plan re-cuts them (FP32 and digit images alike)."""
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    p64 = t.plan(P["np"], P["maxpoint"], P["maxlevel"])
    p32 = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_MIXED)
    ptc = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_FP64_TC)
    for kappa in (P["kappa"], 0.4, P["kappa"]):
        kp = ibim.kernel_params(kappa, P["dE"], P["dI"], P["tau"])
        a = p64.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
        b = p32.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
        c = ptc.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
        for o in range(4):
            assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 2e-5, (kappa, o)
            assert np.abs(a[o] - c[o]).max() / np.abs(a[o]).max() < 1e-10, (kappa, o)


@pytest.mark.parametrize("shift", [0.1, 0.37])
def test_mixed_near_field_decides_the_cutoff_like_fp64(ctx, shift):
    """Points on a lattice of spacing h (offset by a value FP64 cannot hold exactly) put thousands
    of pairs within rounding of the cutoff r = tau h: the FP32 near field must decide each of them
    as the FP64 kernel does (a pair decided the other way changes its target by O(1))."""
    h = 0.5
    g = np.arange(16) * h + shift
    X, Y, Z = np.meshgrid(g, g, g[:6], indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    rng = np.random.default_rng(3)
    nrm = rng.normal(size=pts.shape)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    w = 1.0 + 0.1 * rng.random(len(pts))
    t = ctx.tube(pts, nrm, w, h)
    kp = ibim.kernel_params(0.1, 80.0, 1.0, 1.0)  # tau = 1: cutoff at exactly the lattice spacing
    dens = np.stack([np.sin(0.3 * np.arange(len(pts)) + k) for k in range(4)])
    a = t.plan(4, 64, 1).apply(ibim.KERNEL_BIE_FUSED, kp, dens)  # level 1: near field only
    b = t.plan(4, 64, 1, precision=ibim.PRECISION_MIXED).apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    for o in range(4):
        assert np.abs(a[o] - b[o]).max() / np.abs(a[o]).max() < 2e-5, o
