"""The FP64 operator with its V-list M2L as exact BF16 digit products on the tensor cores
(IBIM_PRECISION_FP64_TC, the mixed path's refinement residual) against the plain FP64 operator.

Only the V-list M2L differs between the two; its digit truncation (a 42-bit cut into 6 digits of
7 bits, or 7 of 6 bits from order 6 up, under power-of-two row and column scales) leaves about
2^-40 of the row-scale x column-scale product per term, so the FMM outputs agree to ~1e-11 of
their magnitude.  Orders 3, 5 (6 digits) and 6 (7 digits) are covered."""

import numpy as np
import pytest

import ibim
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu

TOL = 1e-10  # max-normalised, per output field


def tube_of(ctx, G):
    s = G["surface"]
    return ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], G["params"]["h"])


@pytest.mark.parametrize("case,order", [("born", None), ("synth30", None), ("p1hje", None), ("cavity", None),
                                        ("p1hje", 6), ("synth30", 3)])
def test_sliced_m2l_matches_fp64(ctx, golden, case, order):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    p = order or P["np"]
    t = tube_of(ctx, G)
    a64 = t.plan(p, P["maxpoint"], P["maxlevel"])
    atc = t.plan(p, P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_FP64_TC)
    assert a64.stats()["v_pairs"] > 0  # the sliced contraction runs
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    a = a64.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    b = atc.apply(ibim.KERNEL_BIE_FUSED, kp, dens)
    for o in range(4):
        err = np.abs(a[o] - b[o]).max() / np.abs(a[o]).max()
        assert err < TOL, (o, err)
    x = probe_vector(len(s))
    y64 = a64.matvec(kp, x)
    ytc = atc.matvec(kp, x)
    assert np.linalg.norm(y64 - ytc) / np.linalg.norm(y64) < TOL


@pytest.mark.parametrize("kernel", [ibim.KERNELS.index(k) for k in ("K1x", "K2", "K3xy", "K4z")])
def test_sliced_m2l_single_kernels(ctx, golden, kernel):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    q = np.sin(0.37 * np.arange(len(s))) * s[:, 6]
    a = t.plan(P["np"], P["maxpoint"], P["maxlevel"]).apply(kernel, kp, q)
    b = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_FP64_TC).apply(kernel, kp, q)
    assert np.abs(a - b).max() / np.abs(a).max() < TOL


def test_sliced_gmres_matches_fp64(ctx, golden):
    """GMRES on the sliced operator takes the FP64 path's iterations and reaches its solution."""
    G = golden("synth30")
    P = G["params"]
    s = G["surface"]
    t = tube_of(ctx, G)
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    p64 = t.plan(P["np"], P["maxpoint"], P["maxlevel"])
    ptc = t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=ibim.PRECISION_FP64_TC)
    b = p64.rhs(kp, G["centers"], G["charges"])
    x64, r64 = p64.gmres(kp, b, restart=P["restart"], maxiter=P["maxiter"], tol=P["tol"])
    xtc, rtc = ptc.gmres(kp, b, restart=P["restart"], maxiter=P["maxiter"], tol=P["tol"],
                         precision=ibim.PRECISION_FP64_TC)
    assert rtc["iters"] == r64["iters"]
    assert np.linalg.norm(xtc - x64) / np.linalg.norm(x64) < 1e-9


def test_unknown_precision_rejected(ctx, golden):
    G = golden("born")
    P = G["params"]
    t = tube_of(ctx, G)
    with pytest.raises(ibim.IbimError) as e:
        t.plan(P["np"], P["maxpoint"], P["maxlevel"], precision=7)
    assert e.value.status == ibim.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("case", ["synth30", "p1hje"])
def test_whole_solve_with_sliced_m2l(ctx, golden, case):
    """ibim_config.precision = FP64_TC: FP64 level set and GMRES on the sliced operator reproduce
    the FP64 solve (same iterations, energy to 1e-9)."""
    from conftest import config_for

    G = golden(case)
    P = G["params"]
    r64 = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(P, ibim.PRECISION_FP64))
    rtc = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(P, ibim.PRECISION_FP64_TC))
    assert rtc["n_points"] == r64["n_points"]
    assert rtc["gmres_iters"] == r64["gmres_iters"]
    assert abs(rtc["energy"] - r64["energy"]) <= 1e-9 * abs(r64["energy"])
