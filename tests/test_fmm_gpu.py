"""CUDA FMM (tree, lists, 16 kernels, fused BIE operator) against the reference's golden outputs
and the oracle."""

import numpy as np
import pytest

import ibim
import oracle as O
from test_oracle_golden import KD, bie_densities, fused_to_reference, probe_vector

pytestmark = pytest.mark.gpu
CASES = ["born", "synth30", "p1hje", "synth300"]


def tube_of(ctx, G):
    s = G["surface"]
    return ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], G["params"]["h"])


def kparams(P):
    return ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])


@pytest.mark.parametrize("case", CASES + ["cavity"])
def test_plan_lists_match_reference(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    nodes = plan.lists()
    assert len(nodes) == len(G["tree_level"])
    for i, nd in enumerate(nodes):
        for c in "UVWX":
            p = G[f"tree_{c}_ptr"]
            assert np.array_equal(np.sort(G[f"tree_{c}_idx"][p[i]:p[i + 1]]), nd[c])


@pytest.mark.parametrize("case", CASES)
def test_fused_fmm_matches_16_reference_fmms(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    kp = kparams(P)
    idx = G["sample_idx"]
    for k in range(16):
        if G["fmm16_absmax"][k] == 0:
            continue
        d = np.zeros_like(dens)
        d[KD[k]] = dens[KD[k]]
        v = fused_to_reference(plan.apply(ibim.KERNEL_BIE_FUSED, kp, d), k)
        err = np.abs(v[idx] - G["fmm16_sample"][k]).max() / G["fmm16_absmax"][k]
        assert err < 1e-10, (k, err)


@pytest.mark.parametrize("k", range(16))
def test_single_kernel_api(ctx, golden, k):
    G = golden("synth30")
    P = G["params"]
    s = G["surface"]
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    v = plan.apply(k, kparams(P), dens[KD[k]])
    err = np.abs(v[G["sample_idx"]] - G["fmm16_sample"][k]).max() / G["fmm16_absmax"][k]
    assert err < 1e-10, err


def test_unsupported_kernel_is_rejected(ctx, golden):
    G = golden("born")
    P = G["params"]
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    with pytest.raises(ibim.IbimError) as e:
        plan.apply(42, kparams(P), np.zeros(len(G["surface"])))
    assert e.value.status == ibim.ERR_UNSUPPORTED_KERNEL


@pytest.mark.parametrize("case", ["synth30", "p1hje"])
def test_matvec_matches_oracle(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    x = probe_vector(len(s))
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    y = plan.matvec(kparams(P), x)
    bp = O.bie_params(P["np"], P["maxpoint"], P["maxlevel"], P["restart"], P["maxiter"], P["kappa"], P["dE"], P["dI"],
                      P["tau"], P["tol"], 0)
    yr = O.matvec(s, P["h"], bp, x)
    assert np.abs(y - yr).max() / np.abs(yr).max() < 1e-11


def test_atom_targets_match_oracle(ctx, golden):
    """Targets that are not the sources (polarizeMap's atom centres, electric.cpp:468-478)."""
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    atoms = G["centers"]
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"], targets=atoms)
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    out = plan.apply(ibim.KERNEL_BIE_FUSED, kparams(P), dens)
    T = O.Tree(s[:, :3], atoms, P["maxpoint"], P["maxlevel"])
    ref = T.fmm(P["np"], O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * P["h"]), 16, dens)
    assert np.abs(out - ref).max() / np.abs(ref).max() < 1e-11


def test_rhs_matches_reference(ctx, golden):
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    N = len(s)
    plan = tube_of(ctx, G).plan(P["np"], P["maxpoint"], P["maxlevel"])
    b = plan.rhs(kparams(P), G["centers"], G["charges"])
    idx = G["sample_idx"]
    bs = np.concatenate([b[idx], b[N + idx]])
    assert np.abs(bs - G["rhs_sample"]).max() / np.abs(G["rhs_sample"]).max() < 1e-13
