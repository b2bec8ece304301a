"""The oracle (C restatement of the reference, oracle/ibim_oracle.c) against the reference's own
outputs (tests/golden/*.npz from tests/golden/make_golden.py).  CPU only."""

import numpy as np
import pytest

import oracle as O
from conftest import grid_stats

LS_CASES = ["born", "synth30", "cavity", "p1hje", "synth300"]
KD = [0, 1, 2, 3, 0, 1, 2, 0, 1, 2, 1, 2, 0, 3, 3, 3]
K3F1 = [0, 1, 2, 0, 1, 2, 0, 1, 2]
K3F2 = [0, 1, 2, 1, 2, 0, 1, 2, 0]


def fused_to_reference(out4, k):
    """Reference kernel k from a fused FMM whose only non-zero density is slot KD[k]."""
    if k <= 2:
        return out4[0]
    if k == 3:
        return -out4[0]
    if k >= 13:
        return -out4[1 + k - 13]
    b = KD[k]
    a = K3F1[k - 4] if K3F2[k - 4] == b else K3F2[k - 4]
    return out4[1 + a]


def probe_vector(N):
    i = np.arange(N)
    return np.concatenate([np.sin(0.37 * i) + 0.25, np.cos(0.11 * i) - 0.5])


def bie_densities(s, h, phi):
    N = len(s)
    w = s[:, 6] * h ** 3
    return np.stack([phi[:N] * s[:, 3] * w, phi[:N] * s[:, 4] * w, phi[:N] * s[:, 5] * w, phi[N:] * w])


@pytest.mark.parametrize("case", LS_CASES)
def test_levelset_and_surface(golden, case):
    G = golden(case)
    P = G["params"]
    g, steps = O.levelset(G["centers"], G["radii"], P["lo"], P["h"], P["n"], reinit_t=P["reinit_t"],
                          thickness=P["thickness"], thres=P["thres"], init=P["init"])
    st = grid_stats(g)
    np.testing.assert_allclose(st, G["gridstats_reinit2"], rtol=1e-11)
    s, inc = O.surface(g, P["lo"], P["h"], P["thickness"])
    assert inc == P["scalars"].get("INCLUSION", 0)
    assert len(s) == len(G["surface"])
    np.testing.assert_allclose(s, G["surface"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("case", LS_CASES)
def test_tree_lists(golden, case):
    G = golden(case)
    P = G["params"]
    pts = G["surface"][:, :3]
    T = O.Tree(pts, pts, P["maxpoint"], P["maxlevel"])
    assert T.nnodes == len(G["tree_level"])
    for i in range(T.nnodes):
        ints, cr = T.node(i)
        ref = [G["tree_level"][i], G["tree_parent"][i], G["tree_leaf"][i], G["tree_empty"][i], G["tree_nsrc"][i],
               G["tree_ntgt"][i]]
        assert list(ints) == [int(v) for v in ref]
        np.testing.assert_allclose(cr[:3], G["tree_center"][i], rtol=0, atol=1e-12)
        L = T.lists(i)
        for w, c in enumerate("UVWX"):
            p = G[f"tree_{c}_ptr"]
            assert np.array_equal(np.sort(G[f"tree_{c}_idx"][p[i]:p[i + 1]]), L[w])


@pytest.mark.parametrize("case", ["born", "synth30", "p1hje"])
def test_fmm_16_kernels(golden, case):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    N = len(s)
    h = P["h"]
    pts = s[:, :3]
    T = O.Tree(pts, pts, P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, h, probe_vector(N))
    kp = O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * h)
    idx = G["sample_idx"]
    full = T.fmm(P["np"], kp, 16, dens)
    for k in range(16):
        if G["fmm16_absmax"][k] == 0:
            continue  # K2 / K3 vanish at kappa = 0
        d = np.zeros_like(dens)
        d[KD[k]] = dens[KD[k]]
        v = fused_to_reference(T.fmm(P["np"], kp, 16, d), k)
        err = np.abs(v[idx] - G["fmm16_sample"][k]).max() / G["fmm16_absmax"][k]
        assert err < 1e-12, (k, err)
    assert np.all(np.isfinite(full))


def fused_field_of_reference(G, f):
    """Field f of the fused FMM with all four densities set, as the signed sum of the reference's
    16 single-kernel FMM samples (F = K1 m - K2 psi, G_a = sum_b K3ab m_b - K4a psi)."""
    total = np.zeros(G["fmm16_sample"].shape[1])
    for k in range(16):
        if k <= 2:
            fk, sg = 0, 1.0
        elif k == 3:
            fk, sg = 0, -1.0
        elif k >= 13:
            fk, sg = 1 + k - 13, -1.0
        else:
            b = KD[k]
            a = K3F1[k - 4] if K3F2[k - 4] == b else K3F2[k - 4]
            fk, sg = 1 + a, 1.0
        if fk == f:
            total += sg * G["fmm16_sample"][k]
    return total


def test_fused_fmm_on_benchmark_shaped_protein(golden):
    """One fused FMM of the oracle on the 300-atom protein (p = 5, leaf 128, kappa 0.125, six tree
    levels, an X list) against the sums of the reference's 16 single-kernel FMMs."""
    G = golden("synth300")
    P = G["params"]
    s = G["surface"]
    pts = s[:, :3]
    T = O.Tree(pts, pts, P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    kp = O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * P["h"])
    out = T.fmm(P["np"], kp, 16, dens)
    idx = G["sample_idx"]
    for f in range(4):
        ref = fused_field_of_reference(G, f)
        assert np.abs(out[f][idx] - ref).max() / np.abs(ref).max() < 1e-12, f


def test_fmm_at_chosen_targets(golden):
    """The oracle's FMM evaluated for chosen targets only (the downward pass for their leaves and
    those leaves' ancestors) equals the full FMM there bit for bit (1hje), and on the 300-atom
    protein it matches the sums of the reference's 16 single-kernel FMMs at the golden sample."""
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    T = O.Tree(s[:, :3], s[:, :3], P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    kp = O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * P["h"])
    full = T.fmm(P["np"], kp, 16, dens)
    sel = np.arange(3, len(s), 97)
    at, nleaf = T.fmm_at(P["np"], kp, 16, dens, sel)
    assert 0 < nleaf < T.nnodes
    assert np.array_equal(at, full[:, sel])
    G = golden("synth300")
    P = G["params"]
    s = G["surface"]
    T = O.Tree(s[:, :3], s[:, :3], P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, P["h"], probe_vector(len(s)))
    kp = O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * P["h"])
    idx = G["sample_idx"]
    at, _ = T.fmm_at(P["np"], kp, 16, dens, idx)
    for f in range(4):
        ref = fused_field_of_reference(G, f)
        assert np.abs(at[f] - ref).max() / np.abs(ref).max() < 1e-12, f


def test_fmm_scalar_kernel(golden):
    G = golden("born")
    P = G["params"]
    s = G["surface"]
    N = len(s)
    h = P["h"]
    T = O.Tree(s[:, :3], s[:, :3], P["maxpoint"], P["maxlevel"])
    dens = bie_densities(s, h, probe_vector(N))
    kp = O.KParams(P["kappa"], P["dE"], P["dI"], P["tau"] * h)
    v = T.fmm(P["np"], kp, 0, dens[0])[0]
    err = np.abs(v[G["sample_idx"]] - G["fmm16_sample"][0]).max() / G["fmm16_absmax"][0]
    assert err < 1e-12


@pytest.mark.parametrize("case", ["born", "p1hje"])
def test_solve_energy(golden, case):
    G = golden(case)
    P = G["params"]
    s = G["surface"]
    N = len(s)
    bp = O.bie_params(P["np"], P["maxpoint"], P["maxlevel"], P["restart"], P["maxiter"], P["kappa"], P["dE"], P["dI"],
                      P["tau"], P["tol"], 0)
    b = O.rhs(s, G["centers"], G["charges"], bp)
    idx = G["sample_idx"]
    bs = np.concatenate([b[idx], b[N + idx]])
    assert np.abs(bs - G["rhs_sample"]).max() / np.abs(G["rhs_sample"]).max() < 1e-13
    r = O.solve(s, P["h"], G["centers"], G["charges"], bp)
    assert r["rc"] == 0
    assert r["matvecs"] == int(P["scalars"]["REF_MATVECS"])
    x = r["x"]
    ref = G["solution_sample"]
    assert np.abs(np.concatenate([x[idx], x[N + idx]]) - ref).max() / np.abs(ref).max() < 1e-12
    pot = G["atom_potential"]
    assert np.abs(r["atom_pot"] - pot).max() / np.abs(pot).max() < 1e-12
    E = P["scalars"]["REF_ENERGY_RESTATED"]
    assert abs(r["energy"] - E) / abs(E) < 1e-12


def test_reference_structured_matvec_equals_fused(golden):
    """Mode 1 (16 scalar FMMs, a tree per FMM, as electric.cpp does) equals the fused mode."""
    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    x = probe_vector(len(s))
    args = (P["np"], P["maxpoint"], P["maxlevel"], P["restart"], P["maxiter"], P["kappa"], P["dE"], P["dI"], P["tau"],
            P["tol"])
    y0 = O.matvec(s, P["h"], O.bie_params(*args, 0), x)
    y1 = O.matvec(s, P["h"], O.bie_params(*args, 1), x)
    assert np.abs(y0 - y1).max() / np.abs(y1).max() < 1e-13


def test_born_energy_near_analytic(golden):
    """The reference's Born ion energy is within its first-order discretisation error of Born."""
    G = golden("born")
    E = G["params"]["scalars"]["REF_ENERGY_RESTATED"]
    born = -(1.0 / (8 * np.pi * 2.0)) * (1.0 - 1.0 / 80.0)
    assert abs(E - born) / abs(born) < 0.05
