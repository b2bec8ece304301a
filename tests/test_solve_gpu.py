"""GMRES, polarization energy and the whole path against the reference's golden outputs."""

import os
import tempfile

import numpy as np
import pytest

import ibim
from conftest import config_for

pytestmark = pytest.mark.gpu


def tube_of(ctx, G):
    s = G["surface"]
    return ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], G["params"]["h"])


@pytest.mark.parametrize("case", ["born", "synth30", "p1hje", "synth300"])
def test_electric_matches_reference(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    r = tube_of(ctx, G).electric(G["centers"], G["charges"], config_for(P), want_x=True)
    E = P["scalars"]["REF_ENERGY_RESTATED"]
    assert r["gmres_status"] == 0
    assert abs(r["energy"] - E) / abs(E) < 1e-9
    pot = G["atom_potential"]
    assert np.abs(r["atom_potential"] - pot).max() / np.abs(pot).max() < 1e-9
    N = len(G["surface"])
    idx = G["sample_idx"]
    x = np.concatenate([r["x"][idx], r["x"][N + idx]])
    assert np.abs(x - G["solution_sample"]).max() / np.abs(G["solution_sample"]).max() < 1e-8
    # the reference also applies the operator to x0 = 0 (gmres.cpp:92); that product is zero
    assert r["gmres_iters"] == int(P["scalars"]["REF_MATVECS"]) - 1


# Tube points of the Born ion that lie on the sphere's symmetry planes sit exactly on the octree's
# split planes (x < centre ? 0 : 1, bbfmm.cpp:108-111); ulp-level rounding differences between
# the reference's x86 -Ofast build and the GPU pick either side, which changes the tree and so
# the FMM approximation (not the tube: it agrees to 1e-9).  Asymmetric molecules have no such
# points.  Against the oracle run on the GPU's own tube the trees are identical.
FULL_TOL = {"born": 1e-4, "synth30": 1e-7, "p1hje": 1e-7, "synth300": 1e-6}


@pytest.mark.parametrize("case", ["born", "synth30", "p1hje", "synth300"])
def test_full_solve_matches_reference(ctx, golden, case):
    G = golden(case)
    P = G["params"]
    r = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(P))
    assert r["n_points"] == len(G["surface"])
    E = P["scalars"]["REF_ENERGY_RESTATED"]
    assert abs(r["energy"] - E) / abs(E) < FULL_TOL[case]
    assert abs(r["area"] - (G["surface"][:, 6] * P["h"] ** 3).sum()) < 1e-9 * r["area"]


@pytest.mark.parametrize("case", ["born", "p1hje"])
def test_full_solve_matches_oracle_on_own_tube(ctx, golden, case):
    import oracle as O

    G = golden(case)
    P = G["params"]
    cfg = config_for(P)
    r = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    g, _ = ctx.levelset(G["centers"], G["radii"], cfg)
    s = g.surface(P["thickness"]).surface7()
    bp = O.bie_params(P["np"], P["maxpoint"], P["maxlevel"], P["restart"], P["maxiter"], P["kappa"], P["dE"], P["dI"],
                      P["tau"], P["tol"], 0)
    ro = O.solve(s, P["h"], G["centers"], G["charges"], bp)
    assert abs(r["energy"] - ro["energy"]) / abs(ro["energy"]) < 1e-9


def test_born_analytic(ctx, golden):
    G = golden("born")
    r = ctx.solve(G["centers"], G["charges"], G["radii"], config_for(G["params"]))
    born = -(1.0 / (8 * np.pi * 2.0)) * (1.0 - 1.0 / 80.0)
    assert abs(r["energy"] - born) / abs(born) < 0.05


def test_repeat_solves_agree(ctx, golden):
    G = golden("p1hje")
    cfg = config_for(G["params"])
    a = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)["energy"]
    b = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)["energy"]
    assert abs(a - b) <= 1e-12 * abs(a)


def test_pqr_entry_point(ctx, golden):
    G = golden("p1hje")
    import synth

    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "m.pqr")
        synth.Molecule(G["centers"], G["charges"], G["radii"]).to_pqr(path)
        r = ctx.solve_pqr(path, config_for(G["params"]))
    E = G["params"]["scalars"]["REF_ENERGY_RESTATED"]
    assert abs(r["energy"] - E) / abs(E) < 1e-7


def test_error_statuses(ctx, golden):
    G = golden("born")
    cfg = config_for(G["params"])
    cfg.np = 1
    with pytest.raises(ibim.IbimError) as e:
        ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    assert e.value.status == ibim.ERR_INVALID_ARGUMENT
    with pytest.raises(ibim.IbimError) as e:
        ctx.solve_pqr("/nonexistent/file.pqr", config_for(G["params"]))
    assert e.value.status == ibim.ERR_IO


def test_gmres_nonconvergence_reported(ctx, golden):
    G = golden("synth30")
    cfg = config_for(G["params"])
    cfg.maxiter = 2
    r = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    assert r["gmres_status"] == 1 and r["gmres_iters"] == 2


def test_born_gap_comes_from_points_on_split_planes(ctx, golden):
    """The Born ion's whole-path energy differs from the reference's by ~3e-5 while its tube agrees
    to 1e-9.  The octree splits at geometric centres of the points' bounding box (bbfmm.cpp:44-
    108, `x < centre ? 0 : 1`), and the symmetric ion puts tube points on those planes, where a
    1e-9 difference picks the other side.  Snapping only those points (and the six points that
    fix the bounding box) to the reference's coordinates gives the reference's tree, and the
    energy then agrees to 1e-6: the gap comes only from the split-plane points."""
    G = golden("born")
    P = G["params"]
    cfg = config_for(P)
    g, _ = ctx.levelset(G["centers"], G["radii"], cfg)
    ours = g.surface(P["thickness"]).surface7()
    g.close()
    ref = G["surface"]
    assert ours.shape == ref.shape
    assert np.abs(ours - ref).max() < 1e-9
    # split planes of the reference's tree: the centres of its internal nodes, per axis
    internal = G["tree_leaf"] == 0
    near = np.zeros(len(ref), bool)
    for a in range(3):
        planes = np.unique(G["tree_center"][internal, a])
        k = np.clip(np.searchsorted(planes, ref[:, a]), 1, len(planes) - 1)
        d = np.minimum(np.abs(ref[:, a] - planes[k - 1]), np.abs(ref[:, a] - planes[k]))
        near |= d < 1e-7
    for a in range(3):  # the points that fix the bounding box (the root's centre and radius)
        near |= (ref[:, a] - ref[:, a].min() < 1e-7) | (ref[:, a].max() - ref[:, a] < 1e-7)
    snapped = ours.copy()
    snapped[near] = ref[near]
    E = P["scalars"]["REF_ENERGY_RESTATED"]

    def energy(s7):
        t = ctx.tube(s7[:, :3], s7[:, 3:6], s7[:, 6], P["h"])
        r = t.electric(G["centers"], G["charges"], cfg)
        t.close()
        return r["energy"]

    e_ours, e_snap = energy(ours), energy(snapped)
    assert abs(e_snap - E) / abs(E) < 1e-6, (e_ours, e_snap, E, int(near.sum()))
    assert abs(e_ours - E) / abs(E) < FULL_TOL["born"]
    # the ion's tube points come from lattice points, so whole grid lines lie on the planes: about
    # an eighth of the points are within 1e-7 of one, the rest land where the reference puts them
    assert near.sum() < 0.2 * len(ref), near.sum()


def test_empty_tube_is_an_error_and_the_context_stays_usable(ctx, golden):
    """An atom far outside the grid leaves the level set without tube points: the solve reports
    an invalid argument before any launch over the (empty) tube, and the same context then solves
    normally."""
    G = golden("born")
    cfg = config_for(G["params"])
    with pytest.raises(ibim.IbimError) as e:
        ctx.solve(np.array([[1000.0, 1000.0, 1000.0]]), np.ones(1), np.full(1, 2.0), cfg)
    assert e.value.status == ibim.ERR_INVALID_ARGUMENT
    r = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    E = G["params"]["scalars"]["REF_ENERGY_RESTATED"]
    assert abs(r["energy"] - E) / abs(E) < FULL_TOL["born"]
