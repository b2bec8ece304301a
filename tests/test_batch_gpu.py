"""Many molecules in lock-step waves (ibim_batch_solve): one merged plan per wave, one launch per
FMM stage for all of its molecules, GMRES advanced together.  Each molecule's energy must be the
one its own solve gives (the same mixed-precision path), within 1e-6, and the FP64 path's within
the metric's 1e-4; kappa differs per molecule, so the near-field kernels' per-molecule constants
are exercised.  The operator batched is dmapping (electric.cpp:294-388)."""

import numpy as np
import pytest

import ibim
import workloads

pytestmark = pytest.mark.gpu

SIZES = [(40, 0.0), (75, 0.05), (120, 0.125), (30, 0.15), (200, 0.1), (60, 0.08)]


def molecules(order=4, maxpoint=64):
    ws = [workloads.protein(n, 7_000_000 + k, h=0.5, order=order, maxpoint=maxpoint, kappa=kap)
          for k, (n, kap) in enumerate(SIZES)]
    return ws, [(w.mol.centers, w.mol.charges, w.mol.radii) for w in ws], \
        [w.config(ibim.PRECISION_MIXED) for w in ws]


@pytest.fixture(scope="module")
def solo(ctx):
    ws, mols, cfgs = molecules()
    return [ctx.solve(*m, c) for m, c in zip(mols, cfgs)]


@pytest.mark.parametrize("max_wave", [4, 6])
def test_batch_matches_solo_solves(ctx, solo, max_wave):
    ws, mols, cfgs = molecules()
    res, st, info = ctx.batch_solve(mols, cfgs, max_wave=max_wave, workers=3)
    assert st == [0] * len(mols)
    assert info["waves"] == (2 if max_wave == 4 else 1)
    assert info["largest_wave"] == min(max_wave, len(mols))
    for r, s in zip(res, solo):
        assert r["gmres_status"] == 0 and r["residual"] < 1e-6
        assert r["n_points"] == s["n_points"] and abs(r["area"] - s["area"]) <= 1e-12 * s["area"]
        assert abs(r["energy"] - s["energy"]) <= 1e-6 * abs(s["energy"]), (r["energy"], s["energy"])
        # the same Arnoldi steps give or take one (reductions of another shape near the threshold)
        assert abs(r["gmres_iters"] - s["gmres_iters"]) <= 1
    # a merged matvec serves every molecule of the wave
    assert info["merged_mixed_matvecs"] < sum(r["matvecs"] - r["matvecs_fp64"] for r in res)


def test_batch_energy_within_tolerance_of_fp64(ctx):
    ws, mols, cfgs = molecules()
    res, st, _ = ctx.batch_solve(mols[:3], cfgs[:3], max_wave=3, workers=2)
    for w, m, r in zip(ws[:3], mols[:3], res):
        e64 = ctx.solve(*m, w.config(ibim.PRECISION_FP64))["energy"]
        assert abs(r["energy"] - e64) <= 1e-4 * abs(e64)


def test_batch_budget_smaller_than_a_molecule_runs_one_at_a_time(ctx, solo):
    ws, mols, cfgs = molecules()
    res, st, info = ctx.batch_solve(mols[:3], cfgs[:3], max_wave=8, hbm_budget_bytes=1.0, workers=2)
    assert st == [0, 0, 0]
    assert info["waves"] == 3 and info["largest_wave"] == 1
    for r, s in zip(res, solo[:3]):
        assert abs(r["energy"] - s["energy"]) <= 1e-6 * abs(s["energy"])


def test_batch_rejects_mixed_shapes(ctx):
    ws, mols, cfgs = molecules()
    cfgs[1].np = 5
    with pytest.raises(ibim.IbimError) as e:
        ctx.batch_solve(mols[:2], cfgs[:2])
    assert e.value.status == ibim.ERR_INVALID_ARGUMENT


def test_single_molecule_batch(ctx, solo):
    """A batch of one molecule is one wave of one: the molecule's own solve."""
    ws, mols, cfgs = molecules()
    res, st, info = ctx.batch_solve(mols[:1], cfgs[:1], max_wave=6, workers=1, wave_slots=1)
    assert st == [0] and info["waves"] == 1 and info["largest_wave"] == 1
    assert abs(res[0]["energy"] - solo[0]["energy"]) <= 1e-6 * abs(solo[0]["energy"])
