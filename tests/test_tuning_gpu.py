"""Tuned launch parameters change only the partition of the work: a solve under extreme rows
(other launch form, small and large segments) gives the default's energy within 1e-7 (atomic
accumulation order), and the autotuner returns a valid row."""

import os

import pytest

import ibim
import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_table():
    yield
    lib = ibim.lib()
    lib.ibim_tuning_clear()
    if os.path.exists(ibim.TUNING_TABLE):
        lib.ibim_tuning_load(ibim.TUNING_TABLE.encode())


@pytest.mark.parametrize("row", [(1 << 15, 1 << 13, 4), (1 << 18, 1 << 16, 2), (1 << 16, 1 << 15, 0),
                                 (1 << 17, 1 << 14, 6), (1 << 17, 1 << 14, 7)])
def test_solve_under_other_launch_parameters(ctx, restore_table, row):
    W = workloads.protein(400, 9_000_400, h=0.5, order=5)
    cfg = W.config(ibim.PRECISION_MIXED)
    lib = ibim.lib()
    lib.ibim_tuning_clear()
    ref = ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, cfg)
    assert lib.ibim_tuning_set(5, 0, *row) == ibim.OK
    r = ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, cfg)
    assert r["gmres_status"] == 0
    assert abs(r["energy"] - ref["energy"]) <= 1e-7 * abs(ref["energy"])


def test_autotune_returns_a_row(ctx, restore_table):
    W = workloads.protein(120, 9_000_120, h=0.5, order=4, maxpoint=64)
    cfg = W.config(ibim.PRECISION_MIXED)
    r = ctx.autotune(W.mol.centers, W.mol.charges, W.mol.radii, cfg, reps=2, install_min_points=0)
    # the default, three other launch forms (4, and the CTA-pair forms 6 and 7), three sizes of
    # each near-field segment; two more when a winner other than the defaults is re-measured
    assert r["candidates"] in (10, 12) and r["points"] > 0
    assert r["tc_form"] in (2, 4, 6, 7) and r["best_ms"] <= r["default_ms"]
    assert ibim.tuning_get(4, r["points"]) == dict(near_seg_pairs=r["near_seg_pairs"],
                                                   nearff_seg_pairs=r["nearff_seg_pairs"], tc_form=r["tc_form"])
