"""Request loop (ibim_server): solves admitted by an HBM budget in two phases, run concurrently
(pool) or in lock-step waves.  Each result is the same alone and in the mix: FP64 to 1e-10 (only
atomic summation order differs), mixed to 1e-6."""

import numpy as np
import pytest

import ibim
import workloads

pytestmark = pytest.mark.gpu

SIZES = [(60, 11), (150, 12), (300, 13)]


def molecules():
    return [workloads.protein(n, seed, h=0.5, order=4) for n, seed in SIZES]


@pytest.mark.parametrize("precision,tol", [(ibim.PRECISION_FP64, 1e-10), (ibim.PRECISION_MIXED, 1e-6)])
def test_results_alone_and_in_the_mix(ctx, precision, tol):
    ws = molecules()
    alone = [ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, W.config(precision)) for W in ws]
    srv = ibim.Server(0, slots=3, hbm_budget_bytes=150e9)
    try:
        ids = [srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, W.config(precision)) for W in ws]
        mix = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["submitted"] == 3 and st["completed"] == 3 and st["in_flight"] == 0 and st["queued"] == 0
    for a, m in zip(alone, mix):
        assert m["n_points"] == a["n_points"]
        assert m["gmres_iters"] == a["gmres_iters"]
        assert abs(m["energy"] - a["energy"]) <= tol * abs(a["energy"])
        assert m["latency_ms"] >= m["run_ms"] > 0


@pytest.mark.parametrize("lockstep", [False, True])
def test_fmm_phase_admitted_by_its_real_size(ctx, lockstep):
    """The FMM phase is admitted by the bytes of the request's own tree (exact operator, node and
    point counts), which here exceed what a point count guessed from the grid (a twentieth of the
    cells) would give: with a budget that fits one FMM phase but not two, the peak admitted bytes
    stay within the budget and reach the real size, and every result is right."""
    ws = molecules()
    cfgs = [W.config(ibim.PRECISION_MIXED) for W in ws]
    alone = [ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, c) for W, c in zip(ws, cfgs)]
    real = [ibim.fmm_bytes_estimate(c, a["n_points"]) for c, a in zip(cfgs, alone)]
    guessed = [ibim.fmm_bytes_estimate(c, int(np.prod(list(c.n)) / 20)) for c in cfgs]
    assert all(r > g for r, g in zip(real, guessed))
    budget = 1.5 * max(real)
    srv = ibim.Server(0, slots=3, hbm_budget_bytes=budget, lockstep=lockstep, max_wave=4)
    try:
        ids = [srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, c) for W, c in zip(ws, cfgs)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == 3 and st["in_flight"] == 0
    assert 0.5 * max(real) <= st["peak_bytes"] <= budget
    for r, a in zip(res, alone):
        assert r["gmres_status"] == 0
        assert abs(r["energy"] - a["energy"]) <= 1e-6 * abs(a["energy"])


def test_lockstep_loop_matches_alone_and_batches(ctx):
    """Lock-step loop: requests submitted together are solved in shared waves, each result the one
    its own solve gives (mixed path, 1e-6)."""
    ws = molecules()
    cfgs = [W.config(ibim.PRECISION_MIXED) for W in ws]
    alone = [ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, c) for W, c in zip(ws, cfgs)]
    srv = ibim.Server(0, slots=3, hbm_budget_bytes=150e9, lockstep=True, max_wave=8)
    try:
        ids = [srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, c) for W, c in zip(ws, cfgs)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == 3 and 1 <= st["waves"] <= 3
    for r, a in zip(res, alone):
        assert r["n_points"] == a["n_points"]
        assert abs(r["energy"] - a["energy"]) <= 1e-6 * abs(a["energy"])
        assert r["latency_ms"] >= r["run_ms"] > 0


def test_lockstep_loop_rejects_fp64_requests(ctx):
    W = molecules()[0]
    srv = ibim.Server(0, slots=2, hbm_budget_bytes=150e9, lockstep=True)
    try:
        rid = srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_FP64))
        with pytest.raises(ibim.IbimError) as e:
            srv.wait(rid)
        assert e.value.status == ibim.ERR_INVALID_ARGUMENT
        ok = srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_MIXED))
        assert srv.wait(ok)["gmres_status"] == 0
    finally:
        srv.close()


def test_failed_request_reports_its_error(ctx):
    W = molecules()[0]
    cfg = W.config(ibim.PRECISION_FP64)
    cfg.np = 1  # outside [2, 8]
    srv = ibim.Server(0, slots=2, hbm_budget_bytes=150e9)
    try:
        rid = srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, cfg)
        with pytest.raises(ibim.IbimError) as e:
            srv.wait(rid)
        assert e.value.status == ibim.ERR_INVALID_ARGUMENT
        ok = srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_FP64))
        assert srv.wait(ok)["gmres_status"] == 0
    finally:
        srv.close()
