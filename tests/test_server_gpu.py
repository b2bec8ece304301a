"""Request loop (ibim_server): concurrent solves admitted by an HBM budget.  Each result is the
same alone and in the mix: FP64 to 1e-10 (only atomic summation order differs), mixed to 1e-6."""

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


def test_budget_serialises_requests(ctx):
    """With a budget below two requests' footprint the loop runs them one at a time."""
    ws = molecules()
    cfgs = [W.config(ibim.PRECISION_MIXED) for W in ws]
    est = [ibim.request_bytes_estimate(c) for c in cfgs]
    budget = 1.01 * max(est)
    srv = ibim.Server(0, slots=3, hbm_budget_bytes=budget)
    try:
        ids = [srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, c) for W, c in zip(ws, cfgs)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert all(r["gmres_status"] == 0 for r in res)
    assert st["peak_bytes"] <= budget
    # in order of submission, each request started after the previous one finished
    assert all(res[k + 1]["latency_ms"] - res[k + 1]["run_ms"] >= res[k]["run_ms"] * 0.99 for k in range(2))


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
