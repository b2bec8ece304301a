"""Parity at the benchmark's own size: the 2,000-atom synthetic protein (h = 0.5 A, a 144 x 145 x 150
grid, 408,726 tube points, p = 5, leaves of at most 128 points, 15,193 tree nodes).

* The FP64 level set and tube against the oracle's: the same points, normals and weights.
* The plan's octree lists against the oracle's tree, node by node.
* One fused FMM (the 4 x 4 BIE block of the 16 reference kernels) on the oracle's tube against
  the oracle's FMM, for the FP64 operator, the FP64-class one (digit-sliced tensor-core M2L and
  float-float near field: the mixed path's refinement residual) and the mixed one (scaled FP16
  tensor-core M2L, FP32 near field).  The oracle evaluates the downward pass for the leaves of a
  spread sample of targets and their ancestors (its FMM at those targets, bit for bit).

The oracle's full-size level set and this FMM take a few seconds on 16 host cores."""

import numpy as np
import pytest

import ibim
import oracle as O
import workloads
from test_oracle_golden import bie_densities, probe_vector

pytestmark = pytest.mark.gpu

# operator tolerances, relative to the largest field value at the sampled targets
# (measured on GB300: 1.6e-15, 8.4e-13 and 1.0e-6)
FMM_TOL = {ibim.PRECISION_FP64: 1e-12, ibim.PRECISION_FP64_TC: 1e-11, ibim.PRECISION_MIXED: 1e-5}


@pytest.fixture(scope="module")
def bench_case(ctx):
    W = workloads.protein(2000, 1_000_000, 0.5, 5)
    cfg = W.config(ibim.PRECISION_FP64)
    lo = [cfg.lo[i] for i in range(3)]
    n = [cfg.n[i] for i in range(3)]
    g_ref, steps = O.levelset(W.mol.centers, W.mol.radii, lo, cfg.h, n, band=cfg.band, init=cfg.init,
                              probe=cfg.probe, reinit_t=cfg.reinit_t, thickness=cfg.thickness, thres=cfg.thres)
    s_ref, inc_ref = O.surface(g_ref, lo, cfg.h, cfg.thickness)
    return W, cfg, s_ref, inc_ref, steps


def test_levelset_and_tube_match_oracle(ctx, bench_case):
    W, cfg, s_ref, inc_ref, steps = bench_case
    g, st = ctx.levelset(W.mol.centers, W.mol.radii, cfg)
    t = g.surface(cfg.thickness)
    s = t.surface7()
    assert list(st) == list(steps)
    assert t.inclusion == inc_ref
    assert len(s) == len(s_ref) == 408726
    assert np.abs(s - s_ref).max() < 1e-9


def test_plan_lists_match_oracle_tree(ctx, bench_case):
    W, cfg, s_ref, _, _ = bench_case
    plan = ctx.tube(s_ref[:, :3], s_ref[:, 3:6], s_ref[:, 6], cfg.h).plan(W.np_, W.maxpoint, W.maxlevel)
    nodes = plan.lists()
    T = O.Tree(s_ref[:, :3], s_ref[:, :3], W.maxpoint, W.maxlevel)
    assert len(nodes) == T.nnodes == 15193
    for i, nd in enumerate(nodes):
        ints, _ = T.node(i)
        assert [nd["level"], nd["parent"], nd["leaf"], nd["empty"], nd["nsrc"]] == [int(x) for x in ints[:5]], i
        ref = T.lists(i)
        for w, c in enumerate("UVWX"):
            assert np.array_equal(np.sort(ref[w]), np.sort(nd[c])), (i, c)


@pytest.mark.parametrize("precision", [ibim.PRECISION_FP64, ibim.PRECISION_FP64_TC, ibim.PRECISION_MIXED])
def test_fused_fmm_matches_oracle(ctx, bench_case, precision):
    W, cfg, s_ref, _, _ = bench_case
    N = len(s_ref)
    dens = bie_densities(s_ref, cfg.h, probe_vector(N))
    plan = ctx.tube(s_ref[:, :3], s_ref[:, 3:6], s_ref[:, 6], cfg.h).plan(W.np_, W.maxpoint, W.maxlevel,
                                                                             precision=precision)
    out = plan.apply(ibim.KERNEL_BIE_FUSED, ibim.kernel_params(W.kappa, W.dE, W.dI, W.tau), dens)
    sel = np.arange(7, N, 1500)
    T = O.Tree(s_ref[:, :3], s_ref[:, :3], W.maxpoint, W.maxlevel)
    ref, nleaf = T.fmm_at(W.np_, O.KParams(W.kappa, W.dE, W.dI, W.tau * cfg.h), 16, dens, sel)
    assert nleaf > 200
    err = np.abs(out[:, sel] - ref).max() / np.abs(ref).max()
    print(f"precision {precision}: {len(sel)} targets in {nleaf} leaves, relative error {err:.2e}")
    assert err < FMM_TOL[precision], err
