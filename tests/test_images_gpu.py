"""One pass over the float-float M2L operators makes both tensor-core images of a mixed solve:
the scaled FP16 tiles and row scales of the mixed contraction and the digit tiles and row scales
of the FP64-class refinement residual.  With IBIM_CHECK_IMAGES=1 (read on every solve) the
library also builds them with the separate scale and pack kernels from the same operators and
compares the two word for word; any difference fails the solve.  Orders 4 and 5 cut the operators
into 6 digits of 7 bits, order 6 into 7 digits of 6 bits."""

import pytest

from conftest import config_for, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,order", [("p1hje", None), ("synth30", None), ("synth30", 6)])
def test_one_pass_images_equal_the_separate_passes(ctx, case, order, monkeypatch):
    import ibim

    G = load_golden(case)
    cfg = config_for(G["params"], ibim.PRECISION_MIXED)
    if order:
        cfg.np = order
    monkeypatch.setenv("IBIM_CHECK_IMAGES", "1")
    checked = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)  # raises when a word differs
    monkeypatch.delenv("IBIM_CHECK_IMAGES")
    plain = ctx.solve(G["centers"], G["charges"], G["radii"], cfg)
    # the checked solve keeps the separate passes' images: equal images, equal solves (up to the
    # run-to-run order of the mixed path's FP32 atomic sums)
    assert checked["gmres_iters"] == plain["gmres_iters"]
    assert abs(checked["energy"] - plain["energy"]) <= 1e-6 * abs(plain["energy"])
