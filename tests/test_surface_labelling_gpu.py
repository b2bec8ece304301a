"""The surface's exterior (the reference's BFS from cell 0, levelset.cpp:444-524) found by
connected-component labelling on the GPU, against the oracle's BFS on grids built to stress it:
random fields with many small passable components and enclosed tube cells, the same with cell 0
impassable (only cell 0 is visited, so every tube cell is a cavity), and nested spherical shells
around a closed cavity.  Rows of 31, 32, 33, 65 and 70 cells cover the warp segments of the
run-start scan.  Equal tube points (all seven columns within 1e-9) and equal cavity counts."""

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

H = 0.5
THICKNESS = 2


def compare(ctx, phi):
    n = phi.shape
    lo = (-1.0, -2.0, -3.0)
    g = ctx.grid(n, lo, H)
    g.upload(phi)
    t = g.surface(THICKNESS)
    s = t.surface7()
    s_ref, inc_ref = O.surface(phi.copy(), lo, H, THICKNESS)
    assert t.inclusion == inc_ref
    assert len(s) == len(s_ref)
    if len(s):
        assert np.abs(s - s_ref).max() < 1e-9
    return len(s), inc_ref


@pytest.mark.parametrize("shape", [(9, 11, 31), (7, 6, 32), (8, 5, 33), (6, 7, 65), (5, 9, 70)])
@pytest.mark.parametrize("low", [-2.5, -4.0])  # passable fractions 0.7 and 0.33 (near percolation)
def test_random_fields(ctx, shape, low):
    rng = np.random.default_rng(sum(shape))
    tw = THICKNESS * H
    phi = rng.uniform(low * tw, (low + 4.5 if low < -3 else 2.5) * tw, size=shape)
    phi[0, 0, 0] = 0.5 * tw  # the BFS starts from a passable tube cell
    npts, inc = compare(ctx, phi)
    assert npts > 0
    phi[0, 0, 0] = -10.0  # cell 0 impassable: every tube cell is a cavity
    npts2, inc2 = compare(ctx, phi)
    assert npts2 == 0 and inc2 > 0


def test_nested_shells_enclose_a_cavity(ctx):
    n = (40, 44, 70)
    i, j, k = np.meshgrid(*(np.arange(m) for m in n), indexing="ij")
    r = np.sqrt((i - 20.0) ** 2 + (j - 22.0) ** 2 + (k - 35.0) ** 2) * H
    # outside positive; a wall between radii 5 and 9 whose middle (6 < r < 8, four cells thick) is
    # below -tw, so nothing passes it; a hollow between radii 2 and 5; a core below radius 2.
    # The hollow's tube cells cannot be reached from cell 0 and become cavities.
    phi = np.where(r > 9.0, r - 9.0, np.where(r > 5.0, -np.minimum(r - 5.0, 9.0 - r),
                                               np.where(r > 2.0, np.minimum(r - 2.0, 5.0 - r), r - 2.0)))
    npts, inc = compare(ctx, phi)
    assert npts > 0 and inc > 0
