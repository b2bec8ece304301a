"""ibim_levelset_evolve_static: level-set evolution that allocates no device memory.

Callers that reserve all device memory in their own pool, or that must never enter the CUDA
allocator during a run, pass their own device grid; the two stage buffers come from a fixed
array inside the library (at most 524,288 cells).  This checks it through the C ABI against
ibim_levelset_evolve (which allocates its stage buffers) on two calls in a row, and that a grid
above the limit is rejected.  Kept in a file of its own, collected last.
"""

import ctypes

import numpy as np
import pytest

import ibim

pytestmark = pytest.mark.gpu

N, LO, H = (40, 44, 36), (-6.0, -6.6, -5.4), 0.3
CENTERS = np.array([[0.3, -0.2, 0.1], [1.9, 0.4, -0.5]])
RADII = np.array([2.0, 1.6])


def test_static_evolve_matches_allocating_evolve():
    torch = pytest.importorskip("torch")
    ctx = ibim.Context(0)
    g = ctx.grid(N, LO, H, -80.0)
    g.expand(CENTERS, RADII)
    dev = torch.tensor(g.download(), dtype=torch.float64, device="cuda").contiguous()
    fn = ibim.lib().ibim_levelset_evolve_static
    for call in range(2):
        g.evolve(1.4, 1.0, 0.2)
        st = fn(ctypes.c_void_p(dev.data_ptr()), N[0], N[1], N[2], H, 1.4, 1.0, 0.2, None)
        assert st == ibim.OK, ibim.lib().ibim_last_error().decode()
        torch.cuda.synchronize()
        a = g.download()
        b = dev.cpu().numpy()
        # same kernels and arithmetic: the results agree to the last bit
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(a).max()), call
    g.close()
    ctx.close()


def test_static_evolve_rejects_grids_above_the_limit():
    torch = pytest.importorskip("torch")
    dev = torch.zeros(8, dtype=torch.float64, device="cuda")
    fn = ibim.lib().ibim_levelset_evolve_static
    st = fn(ctypes.c_void_p(dev.data_ptr()), 100, 100, 100, 0.5, 1.4, 1.0, 0.2, None)
    assert st == ibim.ERR_INVALID_ARGUMENT
    assert "524288" in ibim.lib().ibim_last_error().decode()
