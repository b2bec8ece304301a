"""The C ABI without a GPU: the library loads, exports every entry point include/ibim.h declares,
its host-side tree builder reproduces the reference's trees, and compute calls fail loudly (no
CPU fallback) when no GPU is present."""

import os
import re

import numpy as np
import pytest

import ibim
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ibim.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ibim_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ibim.lib()
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(ibim.EXPORTS) == names


def test_status_strings():
    lib = ibim.lib()
    assert lib.ibim_status_string(ibim.OK) == b"ok"
    assert lib.ibim_status_string(ibim.ERR_UNSUPPORTED_KERNEL) == b"unsupported kernel"


def test_config_defaults_follow_input_cfg():
    cfg = ibim.default_config()
    assert (cfg.np, cfg.maxpoint, cfg.maxlevel, cfg.restart, cfg.maxiter) == (4, 160, 10, 40, 100)
    assert cfg.kp.dE == 80.0 and cfg.kp.dI == 1.0 and abs(cfg.kp.kappa - 0.1257) < 1e-15
    assert cfg.band == 8 and cfg.probe == 1.4


@pytest.mark.parametrize("case", ["born", "synth30", "cavity", "p1hje"])
def test_host_tree_matches_reference(golden, case):
    """csrc/tree.cpp (integer lattice lists) against the reference's own trees (bbfmm.cpp)."""
    G = golden(case)
    P = G["params"]
    nodes = ibim.tree_lists_host(G["surface"][:, :3], P["maxpoint"], P["maxlevel"])
    assert len(nodes) == len(G["tree_level"])
    for i, nd in enumerate(nodes):
        assert [nd["level"], nd["parent"], nd["leaf"], nd["empty"], nd["nsrc"]] == [
            int(G["tree_level"][i]), int(G["tree_parent"][i]), int(G["tree_leaf"][i]), int(G["tree_empty"][i]),
            int(G["tree_nsrc"][i])]
        for c in "UVWX":
            p = G[f"tree_{c}_ptr"]
            assert np.array_equal(np.sort(G[f"tree_{c}_idx"][p[i]:p[i + 1]]), nd[c]), (i, c)


@pytest.mark.parametrize("n,maxpoint", [(300_000, 80), (70_000, 40)])
def test_host_tree_large_matches_oracle(n, maxpoint):
    """Point sets large enough that the top levels are partitioned by all threads (ranges of 16k
    points and more) give the oracle's tree and lists (the restated bbfmm::tree::populate)."""
    import oracle as O

    rng = np.random.default_rng(n)
    v = rng.normal(size=(n, 3))
    pts = 20.0 * v / np.linalg.norm(v, axis=1, keepdims=True) + rng.normal(scale=0.7, size=(n, 3))
    pts[: n // 10] *= 0.4  # a denser inner shell: uneven octants
    nodes = ibim.tree_lists_host(pts, maxpoint, 10)
    T = O.Tree(pts, pts, maxpoint, 10)
    assert len(nodes) == T.nnodes
    for i, nd in enumerate(nodes):
        ints, _ = T.node(i)
        assert [nd["level"], nd["parent"], nd["leaf"], nd["empty"], nd["nsrc"]] == [int(x) for x in ints[:5]], i
        L = T.lists(i)
        for w, c in enumerate("UVWX"):
            assert np.array_equal(L[w], nd[c]), (i, c)


def test_tree_rejects_bad_arguments():
    with pytest.raises(ibim.IbimError) as e:
        ibim.tree_lists_host(np.zeros((4, 3)), 0)
    assert e.value.status == ibim.ERR_INVALID_ARGUMENT


def test_no_gpu_means_an_error_not_a_fallback():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(ibim.IbimError) as e:
        ibim.Context(0)
    assert e.value.status == ibim.ERR_CUDA


def test_server_without_gpu_and_bad_arguments():
    lib = ibim.lib()
    import ctypes as C

    h = C.c_void_p()
    assert lib.ibim_server_create(0, 0, 1e9, C.byref(h)) == ibim.ERR_INVALID_ARGUMENT
    assert lib.ibim_server_create(0, 2, -1.0, C.byref(h)) == ibim.ERR_INVALID_ARGUMENT
    try:
        import torch

        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    assert lib.ibim_server_create(0, 2, 1e9, C.byref(h)) == ibim.ERR_CUDA


def test_request_footprint_estimate_grows_with_the_problem():
    small = ibim.default_config(n=[64, 64, 64], np=4, maxpoint=64)
    big = ibim.default_config(n=[256, 256, 256], np=6, maxpoint=64)
    mixed = ibim.default_config(n=[64, 64, 64], np=4, maxpoint=64, precision=ibim.PRECISION_MIXED)
    a, b, c = (ibim.request_bytes_estimate(x) for x in (small, big, mixed))
    assert 0 < a < b and c > a
