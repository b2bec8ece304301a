"""Shared test setup: import paths, golden fixtures, the `gpu` marker."""

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ibim-levelset_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d.pop("params_json")))
    return d


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_golden(name)
        return cache[name]

    return get


@pytest.fixture(scope="session")
def ctx():
    import ibim

    c = ibim.Context(0)
    yield c
    c.close()


def config_for(P, precision=0):
    """ibim.Config from a golden fixture's parameters."""
    import ibim

    return ibim.default_config(lo=P["lo"], h=P["h"], n=P["n"], band=P["band"], init=P["init"], probe=P["probe"],
                               reinit_t=P["reinit_t"], thickness=P["thickness"], thres=P["thres"], np=P["np"],
                               maxpoint=P["maxpoint"], maxlevel=P["maxlevel"], kappa=P["kappa"], dE=P["dE"],
                               dI=P["dI"], tau=P["tau"], restart=P["restart"], maxiter=P["maxiter"], tol=P["tol"],
                               precision=precision)


def grid_stats(a):
    return np.array([a.sum(), np.abs(a).sum(), a.max(), a.min(), (a * a).sum()])


def _build_if_stale():
    """Rebuild libibim_gb300.so when a source is newer (no-op when fresh; skipped without nvcc)."""
    import importlib.util
    import shutil

    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        return
    spec = importlib.util.spec_from_file_location("ibim_gb300_build",
                                                  os.path.join(ROOT, "ibim-levelset_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_build_if_stale()
