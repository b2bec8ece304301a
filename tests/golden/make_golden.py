"""Generate the golden fixtures in tests/golden/ by running the reference's own CPU code.

The reference (ibim-levelset) has no tests or golden vectors of its own, so the fixtures
come from the reference itself: `make -C oracle ref` compiles its unmodified sources into
oracle/_ref/ibim_ref (driver: oracle/ref/ref_driver.cpp), and this script runs it on a few
small cases and packs what it dumps into one .npz per case:

  born     one ion (R=2 A, q=+1), 64^3 grid over [-6,6)^3, p=4, leaf<=64, kappa=0
  synth30  30-atom synthetic protein (seed 7), h=0.5 A, p=5, kappa=0.125, eps 2/80
  cavity   closed shell of 110 atoms around an empty core (exercises the cavity fill)
  p1hje    the reference's data/1hje.pqr (174 atoms) at h=0.75 A, p=4, kappa=0.1257
  synth300 300-atom synthetic protein (seed 300,000), h=0.5 A, p=5, kappa=0.125, eps 2/80, leaf<=128:
           the benchmark protein's settings at a size with a deep tree and a real X list

Run where the reference sources are, naming their directory:
  IBIM_REFERENCE=<reference source dir> python tests/golden/make_golden.py [case ...]
"""

from __future__ import annotations

import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ibim-levelset_gb300"))
import synth  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ibim_ref")
REF_DIR = os.environ.get("IBIM_REFERENCE", "")
REF_DATA = os.path.join(REF_DIR, "data") if REF_DIR else ""
NSAMPLE = 768


def cavity_shell() -> synth.Molecule:
    """110 atoms (R=2 A) on a Fibonacci sphere of radius 8 A: a closed shell with a hollow core."""
    n = 110
    k = np.arange(n) + 0.5
    z = 1.0 - 2.0 * k / n
    phi = math.pi * (1.0 + 5 ** 0.5) * k
    s = np.sqrt(1.0 - z * z)
    c = 8.0 * np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)
    q = np.where(np.arange(n) % 2 == 0, 0.5, -0.5)
    return synth.Molecule(c, q, np.full(n, 2.0))


def cases():
    out = {}
    g = synth.born_geometry()
    out["born"] = dict(mol=synth.born_ion(), geo=g, thickness=3, np_=4, maxpoint=64, kappa=0.0, dI=1.0,
                       dE=80.0, solve=True, fmm=True, reinit_steps=20)
    m = synth.synthetic_protein(30, 7)
    out["synth30"] = dict(mol=m, geo=synth.padded_geometry(m, 0.5), thickness=2, np_=5, maxpoint=64,
                          kappa=0.125, dI=2.0, dE=80.0, solve=True, fmm=True, reinit_steps=20)
    m = cavity_shell()
    out["cavity"] = dict(mol=m, geo=synth.padded_geometry(m, 0.5), thickness=2, np_=4, maxpoint=64,
                         kappa=0.1, dI=2.0, dE=80.0, solve=False, fmm=True, reinit_steps=20)
    m = synth.synthetic_protein(300, 300_000)
    out["synth300"] = dict(mol=m, geo=synth.padded_geometry(m, 0.5), thickness=2, np_=5, maxpoint=128,
                           kappa=0.125, dI=2.0, dE=80.0, solve=True, fmm=True, reinit_steps=20)
    if REF_DATA and os.path.exists(os.path.join(REF_DATA, "1hje.pqr")):
        m = synth.Molecule.from_pqr(os.path.join(REF_DATA, "1hje.pqr"))
        out["p1hje"] = dict(mol=m, geo=synth.padded_geometry(m, 0.75), thickness=2, np_=4, maxpoint=80,
                            kappa=0.1257, dI=1.0, dE=80.0, solve=True, fmm=True, reinit_steps=20)
    return out


def parse_tree(path):
    rows = [ln.split() for ln in open(path)]
    n = len(rows)
    level = np.zeros(n, np.int32)
    parent = np.zeros(n, np.int32)
    leaf = np.zeros(n, np.int8)
    empty = np.zeros(n, np.int8)
    nsrc = np.zeros(n, np.int32)
    ntgt = np.zeros(n, np.int32)
    center = np.zeros((n, 3))
    radius = np.zeros((n, 3))
    lists = {c: ([0], []) for c in "UVWX"}
    for i, r in enumerate(rows):
        level[i], parent[i], leaf[i], empty[i], nsrc[i], ntgt[i] = (int(v) for v in r[1:7])
        center[i] = [float(v) for v in r[7:10]]
        radius[i] = [float(v) for v in r[10:13]]
        p = 13
        for c in "UVWX":
            assert r[p] == c
            cnt = int(r[p + 1])
            lists[c][1].extend(int(v) for v in r[p + 2:p + 2 + cnt])
            lists[c][0].append(len(lists[c][1]))
            p += 2 + cnt
    d = dict(tree_level=level, tree_parent=parent, tree_leaf=leaf, tree_empty=empty, tree_nsrc=nsrc,
             tree_ntgt=ntgt, tree_center=center, tree_radius=radius)
    for c in "UVWX":
        d[f"tree_{c}_ptr"] = np.asarray(lists[c][0], np.int32)
        d[f"tree_{c}_idx"] = np.asarray(lists[c][1], np.int32)
    return d


def stats(a):
    return np.array([a.sum(), np.abs(a).sum(), a.max(), a.min(), (a * a).sum()])


def run_case(name, c):
    geo = c["geo"]
    with tempfile.TemporaryDirectory() as td:
        pqr = os.path.join(td, "mol.pqr")
        c["mol"].to_pqr(pqr)
        # the reference reads the PQR text back; use exactly what it read
        mol = synth.Molecule.from_pqr(pqr)
        rt = synth.reinit_time(c["reinit_steps"], geo.h)
        args = [REF_BIN, f"pqr={pqr}", f"out={td}", f"lox={geo.lo[0]!r}", f"loy={geo.lo[1]!r}",
                f"loz={geo.lo[2]!r}", f"nx={geo.n[0]}", f"ny={geo.n[1]}", f"nz={geo.n[2]}", f"h={geo.h!r}",
                f"reinit_t={rt!r}", f"lvlset_thickness={c['thickness']}", "lvlset_thres=1e-4",
                f"fmm_np={c['np_']}", f"fmm_maxpoint={c['maxpoint']}", "fmm_maxlevel=10",
                f"solvent_kappa={c['kappa']!r}", f"solvent_dI={c['dI']!r}", f"solvent_dE={c['dE']!r}",
                "tau=1.0", "gmres_restart=30", "gmres_maxiter=100", "gmres_tol=1e-6", "dump_grids=1",
                f"fmm_test={int(c['fmm'])}", f"solve={int(c['solve'])}"]
        env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count()))
        res = subprocess.run(args, capture_output=True, text=True, env=env, check=True)
        scal = {}
        for ln in res.stdout.splitlines():
            if ln.startswith("REF_"):
                k, v = ln.split()
                scal[k] = float(v)
            if "INCLUSION" in ln:
                scal["INCLUSION"] = int(ln.split()[1])
        N = int(scal["REF_N"])
        ncell = geo.cells
        d = dict(centers=mol.centers, charges=mol.charges, radii=mol.radii)
        for st in ("expand", "evolve", "reinit1", "reinit2", "surface"):
            gr = np.fromfile(os.path.join(td, f"grid_{st}.bin"), dtype=np.float64)
            assert gr.size == ncell
            d[f"gridstats_{st}"] = stats(gr)
        d["surface"] = np.fromfile(os.path.join(td, "surface.bin"), dtype=np.float64).reshape(N, 7)
        rng = np.random.default_rng(1234)
        idx = np.sort(rng.choice(N, size=min(NSAMPLE, N), replace=False)).astype(np.int64)
        d["sample_idx"] = idx
        if c["fmm"]:
            f16 = np.fromfile(os.path.join(td, "fmm16.bin"), dtype=np.float64).reshape(16, N)
            d["fmm16_sample"] = f16[:, idx]
            d["fmm16_norm"] = np.linalg.norm(f16, axis=1)
            d["fmm16_absmax"] = np.abs(f16).max(axis=1)
            d.update(parse_tree(os.path.join(td, "tree.txt")))
        if c["solve"]:
            rhs = np.fromfile(os.path.join(td, "rhs.bin"), dtype=np.float64)
            sol = np.fromfile(os.path.join(td, "solution.bin"), dtype=np.float64)
            d["rhs_sample"] = np.concatenate([rhs[idx], rhs[N + idx]])
            d["rhs_norm"] = np.array([np.linalg.norm(rhs)])
            d["solution_sample"] = np.concatenate([sol[idx], sol[N + idx]])
            d["solution_norm"] = np.array([np.linalg.norm(sol[:N]), np.linalg.norm(sol[N:])])
            d["atom_potential"] = np.fromfile(os.path.join(td, "atom_potential.bin"), dtype=np.float64)
        params = dict(lo=list(geo.lo), h=geo.h, n=list(geo.n), band=8, probe=1.4,
                      init=-2.0 * max(geo.n), reinit_t=rt, thickness=c["thickness"], thres=1e-4,
                      np=c["np_"], maxpoint=c["maxpoint"], maxlevel=10, kappa=c["kappa"], dI=c["dI"],
                      dE=c["dE"], tau=1.0, restart=30, maxiter=100, tol=1e-6, scalars=scal)
        d["params_json"] = np.array(json.dumps(params))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print(name, "N", N, scal)


def main():
    if not os.path.exists(REF_BIN):
        if not REF_DIR:
            sys.exit("set IBIM_REFERENCE to the reference's source directory")
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF_DIR}"], check=True)
    want = sys.argv[1:]
    for name, c in cases().items():
        if want and name not in want:
            continue
        run_case(name, c)


if __name__ == "__main__":
    main()
