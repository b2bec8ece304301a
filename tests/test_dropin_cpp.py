"""The reference's main.cpp sequence written against the C++ drop-in classes
(include/ibim/dropin.hpp) compiles against the library here, and on a GPU reproduces the
reference's energy and writes the reference's output files (electric.cpp:420-427 potent_file,
2N lines; electric.cpp:491-497 energy_file, M lines; levelset.cpp:39-52 Grid::output, one value
per line in i, j, k order; levelset.cpp:593-601 Surface::output, "x y z" per tube point)."""

import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

LIB_DIR = os.path.join(ROOT, "ibim-levelset_gb300", "_build")
SRC = os.path.join(ROOT, "tests", "cpp", "main_dropin.cpp")
SRC_GMRES = os.path.join(ROOT, "tests", "cpp", "main_gmres.cpp")


def compile_dropin(out_dir, src=SRC):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0])
    cmd = ["g++", "-std=c++14", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), src, "-L", LIB_DIR,
           "-libim_gb300", f"-Wl,-rpath,{LIB_DIR}", "-o", exe]
    cuda_lib = "/usr/local/cuda/lib64"
    if os.path.isdir(cuda_lib):
        cmd += [f"-Wl,-rpath-link,{cuda_lib}", f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dropin_compiles_and_links():
    with tempfile.TemporaryDirectory() as td:
        assert os.path.exists(compile_dropin(td))
        assert os.path.exists(compile_dropin(td, SRC_GMRES))


def write_cfg(td, G, extra=""):
    import synth

    P = G["params"]
    pqr = os.path.join(td, "m.pqr")
    synth.Molecule(G["centers"], G["charges"], G["radii"]).to_pqr(pqr)
    n = max(P["n"])
    lo = min(P["lo"])
    cfg = os.path.join(td, "input.cfg")
    with open(cfg, "w") as f:
        f.write(f"pqr_file = {pqr}\nlo = {lo!r}\nh = {P['h']!r}\nn = {n}\nreinit_step = {P['reinit_t']!r}\n"
                f"lvlset_thickness = {P['thickness']}\nlvlset_thres = {P['thres']}\nfmm_np = {P['np']}\n"
                f"fmm_maxpoint = {P['maxpoint']}\nfmm_maxlevel = {P['maxlevel']}\ntau = {P['tau']}\n"
                f"solvent_kappa = {P['kappa']!r}\nsolvent_dE = {P['dE']!r}\nsolvent_dI = {P['dI']!r}\n"
                f"gmres_restart = {P['restart']}\ngmres_maxiter = {P['maxiter']}\ngmres_tol = {P['tol']}\n" + extra)
    return cfg, n, lo


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["synth30", "p1hje"])
def test_dropin_gmres_closure_reproduces_reference(golden, case):
    """GMRES(FullMap, start, load, m, max_iter, tol) called as electric.cpp:415 calls it, with the
    closure on the drop-in BIE operator and the fixture's own box: the reference's number of
    operator applications (its GMRES applies the operator to x0 = 0 too) and its solution."""
    G = golden(case)
    P = G["params"]
    with tempfile.TemporaryDirectory() as td:
        exe = compile_dropin(td, SRC_GMRES)
        out = os.path.join(td, "solution.bin")
        box = "".join(f"n{a} = {P['n'][i]}\nlo{a} = {P['lo'][i]!r}\n" for i, a in enumerate("xyz"))
        cfg, _, _ = write_cfg(td, G, f"out_file = {out}\n" + box)
        r = subprocess.run([exe, cfg], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        vals = dict(ln.split()[:2] for ln in r.stdout.splitlines() if ln.startswith("DROPIN_"))
        assert int(vals["DROPIN_GMRES_RC"]) == 0
        N = len(G["surface"])
        assert int(vals["DROPIN_POINTS"]) == N
        assert int(vals["DROPIN_MATVECS"]) == int(P["scalars"]["REF_MATVECS"])
        x = np.fromfile(out, dtype=np.float64)
        assert x.shape == (2 * N,)
        idx = G["sample_idx"]
        xs = np.concatenate([x[idx], x[N + idx]])
        assert np.abs(xs - G["solution_sample"]).max() / np.abs(G["solution_sample"]).max() < 1e-8


@pytest.mark.gpu
def test_dropin_main_reproduces_reference(golden):
    import synth

    G = golden("p1hje")
    P = G["params"]
    assert P["n"][0] == P["n"][1] == P["n"][2] or True
    with tempfile.TemporaryDirectory() as td:
        exe = compile_dropin(td)
        pqr = os.path.join(td, "m.pqr")
        synth.Molecule(G["centers"], G["charges"], G["radii"]).to_pqr(pqr)
        n = max(P["n"])
        lo = min(P["lo"])
        cfg = os.path.join(td, "input.cfg")
        with open(cfg, "w") as f:
            f.write(f"pqr_file = {pqr}\nlo = {lo!r}\nh = {P['h']!r}\nn = {n}\nreinit_step = {P['reinit_t']!r}\n"
                    f"lvlset_thickness = {P['thickness']}\nlvlset_thres = {P['thres']}\nfmm_np = {P['np']}\n"
                    f"fmm_maxpoint = {P['maxpoint']}\nfmm_maxlevel = {P['maxlevel']}\ntau = {P['tau']}\n"
                    f"solvent_kappa = {P['kappa']!r}\nsolvent_dE = {P['dE']!r}\nsolvent_dI = {P['dI']!r}\n"
                    f"gmres_restart = {P['restart']}\ngmres_maxiter = {P['maxiter']}\ngmres_tol = {P['tol']}\n"
                    f"potent_file = {td}/potential.txt\nenergy_file = {td}/energy.txt\n"
                    f"grid_file = {td}/output.grid\nnode_file = {td}/output.node\n")
        r = subprocess.run([exe, cfg], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        vals = dict(ln.split()[:2] for ln in r.stdout.splitlines() if ln.startswith("DROPIN_"))
        E = float(vals["DROPIN_ENERGY"])
        assert abs(E) > 0
        # a cubic box of side max(n) around the fixture's box: same molecule, same h
        import ibim
        from conftest import config_for

        ctx = ibim.Context(0)
        cfgp = config_for(dict(P, lo=[lo] * 3, n=[n] * 3, init=-2.0 * n))
        ref = ctx.solve(G["centers"], G["charges"], G["radii"], cfgp)
        ctx.close()
        assert int(vals["DROPIN_POINTS"]) == ref["n_points"]
        assert abs(E - ref["energy"]) / abs(ref["energy"]) < 1e-9
        npts = ref["n_points"]
        pot = np.loadtxt(os.path.join(td, "potential.txt"))
        assert pot.shape == (2 * npts,) and np.all(np.isfinite(pot))
        atom = np.loadtxt(os.path.join(td, "energy.txt"))
        assert atom.shape == (len(G["charges"]),)
        # the files carry 6 significant digits (default stream precision), as the reference's do
        assert abs(0.5 * np.dot(atom, G["charges"]) - E) <= 1e-5 * np.sum(np.abs(0.5 * atom * G["charges"]))
        grid = np.loadtxt(os.path.join(td, "output.grid"))
        assert grid.shape == (n ** 3,)
        nodes = np.loadtxt(os.path.join(td, "output.node"))
        assert nodes.shape == (npts, 3)
