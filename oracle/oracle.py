"""ORACLE — test infrastructure only.

ctypes binding of the C restatement in oracle/ibim_oracle.c (the reference's CPU algorithm
for the IBIM Poisson-Boltzmann path).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it, as the checker; the product never imports it.

`build()` compiles oracle/_build/libibim_oracle.so with gcc (OpenMP), the checker's exact
build, and oracle/_build/libibim_oracle_timing.so, the same source with -ffast-math: the
reference is built -Ofast, and the CPU-baseline leg times this build (`use_timing_build()`),
whose outputs are discarded.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libibim_oracle.so")
TIMING_LIB_PATH = os.path.join(HERE, "_build", "libibim_oracle_timing.so")

_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ibim_oracle.c")
    newest = max(os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ibim_oracle.h")))
    for path, flags in ((LIB_PATH, ["-ffp-contract=off"]), (TIMING_LIB_PATH, ["-ffast-math"])):
        if force or not os.path.exists(path) or os.path.getmtime(path) < newest:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            subprocess.run(["gcc", "-O3", "-fPIC", "-fopenmp", "-std=c11", *flags, "-shared", "-o", path, src, "-lm"],
                           check=True)
    return LIB_PATH


_lib_path = LIB_PATH


def use_timing_build() -> None:
    """Bind the module to the -ffast-math build for the rest of the process (CPU-baseline timing
    only: its results are not the checker's)."""
    global _lib, _lib_path
    build()
    if _lib_path != TIMING_LIB_PATH:
        _lib, _lib_path = None, TIMING_LIB_PATH


class KParams(C.Structure):
    _fields_ = [("kappa", C.c_double), ("dE", C.c_double), ("dI", C.c_double), ("vr", C.c_double)]


class BieParams(C.Structure):
    _fields_ = [("np", C.c_int), ("maxpoint", C.c_int), ("maxlevel", C.c_int), ("restart", C.c_int),
                ("maxiter", C.c_int), ("kappa", C.c_double), ("dE", C.c_double), ("dI", C.c_double),
                ("tau", C.c_double), ("tol", C.c_double), ("mode", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_lib_path)
        L.orc_expand.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, _dp, _dp, C.c_int, C.c_double]
        L.orc_evolve.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_reinitialize.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_double]
        L.orc_reinitialize.restype = C.c_int
        L.orc_count_gradient.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _dp,
                                         C.POINTER(C.c_long)]
        L.orc_count_gradient.restype = C.c_long
        L.orc_levelset_build.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_int, C.c_double, _dp, _dp, C.c_int, C.c_double, C.c_double,
                                         C.c_int, C.c_double, _ip]
        L.orc_surface.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.c_int, _dp, C.c_long, C.POINTER(C.c_long)]
        L.orc_surface.restype = C.c_long
        L.orc_tree_build.argtypes = [_dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int]
        L.orc_tree_build.restype = C.c_void_p
        L.orc_tree_free.argtypes = [C.c_void_p]
        L.orc_tree_nnodes.argtypes = [C.c_void_p]
        L.orc_tree_nnodes.restype = C.c_int
        L.orc_tree_node.argtypes = [C.c_void_p, C.c_int, _ip, _dp]
        L.orc_tree_list.argtypes = [C.c_void_p, C.c_int, C.c_int, _ip, C.c_int]
        L.orc_tree_list.restype = C.c_int
        L.orc_fmm.argtypes = [C.c_void_p, C.c_int, C.POINTER(KParams), C.c_int, _dp, _dp]
        L.orc_fmm_sample.argtypes = [C.c_void_p, C.c_int, C.POINTER(KParams), C.c_int, _dp, _dp, C.c_int]
        L.orc_fmm_targets.argtypes = [C.c_void_p, C.c_int, C.POINTER(KParams), C.c_int, _dp, _dp, _ip, C.c_int]
        L.orc_fmm_targets.restype = C.c_int
        L.orc_rhs.argtypes = [_dp, C.c_long, _dp, _dp, C.c_int, C.POINTER(BieParams), _dp]
        L.orc_matvec.argtypes = [_dp, C.c_long, C.c_double, C.POINTER(BieParams), _dp, _dp]
        L.orc_solve.argtypes = [_dp, C.c_long, C.c_double, _dp, _dp, C.c_int, C.POINTER(BieParams), _dp, _dp, _dp,
                                _ip, _ip]
        L.orc_solve.restype = C.c_int
        L.orc_gmres.argtypes = [ORC_OP, C.c_void_p, C.c_long, _dp, _dp, C.c_int, C.c_int, C.c_double, _ip, _ip]
        L.orc_gmres.restype = C.c_int
        _lib = L
    return _lib


# void (*orc_op)(void *ctx, const double *x, double *y)
ORC_OP = C.CFUNCTYPE(None, C.c_void_p, _dp, _dp)


def _p(a):
    return a.ctypes.data_as(_dp)


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def levelset(centers, radii, lo, h, n, *, band=8, init=None, probe=1.4, reinit_t=1.0, thickness=3, thres=1e-4):
    """main.cpp:45-60 pipeline (s = 1).  Returns (grid (nx,ny,nz), reinit steps (2,))."""
    nx, ny, nz = (int(v) for v in n)
    if init is None:
        init = -2.0 * max(nx, ny, nz)
    g = np.empty((nx, ny, nz))
    c = _c(centers).reshape(-1, 3)
    r = _c(radii)
    steps = np.zeros(2, np.int32)
    lib().orc_levelset_build(_p(g), nx, ny, nz, lo[0], lo[1], lo[2], h, band, init, _p(c), _p(r), len(r), probe,
                             reinit_t, thickness, thres, steps.ctypes.data_as(_ip))
    return g, steps


def expand(g, centers, radii, lo, h, *, band=8, probe=1.4):
    c = _c(centers).reshape(-1, 3)
    r = _c(radii)
    nx, ny, nz = g.shape
    lib().orc_expand(_p(g), nx, ny, nz, lo[0], lo[1], lo[2], h, band, _p(c), _p(r), len(r), probe)


def evolve(g, h, final_t=1.4, vel=1.0, cfl=0.2):
    nx, ny, nz = g.shape
    lib().orc_evolve(_p(g), nx, ny, nz, h, final_t, vel, cfl)


def reinitialize(g, phi0, h, final_t, *, thickness=3, thres=1e-4, vel=1.0, cfl=0.5):
    nx, ny, nz = g.shape
    return lib().orc_reinitialize(_p(g), _p(_c(phi0)), nx, ny, nz, h, final_t, vel, cfl, thickness, thres)


def count_gradient(g, h, thickness, thres):
    nx, ny, nz = g.shape
    acc = C.c_double(0)
    tot = C.c_long(0)
    bad = lib().orc_count_gradient(_p(_c(g)), nx, ny, nz, h, float(thickness), thres, C.byref(acc), C.byref(tot))
    return bad, tot.value, acc.value


def surface(g, lo, h, thickness):
    """Surface(Grid&, levelset&, 1).  Modifies g in place.  Returns (points (N,7), inclusion count)."""
    nx, ny, nz = g.shape
    cap = max(1024, int(np.count_nonzero(np.abs(g) < thickness * h)) + 16)
    out = np.empty((cap, 7))
    inc = C.c_long(0)
    n = lib().orc_surface(_p(g), nx, ny, nz, lo[0], lo[1], lo[2], h, thickness, _p(out), cap, C.byref(inc))
    assert n <= cap
    return out[:n].copy(), inc.value


class Tree:
    """bbfmm::tree built by the restated tree::populate (sources, targets: (n,3))."""

    def __init__(self, src, tgt, maxpoint, maxlevel=10):
        self.src = _c(src).reshape(-1, 3)
        self.tgt = _c(tgt).reshape(-1, 3)
        self.ptr = lib().orc_tree_build(_p(self.src), len(self.src), _p(self.tgt), len(self.tgt), maxpoint,
                                        maxlevel)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().orc_tree_free(self.ptr)
            self.ptr = None

    @property
    def nnodes(self):
        return lib().orc_tree_nnodes(self.ptr)

    def node(self, i):
        ints = np.zeros(6, np.int32)
        cr = np.zeros(6)
        lib().orc_tree_node(self.ptr, i, ints.ctypes.data_as(_ip), _p(cr))
        return ints, cr

    def lists(self, i):
        out = []
        buf = np.zeros(4096, np.int32)
        for w in range(4):
            n = lib().orc_tree_list(self.ptr, i, w, buf.ctypes.data_as(_ip), len(buf))
            assert n <= len(buf)
            out.append(buf[:n].copy())
        return out

    def fmm(self, p, kparams: KParams, kernel: int, dens, sample_stride: int = 1):
        """One FMM; sample_stride > 1 runs the downward pass on every stride-th node only
        (a timing sample whose output is incomplete)."""
        nd = 4 if kernel == 16 else 1
        d = _c(dens).reshape(nd, len(self.src))
        out = np.zeros((nd, len(self.tgt)))
        if sample_stride > 1:
            lib().orc_fmm_sample(self.ptr, p, C.byref(kparams), kernel, _p(d), _p(out), sample_stride)
        else:
            lib().orc_fmm(self.ptr, p, C.byref(kparams), kernel, _p(d), _p(out))
        return out

    def fmm_at(self, p, kparams: KParams, kernel: int, dens, targets):
        """orc_fmm at the given target indices only: the downward pass runs for the leaves that hold
        them and those leaves' ancestors.  Returns (values at the targets, no x len(targets);
        number of leaves evaluated)."""
        nd = 4 if kernel == 16 else 1
        d = _c(dens).reshape(nd, len(self.src))
        sel = np.ascontiguousarray(targets, dtype=np.int32)
        out = np.zeros((nd, len(self.tgt)))
        nleaf = lib().orc_fmm_targets(self.ptr, p, C.byref(kparams), kernel, _p(d), _p(out), sel.ctypes.data_as(_ip),
                                      len(sel))
        return out[:, sel], nleaf


def bie_params(np_=4, maxpoint=64, maxlevel=10, restart=30, maxiter=100, kappa=0.0, dE=80.0, dI=1.0, tau=1.0,
               tol=1e-6, mode=0) -> BieParams:
    return BieParams(np_, maxpoint, maxlevel, restart, maxiter, kappa, dE, dI, tau, tol, mode)


def rhs(surf7, centers, charges, bp: BieParams):
    s = _c(surf7)
    N = len(s)
    b = np.zeros(2 * N)
    c = _c(centers).reshape(-1, 3)
    q = _c(charges)
    lib().orc_rhs(_p(s), N, _p(c), _p(q), len(q), C.byref(bp), _p(b))
    return b


def matvec(surf7, h, bp: BieParams, x):
    s = _c(surf7)
    y = np.zeros(2 * len(s))
    lib().orc_matvec(_p(s), len(s), h, C.byref(bp), _p(_c(x)), _p(y))
    return y


def solve(surf7, h, centers, charges, bp: BieParams):
    """electric() after Surface: returns dict(x, atom_pot, energy, rc, iters, matvecs)."""
    s = _c(surf7)
    N = len(s)
    c = _c(centers).reshape(-1, 3)
    q = _c(charges)
    x = np.zeros(2 * N)
    pot = np.zeros(len(q))
    E = C.c_double(0)
    it = C.c_int(0)
    mv = C.c_int(0)
    rc = lib().orc_solve(_p(s), N, h, _p(c), _p(q), len(q), C.byref(bp), _p(x), _p(pot), C.byref(E), C.byref(it),
                         C.byref(mv))
    return dict(x=x, atom_pot=pot, energy=E.value, rc=rc, iters=it.value, matvecs=mv.value)


def gmres(apply, b, x0=None, m=30, max_iter=100, tol=1e-6):
    """Restarted GMRES of gmres.cpp:50-164 (orc_gmres) on an operator apply(x) -> y given in numpy.
    Returns (x, status, iters, matvecs); matvecs counts the first product A x0 as the reference does."""
    b = _c(b)
    n = len(b)
    x = np.zeros(n) if x0 is None else _c(x0).copy()

    def op(_ctx, xp, yp):
        y = np.asarray(apply(np.ctypeslib.as_array(xp, shape=(n,)).copy()), dtype=np.float64)
        np.ctypeslib.as_array(yp, shape=(n,))[:] = y

    fn = ORC_OP(op)
    it, mv = C.c_int(0), C.c_int(0)
    rc = lib().orc_gmres(fn, None, n, _p(x), _p(b), m, max_iter, tol, C.byref(it), C.byref(mv))
    return x, rc, it.value, mv.value
