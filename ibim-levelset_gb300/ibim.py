"""Python binding of libibim_gb300.so (the C ABI in include/ibim.h).

Mirrors the reference's interfaces for the IBIM Poisson-Boltzmann path:
  Grid / levelset (levelset.h:12-60)  -> Context.grid(), Grid.expand/evolve/reinitialize/...
  Surface (levelset.h:62-72)          -> Grid.surface() -> Tube
  bbfmm::kernel (bbfmm.h:200-270)     -> Tube.plan() -> Plan.apply(kernel, ...)
  GMRES (gmres.h:20-21)               -> Plan.gmres()
  electric (electric.h:13)            -> Tube.electric()
  main.cpp:45-77                      -> Context.solve()
The library has no CPU fallback: without a GPU, every compute call raises IbimError.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libibim_gb300.so")
TUNING_TABLE = os.path.join(HERE, "tuning_gb300.txt")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_UNSUPPORTED_KERNEL = 4
ERR_LIMIT = 5
ERR_IO = 6
ERR_CALLBACK = 7

KERNELS = ["K1x", "K1y", "K1z", "K2", "K3xx", "K3yy", "K3zz", "K3xy", "K3yz", "K3zx", "K3yx", "K3zy", "K3xz",
           "K4x", "K4y", "K4z"]
KERNEL_BIE_FUSED = 16
PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_FP64_TC = 2

# every symbol include/ibim.h declares
EXPORTS = [
    "ibim_ctx_create", "ibim_ctx_destroy", "ibim_last_error", "ibim_status_string", "ibim_config_default",
    "ibim_grid_create", "ibim_grid_destroy", "ibim_grid_upload", "ibim_grid_download", "ibim_grid_scale",
    "ibim_grid_copy", "ibim_levelset_expand", "ibim_levelset_evolve", "ibim_levelset_reinitialize",
    "ibim_levelset_count_gradient", "ibim_levelset_build", "ibim_surface_extract", "ibim_surface_extract_jacobian",
    "ibim_tube_create",
    "ibim_tube_destroy", "ibim_tube_size", "ibim_tube_download", "ibim_fmm_plan", "ibim_plan_destroy",
    "ibim_plan_stats", "ibim_plan_lists", "ibim_fmm_apply", "ibim_bie_matvec", "ibim_bie_rhs", "ibim_gmres_solve",
    "ibim_electric", "ibim_solve", "ibim_solve_dev", "ibim_solve_pqr", "ibim_tree_lists_host", "ibim_ctx_stream",
    "ibim_ctx_trim",
    "ibim_launch_count", "ibim_profile_enable", "ibim_profile_read", "ibim_profile_work", "ibim_measure_peak",
    "ibim_levelset_evolve_static", "ibim_server_create", "ibim_server_destroy", "ibim_server_submit",
    "ibim_server_poll", "ibim_server_wait", "ibim_server_stats", "ibim_request_bytes_estimate", "ibim_gmres_host",
    "ibim_grid_set_geometry", "ibim_batch_solve", "ibim_server_create_lockstep", "ibim_fmm_bytes_estimate",
    "ibim_tuning_set", "ibim_tuning_clear", "ibim_tuning_get", "ibim_tuning_load", "ibim_autotune",
]
PROFILE_CATEGORIES = ["expand", "weno_stage", "count_gradient", "flood_fill", "tube_extract", "m2l_operators", "p2m",
                      "m2m", "m2l_v", "m2l_x", "l2l", "near_l2p", "rhs", "gmres_vectors", "m2l_v_fp64", "m2l_x_fp64",
                      "near_l2p_fp64", "m2l_v_sliced", "l2p", "l2p_fp64", "near_ff"]


class IbimError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class KernelParams(C.Structure):
    _fields_ = [("kappa", C.c_double), ("dE", C.c_double), ("dI", C.c_double), ("tau", C.c_double),
                ("k3_scaled", C.c_int)]


class Config(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("h", C.c_double), ("n", C.c_int * 3), ("band", C.c_int),
                ("init", C.c_double), ("probe", C.c_double), ("reinit_t", C.c_double), ("thickness", C.c_int),
                ("thres", C.c_double), ("np", C.c_int), ("maxpoint", C.c_int), ("maxlevel", C.c_int),
                ("kp", KernelParams), ("restart", C.c_int), ("maxiter", C.c_int), ("tol", C.c_double),
                ("precision", C.c_int), ("jacobian", C.c_int)]


class Result(C.Structure):
    _fields_ = [("energy", C.c_double), ("area", C.c_double), ("n_points", C.c_long), ("inclusion", C.c_long),
                ("reinit_steps", C.c_int * 2), ("gmres_iters", C.c_int), ("matvecs", C.c_int),
                ("matvecs_fp64", C.c_int), ("gmres_status", C.c_int), ("refinements", C.c_int),
                ("residual", C.c_double), ("t_levelset_ms", C.c_double), ("t_surface_ms", C.c_double),
                ("t_plan_ms", C.c_double), ("t_solve_ms", C.c_double), ("t_energy_ms", C.c_double),
                ("grid_cells", C.c_long), ("levelset_stages", C.c_int), ("fmm_nodes", C.c_long),
                ("fmm_v_pairs", C.c_long), ("fmm_x_pairs", C.c_long), ("fmm_near_pairs", C.c_long),
                ("fmm_operators", C.c_long), ("t_tree_ms", C.c_double), ("t_operators_ms", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["reinit_steps"] = list(self.reinit_steps)
        return d


_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_vp = C.c_void_p
# int (*ibim_apply_fn)(void *user, const double *x, double *y, long n)
APPLY_FN = C.CFUNCTYPE(C.c_int, _vp, _dp, _dp, C.c_long)


def lib():
    """Load the shared library (built by build.py; fails loudly when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libibim_gb300.so not built ({LIB_PATH}); run ibim-levelset_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    sig = {
        "ibim_ctx_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
        "ibim_ctx_destroy": ([_vp], C.c_int),
        "ibim_last_error": ([], C.c_char_p),
        "ibim_status_string": ([C.c_int], C.c_char_p),
        "ibim_config_default": ([C.POINTER(Config)], None),
        "ibim_grid_create": ([_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                              C.c_double, C.POINTER(_vp)], C.c_int),
        "ibim_grid_destroy": ([_vp], C.c_int),
        "ibim_grid_upload": ([_vp, _dp], C.c_int),
        "ibim_grid_download": ([_vp, _dp], C.c_int),
        "ibim_grid_scale": ([_vp, C.c_double], C.c_int),
        "ibim_grid_set_geometry": ([_vp, C.c_double, C.c_double, C.c_double, C.c_double], C.c_int),
        "ibim_batch_solve": ([_vp, C.c_int, _ip, _dp, _dp, _dp, C.POINTER(Config), C.c_int, C.c_int, C.c_double,
                              C.c_int, C.POINTER(Result), _ip, _dp, _dp], C.c_int),
        "ibim_grid_copy": ([_vp, _vp], C.c_int),
        "ibim_levelset_expand": ([_vp, _dp, _dp, C.c_int, C.c_double, C.c_int], C.c_int),
        "ibim_levelset_evolve": ([_vp, C.c_double, C.c_double, C.c_double], C.c_int),
        "ibim_levelset_reinitialize": ([_vp, _vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, _ip],
                                       C.c_int),
        "ibim_levelset_count_gradient": ([_vp, C.c_double, C.c_double, _lp, _lp, _dp], C.c_int),
        "ibim_levelset_build": ([_vp, _dp, _dp, C.c_int, C.POINTER(Config), C.POINTER(_vp), _ip], C.c_int),
        "ibim_surface_extract": ([_vp, C.c_int, C.POINTER(_vp), _lp, _lp], C.c_int),
        "ibim_surface_extract_jacobian": ([_vp, C.c_int, C.c_int, C.POINTER(_vp), _lp, _lp], C.c_int),
        "ibim_tube_create": ([_vp, _dp, _dp, _dp, C.c_long, C.c_double, C.POINTER(_vp)], C.c_int),
        "ibim_tube_destroy": ([_vp], C.c_int),
        "ibim_tube_size": ([_vp], C.c_long),
        "ibim_tube_download": ([_vp, _dp, _dp, _dp], C.c_int),
        "ibim_fmm_plan": ([_vp, _dp, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
        "ibim_plan_destroy": ([_vp], C.c_int),
        "ibim_plan_stats": ([_vp, _lp], C.c_int),
        "ibim_plan_lists": ([_vp, C.c_int, _ip, C.c_long, _lp], C.c_int),
        "ibim_fmm_apply": ([_vp, C.c_int, C.POINTER(KernelParams), _dp, _dp], C.c_int),
        "ibim_bie_matvec": ([_vp, C.POINTER(KernelParams), _dp, _dp], C.c_int),
        "ibim_bie_rhs": ([_vp, C.POINTER(KernelParams), _dp, _dp, C.c_int, _dp], C.c_int),
        "ibim_gmres_solve": ([_vp, C.POINTER(KernelParams), _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int, _ip,
                              _ip, _dp], C.c_int),
        "ibim_electric": ([_vp, _dp, _dp, C.c_int, C.POINTER(Config), _dp, _dp, C.POINTER(Result)], C.c_int),
        "ibim_solve": ([_vp, _dp, _dp, _dp, C.c_int, C.POINTER(Config), C.POINTER(Result)], C.c_int),
        "ibim_solve_dev": ([_vp, _vp, _vp, _vp, C.c_int, C.POINTER(Config), C.POINTER(Result)], C.c_int),
        "ibim_solve_pqr": ([_vp, C.c_char_p, C.POINTER(Config), C.POINTER(Result)], C.c_int),
        "ibim_tree_lists_host": ([_dp, C.c_long, C.c_int, C.c_int, _ip, C.c_long, _lp], C.c_int),
        "ibim_ctx_stream": ([_vp], _vp),
        "ibim_ctx_trim": ([_vp], C.c_int),
        "ibim_launch_count": ([], C.c_long),
        "ibim_profile_enable": ([_vp, C.c_uint], C.c_int),
        "ibim_profile_read": ([_vp, _dp, _lp, C.c_int], C.c_int),
        "ibim_profile_work": ([_vp, _dp, _dp, C.c_int], C.c_int),
        "ibim_measure_peak": ([_vp, C.c_int, _dp], C.c_int),
        "ibim_levelset_evolve_static": ([_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_double, _vp], C.c_int),
        "ibim_server_create": ([C.c_int, C.c_int, C.c_double, C.POINTER(_vp)], C.c_int),
        "ibim_server_destroy": ([_vp], C.c_int),
        "ibim_server_submit": ([_vp, _dp, _dp, _dp, C.c_int, C.POINTER(Config), _lp], C.c_int),
        "ibim_server_poll": ([_vp, C.c_long, _ip, _ip, C.POINTER(Result), _dp, _dp], C.c_int),
        "ibim_server_wait": ([_vp, C.c_long, _ip, C.POINTER(Result), _dp, _dp], C.c_int),
        "ibim_server_stats": ([_vp, _dp], C.c_int),
        "ibim_request_bytes_estimate": ([C.POINTER(Config)], C.c_double),
        "ibim_fmm_bytes_estimate": ([C.POINTER(Config), C.c_long], C.c_double),
        "ibim_tuning_set": ([C.c_int, C.c_long, C.c_long, C.c_long, C.c_int], C.c_int),
        "ibim_tuning_clear": ([], C.c_int),
        "ibim_tuning_get": ([C.c_int, C.c_long, _lp], C.c_int),
        "ibim_tuning_load": ([C.c_char_p], C.c_int),
        "ibim_autotune": ([_vp, _dp, _dp, _dp, C.c_int, C.POINTER(Config), C.c_int, C.c_long, _dp], C.c_int),
        "ibim_server_create_lockstep": ([C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(_vp)], C.c_int),
        "ibim_gmres_host": ([_vp, C.c_long, APPLY_FN, _vp, _dp, _dp, C.c_int, C.c_int, C.c_double, _ip, _ip, _ip,
                             _dp], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    # the launch-parameter table measured on GB300 by autotune.py
    if os.path.exists(TUNING_TABLE):
        _check(L.ibim_tuning_load(TUNING_TABLE.encode()))
    return L


def launch_count() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(lib().ibim_launch_count())


def _check(st: int):
    if st != OK:
        raise IbimError(st, lib().ibim_last_error().decode())


def _p(a):
    return a.ctypes.data_as(_dp)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def default_config(**kw) -> Config:
    cfg = Config()
    lib().ibim_config_default(C.byref(cfg))
    for k, v in kw.items():
        if k == "lo":
            cfg.lo = (C.c_double * 3)(*v)
        elif k == "n":
            cfg.n = (C.c_int * 3)(*v)
        elif k in ("kappa", "dE", "dI", "tau", "k3_scaled"):
            setattr(cfg.kp, k, v)
        else:
            setattr(cfg, k, v)
    return cfg


def kernel_params(kappa=0.0, dE=80.0, dI=1.0, tau=1.0, k3_scaled=0) -> KernelParams:
    """k3_scaled = 1 selects the opt-in K3 / (4 pi); 0 is the reference."""
    return KernelParams(kappa, dE, dI, tau, k3_scaled)


class Context:
    """One GPU, one stream (ibim_ctx)."""

    def __init__(self, device: int = 0):
        h = _vp()
        _check(lib().ibim_ctx_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ibim_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        return int(lib().ibim_ctx_stream(self.h) or 0)

    def trim(self):
        """Return the device memory cached by finished solves to the driver."""
        _check(lib().ibim_ctx_trim(self.h))

    def profile(self, categories):
        """Enable CUDA-event timing of the named kernel categories (PROFILE_CATEGORIES)."""
        mask = 0
        for c in categories:
            mask |= 1 << PROFILE_CATEGORIES.index(c)
        _check(lib().ibim_profile_enable(self.h, mask))

    def profile_read(self) -> dict:
        """{category: dict(ms, launches, flops, bytes)} since the last read; clears the counters."""
        n = len(PROFILE_CATEGORIES)
        ms = (C.c_double * n)()
        ln = (C.c_long * n)()
        fl = (C.c_double * n)()
        by = (C.c_double * n)()
        _check(lib().ibim_profile_work(self.h, fl, by, n))
        _check(lib().ibim_profile_read(self.h, ms, ln, n))
        return {c: dict(ms=ms[i], launches=ln[i], flops=fl[i], bytes=by[i]) for i, c in enumerate(PROFILE_CATEGORIES)
                if ln[i]}

    def measure_peak(self, kind: str) -> float:
        v = C.c_double(0)
        _check(lib().ibim_measure_peak(self.h, {"fp64": 0, "fp32": 1}[kind], C.byref(v)))
        return v.value

    def gmres(self, apply, b, x0=None, restart=30, maxiter=100, tol=1e-6):
        """GMRES (gmres.h:20-21) on any operator `apply(x) -> y` evaluated on the host (numpy in,
        numpy out); the Krylov basis and the orthogonalisation run on the device."""
        b = _c(b)
        n = len(b)
        x = np.zeros_like(b) if x0 is None else _c(x0).copy()
        err = []

        def tramp(_user, xp, yp, nn):
            try:
                xin = np.ctypeslib.as_array(xp, shape=(nn,))
                y = np.asarray(apply(xin.copy()), dtype=np.float64).reshape(nn)
                np.ctypeslib.as_array(yp, shape=(nn,))[:] = y
                return 0
            except Exception as e:  # the callback must not raise through C
                err.append(e)
                return 1

        fn = APPLY_FN(tramp)
        it, mv, st, res = C.c_int(0), C.c_int(0), C.c_int(0), C.c_double(0)
        rc = lib().ibim_gmres_host(self.h, n, fn, None, _p(b), _p(x), restart, maxiter, tol, C.byref(it), C.byref(mv),
                                   C.byref(st), C.byref(res))
        if err:
            raise err[0]
        _check(rc)
        return x, dict(iters=it.value, matvecs=mv.value, status=st.value, residual=res.value)

    def batch_solve(self, molecules, cfgs, max_wave=6, hbm_budget_bytes=150e9, workers=4, wave_slots=3,
                    check=True):
        """Many molecules in lock-step waves (ibim_batch_solve).  molecules: list of (centers, charges,
        radii); cfgs: one Config per molecule.  Returns (results, statuses, info)."""
        n = len(molecules)
        na = np.array([len(np.asarray(q)) for _, q, _ in molecules], dtype=np.int32)
        cen = _c(np.concatenate([np.asarray(c, dtype=np.float64).reshape(-1, 3) for c, _, _ in molecules]))
        chg = _c(np.concatenate([np.asarray(q, dtype=np.float64).ravel() for _, q, _ in molecules]))
        rad = _c(np.concatenate([np.asarray(r, dtype=np.float64).ravel() for _, _, r in molecules]))
        carr = (Config * n)(*cfgs)
        res = (Result * n)()
        st = np.zeros(n, dtype=np.int32)
        done = np.zeros(n)
        info = np.zeros(9)
        rc = lib().ibim_batch_solve(self.h, n, na.ctypes.data_as(_ip), _p(cen), _p(chg), _p(rad), carr, max_wave,
                                    wave_slots, hbm_budget_bytes, workers, res, st.ctypes.data_as(_ip), _p(done),
                                    _p(info))
        if check:
            _check(rc)
        keys = ["waves", "largest_wave", "peak_bytes", "merged_mixed_matvecs", "merged_fp64_matvecs",
                "active_fraction", "wave_ms", "prepared_bytes", "admitted_estimate_bytes"]
        out = [r.as_dict() for r in res]
        for r, t in zip(out, done.tolist()):
            r["done_ms"] = t
        return out, st.tolist(), dict(zip(keys, info.tolist()))

    def autotune(self, centers, charges, radii, cfg: Config, reps=5, install_min_points=-1) -> dict:
        """Time candidate launch parameters on this molecule (ibim_autotune); the best, with the
        default's cost.  install_min_points >= 0 adds it to the table as (cfg.np, install_min_points)."""
        c = _c(centers).reshape(-1, 3)
        q = _c(charges)
        r = _c(radii)
        rep = np.zeros(7)
        _check(lib().ibim_autotune(self.h, _p(c), _p(q), _p(r), len(q), C.byref(cfg), reps, install_min_points,
                                   _p(rep)))
        return dict(points=int(rep[0]), near_seg_pairs=int(rep[1]), nearff_seg_pairs=int(rep[2]),
                    tc_form=int(rep[3]), best_ms=rep[4], default_ms=rep[5], candidates=int(rep[6]))

    def grid(self, n, lo, h, value=0.0) -> "Grid":
        g = _vp()
        _check(lib().ibim_grid_create(self.h, int(n[0]), int(n[1]), int(n[2]), lo[0], lo[1], lo[2], h, value,
                                      C.byref(g)))
        return Grid(self, g, tuple(int(v) for v in n))

    def levelset(self, centers, radii, cfg: Config):
        """main.cpp:45-60: returns (Grid, reinit steps (2,))."""
        c = _c(centers).reshape(-1, 3)
        r = _c(radii)
        g = _vp()
        steps = (C.c_int * 2)()
        _check(lib().ibim_levelset_build(self.h, _p(c), _p(r), len(r), C.byref(cfg), C.byref(g), steps))
        return Grid(self, g, tuple(cfg.n)), list(steps)

    def tube(self, points, normals, weights, h) -> "Tube":
        p = _c(points).reshape(-1, 3)
        n = _c(normals).reshape(-1, 3)
        w = _c(weights)
        t = _vp()
        _check(lib().ibim_tube_create(self.h, _p(p), _p(n), _p(w), len(w), h, C.byref(t)))
        return Tube(self, t)

    def solve(self, centers, charges, radii, cfg: Config) -> dict:
        c = _c(centers).reshape(-1, 3)
        q = _c(charges)
        r = _c(radii)
        res = Result()
        _check(lib().ibim_solve(self.h, _p(c), _p(q), _p(r), len(q), C.byref(cfg), C.byref(res)))
        return res.as_dict()

    def solve_dev(self, centers_ptr: int, charges_ptr: int, radii_ptr: int, natoms: int, cfg: Config) -> dict:
        res = Result()
        _check(lib().ibim_solve_dev(self.h, _vp(centers_ptr), _vp(charges_ptr), _vp(radii_ptr), natoms, C.byref(cfg),
                                    C.byref(res)))
        return res.as_dict()

    def solve_pqr(self, path: str, cfg: Config) -> dict:
        res = Result()
        _check(lib().ibim_solve_pqr(self.h, path.encode(), C.byref(cfg), C.byref(res)))
        return res.as_dict()


class Grid:
    """levelset.h:12-60 (Grid + levelset) on the device."""

    def __init__(self, ctx, h, n):
        self.ctx, self.h, self.n = ctx, h, n

    def close(self):
        if getattr(self, "h", None):
            lib().ibim_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def upload(self, a):
        a = _c(a)
        assert a.size == int(np.prod(self.n))
        _check(lib().ibim_grid_upload(self.h, _p(a)))

    def download(self):
        out = np.empty(self.n)
        _check(lib().ibim_grid_download(self.h, _p(out)))
        return out

    def scale(self, s):
        _check(lib().ibim_grid_scale(self.h, s))

    def copy_from(self, other: "Grid"):
        _check(lib().ibim_grid_copy(self.h, other.h))

    def expand(self, centers, radii, probe=1.4, band=8):
        c = _c(centers).reshape(-1, 3)
        r = _c(radii)
        _check(lib().ibim_levelset_expand(self.h, _p(c), _p(r), len(r), probe, band))

    def evolve(self, final_t, vel=1.0, cfl=0.2):
        _check(lib().ibim_levelset_evolve(self.h, final_t, vel, cfl))

    def reinitialize(self, phi0: "Grid", final_t, vel=1.0, cfl=0.5, thickness=2, thres=1e-4) -> int:
        st = C.c_int(0)
        _check(lib().ibim_levelset_reinitialize(self.h, phi0.h, final_t, vel, cfl, thickness, thres, C.byref(st)))
        return st.value

    def count_gradient(self, thickness, thres):
        bad, tot, acc = C.c_long(0), C.c_long(0), C.c_double(0)
        _check(lib().ibim_levelset_count_gradient(self.h, float(thickness), thres, C.byref(bad), C.byref(tot),
                                                  C.byref(acc)))
        return bad.value, tot.value, acc.value

    def surface(self, thickness, jacobian=False) -> "Tube":
        """Tube quadrature (Surface); jacobian=True multiplies the weights by the surface Jacobian."""
        t = _vp()
        n, inc = C.c_long(0), C.c_long(0)
        if jacobian:
            _check(lib().ibim_surface_extract_jacobian(self.h, thickness, 1, C.byref(t), C.byref(n), C.byref(inc)))
        else:
            _check(lib().ibim_surface_extract(self.h, thickness, C.byref(t), C.byref(n), C.byref(inc)))
        tb = Tube(self.ctx, t)
        tb.inclusion = inc.value
        return tb


class Tube:
    """Surface (levelset.h:62-72): tube points, normals and cosine weights on the device."""

    def __init__(self, ctx, h):
        self.ctx, self.h = ctx, h
        self.inclusion = 0

    def close(self):
        if getattr(self, "h", None):
            lib().ibim_tube_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __len__(self):
        return int(lib().ibim_tube_size(self.h))

    def download(self):
        n = len(self)
        p = np.empty((n, 3))
        q = np.empty((n, 3))
        w = np.empty(n)
        _check(lib().ibim_tube_download(self.h, _p(p), _p(q), _p(w)))
        return p, q, w

    def surface7(self):
        p, q, w = self.download()
        return np.concatenate([p, q, w[:, None]], axis=1)

    def plan(self, order, maxpoint, maxlevel=10, targets=None, precision=PRECISION_FP64) -> "Plan":
        pl = _vp()
        if targets is None:
            _check(lib().ibim_fmm_plan(self.h, None, 0, order, maxpoint, maxlevel, precision, C.byref(pl)))
            nt = len(self)
        else:
            t = _c(targets).reshape(-1, 3)
            _check(lib().ibim_fmm_plan(self.h, _p(t), len(t), order, maxpoint, maxlevel, precision, C.byref(pl)))
            nt = len(t)
        return Plan(self, pl, len(self), nt)

    def electric(self, centers, charges, cfg: Config, want_x=False):
        c = _c(centers).reshape(-1, 3)
        q = _c(charges)
        res = Result()
        n = len(self)
        x = np.empty(2 * n) if want_x else None
        pot = np.empty(len(q))
        _check(lib().ibim_electric(self.h, _p(c), _p(q), len(q), C.byref(cfg), _p(x) if want_x else None, _p(pot),
                                   C.byref(res)))
        d = res.as_dict()
        d["atom_potential"] = pot
        if want_x:
            d["x"] = x
        return d


class Plan:
    """bbfmm tree + lists + operators over a tube (bbfmm.h:149-270)."""

    def __init__(self, tube, h, ns, nt):
        self.tube, self.h, self.ns, self.nt = tube, h, ns, nt

    def close(self):
        if getattr(self, "h", None):
            lib().ibim_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def stats(self):
        s = (C.c_long * 8)()
        _check(lib().ibim_plan_stats(self.h, s))
        keys = ["nodes", "levels", "leaves", "v_pairs", "x_pairs", "near_pairs", "operators", "target_leaves"]
        return dict(zip(keys, list(s)))

    def apply(self, kernel: int, kp: KernelParams, dens):
        rows = 4 if kernel == KERNEL_BIE_FUSED else 1
        d = _c(dens).reshape(rows, self.ns)
        out = np.empty((rows, self.nt))
        _check(lib().ibim_fmm_apply(self.h, kernel, C.byref(kp), _p(d), _p(out)))
        return out if rows == 4 else out[0]

    def matvec(self, kp: KernelParams, x):
        x = _c(x)
        y = np.empty_like(x)
        _check(lib().ibim_bie_matvec(self.h, C.byref(kp), _p(x), _p(y)))
        return y

    def rhs(self, kp: KernelParams, centers, charges):
        c = _c(centers).reshape(-1, 3)
        q = _c(charges)
        b = np.empty(2 * self.ns)
        _check(lib().ibim_bie_rhs(self.h, C.byref(kp), _p(c), _p(q), len(q), _p(b)))
        return b

    def gmres(self, kp: KernelParams, b, x0=None, restart=30, maxiter=100, tol=1e-6, precision=PRECISION_FP64):
        b = _c(b)
        x = np.zeros_like(b) if x0 is None else _c(x0).copy()
        it, st, res = C.c_int(0), C.c_int(0), C.c_double(0)
        _check(lib().ibim_gmres_solve(self.h, C.byref(kp), _p(b), _p(x), restart, maxiter, tol, precision,
                                      C.byref(it), C.byref(st), C.byref(res)))
        return x, dict(iters=it.value, status=st.value, residual=res.value)

    def lists(self):
        """Tree + U/V/W/X lists in the reference's node numbering (inspection)."""
        return _read_lists(lambda buf, cap, need: lib().ibim_plan_lists(self.h, 0, buf, cap, need))


def _read_lists(call):
    need = C.c_long(0)
    st = call(None, 0, C.byref(need))
    if st != OK:
        raise IbimError(st, lib().ibim_last_error().decode())
    buf = np.zeros(need.value, np.int32)
    _check(call(buf.ctypes.data_as(_ip), need.value, C.byref(need)))
    return decode_lists(buf)


def decode_lists(buf):
    """Layout of ibim_plan_lists: nnodes, then per node (reference numbering):
    level, parent, leaf, empty, nsrc, then |U| U..., |V| V..., |W| W..., |X| X..."""
    nn = int(buf[0])
    pos = 1
    nodes = []
    for _ in range(nn):
        level, parent, leaf, empty, nsrc = (int(v) for v in buf[pos:pos + 5])
        pos += 5
        L = []
        for _w in range(4):
            k = int(buf[pos])
            L.append(buf[pos + 1:pos + 1 + k].copy())
            pos += 1 + k
        nodes.append(dict(level=level, parent=parent, leaf=leaf, empty=empty, nsrc=nsrc, U=L[0], V=L[1], W=L[2],
                          X=L[3]))
    return nodes


def tree_lists_host(points, maxpoint, maxlevel=10):
    """The host tree builder on (n,3) points, without a GPU (for inspection and tests)."""
    p = _c(points).reshape(-1, 3)
    return _read_lists(lambda buf, cap, need: lib().ibim_tree_lists_host(_p(p), len(p), maxpoint, maxlevel, buf, cap,
                                                                         need))


@dataclass
class Workload:
    """A solve request: atoms + config."""

    centers: np.ndarray
    charges: np.ndarray
    radii: np.ndarray
    cfg: Config


class Server:
    """Request loop on one GPU (ibim_server): requests admitted by an HBM budget in two phases, run
    as concurrent whole solves (`slots` threads), or with lockstep=True prepared by `slots` threads
    and solved in waves of up to max_wave requests on merged plans (ibim_server_create_lockstep)."""

    STAT_KEYS = ["submitted", "completed", "in_flight", "queued", "bytes_in_flight", "peak_bytes", "budget",
                 "waves"]

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget_bytes: float = 150e9, lockstep: bool = False,
                 max_wave: int = 32):
        h = _vp()
        if lockstep:
            _check(lib().ibim_server_create_lockstep(device, slots, max_wave, float(hbm_budget_bytes), C.byref(h)))
        else:
            _check(lib().ibim_server_create(device, slots, float(hbm_budget_bytes), C.byref(h)))
        self.h = h

    def submit(self, centers, charges, radii, cfg: Config) -> int:
        c = _c(centers).reshape(-1, 3)
        q = _c(charges)
        r = _c(radii)
        rid = C.c_long(0)
        _check(lib().ibim_server_submit(self.h, _p(c), _p(q), _p(r), len(q), C.byref(cfg), C.byref(rid)))
        return rid.value

    def _out(self, st, res, lat, run):
        if st.value != OK:
            raise IbimError(st.value, lib().ibim_last_error().decode())
        d = res.as_dict()
        d.update(latency_ms=lat.value, run_ms=run.value)
        return d

    def poll(self, rid: int):
        """The result dict once the request has finished (collecting it), else None."""
        done, st, res, lat, run = C.c_int(0), C.c_int(0), Result(), C.c_double(0), C.c_double(0)
        _check(lib().ibim_server_poll(self.h, rid, C.byref(done), C.byref(st), C.byref(res), C.byref(lat),
                                      C.byref(run)))
        return self._out(st, res, lat, run) if done.value else None

    def wait(self, rid: int) -> dict:
        st, res, lat, run = C.c_int(0), Result(), C.c_double(0), C.c_double(0)
        _check(lib().ibim_server_wait(self.h, rid, C.byref(st), C.byref(res), C.byref(lat), C.byref(run)))
        return self._out(st, res, lat, run)

    def stats(self) -> dict:
        s = (C.c_double * 8)()
        _check(lib().ibim_server_stats(self.h, s))
        return dict(zip(self.STAT_KEYS, list(s)))

    def close(self):
        if getattr(self, "h", None):
            lib().ibim_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def request_bytes_estimate(cfg: Config) -> float:
    return float(lib().ibim_request_bytes_estimate(C.byref(cfg)))


def tuning_get(order: int, npoints: int) -> dict:
    out = (C.c_long * 3)()
    _check(lib().ibim_tuning_get(order, npoints, out))
    return dict(near_seg_pairs=out[0], nearff_seg_pairs=out[1], tc_form=out[2])


def fmm_bytes_estimate(cfg: Config, npoints: int) -> float:
    return float(lib().ibim_fmm_bytes_estimate(C.byref(cfg), int(npoints)))
