"""GMRES on a caller's operator (ibim_gmres_host, the reference's GMRES(std::function<Vector(Vector&)>,
...) of gmres.h:20-21): Krylov basis on the GPU, products through a host callback.  Checked
against the oracle's restatement of gmres.cpp:50-164 on the same operator: the same iteration and
product counts, the same solution; through the restart path and from a nonzero initial guess;
a failing callback ends the solve with its own status."""

import ctypes

import numpy as np
import pytest

import ibim
import oracle as O

pytestmark = pytest.mark.gpu


def dense_operator(n, seed):
    rng = np.random.default_rng(seed)
    A = np.eye(n) + 0.6 * rng.standard_normal((n, n)) / np.sqrt(n)
    return A, rng.standard_normal(n)


@pytest.mark.parametrize("restart,x0", [(40, False), (7, False), (7, True)])
def test_host_gmres_matches_oracle_gmres(ctx, restart, x0):
    A, b = dense_operator(300, 11)
    x_init = np.linspace(-1.0, 1.0, 300) if x0 else None
    calls = [0]

    def apply(x):
        calls[0] += 1
        return A @ x

    x, info = ctx.gmres(apply, b, x0=x_init, restart=restart, maxiter=300, tol=1e-10)
    xo, rc, it, mv = O.gmres(lambda v: A @ v, b, x0=x_init, m=restart, max_iter=300, tol=1e-10)
    assert info["status"] == 0 and rc == 0
    assert info["matvecs"] == mv == calls[0]
    assert info["iters"] == it
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
    assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()


def test_host_gmres_reports_nonconvergence(ctx):
    A, b = dense_operator(200, 5)
    x, info = ctx.gmres(lambda v: A @ v, b, restart=5, maxiter=12, tol=1e-14)
    assert info["status"] == 1 and info["iters"] == 12


def test_host_gmres_callback_failure_is_reported(ctx):
    A, b = dense_operator(64, 3)
    n = len(b)

    def failing(_user, xp, yp, nn):
        return 1

    fn = ibim.APPLY_FN(failing)
    x = np.zeros(n)
    it, mv, st, res = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = ibim.lib().ibim_gmres_host(ctx.h, n, fn, None, b.ctypes.data_as(dp), x.ctypes.data_as(dp), 10, 10, 1e-8,
                                    ctypes.byref(it), ctypes.byref(mv), ctypes.byref(st), ctypes.byref(res))
    assert rc == ibim.ERR_CALLBACK
    assert np.all(x == 0)
    with pytest.raises(ZeroDivisionError):
        ctx.gmres(lambda v: 1 / 0, b)


def test_host_gmres_on_the_bie_operator_reproduces_reference(ctx, golden):
    """The closure of electric.cpp:390-392 (dmapping) applied through ibim_bie_matvec: the
    reference's product count and solution on the 1hje fixture."""
    from conftest import config_for

    G = golden("p1hje")
    P = G["params"]
    s = G["surface"]
    tube = ctx.tube(s[:, :3], s[:, 3:6], s[:, 6], P["h"])
    plan = tube.plan(P["np"], P["maxpoint"], P["maxlevel"])
    kp = ibim.kernel_params(P["kappa"], P["dE"], P["dI"], P["tau"])
    b = plan.rhs(kp, G["centers"], G["charges"])
    x, info = ctx.gmres(lambda v: plan.matvec(kp, v), b, restart=P["restart"], maxiter=P["maxiter"], tol=P["tol"])
    assert info["status"] == 0
    assert info["matvecs"] == int(P["scalars"]["REF_MATVECS"])
    N = len(s)
    idx = G["sample_idx"]
    xs = np.concatenate([x[idx], x[N + idx]])
    assert np.abs(xs - G["solution_sample"]).max() / np.abs(G["solution_sample"]).max() < 1e-8
    assert config_for(P).restart == P["restart"]
