"""The optimisers behind TrainMap on host test problems (no GPU), through
mpgb_optimizer_self_test: SLSQP's unconstrained iteration (LD_SLSQP, the
reference's default algorithm) and the limited-memory BFGS (LD_LBFGS), with
and without the diagonal scaling TrainMap's preconditioner supplies.  The
problems are the extended Rosenbrock function (minimum 0 at all ones) and an
ill-conditioned quadratic (condition number 1e4, minimum 0 at all ones)."""
import ctypes as C

import numpy as np
import pytest

SLSQP, LBFGS = 0, 1


@pytest.fixture(scope="module")
def lib():
    import mpart_gb300
    return mpart_gb300.load()


def run(lib, alg, problem, n, iters, dinv=None):
    x = np.zeros(n)
    f = C.c_double()
    it, ev = C.c_int(), C.c_int()
    d = None if dinv is None else np.ascontiguousarray(dinv, dtype=np.float64)
    rc = lib.mpgb_optimizer_self_test(alg, problem, n, iters,
                                      None if d is None else d.ctypes.data_as(C.POINTER(C.c_double)),
                                      x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(f), C.byref(it), C.byref(ev))
    assert rc == 0
    return x, f.value, it.value, ev.value


@pytest.mark.parametrize("alg", [SLSQP, LBFGS])
def test_rosenbrock(lib, alg):
    x, f, it, ev = run(lib, alg, 0, 10, 2000)
    assert f < 1e-10 and np.allclose(x, 1.0, atol=1e-5), (f, it, ev)


def test_slsqp_bfgs_beats_limited_memory_on_ill_conditioned_quadratic(lib):
    """The full BFGS matrix learns the 1e4 spread of curvatures; the
    quadratic is solved to 1e-10 by both, the dense update in far fewer
    iterations."""
    _, f1, it1, _ = run(lib, SLSQP, 1, 30, 500)
    _, f2, it2, _ = run(lib, LBFGS, 1, 30, 5000)
    assert f1 < 1e-10 and f2 < 1e-10
    assert it1 < it2


def test_lbfgs_diagonal_scaling(lib):
    """With the exact inverse diagonal the quadratic is solved at once; the
    scaling is what TrainMap's preconditioner estimates from squared per-point
    gradients."""
    n = 30
    w = 10.0 ** (4.0 * np.arange(n) / (n - 1))
    x, f, it, _ = run(lib, LBFGS, 1, n, 100, dinv=1.0 / w)
    assert f < 1e-20 and it <= 2 and np.allclose(x, 1.0)
    _, f0, it0, _ = run(lib, LBFGS, 1, n, 100)
    assert it0 > 5 * it


def test_bad_arguments(lib):
    x = np.zeros(3)
    f = C.c_double()
    it, ev = C.c_int(), C.c_int()
    P = C.POINTER(C.c_double)
    assert lib.mpgb_optimizer_self_test(LBFGS, 0, 3, 10, None, x.ctypes.data_as(P), C.byref(f), C.byref(it),
                                        C.byref(ev)) != 0  # Rosenbrock needs an even n
    assert lib.mpgb_optimizer_self_test(7, 1, 3, 10, None, x.ctypes.data_as(P), C.byref(f), C.byref(it),
                                        C.byref(ev)) != 0  # unknown algorithm
