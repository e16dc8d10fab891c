"""Adaptive transport maps (TrainMapAdaptive) and the reference-style
TrainMap(map, objective, options) entry point.

CPU: the reduced margin against a brute-force definition, and the option
defaults of MParT/TrainMap.h and MParT/TrainMapAdaptive.h.  GPU: the
reference's own Python tests for these entry points
(bindings/python/tests/test_TrainMapAdaptive.py and test_TrainMap.py: banana
samples, seed 43, a test objective below 5 and a Kolmogorov-Smirnov statistic
of the pulled-back test samples below 0.1), with AdaptiveClenshawCurtis
quadrature in place of the reference's default AdaptiveSimpson."""
import itertools
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def M():
    import mpart_gb300
    mpart_gb300.load()
    return mpart_gb300


def _brute_reduced_margin(terms, length):
    s = set(terms)
    top = max(max(t) for t in terms) + 1
    out = set()
    for m in itertools.product(range(top + 1), repeat=length):
        if m in s:
            continue
        back = [m[:d] + (m[d] - 1,) + m[d + 1:] for d in range(length) if m[d] > 0]
        if back and all(b in s for b in back):
            out.add(m)
    return out


def test_reduced_margin_matches_definition(M):
    rng = np.random.default_rng(0)
    for length in (1, 2, 3, 4):
        s = M.MultiIndexSet.CreateTotalOrder(length, 0)
        for _ in range(12):
            rm = [tuple(int(v) for v in m) for m in s.ReducedMargin()]
            assert len(rm) == len(set(rm))
            assert set(rm) == _brute_reduced_margin(s._terms, length)
            s += rm[rng.integers(len(rm))]  # stays downward closed
    # the reference's order (entries by first appearance; Expand: the frontier's
    # terms in order, each one's forward neighbours by first appearance, a term
    # reached twice returned twice); tests/test_reference_pins.py checks it
    # against the reference's MultiIndexSet on many sets
    s = M.MultiIndexSet.CreateTotalOrder(2, 1)
    assert [tuple(int(v) for v in m) for m in s.ReducedMargin()] == [(1, 1), (0, 2), (2, 0)]
    assert s.Expand() == [3, 4, 3, 5]
    assert [tuple(int(v) for v in t) for t in s._terms][3:] == [(1, 1), (0, 2), (2, 0)]


def test_option_defaults(M):
    t = M.TrainOptions()  # MParT/TrainMap.h:19-37
    assert (t.opt_ftol_rel, t.opt_ftol_abs, t.opt_xtol_rel, t.opt_xtol_abs, t.opt_maxeval) == (1e-3, 1e-3, 1e-4,
                                                                                               1e-4, 1000)
    a = M.ATMOptions()  # MParT/TrainMapAdaptive.h:19-27
    assert a.maxPatience == 10 and a.maxSize == 2 ** 31 - 1 and a.maxDegrees is None
    assert a.quadType == M.QuadTypes.AdaptiveSimpson and a.opt_maxeval == 1000


def _banana(n, seed=43):
    np.random.seed(seed)
    s = np.random.randn(2, n)
    return np.vstack([s[0], s[1] + s[0] ** 2])


def _ks(tmap, test):
    import torch
    y = tmap.Evaluate(torch.as_tensor(test, device="cuda")).cpu().numpy()
    srt = np.sort(y.flatten())
    cdf = (1 + np.vectorize(math.erf)(srt / np.sqrt(2))) / 2
    ecdf = (np.arange(y.size) + 1) / y.size
    return np.abs(cdf - ecdf).max()


@pytest.mark.gpu
def test_train_map_adaptive_banana(gpu):
    M = gpu
    samples = _banana(5000)
    test, train = samples[:, :1000], samples[:, 1000:]
    obj = M.CreateGaussianKLObjective(train, test)
    opts = M.ATMOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis)
    msets = [M.MultiIndexSet.CreateTotalOrder(d + 1, 1) for d in range(2)]
    first = M.TriangularMap([M.CreateComponent(m.Fix(), opts) for m in msets], True)
    M.TrainMap(first, obj, opts)
    tmap = M.TrainMapAdaptive(msets, obj, opts)
    assert msets[1].Size() > 3
    assert obj.TestError(tmap) < 5.0
    assert _ks(tmap, test) < 0.1
    # the selected sets are downward closed and the result is no worse than the start
    for m in msets:
        terms = set(m._terms)
        for t in terms:
            for d in range(len(t)):
                if t[d]:
                    assert t[:d] + (t[d] - 1,) + t[d + 1:] in terms
    assert tmap.atm_result["best_test_error"] <= obj.TestError(first) + 1e-12
    assert tmap.atm_result["final_test_error"] <= tmap.atm_result["best_test_error"] + 1e-3
    assert tmap.numCoeffs == sum(m.Size() for m in msets)


@pytest.mark.gpu
def test_train_map_with_objective_and_options(gpu):
    M = gpu
    samples = _banana(20000)
    test, train = samples[:, :4000], samples[:, 4000:]
    obj2 = M.CreateGaussianKLObjective(train, test)
    obj1 = M.CreateGaussianKLObjective(train, test, 1)
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis)
    map2 = M.CreateTriangular(2, 2, 2, opts)
    map1 = M.CreateComponent(M.FixedMultiIndexSet(2, 2), opts)
    M.TrainMap(map2, obj2, M.TrainOptions())
    M.TrainMap(map1, obj1, M.TrainOptions())
    assert obj1.TestError(map1) < 5.0
    assert obj2.TestError(map2) < 5.0
    assert _ks(map1, test) < 0.1
    assert _ks(map2, test) < 0.1


@pytest.mark.gpu
def test_train_map_starts_unset_coefficients_at_one(gpu):
    """src/TrainMap.cpp:168-176: a map whose coefficients were never set starts
    from ones."""
    import torch
    M = gpu
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis)
    X = torch.as_tensor(_banana(2000), device="cuda")
    maps = []
    for start in (None, 1.0):
        comps = [M.CreateComponent(M.FixedMultiIndexSet(d + 1, 2), opts) for d in range(2)]
        tri = M.TriangularMap(comps, False)
        if start is not None:
            tri.SetCoeffs(np.full(tri.numCoeffs, start))
        loss, res = M.TrainMap(tri, X, max_iters=5)
        assert np.isfinite(loss).all()
        maps.append(np.asarray(tri.CoeffMap()))
    np.testing.assert_array_equal(maps[0], maps[1])


def test_expand_and_options_errors(M):
    """Bad arguments are refused on the host: an Expand of a zero-length set
    through the C ABI, an optimiser name this library does not provide."""
    import ctypes as C
    lib = M.load()
    n = C.c_uint()
    assert lib.mpgb_multi_index_expand(0, 0, None, C.byref(n), None, C.byref(n), None, 0) != 0
    with pytest.raises(ValueError):
        M.TrainOptions(opt_alg="LN_COBYLA")._train_c()
    assert M.TrainOptions()._train_c().algorithm == 0 and M.TrainOptions(opt_alg="LD_LBFGS")._train_c().algorithm == 1
