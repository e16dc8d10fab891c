"""Pins of the oracle's sigmoid expansions (Sigmoid1d, CreateSigmoid's
parameters, RectifiedMultivariateExpansion, UnivariateExpansion) against the
reference's own tests (no GPU).  Each test names the reference test it
restates."""
import math

import numpy as np
import pytest

SUPPORT = 100.0


def _multi_sigmoid_params(num_sigmoids=3, edge_bound=3.0):
    # tests/Test_Sigmoid.cpp:181-199 (also Test_RectifiedMultivariateExpansion.cpp:268-283):
    # integer division in 4*(-(k-1)/2 + i) as in the C++ source.
    n = 2 + num_sigmoids * (num_sigmoids + 1) // 2
    c, w, wt = np.zeros(n), np.zeros(n), np.zeros(n)
    c[0], w[0], wt[0] = -edge_bound, 2 * edge_bound / 10, 1.0
    c[1], w[1], wt[1] = edge_bound, 2 * edge_bound / 10, 1.0
    idx = 2
    for k in range(1, num_sigmoids + 1):
        for i in range(k):
            c[idx] = 4 * (-((k - 1) // 2) + i)
            w[idx] = 1 / (i + 1.0)
            wt[idx] = 1.0 / k
            idx += 1
    starts = np.array([2 + k * (k + 1) // 2 for k in range(num_sigmoids)], np.uint32)
    return c, w, wt, starts


def _check_gradients(O, prm, order, fd=1e-7):
    # TestSigmoidGradients (tests/Test_Sigmoid.cpp:14-70).
    for x in np.linspace(-3.0, 3.0, 100):
        v, _, _ = O.sigmoid_eval(prm, x, order, 0)
        vp, _, _ = O.sigmoid_eval(prm, x + fd, order, 0)
        v1, d1, _ = O.sigmoid_eval(prm, x, order, 1)
        v1p, d1p, _ = O.sigmoid_eval(prm, x + fd, order, 1)
        v2, d12, d2 = O.sigmoid_eval(prm, x, order, 2)
        np.testing.assert_array_equal(v1, v)
        np.testing.assert_array_equal(v2, v)
        np.testing.assert_array_equal(d12, d1)
        fdd = (vp - v) / fd
        fdd2 = (d1p - d1) / fd
        for j in range(order + 1):
            for calc, ref in ((d1[j], fdd[j]), (d2[j], fdd2[j])):
                if ref == 0.0:
                    assert abs(calc) <= 1e-12
                else:
                    assert abs(calc - ref) <= math.sqrt(fd) * max(abs(calc), abs(ref))


# tests/Test_Sigmoid.cpp:92-119 -- sizes that cannot form a Linear sum.
def test_sigmoid_initialization(oracle):
    O = oracle
    for n in (0, 1, 2 + 1 + 2 + 3 + 5, 2 + (1 + 3)):
        with pytest.raises(ValueError):
            O.sigmoid_from_centers(np.zeros(n)) if n >= 2 else O.sigmoid_eval(
                (np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(0, np.uint32)), 0.0, 0)
    # two centers: affine + 2 edge terms; three: one sigmoid
    assert len(O.sigmoid_from_centers(np.zeros(2))[3]) == 0
    prm = O.sigmoid_from_centers(np.zeros(3))
    assert list(prm[3]) == [2]
    O.sigmoid_eval(prm, 0.0, 4)
    with pytest.raises(ValueError):
        O.sigmoid_eval(prm, 0.0, 5)  # order 1 + 2 + 1 = 4


# tests/Test_Sigmoid.cpp:121-179 -- one sigmoid, known values at -100, 0, 100.
def test_single_sigmoid_known_values(oracle):
    O = oracle
    prm = (np.zeros(3), np.ones(3), np.ones(3), np.array([2], np.uint32))
    expect = [[1.0, -SUPPORT, -SUPPORT, 0.0, 0.0], [1.0, 0.0, -math.log(2), math.log(2), 0.5],
              [1.0, SUPPORT, 0.0, SUPPORT, 1.0]]
    for x, e in zip((-SUPPORT, 0.0, SUPPORT), expect):
        v = O.sigmoid_eval(prm, x, 4, 0)[0]
        for a, b in zip(v, e):
            if b == 0.0:
                assert a == 0.0
            else:
                assert abs(a - b) <= 1e-12 * abs(b)
    prev = 0.0
    for x in np.linspace(-5.0, 5.0, 100):
        v = O.sigmoid_eval(prm, x, 4, 0)[0]
        assert v[0] == 1.0 and v[1] == x and v[3] > prev
        prev = v[3]
    _check_gradients(O, prm, 4)


# tests/Test_Sigmoid.cpp:181-248 -- three sigmoid terms: limits and monotonicity.
def test_multiple_sigmoids(oracle):
    O = oracle
    prm = _multi_sigmoid_params()
    order = 6
    edge = 3.0
    lo = O.sigmoid_eval(prm, -SUPPORT, order, 0)[0]
    hi = O.sigmoid_eval(prm, SUPPORT, order, 0)[0]
    exp_lo = [1.0, -SUPPORT, -(SUPPORT - edge) * prm[1][0], 0.0]
    exp_hi = [1.0, SUPPORT, 0.0, (SUPPORT - edge) * prm[1][1]]
    for j in range(4):
        assert lo[j] == exp_lo[j] and hi[j] == exp_hi[j]
    for j in range(4, order + 1):
        assert abs(lo[j]) <= 1e-12 and abs(hi[j] - 1.0) <= 1e-12
    prev = np.zeros(order + 1)
    prev[2] = -2 * SUPPORT
    for x in np.linspace(-5.0, 5.0, 100):
        v = O.sigmoid_eval(prm, x, order, 0)[0]
        assert v[0] == 1.0 and v[1] == x
        assert (v[2:] > prev[2:]).all()
        prev = v
    _check_gradients(O, prm, order)


# src/MapFactory.cpp:181-254 -- the factory's widths and weights.
def test_sigmoid_factory_parameters(oracle):
    O = oracle
    c = np.array([-3.0, 3.0, 0.0, -1.0, 1.0, -2.0, 0.0, 2.0])  # Linear, three sigmoid terms
    oc, w, wt, st = O.sigmoid_from_centers(c, 1.5, O.SUM_LINEAR)
    np.testing.assert_array_equal(oc, c)
    assert list(st) == [2, 3, 5]
    assert w[0] == 1.5 and w[1] == 1.5 and wt[0] == 1 / 1.5 and wt[1] == 1 / 1.5
    # term i has i + 1 sigmoids; widths 2 / (next - prev) for all but its last (width 0)
    assert w[2] == 0.0
    assert w[3] == 2 / (c[1] - c[0]) and w[4] == 0.0
    assert w[5] == 2 / (c[5] - c[0]) and w[6] == 2 / (c[1] - c[5]) and w[7] == 0.0
    assert (wt[2:] == 1.0).all()
    # Constant: interior centers sorted, neighbour spacings
    c2 = np.array([-3.0, 3.0, 1.0, -1.0, 0.5])
    oc, w, wt, st = O.sigmoid_from_centers(c2, 2.0, O.SUM_CONSTANT)
    np.testing.assert_array_equal(oc, [-3.0, 3.0, -1.0, 0.5, 1.0])
    assert list(st) == [2, 3, 4]
    assert w[2] == 4.0 / (0.5 + 1.0) and w[3] == 8.0 / (1.0 + 1.0) and w[4] == 4.0 / (1.0 - 0.5)
    oc, w, wt, st = O.sigmoid_from_centers(np.array([-3.0, 3.0, 0.2]), 2.0, O.SUM_CONSTANT)
    assert w[2] == 8.0 / 6.0


# bindings/python/tests/test_MapFactory.py:104-137 -- sizes of the factory's sets.
def test_sigmoid_mset_sizes(oracle):
    O = oracle
    num_sig, deg, dim = 5, 3, 6
    s, d, o = O.sigmoid_mset(dim, deg, deg, num_sig)
    assert len(s) - 1 == (num_sig + 4) * math.comb(dim - 1 + deg, dim - 1)
    # first block: leading total order x {0}; second: leading cross order x {1..n+3}
    n1 = math.comb(dim - 1 + deg, deg)
    for t in range(n1):
        assert (d[s[t]:s[t + 1]] < dim - 1).all()
    for t in range(n1, len(s) - 1):
        assert d[s[t + 1] - 1] == dim - 1
        assert o[s[t + 1] - 1] == 1 + (t - n1) % (num_sig + 3)
    s1, _, o1 = O.sigmoid_mset(1, deg, deg, num_sig)
    assert len(s1) - 1 == num_sig + 4 and list(o1) == list(range(1, num_sig + 4))


def _comp(O, dim, order, params, pos=None):
    pos = O.POS_SOFTPLUS if pos is None else pos
    s, d, o = O.total_order(dim, order)
    return O.OracleSigmoidComponent(dim, s, d, o, params, pos), (s, d, o)


def _index(s, d, o, multi):
    for t in range(len(s) - 1):
        m = [0] * len(multi)
        for i in range(s[t], s[t + 1]):
            m[d[i]] = int(o[i])
        if m == list(multi):
            return t
    raise KeyError(multi)


def _hf(O, k, x):
    import ctypes as C
    v = np.zeros(k + 1)
    O.lib().orc_basis(2, 1, 0, k, x, v.ctypes.data_as(C.POINTER(C.c_double)), v.ctypes.data_as(
        C.POINTER(C.c_double)), v.ctypes.data_as(C.POINTER(C.c_double)))
    return v[k]


# tests/Test_RectifiedMultivariateExpansion.cpp:157-266 -- one sigmoid: the
# diagonal shapes (up to the constant that the rectified empty product gives),
# the leading-input terms, and SoftPlus(leading) * diagonal.
def test_single_sigmoid_rectified_expansion(oracle):
    O = oracle
    prm = (np.array([-1.0, 1.0, 0.0]), np.ones(3), np.ones(3), np.array([2], np.uint32))
    comp, (s, d, o) = _comp(O, 2, 4, prm)
    N = 20
    h = (N - 1) / 2
    grid = np.array([3 * (i - h) / h for i in range(N)])
    pts = np.zeros((2, N + 1))
    pts[0, :N], pts[1, :N] = -grid, grid
    pts[1, N] = 1.0
    edge_inv = math.log(math.e - 1) + 1
    sp = lambda x: O.lib().orc_posfunc(O.POS_SOFTPLUS, 0, x)
    diag = {}
    for order in range(1, 5):
        c = np.zeros(len(s) - 1)
        c[_index(s, d, o, (0, order))] = 1.0
        ev = comp.evaluate(c, pts)
        prop = abs(ev[N])
        for i in range(N):
            y = grid[i]
            ref = {1: y, 2: -sp(-(y + 1)), 3: sp(y - 1), 4: 0.5 + 0.5 * math.tanh(y / 2)}[order]
            val = ev[i] / prop
            diag[order, i] = val
            assert abs(val - ref) <= 1e-14 * abs(ref) + (1e-300 if ref == 0 else 0)
        pts[1, N] = {1: -edge_inv, 2: edge_inv, 3: 100.0, 4: pts[1, N]}[order]
    off = {}
    for k in range(5):
        c = np.zeros(len(s) - 1)
        c[_index(s, d, o, (k, 0))] = 1.0
        ev = comp.evaluate(c, pts)
        for i in range(N):
            ref = _hf(O, k, pts[0, i])
            assert abs(ev[i] - ref) <= 1e-14 * abs(ref)
            off[k, i] = ev[i]
    for t in range(len(s) - 1):
        if d[s[t + 1] - 1] != 1 if s[t + 1] > s[t] else True:
            continue
        m = [0, 0]
        for i in range(s[t], s[t + 1]):
            m[d[i]] = int(o[i])
        c = np.zeros(len(s) - 1)
        c[t] = 1.0
        ev = comp.evaluate(c, pts)
        for i in range(N):
            ref = sp(off[m[0], i]) * diag[m[1], i]
            assert abs(ev[i] - ref) <= 1e-14 * abs(ref)


def _multi_setup(O):
    # tests/Test_RectifiedMultivariateExpansion.cpp:256-318
    dim, order = 3, 4
    s, d, o = O.total_order(dim, order)
    keep = [t for t in range(len(s) - 1) if s[t + 1] > s[t] and d[s[t + 1] - 1] == dim - 1]
    starts, dims, orders = [0], [], []
    for t in keep:
        dims.extend(d[s[t]:s[t + 1]]); orders.extend(o[s[t]:s[t + 1]]); starts.append(len(dims))
    comp = O.OracleSigmoidComponent(dim, starts, dims, orders, _multi_sigmoid_params(), O.POS_SOFTPLUS)
    nc = comp.num_coeffs
    coeffs = np.array([1.0 - c / nc for c in range(nc)])
    N = 20
    pts = np.array([[(j + i - j * i) / (N - 1) for i in range(N)] for j in range(dim)])
    sens = np.array([0.5 if i % 3 else -0.5 for i in range(N)])
    return comp, coeffs, pts, sens


def _rel(a, b, tol):
    return abs(a - b) <= tol * max(abs(a), abs(b))


# tests/Test_RectifiedMultivariateExpansion.cpp:319-429 -- finite-difference
# consistency of every derivative and the inverse.
def test_multiple_sigmoid_rectified_expansion(oracle):
    O = oracle
    comp, c, pts, sens = _multi_setup(O)
    fd = 1e-6
    dim, N = pts.shape
    ev = comp.evaluate(c, pts)
    g = comp.gradient(c, pts, sens)
    for j in range(dim):
        p = pts.copy(); p[j] += fd
        fdd = (comp.evaluate(c, p) - ev) / fd
        for i in range(N):
            assert _rel(g[j, i], fdd[i] * sens[i], 20 * fd)
    cg = comp.coeff_grad(c, pts, sens)
    for j in range(comp.num_coeffs):
        cc = c.copy(); cc[j] += fd
        fdd = (comp.evaluate(cc, pts) - ev) / fd
        for i in range(N):
            if abs(fdd[i]) > fd:
                assert _rel(cg[j, i], fdd[i] * sens[i], 20 * fd)
            else:
                assert abs(cg[j, i] - fdd[i] * sens[i]) <= 1e-9
    ld = comp.logdet(c, pts)
    p = pts.copy(); p[dim - 1] += fd
    for i in range(N):
        assert _rel(ld[i], math.log((comp.evaluate(c, p)[i] - ev[i]) / fd), 20 * fd)
    lg = comp.logdet_input_grad(c, pts)
    for j in range(dim):
        p = pts.copy(); p[j] += fd
        fdd = (comp.logdet(c, p) - ld) / fd
        for i in range(N):
            assert _rel(lg[j, i], fdd[i], 20 * fd)
    lcg = comp.logdet_coeff_grad(c, pts)
    for j in range(comp.num_coeffs):
        cc = c.copy(); cc[j] += fd
        fdd = (comp.logdet(cc, pts) - ld) / fd
        for i in range(N):
            assert _rel(lcg[j, i], fdd[i], 20 * fd)
    xs = np.vstack([pts[:dim - 1], pts[dim - 2:dim - 1]])  # initial guess: the last conditioning input
    inv = comp.inverse(c, xs, ev)
    assert np.abs(inv - pts[dim - 1]).max() <= 1e-6 * (1 + 1e-6)


# MParT/UnivariateExpansion.h -- one input: no rectifier, inverse from 0.
def test_univariate_sigmoid_expansion(oracle):
    O = oracle
    prm = _multi_sigmoid_params()
    s, d, o = O.sigmoid_mset(1, 0, 0, 3)
    comp = O.OracleSigmoidComponent(1, s, d, o, prm)
    c = np.array([0.3, 0.5, 0.2, 0.1, 0.4, 0.3, 0.2])
    x = np.linspace(-4, 4, 33)[None, :]
    ev = comp.evaluate(c, x)
    ref = np.array([sum(ck * vk for ck, vk in zip(c, O.sigmoid_eval(prm, xi, 6, 0)[0])) for xi in x[0]])
    np.testing.assert_allclose(ev, ref, rtol=1e-15, atol=1e-15)
    ld = comp.logdet(c, x)
    dref = np.array([sum(ck * vk for ck, vk in zip(c, O.sigmoid_eval(prm, xi, 6, 1)[1])) for xi in x[0]])
    np.testing.assert_allclose(ld, np.log(dref), rtol=1e-14)
    inv = comp.inverse(c, np.zeros((1, 1)), ev)
    assert np.abs(inv - x[0]).max() <= 1e-6 * (1 + 1e-6)  # xtol, up to the bracket midpoint's rounding
