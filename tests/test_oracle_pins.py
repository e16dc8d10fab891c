"""Pins of the CPU oracle against the reference's own known-answer tests
(no GPU).  Each test names the reference test it restates."""
import math

import numpy as np
import pytest

XS = [-1.0, -0.5, 0.0, 0.1, 1.0]


def _basis(O, kind, normalize, which, p, x):
    import ctypes as C
    v = np.zeros(p + 1); d1 = np.zeros(p + 1); d2 = np.zeros(p + 1)
    dp = C.POINTER(C.c_double)
    O.lib().orc_basis(kind, int(normalize), which, p, x, v.ctypes.data_as(dp), d1.ctypes.data_as(dp),
                      d2.ctypes.data_as(dp))
    return v, d1, d2


# tests/Test_OrthogonalPolynomials.cpp:66-150 -- closed forms He_0..He_4.
def test_probabilist_hermite_closed_forms(oracle):
    for x in XS:
        he = [1.0, x, x * x - 1.0, x ** 3 - 3 * x, x ** 4 - 6 * x * x + 3.0]
        dhe = [0.0, 1.0, 2 * x, 3 * x * x - 3.0, 4 * x ** 3 - 12 * x]
        d2he = [0.0, 0.0, 2.0, 6 * x, 12 * x * x - 12.0]
        for which in (0, 1, 2):
            v, d1, d2 = _basis(oracle, 0, False, which, 4, x)
            np.testing.assert_allclose(v, he, rtol=1e-15, atol=1e-15)
            if which >= 1:
                np.testing.assert_allclose(d1, dhe, rtol=1e-15, atol=1e-15)
            if which == 2:
                np.testing.assert_allclose(d2, d2he, rtol=1e-15, atol=1e-15)


# tests/Test_OrthogonalPolynomials.cpp:11-63 -- normalisation against Gauss-Hermite quadrature.
def test_probabilist_hermite_normalisation(oracle):
    xg, wg = np.polynomial.hermite_e.hermegauss(15)
    for k in range(6):
        vals = np.array([_basis(oracle, 0, True, 0, 5, x)[0][k] for x in xg])
        norm = (wg * vals * vals).sum() / math.sqrt(2 * math.pi)
        # normalised He_k / sqrt(sqrt(2 pi) k!) has squared weighted norm 1/sqrt(2 pi)
        assert norm == pytest.approx(1.0 / math.sqrt(2 * math.pi), rel=1e-7)


# tests/Test_HermiteFunctions.cpp:9-103 -- closed forms psi_0..psi_4 (orders 2..6).
def test_hermite_functions_closed_forms(oracle):
    q = math.pi ** -0.25
    for x in XS:
        e = math.exp(-0.5 * x * x)
        truth = [1.0, x, q * e, math.sqrt(2.0) * q * x * e, 2 ** -0.5 * q * (2 * x * x - 1.0) * e,
                 3 ** -0.5 * q * (2 * x ** 3 - 3 * x) * e, 24 ** -0.5 * q * (4 * x ** 4 - 12 * x * x + 3.0) * e]
        for which in (0, 1, 2):
            v, d1, d2 = _basis(oracle, 2, False, which, 6, x)
            np.testing.assert_allclose(v, truth, rtol=1e-14, atol=1e-15)
        # derivatives by central differences of the closed form
        v, d1, d2 = _basis(oracle, 2, False, 2, 6, x)
        h = 1e-5
        vp = _basis(oracle, 2, False, 0, 6, x + h)[0]
        vm = _basis(oracle, 2, False, 0, 6, x - h)[0]
        np.testing.assert_allclose(d1, (vp - vm) / (2 * h), rtol=1e-8, atol=1e-9)
        np.testing.assert_allclose(d2, (vp - 2 * v + vm) / (h * h), rtol=1e-4, atol=1e-5)


# tests/Test_PositiveBijectors.cpp:13-36
def test_softplus(oracle):
    L = oracle.lib()
    for x in XS:
        assert L.orc_posfunc(1, 0, x) == pytest.approx(math.log(1.0 + math.exp(x)))
        assert L.orc_posfunc(1, 1, x) == pytest.approx(math.exp(x) / (math.exp(x) + 1.0))
    for x in (50.0, 100.0):
        assert L.orc_posfunc(1, 0, x) == pytest.approx(x)
        assert L.orc_posfunc(1, 1, x) == pytest.approx(1.0)
    assert L.orc_posfunc(0, 0, 0.3) == pytest.approx(math.exp(0.3))


# tests/Test_Quadrature.cpp:24-42 -- nested Clenshaw-Curtis points.
def test_cc_nesting(oracle):
    import ctypes as C
    dp = C.POINTER(C.c_double)
    L = oracle.lib()
    for level in (1, 2, 3):
        nc, nf = 2 ** level + 1, 2 ** (level + 1) + 1
        wc, pc, wf, pf = np.zeros(nc), np.zeros(nc), np.zeros(nf), np.zeros(nf)
        L.orc_cc_rule(nc, wc.ctypes.data_as(dp), pc.ctypes.data_as(dp))
        L.orc_cc_rule(nf, wf.ctypes.data_as(dp), pf.ctypes.data_as(dp))
        for i in range(nc):
            assert pc[i] == pf[2 * i]
        assert wc.sum() == pytest.approx(2.0, rel=1e-14)
        assert wf.sum() == pytest.approx(2.0, rel=1e-14)


def _acc(O, fid, level=2, maxsub=10, tol=1e-6, lb=0.0, ub=1.0):
    import ctypes as C
    res = np.zeros(2)
    n = C.c_long(0)
    O.lib().orc_acc_test(fid, level, maxsub, tol, tol, 0, lb, ub, res.ctypes.data_as(C.POINTER(C.c_double)),
                         C.byref(n))
    return res, n.value


# tests/Test_Quadrature.cpp:118-219 -- adaptive Clenshaw-Curtis known answers.
def test_acc_known_answers(oracle):
    res, _ = _acc(oracle, 0)
    assert res[0] == pytest.approx(math.e - 1.0, rel=1e-4)
    res, n = _acc(oracle, 1)
    assert res[0] == pytest.approx(0.5 + math.e - 1.0, rel=1e-4)
    assert n < 300
    res, _ = _acc(oracle, 2)
    assert res[0] == pytest.approx(math.e - 1.0, rel=1e-4)
    assert res[1] == pytest.approx(2 * (math.e - 1.0), rel=1e-4)
    # level 1 (the factory's quadPts = 5) is much tighter on a smooth integrand
    res, _ = _acc(oracle, 0, level=1, maxsub=30, tol=1e-10)
    assert res[0] == pytest.approx(math.e - 1.0, rel=1e-10)


def _quad(O, kind, fid, n=0, maxsub=30, tol=1e-8):
    import ctypes as C
    res = np.zeros(2)
    cnt = C.c_long(0)
    O.lib().orc_quad_test(kind, fid, n, maxsub, tol, tol, 0, 0.0, 1.0, res.ctypes.data_as(C.POINTER(C.c_double)),
                          C.byref(cnt))
    return res, cnt.value


# tests/Test_Quadrature.cpp:45-116 (ClenshawCurtis, 10 points) and :223-324 (AdaptiveSimpson).
def test_cc_and_simpson_known_answers(oracle):
    e1 = math.e - 1.0
    res, n = _quad(oracle, oracle.QUAD_CC, 0, n=10)
    assert res[0] == pytest.approx(e1, rel=1e-8) and n == 10
    res, _ = _quad(oracle, oracle.QUAD_CC, 2, n=10)
    assert res[0] == pytest.approx(e1, rel=1e-8) and res[1] == pytest.approx(2 * e1, rel=1e-8)
    res, _ = _quad(oracle, oracle.QUAD_SIMPSON, 0)
    assert res[0] == pytest.approx(e1, rel=1e-4)
    res, n = _quad(oracle, oracle.QUAD_SIMPSON, 1)
    assert res[0] == pytest.approx(0.5 + e1, rel=1e-4)
    assert n < 150
    res, _ = _quad(oracle, oracle.QUAD_SIMPSON, 2)
    assert res[0] == pytest.approx(e1, rel=1e-4) and res[1] == pytest.approx(2 * e1, rel=1e-4)
    # the adaptive kinds agree with each other on a smooth integrand at tight tolerance
    a, _ = _quad(oracle, oracle.QUAD_ACC, 0, n=1, tol=1e-12)
    s, _ = _quad(oracle, oracle.QUAD_SIMPSON, 0, tol=1e-12)
    assert a[0] == pytest.approx(e1, rel=1e-11) and s[0] == pytest.approx(e1, rel=1e-11)


# tests/Test_RootFinding.cpp:17-113
def test_root_finding(oracle):
    import ctypes as C
    L = oracle.lib()
    info = C.c_int(0)
    sig = lambda z: 1.0 / (math.exp(-z) + 1.0)
    combo = lambda x: sig(2 * (x - 1)) + 3 * sig(x * 0.5) + 0.5 * sig(1.5 * (x + 1))
    cases = [(0, 0.5, 0.0, 0.5), (0, 0.5, 1.0, 0.5), (1, sig(0.5), 0.0, 0.5), (1, sig(0.5), 1.0, 0.5),
             (2, combo(0.5), -5.0, 0.5), (2, combo(0.5), 5.0, 0.5)]
    for fid, yd, x0, xd in cases:
        x = L.orc_rootfind_test(fid, yd, x0, 1e-5, 1e-5, C.byref(info))
        assert x == pytest.approx(xd, rel=2e-5)
        assert info.value == 0
    x = L.orc_rootfind_test(3, 0.0, 0.0, 1e-5, 1e-5, C.byref(info))
    assert math.isnan(x) and info.value == -2
    # FindBracket on the linear function
    xlb, ylb, xub, yub = C.c_double(0.0), C.c_double(0.0), C.c_double(2.0), C.c_double(2.0)
    rc = L.orc_findbracket_test(0, C.byref(xlb), C.byref(ylb), C.byref(xub), C.byref(yub), -1.1)
    assert rc == 0 and xlb.value < -1.1 < xub.value
    rc = L.orc_findbracket_test(3, C.byref(C.c_double(0.0)), C.byref(C.c_double(-1.0)), C.byref(C.c_double(2.0)),
                                C.byref(C.c_double(-1.0)), 0.0)
    assert rc == -1


def _comp(O, dim, order, **kw):
    s, d, o = O.total_order(dim, order)
    return O.OracleComponent(dim, s, d, o, **kw)


# tests/Test_MultivariateExpansionWorker.cpp:67-80 and Test_MonotoneComponent.cpp:34 -- cache sizes.
def test_cache_size_and_term_order(oracle):
    c = _comp(oracle, 1, 1, normalize=False)
    assert c.cache_size == 6
    c = _comp(oracle, 3, 4)
    assert c.cache_size == (4 + 1) * (2 * 3 + 1)
    s, d, o = oracle.total_order(2, 2)
    # terms of the total-order set, last dimension fastest
    terms = []
    for t in range(len(s) - 1):
        m = [0, 0]
        for j in range(s[t], s[t + 1]):
            m[d[j]] = o[j]
        terms.append(tuple(m))
    assert terms == [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (2, 0)]


# tests/Test_MonotoneComponent.cpp:22-60 -- the integrand of f = 1 + x with Exp is e.
def test_integrand_affine_exp(oracle):
    c = _comp(oracle, 1, 1, normalize=False, posfunc=oracle.POS_EXP)
    for t in (0.0, 0.5, -0.5):
        assert c.integrand([1.0, 1.0], [1.0], t, 0)[0] == pytest.approx(math.e, rel=1e-7)
        assert c.integrand([1.0, 1.0], [1.0], t, 1)[0] == pytest.approx(math.e, rel=1e-7)
    # Parameters gradient vs forward differences (:62-84)
    g = c.integrand([1.0, 1.0], [1.0], 0.5, 2)
    for k in range(2):
        cp = np.array([1.0, 1.0]); cp[k] += 1e-4
        fd = (c.integrand(cp, [1.0], 0.5, 0)[0] - g[0]) / 1e-4
        assert g[1 + k] == pytest.approx(fd, rel=1e-4, abs=1e-8)


# tests/Test_MonotoneComponent.cpp:360-440 -- 1-D affine and quadratic closed forms.
def test_component_closed_forms(oracle):
    x = np.array([(i / (20 - 0.5)) * 4.0 + 2.0 for i in range(20)])[None, :]
    c = _comp(oracle, 1, 1, normalize=False, posfunc=oracle.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
    np.testing.assert_allclose(c.evaluate([1.0, 1.0], x), 1 + math.e * x[0], rtol=1e-7)
    c = _comp(oracle, 1, 2, normalize=False, posfunc=oracle.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
    np.testing.assert_allclose(c.evaluate([1.5, 1.0, 0.5], x), 1 + math.e * (np.exp(x[0]) - 1), rtol=1e-7)


# tests/Test_MonotoneComponent.cpp:443-557 -- bracket inverse round trip.
def test_component_inverse_round_trip(oracle):
    x = np.array([(i / 19.0) * 4.0 - 2.0 for i in range(20)])[None, :]
    c = _comp(oracle, 1, 2, normalize=False, posfunc=oracle.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
    coef = [1.5, 1.0, 0.5]
    y = c.evaluate(coef, x)
    xi = c.inverse(coef, x, y)
    np.testing.assert_allclose(xi, x[0], rtol=1e-6, atol=1e-6)
    # one x column broadcast over many ys (:527-556)
    xi = c.inverse(coef, np.zeros((1, 1)), y)
    np.testing.assert_allclose(xi, x[0], rtol=1e-6, atol=1e-6)


def _pts2(n=20):
    p = np.zeros((2, n))
    for i in range(n):
        p[0, i] = (i / (n - 1.0)) * 1.0 - 0.5
        p[1, i] = p[0, i]
    return p


# tests/Test_MonotoneComponent.cpp:561-735 -- FD checks of the Jacobians.
def test_component_jacobians_fd(oracle):
    c = _comp(oracle, 2, 2, normalize=False, posfunc=oracle.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
    coef = 0.1 * np.cos(0.01 * np.arange(c.num_terms))
    pts = _pts2()
    ev = c.evaluate(coef, pts)
    h = 1e-4
    right = pts.copy(); right[1] += h
    fd = (c.evaluate(coef, right) - ev) / h
    np.testing.assert_allclose(c.cont_derivative(coef, pts), fd, rtol=1e-4)
    ev2, jac = c.coeff_jacobian(coef, pts)
    np.testing.assert_allclose(ev2, ev, rtol=1e-12)
    for j in range(c.num_terms):
        cp = coef.copy(); cp[j] += h
        fdj = (c.evaluate(cp, pts) - ev) / h
        np.testing.assert_allclose(jac[j], fdj, rtol=5e-4, atol=1e-4)
    ev3, ij = c.input_jacobian(coef, pts)
    for d in range(2):
        pp = pts.copy(); pp[d] += h
        np.testing.assert_allclose(ij[d], (c.evaluate(coef, pp) - ev) / h, rtol=1e-4, atol=1e-3)
    lg = c.logdet_input_grad(coef, pts)
    ld = c.logdet(coef, pts)
    for d in range(2):
        pp = pts.copy(); pp[d] += 1e-6
        np.testing.assert_allclose(lg[d], (c.logdet(coef, pp) - ld) / 1e-6, rtol=1e-4, atol=1e-5)


# tests/Test_MonotoneComponent.cpp:792-877 -- CoeffGrad is linear in sens; LogDet coefficient gradient vs FD.
def test_component_coeffgrad_and_logdet_grad(oracle):
    c = _comp(oracle, 2, 3, normalize=False, posfunc=oracle.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
    coef = 0.1 * np.cos(0.01 * np.arange(c.num_terms))
    pts = np.tile(np.array([[0.3], [0.5]]), (1, 20))
    sens = 0.25 * (np.arange(20) + 1)
    g = c.coeff_grad(coef, pts, sens)
    for j in range(1, 20):
        np.testing.assert_allclose(g[:, j], (j + 1.0) * g[:, 0], rtol=1e-14)
    pts = np.stack([0.03 * np.arange(20), -0.05 * np.arange(20)])
    ld = c.logdet(coef, pts)
    lg = c.logdet_coeff_grad(coef, pts)
    for i in range(c.num_terms):
        cp = coef.copy(); cp[i] += 1e-4
        np.testing.assert_allclose(lg[i], (c.logdet(cp, pts) - ld) / 1e-4, rtol=1e-5, atol=1e-7)


# tests/Test_TriangularMap.cpp:10-228 -- block consistency, inverse round trip, FD gradients.
def test_triangular_map(oracle):
    tm = oracle.OracleTriangularMap(3, 3, 2, normalize=False)
    rng = np.random.default_rng(3)
    coef = 0.1 * rng.standard_normal(tm.num_coeffs)
    pts = rng.standard_normal((3, 25))
    ev = tm.evaluate(coef, pts)
    cs = tm.split(coef)
    for i, c in enumerate(tm.comps):
        np.testing.assert_array_equal(ev[i], c.evaluate(cs[i], pts[:c.input_dim]))
    ld = tm.logdet(coef, pts)
    np.testing.assert_allclose(ld, sum(c.logdet(cs[i], pts[:c.input_dim]) for i, c in enumerate(tm.comps)),
                               rtol=1e-14)
    xi = tm.inverse(coef, np.zeros((0, 25)), ev)
    np.testing.assert_allclose(xi, pts, atol=1e-5)
    sens = rng.standard_normal((3, 25))
    g = tm.coeff_grad(coef, pts, sens)
    for j in range(tm.num_coeffs):
        cp = coef.copy(); cp[j] += 1e-6
        fd = ((tm.evaluate(cp, pts) - ev) * sens).sum(axis=0) / 1e-6
        np.testing.assert_allclose(g[j], fd, rtol=1e-4, atol=1e-6)


# tests/Test_MapObjective.cpp:98-157 -- FastGaussianReverseKL matches KLObjective gradients.
def test_fast_gaussian_kl_matches_kl(oracle):
    tm = oracle.OracleTriangularMap(1, 1, 4)
    rng = np.random.default_rng(42)
    x = rng.standard_normal((1, 2000))
    for val in (0.1, 0.5, -0.1):
        coef = np.full(tm.num_coeffs, val)
        lf, gf = oracle.fast_gaussian_reverse_kl(tm.comps[0], coef, x)
        lk, gk = oracle.kl_objective(tm, coef, x)
        np.testing.assert_allclose(gf, gk, rtol=1e-12, atol=1e-14)
        # objectives differ by the constant 0.5 log(2 pi)
        assert lk - lf == pytest.approx(0.5 * math.log(2 * math.pi), rel=1e-12)


# Overflow of the Exp rectifier: the reference throws; the oracle flags the point.
def test_integrand_overflow_flag(oracle):
    c = _comp(oracle, 1, 1, normalize=False, posfunc=oracle.POS_EXP)
    out, nev, st = c.evaluate([0.0, 800.0], np.array([[1.0, 0.1]]), return_evals=True)
    assert st[0] == 1 and math.isnan(out[0])
    out, nev, st = c.evaluate([0.0, 1.0], np.array([[float("nan")]]), return_evals=True)
    assert st[0] == 2 and math.isnan(out[0]) and nev[0] <= 3


# tests/Test_MonotoneComponent.cpp:443-557 (inverse round trips), on the
# workloads of the GPU's two-pass inverse test: far roots and targets without
# a root.  The finite roots reproduce their targets.
@pytest.mark.parametrize("basis,pos,scale,rscale,bound", [(0, 1, 0.05, 3.0, 1e-9), (2, 0, 0.1, 2.0, 1e-8)])
def test_inverse_round_trip_far_roots(oracle, basis, pos, scale, rscale, bound):
    om = oracle.OracleTriangularMap(4, 4, 3, basis=basis, normalize=True, posfunc=pos, abs_tol=1e-8, rel_tol=1e-8,
                                    max_sub=30)
    coef = np.random.default_rng(11).normal(0.0, scale, om.num_coeffs)
    r = rscale * np.random.default_rng(12).standard_normal((4, 777))
    x = om.inverse(coef, np.zeros((0, 777)), r, 1e-10, 1e-10)
    ok = ~np.isnan(x).any(axis=0)
    assert ok.sum() > 500 and np.nanmax(np.abs(x)) > 7.0
    back = om.evaluate(coef, np.where(ok, x, 0.0))
    assert np.abs(back - r)[:, ok].max() < bound


def _itp_reference(f, yd, x0, xtol, ftol):
    """MParT/Utilities/RootFinding.h:20-178 (FindBracket, Find_x_ITP,
    InverseSingleBracket) restated in plain Python floats, independently of
    the oracle's C++."""
    xlb = xub = x0
    ylb = yub = f(x0)
    step = 1.0
    if ylb > yd:
        xub, yub = xlb, ylb
        for _ in range(128):
            xlb = xub - step
            ylb = f(xlb)
            if abs((yub - ylb) / (xub - xlb)) < 1e-12 and (xub - xlb) > 10:
                return math.nan
            if ylb > yd:
                yub, xub = ylb, xlb
                step *= 2.0
            else:
                break
        else:
            return math.nan
    else:
        for _ in range(128):
            xub = xlb + step
            yub = f(xub)
            if abs((yub - ylb) / (xub - xlb)) < 1e-12 and (xub - xlb) > 10:
                return math.nan
            if yub < yd:
                ylb, xlb = yub, xub
                step *= 2.0
            else:
                break
        else:
            return math.nan
    if ylb > yd or yub < yd:
        return math.nan
    nhalf = math.ceil(math.log2(0.5 * (xub - xlb) / xtol))
    for it in range(10000):
        xb = 0.5 * (xub + xlb)
        xf = (xub * ylb - xlb * yub) / (ylb - yub)
        sigma = 1.0 if (xb - xf) > 0 else -1.0
        delta = min(0.1 * (xub - xlb) ** 2, abs(xb - xf))
        xf += delta * sigma
        rho = min(xtol * 2.0 ** (nhalf + 1.0 - it) - 0.5 * (xub - xlb), abs(xf - xb))
        xc = xb - sigma * rho
        yc = f(xc)
        if abs(yc - yd) < ftol:
            return xc
        if yc > yd:
            xub, yub = xc, yc
        else:
            xlb, ylb = xc, yc
        if (xub - xlb) < xtol or (yub - ylb) < ftol:
            break
    return 0.5 * (xub + xlb)


def test_itp_sensitivity_to_last_bits(oracle):
    """The oracle's Inverse is the reference's ITP to the bit (an independent
    restatement of RootFinding.h over the oracle's own T gives identical
    roots), and that solver stops at an iterate that moves by up to
    xtol + ytol / slope when T changes in its last bits: with T scaled by
    1 +- 1e-15 a large share of the C1 roots (first component, xtol = ytol =
    1e-6) move by more than xtol.  Any other build of the reference (another
    compiler, FMA contraction, another summation order -- the GPU's among
    them) therefore agrees with it within the solver's tolerance, not within
    xtol."""
    O = oracle
    om = O.OracleTriangularMap(2, 2, 3, normalize=True, posfunc=O.POS_SOFTPLUS, abs_tol=1e-6, rel_tol=1e-6,
                               max_sub=30)
    coef = np.random.default_rng(0).normal(0.0, 0.1, om.num_coeffs)
    x = np.random.default_rng(1).standard_normal((2, 120))
    r = om.evaluate(coef, x)
    comp, c0 = om.comps[0], om.split(coef)[0]
    ref = comp.inverse(c0, x[:1], r[0], 1e-6, 1e-6)
    T = lambda v, s=1.0: float(comp.evaluate(c0, np.array([[v]]))[0]) * s
    moved, ratio = 0, 0.0
    for i in range(x.shape[1]):
        a = _itp_reference(T, r[0, i], x[0, i], 1e-6, 1e-6)
        assert a == ref[i]
        slope = float(comp.cont_derivative(c0, np.array([[a]]))[0])
        for s in (1.0 + 1e-15, 1.0 - 1e-15):
            b = _itp_reference(lambda v: T(v, s), r[0, i], x[0, i], 1e-6, 1e-6)
            moved += abs(a - b) > 1e-6
            ratio = max(ratio, abs(a - b) / (1e-6 + 1e-6 / slope))
    assert moved >= 0.1 * 2 * x.shape[1]
    assert ratio <= 1.0 + 1e-9
