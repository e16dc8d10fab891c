"""Parity of the sm_103a kernels (called through the C ABI) with the CPU
oracle on the same seeded inputs.

Tolerance: an entry passes when |gpu - oracle| <= 1e-10 * max(|oracle|,
1e-6 * max|oracle over the array|); the floor only matters for entries a
million times smaller than the array's largest.  Inverses (the reference's
ITP solver on both sides, or the Newton option) agree within the solver's own
tolerance, component by component (assert_inverse_parity)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def assert_parity(a, b, rtol=RTOL, floor=1e-6, what=""):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if b.size == 0:
        return
    scale = np.nanmax(np.abs(b)) if np.isfinite(b).any() else 1.0
    tol = rtol * np.maximum(np.abs(b), floor * scale)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    bad = ~same & ~(np.abs(a - b) <= tol)
    if bad.any():
        i = np.argmax(np.where(bad, np.abs(a - b) / np.maximum(tol, 1e-300), 0))
        raise AssertionError(f"{what}: {bad.sum()} of {b.size} entries outside tolerance; worst at {np.unravel_index(i, b.shape)}: "
                             f"gpu={a.flat[i]!r} oracle={b.flat[i]!r}")


def assert_inverse_parity(om, coef, x1, r, xi, xtol, ytol, method="Bracket", qtol=None):
    """Component by component: the oracle (the reference's FindBracket + ITP)
    solves component c from the GPU's own solution of the earlier coordinates,
    with NaN (no bracket) at the same points.

    method "Bracket" (ITP on the GPU too) and "Newton" (another iterate of the
    same bracket): the roots agree within the solver's tolerance,
    2 (xtol + ytol / dT_c/dx_c).  The ITP iterates are not compared to the
    bit: the GPU's T differs from the oracle's in the last bits (another
    summation order), and the reference's ITP stops at an iterate that moves
    by up to xtol + ytol / slope under such a change (the oracle's own roots
    do, tests/test_oracle_pins.py::test_itp_sensitivity_to_last_bits).  A
    last-bit change can also flip a borderline accept test of the adaptive
    quadrature and move T by up to the quadrature tolerance qtol: at most
    0.2 % of the points (and at least 2) may differ by up to
    2 (xtol + (ytol + qtol (1 + |r|)) / dT_c/dx_c)."""
    n = r.shape[1]
    if qtol is None:
        qtol = om.comps[0].abs_tol if hasattr(om.comps[0], "abs_tol") else 1e-6
    cs = om.split(coef)
    extra = om.input_dim - om.output_dim
    full = np.zeros((om.input_dim, n))
    full[:x1.shape[0]] = x1
    full[extra:] = xi
    for c, comp in enumerate(om.comps):
        guess = np.zeros((comp.input_dim, n))
        guess[:-1] = full[:comp.input_dim - 1]
        if x1.shape[0] >= comp.input_dim:
            guess[-1] = x1[comp.input_dim - 1]
        ref = comp.inverse(cs[c], guess, r[c], xtol, ytol)
        got = xi[c]
        assert np.array_equal(np.isnan(ref), np.isnan(got)), f"component {c}: NaN pattern differs"
        ok = ~np.isnan(ref)
        pt = guess.copy()
        pt[-1] = np.where(ok, ref, 0.0)
        slope = comp.cont_derivative(cs[c], pt)
        diff = np.abs(got - ref)
        bound = 2.0 * (xtol + ytol / np.maximum(slope, 1e-300))
        loose = 2.0 * (xtol + (ytol + qtol * (1.0 + np.abs(r[c]))) / np.maximum(slope, 1e-300))
        far = ok & (diff > bound)
        assert far.sum() <= max(2, int(0.002 * ok.sum())), \
            f"component {c} ({method}): {far.sum()} of {ok.sum()} roots outside 2 (xtol + ytol / slope) of the " \
            f"oracle's (max ratio {np.max(diff[ok] / bound[ok]):.3e})"
        assert np.all(diff[ok] <= loose[ok]), f"component {c} ({method}): max |dx| {diff[ok].max()}"


def T(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def H(t):
    return t.detach().cpu().numpy()


def opts(M, basis=0, pos=1, tol=1e-6, maxsub=30):
    return M.MapOptions(basisType=M.BasisTypes(basis), posFuncType=M.PosFuncTypes(pos),
                        quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=tol, quadRelTol=tol,
                        quadMaxSub=maxsub)


def oracle_tri(O, inp, out, order, basis=0, pos=1, tol=1e-6, maxsub=30):
    return O.OracleTriangularMap(inp, out, order, basis=basis, normalize=True, posfunc=pos, abs_tol=tol,
                                 rel_tol=tol, max_sub=maxsub)


# ----------------------------------------------------------------------------
# C1: 2 x 2 triangular map, total order 3, ProbabilistHermite + SoftPlus.
# ----------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c1(gpu, oracle):
    M, O = gpu, oracle
    rng0, rng1 = np.random.default_rng(0), np.random.default_rng(1)
    tm = M.CreateTriangular(2, 2, 3, opts(M))
    om = oracle_tri(O, 2, 2, 3)
    coef = rng0.normal(0.0, 0.1, tm.numCoeffs)
    x = rng1.standard_normal((2, 10000))
    tm.SetCoeffs(coef)
    return M, O, tm, om, coef, x


def test_c1_evaluate_logdet(c1):
    M, O, tm, om, coef, x = c1
    y = H(tm.Evaluate(T(x)))
    assert_parity(y, om.evaluate(coef, x), what="Evaluate")
    ld = H(tm.LogDeterminant(T(x)))
    assert_parity(ld, om.logdet(coef, x), what="LogDeterminant")


@pytest.mark.parametrize("method", ["Bracket", "Newton"])
def test_c1_inverse(c1, method):
    M, O, tm, om, coef, x = c1
    r = om.evaluate(coef, x)
    for x1 in (x, np.zeros((0, x.shape[1]))):
        xi = H(tm.Inverse(T(x1), T(r), method=method))
        assert_inverse_parity(om, coef, x1, r, xi, 1e-6, 1e-6, method=method)
        assert np.nanmax(np.abs(xi - x)) < 1e-4


def test_inverse_method_errors(c1):
    M, O, tm, om, coef, x = c1
    with pytest.raises(ValueError):
        tm.Inverse(T(x[:, :4]), T(x[:, :4]), method="Bisect")


def test_c1_coefficient_gradients(c1):
    M, O, tm, om, coef, x = c1
    xs = x[:, :2000]
    sens = np.random.default_rng(7).standard_normal((2, xs.shape[1]))
    g = H(tm.CoeffGrad(T(xs), T(sens)))
    assert_parity(g, om.coeff_grad(coef, xs, sens), what="CoeffGrad")
    lg = H(tm.LogDeterminantCoeffGrad(T(xs)))
    assert_parity(lg, om.logdet_coeff_grad(coef, xs), what="LogDeterminantCoeffGrad")


def test_c1_input_gradients(c1):
    M, O, tm, om, coef, x = c1
    xs = x[:, :2000]
    sens = np.random.default_rng(8).standard_normal((2, xs.shape[1]))
    g = H(tm.Gradient(T(xs), T(sens)))
    assert_parity(g, om.gradient(coef, xs, sens), what="Gradient")
    lg = H(tm.LogDeterminantInputGrad(T(xs)))
    assert_parity(lg, om.logdet_input_grad(coef, xs), what="LogDeterminantInputGrad")


def test_c1_fused_reduced_adjoint(c1):
    import torch
    M, O, tm, om, coef, x = c1
    sens = np.random.default_rng(9).standard_normal((2, x.shape[1]))
    lsens = np.random.default_rng(10).standard_normal(x.shape[1])
    out = torch.zeros(2, x.shape[1], dtype=torch.float64, device="cuda")
    ld = torch.zeros(x.shape[1], dtype=torch.float64, device="cuda")
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device="cuda")
    ig = torch.zeros(2, x.shape[1], dtype=torch.float64, device="cuda")
    tm.FusedForwardAdjointImpl(T(x), sens=T(sens), logdet_sens=T(lsens), out_eval=out, out_logdet=ld,
                               coeff_grad=cg, input_grad=ig)
    assert_parity(H(out), om.evaluate(coef, x), what="fused eval")
    assert_parity(H(ld), om.logdet(coef, x), what="fused logdet")
    ref_cg = om.coeff_grad(coef, x, sens).sum(axis=1) + (om.logdet_coeff_grad(coef, x) * lsens).sum(axis=1)
    assert_parity(H(cg), ref_cg, floor=1e-3, what="fused coefficient gradient")
    ref_ig = om.gradient(coef, x, sens) + om.logdet_input_grad(coef, x) * lsens
    assert_parity(H(ig), ref_ig, what="fused input gradient")


def test_c1_kl_objective(c1):
    M, O, tm, om, coef, x = c1
    loss, grad = tm.KLObjective(T(x))
    cs = om.split(coef)
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim])
        assert_parity(H(loss)[i:i + 1], [l], what=f"KL loss comp {i}")
        assert_parity(H(grad)[om.offsets[i]:om.offsets[i + 1]], g, floor=1e-3, what=f"KL grad comp {i}")


def test_c1_host_buffers_match_device(c1):
    M, O, tm, om, coef, x = c1
    xs = np.ascontiguousarray(x[:, :500])
    y_host = tm.Evaluate(xs)  # numpy in -> staged through the device
    y_dev = H(tm.Evaluate(T(xs)))
    np.testing.assert_array_equal(y_host, y_dev)
    # strided (transposed) host input
    xt = np.asfortranarray(xs)
    np.testing.assert_array_equal(tm.Evaluate(xt), y_dev)


# ----------------------------------------------------------------------------
# C2 (reduced size): one component, D = 8, total order 4 (495 terms).
# ----------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c2(gpu, oracle):
    M, O = gpu, oracle
    ms = M.FixedMultiIndexSet(8, 4)
    comp = M.CreateComponent(ms, opts(M))
    s, d, o = O.total_order(8, 4)
    oc = O.OracleComponent(8, s, d, o)
    coef = np.random.default_rng(0).normal(0.0, 0.05, comp.numCoeffs)
    x = np.random.default_rng(1).standard_normal((8, 3000))
    comp.SetCoeffs(coef)
    return M, O, comp, oc, coef, x


def test_c2_forward(c2):
    M, O, comp, oc, coef, x = c2
    assert comp.numCoeffs == 495
    assert_parity(H(comp.Evaluate(T(x)))[0], oc.evaluate(coef, x), what="C2 Evaluate")
    assert_parity(H(comp.LogDeterminant(T(x))), oc.logdet(coef, x), what="C2 LogDeterminant")


def test_c2_dense_and_reduced_adjoint(c2):
    import torch
    M, O, comp, oc, coef, x = c2
    xs = x[:, :600]
    sens = np.random.default_rng(5).standard_normal((1, xs.shape[1]))
    dense = H(comp.CoeffGrad(T(xs), T(sens)))
    ref = oc.coeff_grad(coef, xs, sens[0])
    assert_parity(dense, ref, what="C2 CoeffGrad dense")
    ldense = H(comp.LogDeterminantCoeffGrad(T(xs)))
    lref = oc.logdet_coeff_grad(coef, xs)
    assert_parity(ldense, lref, what="C2 LogDeterminantCoeffGrad dense")
    cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device="cuda")
    comp.FusedForwardAdjointImpl(T(xs), sens=T(sens), logdet_sens_scale=1.0, coeff_grad=cg)
    assert_parity(H(cg), ref.sum(axis=1) + lref.sum(axis=1), floor=1e-3, what="C2 fused reduced")


def test_c2_central_differences(c2):
    """Coefficient gradient of sum(sens*T) against central differences (h = 1e-6)."""
    import torch
    M, O, comp, oc, coef, x = c2
    xs = x[:, :400]
    sens = np.random.default_rng(6).standard_normal((1, xs.shape[1]))
    cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device="cuda")
    comp.FusedForwardAdjointImpl(T(xs), sens=T(sens), coeff_grad=cg)
    cg = H(cg)
    h = 1e-6
    for j in [0, 1, 7, 100, 250, 494]:
        cp, cm = coef.copy(), coef.copy()
        cp[j] += h
        cm[j] -= h
        comp.SetCoeffs(cp)
        fp = (H(comp.Evaluate(T(xs)))[0] * sens[0]).sum()
        comp.SetCoeffs(cm)
        fm = (H(comp.Evaluate(T(xs)))[0] * sens[0]).sum()
        assert cg[j] == pytest.approx((fp - fm) / (2 * h), rel=1e-5, abs=1e-6)
    comp.SetCoeffs(coef)


# ----------------------------------------------------------------------------
# C3 (reduced size): Hermite functions + Exp, tol 1e-7, banana samples.
# ----------------------------------------------------------------------------
def banana(n, seed):
    rng = np.random.default_rng(seed)
    x1 = rng.standard_normal(n)
    x2 = x1 ** 2 + 0.5 * rng.standard_normal(n)
    xs = [x1, x2]
    for _ in range(4):
        xs.append(0.8 * xs[-1] + 0.6 * rng.standard_normal(n))
    return np.stack(xs)


def test_c3_hermite_functions_exp(gpu, oracle):
    M, O = gpu, oracle
    tm = M.CreateTriangular(4, 4, 5, opts(M, basis=2, pos=0, tol=1e-7))
    om = oracle_tri(O, 4, 4, 5, basis=2, pos=0, tol=1e-7)
    coef = np.random.default_rng(3).normal(0.0, 0.02, tm.numCoeffs)
    tm.SetCoeffs(coef)
    x = banana(800, 11)[:4]
    assert_parity(H(tm.Evaluate(T(x))), om.evaluate(coef, x), what="HF Evaluate")
    assert_parity(H(tm.LogDeterminant(T(x))), om.logdet(coef, x), what="HF LogDeterminant")
    loss, grad = tm.KLObjective(T(x))
    cs = om.split(coef)
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim])
        assert_parity(H(loss)[i:i + 1], [l], what=f"HF KL loss {i}")
        assert_parity(H(grad)[om.offsets[i]:om.offsets[i + 1]], g, floor=1e-3, what=f"HF KL grad {i}")
    sens = np.random.default_rng(4).standard_normal((4, 300))
    assert_parity(H(tm.Gradient(T(x[:, :300]), T(sens))), om.gradient(coef, x[:, :300], sens), what="HF Gradient")


# ----------------------------------------------------------------------------
# C5 (reduced size): 16-D triangular map, total order 3, tol 1e-8, inverse to xtol 1e-10.
# ----------------------------------------------------------------------------
def test_c5_inverse_small(gpu, oracle):
    M, O = gpu, oracle
    tm = M.CreateTriangular(16, 16, 3, opts(M, tol=1e-8))
    om = oracle_tri(O, 16, 16, 3, tol=1e-8)
    coef = np.random.default_rng(0).normal(0.0, 0.03, tm.numCoeffs)
    tm.SetCoeffs(coef)
    r = np.random.default_rng(1).standard_normal((16, 150))
    x1 = np.zeros((0, 150))
    xi = H(tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-10))
    assert_inverse_parity(om, coef, x1, r, xi, 1e-10, 1e-10)
    ok = ~np.isnan(xi).any(axis=0)
    assert ok.sum() >= 140
    back = H(tm.Evaluate(T(np.ascontiguousarray(xi[:, ok]))))
    assert np.max(np.abs(back - r[:, ok])) < 1e-7


def test_c5_inverse_10k(gpu, oracle):
    """C5's map (16-D, total order 3, tol 1e-8, xtol 1e-10) on 10,000 random
    targets: the default ITP solve against the oracle's component by
    component, and the Newton solve within its own bound."""
    M, O = gpu, oracle
    tm = M.CreateTriangular(16, 16, 3, opts(M, tol=1e-8))
    om = oracle_tri(O, 16, 16, 3, tol=1e-8)
    coef = np.random.default_rng(0).normal(0.0, 0.03, tm.numCoeffs)
    tm.SetCoeffs(coef)
    n = 10000
    r = np.random.default_rng(1).standard_normal((16, n))
    x1 = np.zeros((0, n))
    xi = H(tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-10))
    assert_inverse_parity(om, coef, x1, r, xi, 1e-10, 1e-10)
    xn = H(tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-10, method="Newton"))
    assert np.array_equal(np.isnan(xn), np.isnan(xi))
    ok = ~np.isnan(xi).any(axis=0)
    assert ok.sum() >= 0.9 * n
    # Round trip: the solver stops with |T - r| < ytol or with a bracket
    # narrower than xtol, so |T(x) - r| <= ytol + slope * xtol.
    xo = np.ascontiguousarray(xi[:, ok])
    back = H(tm.Evaluate(T(xo)))
    cs = om.split(coef)
    for c, comp in enumerate(om.comps):
        slope = comp.cont_derivative(cs[c], xo[:c + 1])
        assert np.all(np.abs(back[c] - r[c, ok]) <= 2.0 * (1e-10 + slope * 1e-10) + 1e-12), f"component {c}"


@pytest.mark.parametrize("method", ["Bracket", "Newton"])
@pytest.mark.parametrize("basis,pos,scale,rscale", [(0, 1, 0.05, 3.0), (2, 0, 0.1, 2.0)])
def test_inverse_queue_far_and_missing_roots(gpu, oracle, basis, pos, scale, rscale, method):
    """More than 256 targets take the per-component queue solver (points in
    the order of a root estimate, expensive first, one integrand node per lane
    and step).  Wide targets give far roots and targets without a root (NaN,
    as in the reference); the results match the oracle component by
    component and do not depend on the processing order (point ordering off:
    bitwise-equal roots).  The scales keep the integrand finite at the far
    roots (with larger Hermite-function coefficients exp(df) overflows there,
    which the GPU reports as an IntegrandError)."""
    M, O = gpu, oracle
    tm = M.CreateTriangular(4, 4, 3, opts(M, basis=basis, pos=pos, tol=1e-8))
    om = oracle_tri(O, 4, 4, 3, basis=basis, pos=pos, tol=1e-8)
    coef = np.random.default_rng(11).normal(0.0, scale, tm.numCoeffs)
    tm.SetCoeffs(coef)
    n = 777
    r = rscale * np.random.default_rng(12).standard_normal((4, n))
    x1 = np.zeros((0, n))
    xi = H(tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-10, method=method))
    assert_inverse_parity(om, coef, x1, r, xi, 1e-10, 1e-10, method=method)
    # far roots: some lie beyond 7
    assert np.nanmax(np.abs(xi)) > 7.0
    tm.SetPointOrdering(False)
    xu = H(tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-10, method=method))
    tm.SetPointOrdering(True)
    np.testing.assert_array_equal(xu, xi)
    # The small-N path (one launch over all components, lockstep solver) gives
    # the same roots: the same quadratures and the same solver steps.
    xs = np.concatenate([H(tm.Inverse(T(x1[:, k:k + 200]), T(r[:, k:k + 200]), xtol=1e-10, ytol=1e-10,
                                      method=method)) for k in range(0, n, 200)], axis=1)
    np.testing.assert_array_equal(xs, xi)


# ----------------------------------------------------------------------------
# Edge cases and error behaviour.
# ----------------------------------------------------------------------------
def test_empty_and_shape_errors(c1):
    import torch
    M, O, tm, om, coef, x = c1
    e = torch.zeros(2, 0, dtype=torch.float64, device="cuda")
    tm.EvaluateImpl(e, torch.zeros(2, 0, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        tm.EvaluateImpl(T(x[:, :10]), torch.zeros(3, 10, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        tm.SetCoeffs(np.zeros(tm.numCoeffs + 1))


def test_nan_points_and_overflow(gpu, oracle):
    M, O = gpu, oracle
    tm = M.CreateTriangular(1, 1, 1, opts(M, pos=0))
    tm.SetCoeffs(np.array([0.0, 1.0]))
    om = oracle_tri(O, 1, 1, 1, pos=0)
    # A NaN target is not screened by the reference (only NaN inputs are,
    # MonotoneComponent.h:420-426): the solver returns a finite midpoint.
    r = np.array([[0.5, float("nan")]])
    xi = H(tm.Inverse(T(np.zeros((0, 2))), T(r)))
    ref = om.inverse(np.array([0.0, 1.0]), np.zeros((0, 2)), r)
    assert np.all(np.abs(xi - ref) <= 2e-6)
    # A NaN input gives NaN.
    xi = H(tm.Inverse(T(np.array([[float("nan"), 0.0]])), T(np.array([[0.5, 0.5]]))))
    assert math.isnan(xi[0, 0]) and math.isfinite(xi[0, 1])
    y = H(tm.Evaluate(T(np.array([[0.3, float("nan")]]))))
    assert math.isfinite(y[0, 0]) and math.isnan(y[0, 1])
    tm.SetCoeffs(np.array([0.0, 2000.0]))  # exp(2000 / (2 pi)^(1/4)) overflows
    with pytest.raises(M.IntegrandError):
        tm.Evaluate(T(np.array([[1.0]])))
    tm.SetCoeffs(np.array([0.0, 1.0]))
    tm.Evaluate(T(np.array([[1.0]])))  # status cleared, usable again


def test_component_reuse_and_wrap(gpu, oracle):
    import torch
    M, O = gpu, oracle
    c0 = M.CreateComponent(M.FixedMultiIndexSet(1, 2), opts(M))
    c1 = M.CreateComponent(M.FixedMultiIndexSet(2, 2), opts(M))
    c0.SetCoeffs(np.array([0.1, 0.2, 0.3]))
    c1.SetCoeffs(np.linspace(-0.2, 0.2, 6))
    tm = M.TriangularMap([c0, c1], moveCoeffs=True)
    assert tm.numCoeffs == 9
    np.testing.assert_allclose(tm.CoeffMap(), np.r_[[0.1, 0.2, 0.3], np.linspace(-0.2, 0.2, 6)])
    x = np.random.default_rng(2).standard_normal((2, 64))
    y = H(tm.Evaluate(T(x)))
    np.testing.assert_array_equal(y[0], H(c0.Evaluate(T(x[:1])))[0])
    np.testing.assert_array_equal(y[1], H(c1.Evaluate(T(x)))[0])
    w = torch.tensor(tm.CoeffMap() * 2.0, dtype=torch.float64, device="cuda")
    tm.WrapCoeffs(w)
    y2 = H(tm.Evaluate(T(x)))
    assert not np.allclose(y2, y)
    w.copy_(torch.tensor(tm.CoeffMap() / 2.0, device="cuda"))
    np.testing.assert_array_equal(H(tm.Evaluate(T(x))), y)


def test_torch_autograd(gpu, oracle):
    import torch
    M, O = gpu, oracle
    tm = M.CreateTriangular(2, 2, 3, opts(M))
    om = oracle_tri(O, 2, 2, 3)
    coef = np.random.default_rng(0).normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(coef)
    mod = tm.torch(store_coeffs=True, return_logdet=True)
    x = torch.tensor(np.random.default_rng(1).standard_normal((50, 2)), dtype=torch.float64, device="cuda",
                     requires_grad=True)
    y, ld = mod(x)
    loss = (y ** 2).sum() + ld.sum()
    loss.backward()
    xn = H(x).T
    yr = om.evaluate(coef, xn)
    sens = 2 * yr
    ref_c = om.coeff_grad(coef, xn, sens).sum(axis=1) + om.logdet_coeff_grad(coef, xn).sum(axis=1)
    assert_parity(H(mod.coeffs.grad), ref_c, floor=1e-3, what="autograd coeff grad")
    ref_x = om.gradient(coef, xn, sens) + om.logdet_input_grad(coef, xn)
    assert_parity(H(x.grad).T, ref_x, what="autograd input grad")


def test_torch_parameterized_function_base(gpu, oracle):
    """TorchParameterizedFunctionBase (bindings/python/package/torch.py): f(x)
    as a torch module; its coefficient and input gradients are the oracle's."""
    import torch
    M, O = gpu, oracle
    tm = M.CreateTriangular(2, 2, 3, opts(M))
    om = oracle_tri(O, 2, 2, 3)
    coef = np.random.default_rng(2).normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(coef)
    mod = M.TorchParameterizedFunctionBase(tm)
    x = torch.tensor(np.random.default_rng(3).standard_normal((40, 2)), dtype=torch.float64, device="cuda",
                     requires_grad=True)
    y = mod(x)
    (y ** 2).sum().backward()
    xn = H(x).T
    yr = om.evaluate(coef, xn)
    assert_parity(H(y).T, yr, what="TorchParameterizedFunctionBase forward")
    assert_parity(H(mod.coeffs.grad), om.coeff_grad(coef, xn, 2 * yr).sum(axis=1), floor=1e-3,
                  what="TorchParameterizedFunctionBase coeff grad")
    assert_parity(H(x.grad).T, om.gradient(coef, xn, 2 * yr), what="TorchParameterizedFunctionBase input grad")


def test_plain_path_matches_oracle(gpu, oracle):
    """The reference-structured comparator gives the same results."""
    import torch
    M, O = gpu, oracle
    p = M.PlainComponent(8, 4, opts(M))
    s, d, o = O.total_order(8, 4)
    oc = O.OracleComponent(8, s, d, o)
    coef = np.random.default_rng(0).normal(0.0, 0.05, p.numCoeffs)
    x = np.random.default_rng(1).standard_normal((8, 700))
    sens = np.random.default_rng(2).standard_normal(700)
    ev = torch.zeros(700, dtype=torch.float64, device="cuda")
    ld = torch.zeros(700, dtype=torch.float64, device="cuda")
    cg = torch.zeros(p.numCoeffs, dtype=torch.float64, device="cuda")
    p.FwdAdj(T(coef), T(x), T(sens), ev, ld, cg)
    torch.cuda.synchronize()
    assert_parity(H(ev), oc.evaluate(coef, x), what="plain evaluate")
    assert_parity(H(ld), oc.logdet(coef, x), what="plain logdet")
    ref = oc.coeff_grad(coef, x, sens).sum(axis=1) + oc.logdet_coeff_grad(coef, x).sum(axis=1)
    assert_parity(H(cg), ref, floor=1e-3, what="plain reduced adjoint")


# ----------------------------------------------------------------------------
# KL training (C3 layout, reduced size)
# ----------------------------------------------------------------------------
def test_kl_batched_equals_per_component(gpu):
    """The batched launch and one launch per component give identical values."""
    import torch
    M = gpu
    tm = M.CreateTriangular(6, 6, 5, opts(M, basis=2, pos=0, tol=1e-7))
    tm.SetCoeffs(np.random.default_rng(5).normal(0.0, 0.01, tm.numCoeffs))
    x = T(banana(5000, 12))
    # (the first call orders the samples by |x_D|, later ones by the interval
    # counts of the call before: compare calls at the same history)
    tm.KLObjective(x)
    lb, gb = tm.KLObjective(x)
    lb, gb = H(lb), H(gb)
    res = {m: M.KLStepTime(tm, x, mode=m, steps=3, return_values=True) for m in (0, 1, 2, 3)}
    for m in (0, 1, 2):
        assert res[m][0] > 0
        np.testing.assert_array_equal(res[m][1], lb)
        np.testing.assert_array_equal(res[m][2], gb)
    # the reference objective's call sequence (dense outputs): same values to rounding
    assert_parity(res[3][1], lb, what="KL loss, reference call sequence")
    assert_parity(res[3][2], gb, floor=1e-3, what="KL gradient, reference call sequence")
    # graph replays count their kernel nodes: the same launches as direct mode
    counts = []
    for mode in (0, 1):
        n0 = M.launch_count()
        M.KLStepTime(tm, x, mode=mode, steps=5)
        counts.append(M.launch_count() - n0)
    assert counts[0] == counts[1] > 0


def test_launch_count_of_fused_call(c2):
    """A fused call on one component launches the sort (3 kernels), the
    coefficient gather, the fused kernel, the log-det row sum and the
    fixed-order reduction of the partial rows."""
    import torch
    M, O, comp, oc, coef, x = c2
    xs = T(x)
    n = x.shape[1]
    ev = torch.zeros(1, n, dtype=torch.float64, device="cuda")
    ld = torch.zeros(n, dtype=torch.float64, device="cuda")
    cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device="cuda")
    n0 = M.launch_count()
    comp.FusedForwardAdjointImpl(xs, sens=T(np.ones((1, n))), logdet_sens_scale=1.0, out_eval=ev, out_logdet=ld,
                                 coeff_grad=cg)
    assert M.launch_count() - n0 == 7


def test_train_map_matches_oracle_objective(gpu, oracle):
    M, O = gpu, oracle
    x = banana(2000, 13)[:3]
    tm = M.CreateTriangular(3, 3, 3, opts(M, basis=2, pos=0, tol=1e-7))
    loss, res = M.TrainMap(tm, T(x), max_iters=15, mode=0)
    assert res["iterations"] >= 5
    coef = tm.CoeffMap()
    om = oracle_tri(O, 3, 3, 3, basis=2, pos=0, tol=1e-7)
    cs = om.split(coef)
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim])
        assert loss[i] == pytest.approx(l, rel=1e-10)
    # training reduces the objective below its value at zero coefficients
    l0 = [O.fast_gaussian_reverse_kl(c, np.zeros(c.num_coeffs), x[:c.input_dim])[0] for c in om.comps]
    assert np.all(loss < np.array(l0))
    # same trajectory with direct launches and with one launch set per component
    for mode in (1, 2):
        tm2 = M.CreateTriangular(3, 3, 3, opts(M, basis=2, pos=0, tol=1e-7))
        loss2, _ = M.TrainMap(tm2, T(x), max_iters=15, mode=mode)
        np.testing.assert_array_equal(loss2, loss)
        np.testing.assert_array_equal(tm2.CoeffMap(), coef)
    # the reference objective's call sequence (dense outputs, separate
    # reductions) sums in another order: the same objective to rounding
    tm3 = M.CreateTriangular(3, 3, 3, opts(M, basis=2, pos=0, tol=1e-7))
    loss3, _ = M.TrainMap(tm3, T(x), max_iters=15, mode=3)
    np.testing.assert_allclose(loss3, loss, rtol=1e-10)


def test_train_map_preconditioned_lbfgs(gpu, oracle):
    """L-BFGS with the diagonal preconditioner (inverse mean squared per-point
    gradients at the start) on a 3-D order-4 HermiteFunctions + Exp map: it
    goes further than plain L-BFGS in the same iterations, its objective at
    the trained coefficients is the oracle's, and with a gradient-norm
    tolerance it stops once the tolerance is met."""
    M, O = gpu, oracle
    x = banana(4000, 21)[:3]
    mk = lambda: M.CreateTriangular(3, 3, 4, opts(M, basis=2, pos=0, tol=1e-7))
    tp, tq = mk(), mk()
    lp, rp = M.TrainMap(tp, T(x), max_iters=40, max_evals=200, algorithm="LD_LBFGS", precondition=True)
    lq, rq = M.TrainMap(tq, T(x), max_iters=40, max_evals=200, algorithm="LD_LBFGS")
    assert rp["total_loss"] < rq["total_loss"]
    om = oracle_tri(O, 3, 3, 4, basis=2, pos=0, tol=1e-7)
    cs = om.split(tp.CoeffMap())
    for i, c in enumerate(om.comps):
        assert lp[i] == pytest.approx(O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim])[0], rel=1e-10)
    tg = mk()
    _, rg = M.TrainMap(tg, T(x), max_iters=2000, max_evals=6000, gtol=0.05, algorithm="LD_LBFGS",
                       precondition=True)
    # (the tolerance holds per component; the reported norm is over all three)
    assert rg["grad_norm"] <= 0.05 * np.sqrt(3) and rg["iterations"] < 2000


def test_point_ordering_invariance_and_determinism(c2):
    """Grouping points by |x_D| changes only the summation order; repeated
    calls are bitwise identical."""
    import torch
    M, O, comp, oc, coef, x = c2
    xs = T(x)
    sens = T(np.random.default_rng(3).standard_normal((1, x.shape[1])))

    def run():
        ev = torch.zeros(1, x.shape[1], dtype=torch.float64, device="cuda")
        cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device="cuda")
        comp.FusedForwardAdjointImpl(xs, sens=sens, logdet_sens_scale=1.0, out_eval=ev, coeff_grad=cg)
        return H(ev), H(cg)

    e1, g1 = run()
    e2, g2 = run()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(g1, g2)
    comp.SetPointOrdering(False)
    e3, g3 = run()
    comp.SetPointOrdering(True)
    np.testing.assert_array_equal(e1, e3)  # per-point values do not depend on the order
    assert_parity(g3, g1, floor=1e-3, what="ordered vs unordered reduction")


# ----------------------------------------------------------------------------
# The other quadrature rules of MapOptions::quadType: AdaptiveSimpson (the
# reference's default) and the fixed ClenshawCurtis rule.
# ----------------------------------------------------------------------------
@pytest.mark.parametrize("quad,pts", [(1, 5), (0, 5), (0, 9)])
def test_quadrature_kinds_match_oracle(gpu, oracle, quad, pts):
    import torch
    M, O = gpu, oracle
    opt = M.MapOptions(quadType=M.QuadTypes(quad), quadPts=pts, quadAbsTol=1e-7, quadRelTol=1e-7)
    tm = M.CreateTriangular(4, 3, 3, opt)
    om = O.OracleTriangularMap(4, 3, 3, abs_tol=1e-7, rel_tol=1e-7, quad_pts=pts, quad_type=quad)
    rng = np.random.default_rng(40 + quad + pts)
    coef = rng.normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(coef)
    x = rng.standard_normal((4, 1500))
    sens = rng.standard_normal((3, 1500))
    xs = T(x)
    assert_parity(H(tm.Evaluate(xs)), om.evaluate(coef, x), what="Evaluate")
    assert_parity(H(tm.LogDeterminant(xs)), om.logdet(coef, x), what="LogDeterminant")
    assert_parity(H(tm.CoeffGrad(xs, T(sens))), om.coeff_grad(coef, x, sens), what="CoeffGrad")
    assert_parity(H(tm.Gradient(xs, T(sens))), om.gradient(coef, x, sens), what="Gradient")
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device="cuda")
    tm.FusedForwardAdjointImpl(xs, sens=T(sens), logdet_sens_scale=1.0, coeff_grad=cg)
    ref = om.coeff_grad(coef, x, sens).sum(axis=1) + om.logdet_coeff_grad(coef, x).sum(axis=1)
    assert_parity(H(cg), ref, floor=1e-3, what="fused adjoint")
    loss, grad = tm.KLObjective(xs)
    l_ref, g_ref = [], []
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, om.split(coef)[i], x[:c.input_dim])
        l_ref.append(l)
        g_ref.append(g)
    assert_parity(H(loss), np.array(l_ref), what="KL loss")
    assert_parity(H(grad), np.concatenate(g_ref), floor=1e-3, what="KL gradient")
    r = om.evaluate(coef, x)
    xi = H(tm.Inverse(T(x[:1]), T(r), xtol=1e-10, ytol=1e-10))
    assert_inverse_parity(om, coef, x[:1], r, xi, 1e-10, 1e-10)


# ----------------------------------------------------------------------------
# contDeriv = false: log-determinants of the quadrature approximation
# (DiscreteDerivative / DiscreteMixedJacobian).
# ----------------------------------------------------------------------------
@pytest.mark.parametrize("basis,pos,quad", [(0, 1, 2), (2, 0, 2), (0, 1, 1)])
def test_discrete_derivative_matches_oracle(gpu, oracle, basis, pos, quad):
    import torch
    M, O = gpu, oracle
    opt = M.MapOptions(basisType=M.BasisTypes(basis), posFuncType=M.PosFuncTypes(pos), quadType=M.QuadTypes(quad),
                       quadAbsTol=1e-7, quadRelTol=1e-7, contDeriv=False)
    tm = M.CreateTriangular(3, 3, 3, opt)
    om = O.OracleTriangularMap(3, 3, 3, basis=basis, posfunc=pos, abs_tol=1e-7, rel_tol=1e-7, quad_type=quad,
                               cont_deriv=False)
    rng = np.random.default_rng(50 + basis + pos + quad)
    coef = rng.normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(coef)
    x = rng.standard_normal((3, 1200))
    sens = rng.standard_normal((3, 1200))
    xs = T(x)
    assert_parity(H(tm.LogDeterminant(xs)), om.logdet(coef, x), what="discrete LogDeterminant")
    assert_parity(H(tm.LogDeterminantCoeffGrad(xs)), om.logdet_coeff_grad(coef, x),
                  what="discrete LogDeterminantCoeffGrad")
    assert_parity(H(tm.Evaluate(xs)), om.evaluate(coef, x), what="Evaluate")
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device="cuda")
    ld = torch.zeros(1200, dtype=torch.float64, device="cuda")
    tm.FusedForwardAdjointImpl(xs, sens=T(sens), logdet_sens_scale=1.0, out_logdet=ld, coeff_grad=cg)
    ref = om.coeff_grad(coef, x, sens).sum(axis=1) + om.logdet_coeff_grad(coef, x).sum(axis=1)
    assert_parity(H(cg), ref, floor=1e-3, what="discrete fused adjoint")
    assert_parity(H(ld), om.logdet(coef, x), what="discrete fused log-det")
    loss, grad = tm.KLObjective(xs)
    cs = om.split(coef)
    refs = [O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim]) for i, c in enumerate(om.comps)]
    assert_parity(H(loss), np.array([r[0] for r in refs]), what="discrete KL loss")
    assert_parity(H(grad), np.concatenate([r[1] for r in refs]), floor=1e-3, what="discrete KL gradient")
    # as in the reference (MonotoneComponent.h:216-222)
    with pytest.raises(ValueError, match="Discrete derivative"):
        tm.LogDeterminantInputGrad(xs)


def test_nugget_semantics_match_reference(gpu, oracle):
    """With a nonzero nugget the reference's Evaluate integrates g(df) alone
    (EvaluateImpl calls EvaluateSingle without it, MonotoneComponent.h:290)
    while CoeffGrad, Gradient and Inverse integrate g(df) + nugget (:434,
    :721, :794); the fused call, the KL objective and the batch give each
    output the meaning of its reference call (tests/test_reference_pins.py
    pins the oracle to the reference on this)."""
    import torch
    M, O = gpu, oracle
    o = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, nugget=0.3)
    tm = M.CreateTriangular(2, 2, 3, o)
    om = O.OracleTriangularMap(2, 2, 3, nugget=0.3)
    coef = np.random.default_rng(0).normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(coef)
    x = np.random.default_rng(1).standard_normal((2, 3000))
    sens = np.random.default_rng(2).standard_normal((2, 3000))
    assert_parity(H(tm.Evaluate(T(x))), om.evaluate(coef, x), what="Evaluate")
    assert_parity(H(tm.LogDeterminant(T(x))), om.logdet(coef, x), what="LogDeterminant")
    assert_parity(H(tm.CoeffGrad(T(x), T(sens))), om.coeff_grad(coef, x, sens), what="CoeffGrad")
    assert_parity(H(tm.Gradient(T(x), T(sens))), om.gradient(coef, x, sens), what="Gradient")
    r = om.evaluate(coef, x)
    xi = H(tm.Inverse(T(np.zeros((0, 3000))), T(r), xtol=1e-10, ytol=1e-10))
    assert_inverse_parity(om, coef, np.zeros((0, 3000)), r, xi, 1e-10, 1e-10)
    assert np.abs(xi - x).max() > 1e-3  # the inverse solves T + nugget x = r
    # fused call: values as Evaluate, gradient as CoeffGrad + LogDeterminantCoeffGrad
    ev = torch.zeros(2, 3000, dtype=torch.float64, device="cuda")
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device="cuda")
    tm.FusedForwardAdjointImpl(T(x), sens=T(sens), logdet_sens_scale=1.0, out_eval=ev, coeff_grad=cg)
    assert_parity(H(ev), om.evaluate(coef, x), what="fused values")
    ref_cg = om.coeff_grad(coef, x, sens).sum(axis=1) + om.logdet_coeff_grad(coef, x).sum(axis=1)
    assert_parity(H(cg), ref_cg, floor=1e-3, what="fused coefficient gradient")
    # KL objective (FastGaussianReverseKL per component)
    loss, grad = tm.KLObjective(T(x))
    cs = om.split(coef)
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, cs[i], np.ascontiguousarray(x[:c.input_dim]))
        assert_parity(H(loss)[i:i + 1], [l], what=f"KL loss {i}")
        assert_parity(H(grad)[om.offsets[i]:om.offsets[i + 1]], g, floor=1e-3, what=f"KL grad {i}")
