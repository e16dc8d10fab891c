"""Implicit-function derivative of Inverse: the coefficient gradient of a
linear functional L = sum w * x of x = T^{-1}(x1, r), dL/dc = -lambda^T dT/dc
with (dT/dx)^T lambda = w, and the gradients with respect to r and x1.

The oracle's restatement is pinned against central finite differences of its
own Inverse (CPU), and the GPU path is checked against the oracle at the GPU's
solution (1e-10 relative, floored at 1e-3 of the largest entry for the sums
over points) and against central finite differences of the GPU Inverse."""
import numpy as np
import pytest

from test_gpu_parity import H, T, assert_parity, opts, oracle_tri

H_FD = 1e-6


def _problem(O, inp, out, order, n, seed, tol=1e-8, coef_sd=0.03):
    om = oracle_tri(O, inp, out, order, tol=tol)
    coef = np.random.default_rng(seed).normal(0.0, coef_sd, om.num_coeffs)
    rng = np.random.default_rng(seed + 1)
    x1 = rng.standard_normal((inp - out, n))
    r = rng.standard_normal((out, n))
    w = rng.standard_normal((out, n))
    return om, coef, x1, r, w


def test_oracle_inverse_grad_matches_finite_differences(oracle):
    """The restatement against central differences of the oracle's Inverse,
    for coefficients, targets (a shift of one output row) and the fixed inputs."""
    O = oracle
    om, coef, x1, r, w = _problem(O, 4, 2, 3, 40, 7, coef_sd=0.1)
    xtol = ytol = 1e-14
    # Targets outside the range of the map have no inverse (NaN, as in the
    # reference's bracket search); keep the points that have one.
    ok = ~np.isnan(om.inverse(coef, x1, r, xtol, ytol)).any(axis=0)
    assert ok.sum() >= 30
    x1, r, w = x1[:, ok], r[:, ok], w[:, ok]

    def L(c=coef, x1_=x1, r_=r):
        return float((w * om.inverse(c, x1_, r_, xtol, ytol)).sum())

    x = om.inverse(coef, x1, r, xtol, ytol)
    g, pg = O.inverse_coeff_grad(om, coef, np.vstack([x1, x]), w)
    scale = np.abs(g).max()
    for j in np.random.default_rng(3).choice(om.num_coeffs, 8, replace=False):
        e = np.zeros_like(coef)
        e[j] = H_FD
        fd = (L(c=coef + e) - L(c=coef - e)) / (2 * H_FD)
        assert abs(fd - g[j]) <= 1e-6 * scale, (j, fd, g[j])
    for k in range(2):
        e = np.zeros_like(r)
        e[k] = H_FD
        fd = (L(r_=r + e) - L(r_=r - e)) / (2 * H_FD)
        assert fd == pytest.approx(pg[2 + k].sum(), rel=1e-6, abs=1e-8)
    for k in range(2):
        e = np.zeros_like(x1)
        e[k] = H_FD
        fd = (L(x1_=x1 + e) - L(x1_=x1 - e)) / (2 * H_FD)
        assert fd == pytest.approx(pg[k].sum(), rel=1e-6, abs=1e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("inp,out,order,n", [(3, 3, 3, 2000), (4, 2, 3, 2000), (16, 16, 3, 300)])
def test_inverse_coeff_grad_matches_oracle(gpu, oracle, inp, out, order, n):
    M, O = gpu, oracle
    om, coef, x1, r, w = _problem(O, inp, out, order, n, 11)
    tm = M.CreateTriangular(inp, out, order, opts(M, tol=1e-8))
    tm.SetCoeffs(coef)
    x = tm.Inverse(T(x1), T(r), xtol=1e-10, ytol=1e-12)
    # Targets outside the range of the map have no inverse (NaN, the
    # reference's bracket-search result); compare at the others.
    ok = ~np.isnan(H(x)).any(axis=0)
    assert ok.sum() >= 0.8 * n
    x1, r, w, x = x1[:, ok], r[:, ok], w[:, ok], T(H(x)[:, ok])
    cg, gx1, gr = tm.InverseCoeffGrad(T(x1), x, T(w))
    g_ref, pg_ref = O.inverse_coeff_grad(om, coef, np.vstack([x1, H(x)]), w)
    assert_parity(H(cg), g_ref, floor=1e-3, what="dL/dc")
    assert_parity(H(gr), pg_ref[inp - out:], what="dL/dr")
    assert_parity(H(gx1), pg_ref[:inp - out], what="dL/dx1")


@pytest.mark.gpu
def test_inverse_coeff_grad_finite_differences(gpu):
    """Against central differences of the GPU Inverse (h = 1e-6) for a
    conditional map, at the C5 option set (ProbabilistHermite + SoftPlus,
    tol 1e-8, coefficients N(0, 0.03^2))."""
    import torch
    M = gpu
    inp, out, n = 5, 3, 4000
    rng = np.random.default_rng(21)
    tm = M.CreateTriangular(inp, out, 3, opts(M, tol=1e-8))
    coef = rng.normal(0.0, 0.03, tm.numCoeffs)
    x1, r, w = T(rng.standard_normal((inp - out, n))), T(rng.standard_normal((out, n))), T(rng.standard_normal((out, n)))

    def L(c):
        tm.SetCoeffs(c)
        return float((w * tm.Inverse(x1, r, xtol=1e-14, ytol=1e-14)).sum())

    tm.SetCoeffs(coef)
    x = tm.Inverse(x1, r, xtol=1e-14, ytol=1e-14)
    ok = ~torch.isnan(x).any(dim=0)
    assert int(ok.sum()) >= n - 10
    x1, r, w, x = x1[:, ok].contiguous(), r[:, ok].contiguous(), w[:, ok].contiguous(), x[:, ok].contiguous()
    cg = H(tm.InverseCoeffGrad(x1, x, w)[0])
    scale = np.abs(cg).max()
    for j in rng.choice(tm.numCoeffs, 10, replace=False):
        e = np.zeros_like(coef)
        e[j] = H_FD
        fd = (L(coef + e) - L(coef - e)) / (2 * H_FD)
        assert abs(fd - cg[j]) <= 1e-6 * scale, (j, fd, cg[j])
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_inverse_coeff_grad_host_buffers_and_no_input_grad(gpu):
    """Host (numpy) arguments are staged; the gradient alone (no pts_grad) is the same."""
    import torch
    M = gpu
    tm = M.CreateTriangular(3, 3, 3, opts(M, tol=1e-8))
    tm.SetCoeffs(np.random.default_rng(2).normal(0.0, 0.03, tm.numCoeffs))
    rng = np.random.default_rng(4)
    r, w = rng.standard_normal((3, 1000)), rng.standard_normal((3, 1000))
    x = tm.Inverse(T(np.zeros((0, 1000))), T(r), xtol=1e-10, ytol=1e-12)
    cg_dev, _, gr_dev = tm.InverseCoeffGrad(T(np.zeros((0, 1000))), x, T(w))
    cg_host = np.zeros(tm.numCoeffs)
    tm.InverseCoeffGradImpl(H(x), w, cg_host, None)
    np.testing.assert_array_equal(cg_host, H(cg_dev))
    gr_host = np.zeros((3, 1000))
    tm.InverseCoeffGradImpl(H(x), w, None, gr_host)
    np.testing.assert_array_equal(gr_host, H(gr_dev))
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_torch_inverse_backward(gpu):
    """TorchConditionalMapBase.inverse backpropagates through the implicit rule:
    the same gradients as InverseCoeffGrad, zero for the initial-guess columns."""
    import torch
    M = gpu
    tm = M.CreateTriangular(4, 2, 3, opts(M, tol=1e-8))
    rng = np.random.default_rng(8)
    tm.SetCoeffs(rng.normal(0.0, 0.03, tm.numCoeffs))
    mod = tm.torch(store_coeffs=True)
    x = T(rng.standard_normal((500, 4))).requires_grad_(True)
    r = T(rng.standard_normal((500, 2))).requires_grad_(True)
    out = mod.inverse(x, r)
    w = T(rng.standard_normal((500, 2)))
    (out * w).sum().backward()
    cg, gx1, gr = tm.InverseCoeffGrad(x.detach().T[:2].contiguous(), out.detach().T.contiguous(), w.T.contiguous())
    np.testing.assert_array_equal(H(mod.coeffs.grad), H(cg))
    np.testing.assert_array_equal(H(r.grad.T), H(gr))
    np.testing.assert_array_equal(H(x.grad.T[:2]), H(gx1))
    assert not H(x.grad[:, 2:]).any()
