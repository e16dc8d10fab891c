"""GPU parity at the benchmark workloads' own shapes (the oracle on the same
seeded inputs, through the C ABI):

* the KL training map -- 6-D TriangularMap, total order 5 (923 coefficients),
  HermiteFunctions + Exp, tol 1e-7 -- on 50,000 banana samples at fixed
  coefficients: every component's FastGaussianReverseKLObjective value and
  gradient, and the KLObjective through PullbackDensity (value with
  (M/2) log 2 pi, coefficient gradient, TrainError / TestError);
* all 64 maps of the batched-maps workload (dims 2-16, total orders 2-6, up
  to 15,504 terms in a component), each on a sample of its points, through
  one batch call.

The full-size inverse workload's map is checked in test_gpu_parity.py
(test_c5_inverse_10k) and the fused forward + adjoint at 1,000,000 points by
the benchmark itself (its `parity_full` block).  Tolerance as in
test_gpu_parity.py: 1e-10 relative, floored at 1e-6 of the largest entry
(1e-3 for sums over points)."""
import math

import numpy as np
import pytest

from test_gpu_parity import H, T, assert_parity, opts, oracle_tri

pytestmark = pytest.mark.gpu


def banana(n, seed=11, dim=6):
    """x1 ~ N(0,1), x2 = x1^2 + 0.5 N(0,1), x_k = 0.8 x_{k-1} + 0.6 N(0,1)."""
    rng = np.random.default_rng(seed)
    x1 = rng.standard_normal(n)
    xs = [x1, x1 ** 2 + 0.5 * rng.standard_normal(n)]
    while len(xs) < dim:
        xs.append(0.8 * xs[-1] + 0.6 * rng.standard_normal(n))
    return np.stack(xs)


@pytest.fixture(scope="module")
def kl_map(gpu, oracle):
    M, O = gpu, oracle
    tm = M.CreateTriangular(6, 6, 5, opts(M, basis=2, pos=0, tol=1e-7))
    om = oracle_tri(O, 6, 6, 5, basis=2, pos=0, tol=1e-7)
    assert tm.numCoeffs == 923
    # fixed coefficients away from the KL optimum (so that the gradient sums
    # do not cancel): the linear diagonal term x_k of every component
    # (multi-index (0, ..., 0, 1), term 1 of the total-order set) at 1, and
    # N(0, 0.01^2) on the terms whose leading factors have total degree <= 2
    # with at most one phi_1 = x factor.  Products of several unbounded
    # phi_1 factors with random coefficients overflow exp(df) on banana
    # samples, so those terms stay 0.
    coef = np.random.default_rng(3).normal(0.0, 0.01, tm.numCoeffs)
    for k, off in enumerate(om.offsets[:-1]):
        ms = M.FixedMultiIndexSet(k + 1, 5)
        for t in range(ms.Size()):
            m = ms.IndexToMulti(t)
            if sum(1 for v in m[:-1] if v == 1) >= 2 or sum(m[:-1]) > 2:
                coef[off + t] = 0.0
        coef[off + 1] = 1.0
    tm.SetCoeffs(coef)
    return M, O, tm, om, coef


def test_kl_map_per_component_objectives(kl_map):
    M, O, tm, om, coef = kl_map
    x = banana(50_000)
    loss, grad = tm.KLObjective(T(x))
    cs = om.split(coef)
    for i, c in enumerate(om.comps):
        l, g = O.fast_gaussian_reverse_kl(c, cs[i], np.ascontiguousarray(x[:c.input_dim]))
        assert math.isfinite(l)
        assert_parity(H(loss)[i:i + 1], [l], what=f"KL loss {i}")
        assert_parity(H(grad)[om.offsets[i]:om.offsets[i + 1]], g, floor=1e-3, what=f"KL grad {i}")


def test_kl_objective_pullback_density(kl_map):
    """KLObjective::ObjectivePlusCoeffGradImpl with the identity-covariance
    GaussianSamplerDensity through PullbackDensity (src/MapObjective.cpp:54-91,
    src/Distributions/PullbackDensity.cpp:13-37,
    src/Distributions/GaussianSamplerDensity.cpp:21-88)."""
    M, O, tm, om, coef = kl_map
    train, test = banana(50_000, seed=11), banana(20_000, seed=12)
    obj = M.CreateGaussianKLObjective(train, test)
    ref_train, ref_grad = O.kl_objective(om, coef, train)
    ref_test, _ = O.kl_objective(om, coef, test)
    assert_parity([obj.TrainError(tm)], [ref_train], what="KLObjective train value")
    assert_parity([obj.TestError(tm)], [ref_test], what="KLObjective test value")
    assert_parity(H(obj.TrainCoeffGrad(tm)), ref_grad, floor=1e-3, what="KLObjective gradient")
    # the value includes the (M/2) log 2 pi of the Gaussian density
    per_comp = H(tm.KLObjective(T(train))[0]).sum()
    assert obj.TrainError(tm) - per_comp == pytest.approx(3.0 * math.log(2.0 * math.pi), rel=1e-12)


def batch_specs(n_maps=64, seed=17):
    """The batched-maps workload's maps: dims uniform in 2..16, total orders
    uniform in 2..6 (point counts log-uniform in [1e3, 2e5])."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(2, 17, n_maps)
    orders = rng.integers(2, 7, n_maps)
    npts = np.exp(rng.uniform(np.log(1e3), np.log(2e5), n_maps)).astype(int)
    return list(zip(dims.tolist(), orders.tolist(), npts.tolist()))


def test_batch_workload_all_maps_match_oracle(gpu, oracle):
    M, O = gpu, oracle
    rng = np.random.default_rng(18)
    specs = batch_specs()
    maps, pts, sens, coefs = [], [], [], []
    sample = 48
    for d, o, n in specs:
        tm = M.CreateTriangular(d, d, o, opts(M))
        c = rng.normal(0.0, 0.05, tm.numCoeffs)
        tm.SetCoeffs(c)
        maps.append(tm)
        coefs.append(c)
        pts.append(rng.standard_normal((d, n))[:, :sample].copy())
        sens.append(rng.standard_normal((d, n))[:, :sample].copy())
    assert max(m.numCoeffs for m in maps) > 70_000  # a 16-D order-5 map is among them
    B = M.MapBatch(maps)
    import torch
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device="cuda")
    ev = [z(m.outputDim, sample) for m in maps]
    ld = [z(sample) for _ in maps]
    cg = [z(m.numCoeffs) for m in maps]
    B.FusedForwardAdjoint([T(p) for p in pts], [T(s) for s in sens], 1.0, ev, ld, cg)
    for k, ((d, o, n), tm) in enumerate(zip(specs, maps)):
        om = oracle_tri(O, d, d, o)
        x, s, c = pts[k], sens[k], coefs[k]
        assert_parity(H(ev[k]), om.evaluate(c, x), what=f"map {k} ({d}-D, order {o}) Evaluate")
        assert_parity(H(ld[k]), om.logdet(c, x), what=f"map {k} LogDeterminant")
        ref = om.coeff_grad(c, x, s).sum(axis=1) + om.logdet_coeff_grad(c, x).sum(axis=1)
        assert_parity(H(cg[k]), ref, floor=1e-3, what=f"map {k} coefficient adjoint")
