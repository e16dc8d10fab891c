"""Sigmoid expansions on the GPU (RectifiedMultivariateExpansion and
UnivariateExpansion<Sigmoid1d>, built by CreateSigmoidComponent /
CreateSigmoidTriangular) against the oracle on the same seeded inputs,
through the C ABI.  Tolerance as in test_gpu_parity: 1e-10 relative with a
floor at 1e-6 of the array's largest entry (1e-3 for gradients summed over
points, whose partial sums follow the tiles); inverses within the solver's
tolerance."""
import math
import pickle

import numpy as np
import pytest

from test_gpu_parity import H, T, assert_parity

pytestmark = pytest.mark.gpu


def _centers(rng, num_sig, sum_type, bound=3.0):
    if sum_type == 0:
        n = 2 + num_sig * (num_sig + 1) // 2
        c = [-bound, bound]
        for k in range(1, num_sig + 1):
            c += [1.9 * bound * (j - (k - 1) / 2) / max(k - 1, 1) for j in range(k)]
        return np.array(c[:n])
    return np.concatenate([[-bound, bound], np.sort(rng.uniform(-bound, bound, num_sig))])


def _opts(M, pos, sum_type, edge=1.5):
    return M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes(pos),
                        sigmoidBasisSumType=M.SigmoidSumSizeType(sum_type), edgeShape=edge)


def _oracle_comp(O, comp, pos):
    """The oracle twin of a GPU sigmoid component (same set, same parameters)."""
    s, d, o = _mset(comp)
    return O.OracleSigmoidComponent(comp.inputDim, s, d, o, comp.GetSigmoid(), pos)


def _mset(comp):
    import ctypes as C
    from mpart_gb300 import _capi
    L = _capi.load()
    dim, nt, nnz = C.c_uint(), C.c_uint(), C.c_uint()
    _capi.check(L.mpgb_component_multi_index(comp._h, C.byref(dim), C.byref(nt), C.byref(nnz), None, None, None))
    s = np.zeros(nt.value + 1, np.uint32)
    d = np.zeros(max(1, nnz.value), np.uint32)
    o = np.zeros(max(1, nnz.value), np.uint32)
    U = C.POINTER(C.c_uint)
    _capi.check(L.mpgb_component_multi_index(comp._h, None, None, None, s.ctypes.data_as(U), d.ctypes.data_as(U),
                                             o.ctypes.data_as(U)))
    return s, d[:nnz.value], o[:nnz.value]


def _coeffs(rng, comp):
    """Random coefficients, non-negative on the terms with a last-input factor
    (the CoeffBounds lower bounds), so that the expansion is increasing."""
    lb, _ = comp.CoeffBounds()
    c = rng.normal(0.0, 0.3, comp.numCoeffs)
    c[lb == 0.0] = np.abs(c[lb == 0.0]) + 0.05
    return c


CASES = [  # (input dim, total order, cross order, sigmoids, sum type, rectifier)
    (3, 2, 2, 3, 0, 1), (4, 3, 2, 4, 1, 0), (2, 4, 3, 5, 0, 0), (1, 0, 0, 4, 0, 1), (5, 2, 1, 2, 1, 1),
]


@pytest.mark.parametrize("case", CASES, ids=[f"d{c[0]}o{c[1]}x{c[2]}s{c[3]}{'LC'[c[4]]}{'ES'[c[5]]}" for c in CASES])
def test_sigmoid_component_matches_oracle(gpu, oracle, case):
    M, O = gpu, oracle
    dim, order, cross, ns, st, pos = case
    rng = np.random.default_rng(17 + dim)
    comp = M.CreateSigmoidComponent(dim, order, cross, _centers(rng, ns, st), _opts(M, pos, st))
    om = _oracle_comp(O, comp, pos)
    c = _coeffs(rng, comp)
    comp.SetCoeffs(c)
    N = 2000
    x = rng.normal(0.0, 1.5, (dim, N))
    # far tails and the origin (with the Exp rectifier, leading products of
    # order 3 at 40 overflow, where the two sides differ only in inf vs NaN)
    far = 40.0 if pos == 1 else 8.0
    x[:, 0], x[:, 1], x[:, 2] = -far, 0.0, 0.9 * far
    s = rng.normal(size=N)
    xt = T(x)
    assert_parity(H(comp.Evaluate(xt))[0], om.evaluate(c, x), what="Evaluate")
    assert_parity(H(comp.LogDeterminant(xt)), om.logdet(c, x), what="LogDeterminant")
    assert_parity(H(comp.CoeffGrad(xt, T(s[None, :]))), om.coeff_grad(c, x, s), what="CoeffGrad")
    assert_parity(H(comp.LogDeterminantCoeffGrad(xt)), om.logdet_coeff_grad(c, x), what="LogDeterminantCoeffGrad")
    assert_parity(H(comp.Gradient(xt, T(s[None, :]))), om.gradient(c, x, s), what="Gradient")
    assert_parity(H(comp.LogDeterminantInputGrad(xt)), om.logdet_input_grad(c, x), what="LogDeterminantInputGrad")
    # fused forward + reduced adjoint (one pass) equals the sums of the oracle's dense outputs
    import torch
    ev = torch.zeros((1, N), dtype=torch.float64, device="cuda")
    ld = torch.zeros(N, dtype=torch.float64, device="cuda")
    cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device="cuda")
    comp.FusedForwardAdjointImpl(xt, sens=T(s[None, :]), logdet_sens_scale=0.7, out_eval=ev, out_logdet=ld,
                                 coeff_grad=cg)
    ref = om.coeff_grad(c, x, s).sum(axis=1) + 0.7 * om.logdet_coeff_grad(c, x).sum(axis=1)
    assert_parity(H(cg), ref, floor=1e-3, what="fused coefficient adjoint")
    assert_parity(H(ev)[0], om.evaluate(c, x), what="fused Evaluate")
    # inverse: the oracle's ITP root and the GPU's bracketed Newton root within xtol
    r = om.evaluate(c, x)[None, :]
    x1 = x[:dim - 1]
    xi = H(comp.Inverse(T(x1), T(r)))[0]
    guess = np.vstack([x1, np.zeros((1, N))])
    ref = om.inverse(c, guess, r[0])
    assert np.array_equal(np.isnan(ref), np.isnan(xi))
    ok = ~np.isnan(ref)
    # both solvers stop at |dx| < xtol or |dT| < ytol: 2 (xtol + ytol / d_D T)
    pt = np.vstack([x1, np.where(ok, ref, 0.0)])
    bound = 2.0 * (1e-6 + 1e-6 / np.exp(om.logdet(c, pt)))
    assert np.all(np.abs(xi - ref)[ok] <= bound[ok])
    assert np.all(np.abs(xi - x[dim - 1])[ok] <= bound[ok])


def test_sigmoid1d_device_matches_oracle(gpu, oracle):
    M, O = gpu, oracle
    for centers, edge, st in ((np.array([-3.0, 3.0, 0.0, -1.0, 1.0, -2.0, 0.0, 2.0]), 1.5, 0),
                              (np.array([-2.0, 2.5, 1.0, -1.5, 0.3, 0.9]), 0.7, 1)):
        S = M.Sigmoid1d.FromCenters(centers, edge, M.SigmoidSumSizeType(st))
        prm = O.sigmoid_from_centers(centers, edge, st)
        for a, b in zip((S.centers, S.widths, S.weights, S.startInds), prm):
            np.testing.assert_array_equal(a, b)
        xs = np.concatenate([np.linspace(-6, 6, 201), [-100.0, 100.0, 0.0]])
        v, d1, d2 = (H(t) for t in S.Evaluate(xs, S.GetOrder(), 2))
        for j, x in enumerate(xs):
            rv, r1, r2 = O.sigmoid_eval(prm, x, S.GetOrder(), 2)
            assert_parity(v[:, j], rv, floor=1e-12, what=f"values at {x}")
            assert_parity(d1[:, j], r1, floor=1e-12, what=f"first derivatives at {x}")
            assert_parity(d2[:, j], r2, floor=1e-12, what=f"second derivatives at {x}")
        out = np.zeros(S.GetOrder() + 1)
        S.EvaluateAll(out, 0.25)
        np.testing.assert_array_equal(out, H(S.Evaluate([0.25])[0])[:, 0])
    with pytest.raises(ValueError):
        M.Sigmoid1d(np.zeros(3), np.ones(3), np.ones(3)).Evaluate([0.0], 5)


# bindings/python/tests/test_MapFactory.py:104-137
def test_create_sigmoid_maps(gpu):
    M = gpu
    input_dim, num_sigmoid, max_degree = 6, 5, 3
    centers_len = 2 + num_sigmoid * (num_sigmoid + 1) // 2
    centers = np.zeros(centers_len)
    bound = 3.0
    centers[0], centers[1], centers[2] = -bound, bound, 0.0
    idx = 0
    for order in range(2, num_sigmoid + 1):
        for j in range(order):
            centers[idx] = 1.9 * bound * (j - (order - 1) / 2) / (order - 1)
            idx += 1
    opts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions)
    sig = M.CreateSigmoidComponent(input_dim, max_degree, centers, opts)
    lb, ub = sig.CoeffBounds()
    assert np.max(lb) == 0
    assert sig.numCoeffs == (num_sigmoid + 4) * math.comb(input_dim - 1 + max_degree, input_dim - 1)
    mset = M.FixedMultiIndexSet(input_dim, max_degree)
    sig_mset = M.CreateSigmoidComponent(mset, centers, opts)
    assert sig_mset.numCoeffs == mset.Size()
    centers_total = np.column_stack([centers for _ in range(input_dim)])
    tri = M.CreateSigmoidTriangular(input_dim, input_dim, max_degree, centers_total, opts)
    assert tri.numCoeffs == sum((num_sigmoid + 4) * math.comb(d - 1 + max_degree, d - 1)
                                for d in range(1, input_dim + 1))
    lb, ub = tri.CoeffBounds()
    assert np.max(lb) == 0 and np.isinf(ub).all()
    # HandleSigmoidComponentErrors (src/MapFactory.cpp:320-348)
    with pytest.raises(ValueError, match="basis type"):
        M.CreateSigmoidComponent(input_dim, max_degree, centers, M.MapOptions())
    with pytest.raises(ValueError):
        M.CreateSigmoidComponent(2, 2, np.zeros(4), opts)  # 2 + 2 centers do not form a Linear sum


def test_sigmoid_triangular_kl_and_training(gpu, oracle):
    M, O = gpu, oracle
    import torch
    rng = np.random.default_rng(3)
    dim, order, ns = 3, 2, 3
    cen = np.column_stack([_centers(rng, ns, 0) for _ in range(dim)])
    tri = M.CreateSigmoidTriangular(dim, dim, order, cen, _opts(M, 1, 0))
    otri = O.sigmoid_triangular(dim, dim, order, cen, 1.5, 0, O.POS_SOFTPLUS)
    assert tri.numCoeffs == otri.num_coeffs
    lb, _ = tri.CoeffBounds()
    c = rng.normal(0.0, 0.2, tri.numCoeffs)
    c[lb == 0.0] = np.abs(c[lb == 0.0]) + 0.05
    tri.SetCoeffs(c)
    x = rng.normal(size=(dim, 3000))
    xt = T(x)
    assert_parity(H(tri.Evaluate(xt)), otri.evaluate(c, x), what="triangular Evaluate")
    assert_parity(H(tri.LogDeterminant(xt)), otri.logdet(c, x), what="triangular LogDeterminant")
    assert_parity(H(tri.LogDeterminantInputGrad(xt)), otri.logdet_input_grad(c, x), what="LogDeterminantInputGrad")
    # per-component standard-normal reverse KL (FastGaussianReverseKLObjective)
    loss, grad = tri.KLObjective(xt)
    cs = otri.split(c)
    for k, comp in enumerate(otri.comps):
        l_ref, g_ref = O.fast_gaussian_reverse_kl(comp, cs[k], x[:comp.input_dim])
        assert abs(H(loss)[k] - l_ref) <= 1e-10 * abs(l_ref) + 1e-14
        assert_parity(H(grad)[otri.offsets[k]:otri.offsets[k + 1]], g_ref, floor=1e-3, what=f"KL gradient {k}")
    # inverse of the whole map
    r = otri.evaluate(c, x)
    xi = H(tri.Inverse(T(np.zeros((0, x.shape[1]))), T(r)))
    assert np.nanmax(np.abs(xi - x)) <= 1e-5
    # training on banana samples lowers the objective
    np.random.seed(43)
    s = np.random.randn(2, 4000)
    samples = np.vstack([s[0], s[1] + s[0] ** 2])
    tri2 = M.CreateSigmoidTriangular(2, 2, 2, np.column_stack([_centers(rng, 3, 0)] * 2), _opts(M, 1, 0))
    lb2, _ = tri2.CoeffBounds()
    tri2.SetCoeffs(np.where(lb2 == 0.0, 0.1, 0.0))  # at zero coefficients d_D T = 0: log-det -inf
    start = sum(H(tri2.KLObjective(T(samples))[0]))
    res = M.TrainMap(tri2, T(samples), max_iters=60)
    end = sum(H(tri2.KLObjective(T(samples))[0]))
    assert end < start - 0.5 and np.isfinite(end)
    del res


def test_sigmoid_archive_round_trip(gpu):
    M = gpu
    rng = np.random.default_rng(9)
    for m in (M.CreateSigmoidComponent(3, 2, _centers(rng, 3, 1), _opts(M, 0, 1, 0.8)),
              M.CreateSigmoidTriangular(3, 2, 2, np.column_stack([_centers(rng, 2, 0)] * 2), _opts(M, 1, 0)),
              M.CreateSigmoidComponent(1, 0, _centers(rng, 2, 0), _opts(M, 1, 0))):
        m.SetCoeffs(np.abs(rng.normal(0.0, 0.1, m.numCoeffs)))
        x = T(rng.normal(size=(m.inputDim, 300)))
        for back in (M.FromBytes(m.ToBytes()), pickle.loads(pickle.dumps(m))):
            assert type(back) is type(m)
            np.testing.assert_array_equal(np.asarray(back.CoeffMap()), np.asarray(m.CoeffMap()))
            np.testing.assert_array_equal(H(back.Evaluate(x)), H(m.Evaluate(x)))
            np.testing.assert_array_equal(H(back.LogDeterminant(x)), H(m.LogDeterminant(x)))
    with pytest.raises(ValueError):
        M.TriangularMap([M.CreateComponent(M.FixedMultiIndexSet(1, 2)),
                         M.CreateSigmoidComponent(2, 1, _centers(rng, 2, 0),
                                                  _opts(M, 1, 0))], True).Evaluate(T(np.zeros((2, 4))))


def test_sigmoid_map_torch_autograd(gpu, oracle):
    """TorchConditionalMapBase over a sigmoid TriangularMap: the backward pass
    (one fused adjoint call) against the oracle's CoeffGrad + LogDeterminantCoeffGrad
    and Gradient + LogDeterminantInputGrad."""
    M, O = gpu, oracle
    import torch
    rng = np.random.default_rng(21)
    dim, order = 3, 2
    cen = np.column_stack([_centers(rng, 3, 1) for _ in range(dim)])
    tri = M.CreateSigmoidTriangular(dim, dim, order, cen, _opts(M, 0, 1))
    otri = O.sigmoid_triangular(dim, dim, order, cen, 1.5, 1, O.POS_EXP)
    lb, _ = tri.CoeffBounds()
    c = rng.normal(0.0, 0.1, tri.numCoeffs)
    c[lb == 0.0] = np.abs(c[lb == 0.0]) + 0.05
    tri.SetCoeffs(c)
    mod = tri.torch(store_coeffs=True, return_logdet=True)
    x = rng.normal(size=(dim, 1500))
    xt = torch.tensor(x.T, dtype=torch.float64, device="cuda", requires_grad=True)
    y, ld = mod(xt)
    loss = (y * y).sum() + 0.5 * ld.sum()
    loss.backward()
    yo = otri.evaluate(c, x)
    ref_c = otri.coeff_grad(c, x, 2.0 * yo).sum(axis=1) + 0.5 * otri.logdet_coeff_grad(c, x).sum(axis=1)
    ref_x = otri.gradient(c, x, 2.0 * yo) + 0.5 * otri.logdet_input_grad(c, x)
    assert_parity(H(y).T, yo, what="torch forward")
    assert_parity(H(ld), otri.logdet(c, x), what="torch log-determinant")
    assert_parity(H(mod.coeffs.grad), ref_c, floor=1e-3, what="torch coefficient gradient")
    assert_parity(H(xt.grad).T, ref_x, what="torch input gradient")
