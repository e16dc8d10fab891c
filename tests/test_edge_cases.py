"""Edge cases through the C ABI on the GPU: empty inputs on every entry point,
point counts that are not a multiple of the 128-point tile, and strided
(non-contiguous) point matrices, for monotone components and sigmoid
expansions."""
import numpy as np
import pytest

from test_gpu_parity import H, T, assert_parity, oracle_tri, opts

pytestmark = pytest.mark.gpu


def _maps(M, O):
    rng = np.random.default_rng(4)
    mono = M.CreateTriangular(3, 2, 2, opts(M))
    mono.SetCoeffs(rng.normal(0.0, 0.1, mono.numCoeffs))
    omono = oracle_tri(O, 3, 2, 2)
    cen = np.column_stack([np.array([-3.0, 3.0, 0.0, -1.0, 1.0])] * 2)
    sopts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, sigmoidBasisSumType=M.SigmoidSumSizeType.Constant)
    sig = M.CreateSigmoidTriangular(3, 2, 2, cen, sopts)
    lb, _ = sig.CoeffBounds()
    c = rng.normal(0.0, 0.1, sig.numCoeffs)
    c[lb == 0.0] = np.abs(c[lb == 0.0]) + 0.05
    sig.SetCoeffs(c)
    osig = O.sigmoid_triangular(3, 2, 2, cen, 1.5, O.SUM_CONSTANT, O.POS_SOFTPLUS)
    return [(mono, omono), (sig, osig)]


def test_empty_inputs_on_every_entry_point(gpu, oracle):
    import torch
    M = gpu
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device="cuda")
    for m, _ in _maps(M, oracle):
        x = z(m.inputDim, 0)
        assert H(m.Evaluate(x)).shape == (m.outputDim, 0)
        assert H(m.LogDeterminant(x)).shape == (0,)
        assert H(m.CoeffGrad(x, z(m.outputDim, 0))).shape == (m.numCoeffs, 0)
        assert H(m.Gradient(x, z(m.outputDim, 0))).shape == (m.inputDim, 0)
        assert H(m.LogDeterminantCoeffGrad(x)).shape == (m.numCoeffs, 0)
        assert H(m.LogDeterminantInputGrad(x)).shape == (m.inputDim, 0)
        assert H(m.Inverse(z(m.inputDim - m.outputDim, 0), z(m.outputDim, 0))).shape == (m.outputDim, 0)
        cg = torch.full((m.numCoeffs,), 7.0, dtype=torch.float64, device="cuda")
        m.FusedForwardAdjointImpl(x, sens=z(m.outputDim, 0), logdet_sens_scale=1.0, coeff_grad=cg)
        assert not H(cg).any()  # no points: a zero gradient
        with pytest.raises(ValueError):
            m.KLObjective(x)


@pytest.mark.parametrize("n", [1, 127, 129, 257])
def test_ragged_point_counts_match_oracle(gpu, oracle, n):
    M, O = gpu, oracle
    rng = np.random.default_rng(n)
    for m, om in _maps(M, O):
        coef = np.asarray(m.CoeffMap())
        x = rng.standard_normal((m.inputDim, n))
        s = rng.standard_normal((m.outputDim, n))
        assert_parity(H(m.Evaluate(T(x))), om.evaluate(coef, x), what=f"Evaluate n={n}")
        assert_parity(H(m.LogDeterminant(T(x))), om.logdet(coef, x), what=f"LogDeterminant n={n}")
        import torch
        cg = torch.zeros(m.numCoeffs, dtype=torch.float64, device="cuda")
        m.FusedForwardAdjointImpl(T(x), sens=T(s), logdet_sens_scale=1.0, coeff_grad=cg)
        ref = om.coeff_grad(coef, x, s).sum(axis=1) + om.logdet_coeff_grad(coef, x).sum(axis=1)
        assert_parity(H(cg), ref, floor=1e-3, what=f"fused adjoint n={n}")


def test_strided_points_give_the_same_results(gpu, oracle):
    import torch
    M = gpu
    rng = np.random.default_rng(8)
    for m, _ in _maps(M, oracle):
        xn = rng.standard_normal((300, m.inputDim))
        xs = torch.as_tensor(xn, device="cuda").T  # column stride 1 across rows: a transposed view
        xc = xs.contiguous()
        assert not xs.is_contiguous()
        np.testing.assert_array_equal(H(m.Evaluate(xs)), H(m.Evaluate(xc)))
        np.testing.assert_array_equal(H(m.LogDeterminant(xs)), H(m.LogDeterminant(xc)))
        sn = torch.as_tensor(rng.standard_normal((300, m.outputDim)), device="cuda").T
        np.testing.assert_array_equal(H(m.Gradient(xs, sn)), H(m.Gradient(xc, sn.contiguous())))
