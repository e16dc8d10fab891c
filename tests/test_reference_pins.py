"""The oracle against the reference itself (no GPU): MParT's own sources,
compiled unchanged into oracle/_ref (oracle/ref.mk, with the serial Kokkos and
minimal Eigen stand-ins of oracle/ref_shim/), on the same seeded inputs.

Both are built with strict IEEE evaluation order (-ffp-contract=off), so the
oracle's restatement must give the reference's results to the bit: every
entry point of the monotone-component path (Evaluate, LogDeterminant,
CoeffGrad, Gradient, LogDeterminantCoeffGrad, LogDeterminantInputGrad,
Inverse) on the benchmark workloads' maps, and every MapOptions combination
the path supports (AdaptiveClenshawCurtis, AdaptiveSimpson, ClenshawCurtis;
ProbabilistHermite and HermiteFunctions; SoftPlus and Exp; contDeriv; the
nugget).

The reference checkout exists only on the development host; elsewhere these
tests are skipped (the GPU tests compare against the oracle and the committed
fixtures, which tests/golden/make_golden.py takes from the reference)."""
import numpy as np
import pytest

from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference checkout not present")

QUAD = {"AdaptiveClenshawCurtis": 2, "AdaptiveSimpson": 1, "ClenshawCurtis": 0}


def same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, what
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    assert eq.all(), f"{what}: {np.count_nonzero(~eq)} of {a.size} differ (max {np.nanmax(np.abs(a - b)):.3e})"


def pair(O, inp, out, order, basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis",
         tol=1e-6, max_sub=30, nugget=0.0, cont_deriv=True, quad_pts=5):
    ref = R.RefMap(inp, out, order, basis=basis, posfunc=posfunc, quad=quad, abs_tol=tol, rel_tol=tol,
                   max_sub=max_sub, nugget=nugget, cont_deriv=cont_deriv, quad_pts=quad_pts)
    orc = O.OracleTriangularMap(inp, out, order,
                                basis=O.BASIS_HERMITE_FUNCTIONS if basis == "HermiteFunctions" else O.BASIS_PROB_HERMITE,
                                normalize=True, posfunc=O.POS_EXP if posfunc == "Exp" else O.POS_SOFTPLUS,
                                abs_tol=tol, rel_tol=tol, max_sub=max_sub, nugget=nugget, quad_type=QUAD[quad],
                                quad_pts=quad_pts, cont_deriv=cont_deriv)
    return ref, orc


def check_all(ref, orc, coef, x, sens, adjoints=True, inverse=True, xtol=1e-6, ytol=1e-6):
    ref.set_coeffs(coef)
    same(ref.evaluate(x), orc.evaluate(coef, x), "Evaluate")
    same(ref.logdet(x), orc.logdet(coef, x), "LogDeterminant")
    same(ref.logdet_coeff_grad(x), orc.logdet_coeff_grad(coef, x), "LogDeterminantCoeffGrad")
    if adjoints:
        same(ref.coeff_grad(x, sens), orc.coeff_grad(coef, x, sens), "CoeffGrad")
        same(ref.gradient(x, sens), orc.gradient(coef, x, sens), "Gradient")
        if orc.comps[0].cont_deriv:
            same(ref.logdet_input_grad(x), orc.logdet_input_grad(coef, x), "LogDeterminantInputGrad")
    if inverse:
        r = orc.evaluate(coef, x)
        n = x.shape[1]
        extra = orc.input_dim - orc.output_dim
        for x1 in (x, x[:extra]):  # with and without initial guesses
            same(ref.inverse(x1, r, xtol, ytol), orc.inverse(coef, x1 if len(x1) else np.zeros((0, n)), r, xtol, ytol),
                 "Inverse")


def test_c1_map_matches_reference(oracle):
    """2 x 2, total order 3, ProbabilistHermite + SoftPlus, ACC tol 1e-6: the
    small workload on its 10,000 points."""
    O = oracle
    ref, orc = pair(O, 2, 2, 3)
    coef = np.random.default_rng(0).normal(0.0, 0.1, orc.num_coeffs)
    x = np.random.default_rng(1).standard_normal((2, 10000))
    sens = np.random.default_rng(2).standard_normal((2, 10000))
    check_all(ref, orc, coef, x, sens)


def test_c2_component_matches_reference(oracle):
    """One component, dim 8, total order 4 (495 terms), ACC tol 1e-6 / maxSub
    30: the fused-adjoint workload's component on 2,000 of its points."""
    O = oracle
    s, d, o = O.total_order(8, 4)
    ref = R.RefMap(8, starts=s, dims=d, orders=o)
    orc = O.OracleComponent(8, s, d, o)
    assert ref.num_coeffs == 495
    coef = np.random.default_rng(0).normal(0.0, 0.05, 495)
    x = np.random.default_rng(1).standard_normal((8, 2000))
    sens = np.random.default_rng(2).standard_normal((1, 2000))
    ref.set_coeffs(coef)
    same(ref.evaluate(x)[0], orc.evaluate(coef, x), "Evaluate")
    same(ref.logdet(x), orc.logdet(coef, x), "LogDeterminant")
    same(ref.coeff_grad(x, sens), orc.coeff_grad(coef, x, sens[0]), "CoeffGrad")
    same(ref.logdet_coeff_grad(x), orc.logdet_coeff_grad(coef, x), "LogDeterminantCoeffGrad")


def test_kl_map_matches_reference(oracle):
    """6-D TriangularMap, total order 5, HermiteFunctions + Exp, tol 1e-7: the
    KL training map on 1,000 banana samples."""
    O = oracle
    ref, orc = pair(O, 6, 6, 5, basis="HermiteFunctions", posfunc="Exp", tol=1e-7)
    rng = np.random.default_rng(11)
    x1 = rng.standard_normal(1000)
    xs = [x1, x1 ** 2 + 0.5 * rng.standard_normal(1000)]
    while len(xs) < 6:
        xs.append(0.8 * xs[-1] + 0.6 * rng.standard_normal(1000))
    x = np.stack(xs)
    coef = np.random.default_rng(3).normal(0.0, 0.001, orc.num_coeffs)
    sens = np.random.default_rng(4).standard_normal((6, 1000))
    check_all(ref, orc, coef, x, sens, inverse=False)


def test_inverse_map_matches_reference(oracle):
    """16-D TriangularMap, total order 3, ProbabilistHermite + SoftPlus, tol
    1e-8: the inverse workload's map, Inverse of 60 random targets to xtol 1e-10
    (ITP iterates to the bit), and its forward evaluations."""
    O = oracle
    ref, orc = pair(O, 16, 16, 3, tol=1e-8)
    coef = np.random.default_rng(31).normal(0.0, 0.03, orc.num_coeffs)
    r = np.random.default_rng(32).standard_normal((16, 60))
    ref.set_coeffs(coef)
    same(ref.inverse(np.zeros((0, 60)), r, 1e-10, 1e-10), orc.inverse(coef, np.zeros((0, 60)), r, 1e-10, 1e-10),
         "Inverse")
    x = np.random.default_rng(33).standard_normal((16, 200))
    same(ref.evaluate(x), orc.evaluate(coef, x), "Evaluate")
    same(ref.logdet(x), orc.logdet(coef, x), "LogDeterminant")


@pytest.mark.parametrize("kw", [
    dict(quad="AdaptiveSimpson"),
    dict(basis="HermiteFunctions", posfunc="Exp"),
    dict(posfunc="Exp", quad="AdaptiveSimpson"),
    dict(cont_deriv=False),
    dict(nugget=0.3),
    dict(tol=1e-9, max_sub=12),
], ids=lambda kw: ",".join(f"{k}={v}" for k, v in kw.items()))
def test_options_match_reference(oracle, kw):
    O = oracle
    ref, orc = pair(O, 3, 3, 3, **kw)
    coef = np.random.default_rng(5).normal(0.0, 0.1, orc.num_coeffs)
    x = np.random.default_rng(6).standard_normal((3, 1500))
    sens = np.random.default_rng(7).standard_normal((3, 1500))
    check_all(ref, orc, coef, x, sens)


def test_fixed_clenshaw_curtis_matches_reference(oracle):
    """The fixed ClenshawCurtis rule (quadPts 9).  The reference's factory
    gives it maxDim 1 and its SetDim asserts fdim <= maxDim
    (MParT/Quadrature.h:178; the reference's release flags keep asserts), so
    the reference computes only the value-sized quadratures with it:
    Evaluate, LogDeterminant and Inverse."""
    O = oracle
    ref, orc = pair(O, 2, 2, 3, quad="ClenshawCurtis", quad_pts=9)
    coef = np.random.default_rng(0).normal(0.0, 0.1, orc.num_coeffs)
    x = np.random.default_rng(1).standard_normal((2, 2000))
    check_all(ref, orc, coef, x, None, adjoints=False)


def test_nugget_enters_inverse_but_not_evaluate(oracle):
    """The reference's EvaluateImpl calls EvaluateSingle without the nugget
    (MonotoneComponent.h:290), while Inverse passes it
    (MonotoneComponent.h:434), so with a nonzero nugget
    Inverse(Evaluate(x)) != x; the oracle keeps both."""
    O = oracle
    ref, orc = pair(O, 1, 1, 2, nugget=0.5)
    coef = np.array([0.1, 0.5, -0.2])
    ref.set_coeffs(coef)
    x = np.array([[0.3, -1.2, 2.0]])
    y = ref.evaluate(x)
    same(y, orc.evaluate(coef, x), "Evaluate")
    xi = ref.inverse(np.zeros((0, 3)), y, 1e-12, 1e-12)
    same(xi, orc.inverse(coef, np.zeros((0, 3)), y, 1e-12, 1e-12), "Inverse")
    assert np.all(np.abs(xi - x) > 1e-3)


def _grow(rng, length, steps, expand_every=0):
    """A downward-closed set grown from a total-order set the way the adaptive
    loop grows it: one reduced-margin term at a time (and, every expand_every
    steps, a whole Expand)."""
    import mpart_gb300 as M
    s = M.MultiIndexSet.CreateTotalOrder(length, int(rng.integers(0, 3)))
    sets = [list(s._terms)]
    for k in range(steps):
        if expand_every and k % expand_every == expand_every - 1:
            s.Expand()
        else:
            rm = s.ReducedMargin()
            s += rm[rng.integers(len(rm))]
        sets.append(list(s._terms))
    return sets


def test_multi_index_set_order_matches_reference():
    """MultiIndexSet::ReducedMargin and ::Expand, whose order decides which of
    equal KL gradients TrainMapAdaptive picks, against the reference's own
    MultiIndexSet on sets grown as the adaptive loop grows them: the same
    terms in the same order, and Expand's returned indices (a term reached
    from several frontier terms repeated) equal."""
    import mpart_gb300 as M
    rng = np.random.default_rng(5)
    for length in (1, 2, 3, 4, 5):
        for terms in _grow(rng, length, 10, expand_every=4):
            s = M.MultiIndexSet(length, terms)
            got_rm = [tuple(int(v) for v in m) for m in s.ReducedMargin()]
            assert got_rm == R.mset_reduced_margin(terms), (length, terms)
            ref_idx, ref_terms = R.mset_expand(terms)
            got_idx = s.Expand()
            assert got_idx == ref_idx, (length, terms)
            assert [tuple(int(v) for v in t) for t in s._terms] == ref_terms
    # the 2-D total-order-1 set: [1 1] is reached from [0 1] and [1 0]
    assert R.mset_expand([(0, 0), (0, 1), (1, 0)])[0] == [3, 4, 3, 5]


@pytest.mark.parametrize("dim,sum_type,pos", [(1, "Linear", "SoftPlus"), (2, "Linear", "SoftPlus"),
                                              (3, "Constant", "SoftPlus"), (3, "Linear", "Exp")])
def test_sigmoid_expansion_matches_reference(oracle, dim, sum_type, pos):
    """The sigmoid expansions against the reference's own Sigmoid1d,
    RectifiedMultivariateExpansion and UnivariateExpansion (as
    MapFactory::CreateSigmoidComponent assembles them), with the factory's
    widths and weights from the oracle's restatement: every entry point, to
    the bit; the Inverse (the classes' own solvers) to the solver tolerance."""
    O = oracle
    if sum_type == "Linear":
        centers = np.array([-3.0, 3.0, 0.0, -1.0, 1.0, -2.0, 0.0, 2.0])  # three sigmoid terms
        nsig, st = 3, O.SUM_LINEAR
    else:
        centers = np.array([-3.0, 3.0, 1.0, -1.0, 0.5])
        nsig, st = 3, O.SUM_CONSTANT
    oc, w, wt, starts = O.sigmoid_from_centers(centers, 1.5, st)
    s, d, o = O.sigmoid_mset(dim, 2, 2, nsig)
    orc = O.OracleSigmoidComponent(dim, s, d, o, (oc, w, wt, starts), O.POS_EXP if pos == "Exp" else O.POS_SOFTPLUS)
    ref = R.RefSigmoid(dim, s, d, o, oc, w, wt, sum_type, pos)
    assert ref.num_coeffs == orc.num_coeffs and ref.input_dim == dim
    rng = np.random.default_rng(11 + dim)
    # positive coefficients on the terms with a last-input factor keep the map monotone
    diag = np.array([d[s[t + 1] - 1] == dim - 1 if s[t + 1] > s[t] else False for t in range(len(s) - 1)])
    coef = np.where(diag, 0.1 + 0.2 * rng.random(orc.num_coeffs), 0.1 * rng.standard_normal(orc.num_coeffs))
    if dim == 1:
        coef[0] = 0.1 * rng.standard_normal()
    x = rng.standard_normal((dim, 300)) * 1.5
    sens = rng.standard_normal((1, 300))
    ref.set_coeffs(coef)
    same(ref.evaluate(x)[0], orc.evaluate(coef, x), "Evaluate")
    same(ref.logdet(x), orc.logdet(coef, x), "LogDeterminant")
    same(ref.coeff_grad(x, sens), orc.coeff_grad(coef, x, sens), "CoeffGrad")
    same(ref.gradient(x, sens), orc.gradient(coef, x, sens), "Gradient")
    same(ref.logdet_coeff_grad(x), orc.logdet_coeff_grad(coef, x), "LogDeterminantCoeffGrad")
    same(ref.logdet_input_grad(x), orc.logdet_input_grad(coef, x), "LogDeterminantInputGrad")
    r = orc.evaluate(coef, x)
    xi = ref.inverse(x[:dim - 1], r)[0]
    np.testing.assert_allclose(xi, x[dim - 1], atol=1e-5)
