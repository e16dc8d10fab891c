"""Generates the golden fixtures in this directory.

    python tests/golden/make_golden.py

c1, c2, c3 and c5 hold the outputs of the reference itself: MParT's own
sources compiled unchanged into oracle/_ref (oracle/ref.mk; needs the
reference checkout), with the per-component FastGaussianReverseKL loss and
gradient composed from the reference's Evaluate, LogDeterminant, CoeffGrad
and LogDeterminantCoeffGrad as src/MapObjective.cpp:185-234 does (that file
needs Eigen's LU and is not compiled).  Each output is also computed by the
oracle's restatement, which must agree to the bit.  sig (the sigmoid
expansions, whose factory lives in src/MapFactory.cpp with the affine maps)
comes from the oracle.  c2's per-point integrand evaluation counts come from
the oracle (the reference does not count them).

Inputs come from numpy's default_rng with the seeds below and are stored in
the fixtures next to the outputs, so the fixtures do not depend on the
generator.  Configurations follow the benchmark configurations at reduced
point counts:
  c1  2x2 triangular map, total order 3, ProbabilistHermite + SoftPlus, tol 1e-6
  c2  one component, dim 8, total order 4 (495 terms), tol 1e-6
  c3  6-D triangular map, total order 5, HermiteFunctions + Exp, tol 1e-7, banana samples
  c5  16-D triangular map, total order 3, tol 1e-8, inverse to xtol 1e-10
  sig 3-D sigmoid triangular map, total order 2, three sigmoid terms (SoftPlus)

archive holds the reference's ToBytes / pickle archives
(ParameterizedFunctionBase::Save, with the cereal stand-in of
oracle/ref_shim/cereal) of maps built by its factory, by TriangularMap with
moveCoeffs and by WrapCoeffs, each after a sequence of operations (which set
the components' quadrature dimension that the archive records), with the
reference's evaluation of each map and its coefficient archive (the Python
binding's Serialize).  The case table (ARCHIVE_CASES) is stored
in the fixture as JSON.

    python tests/golden/make_golden.py [name ...]   # only the named fixtures
"""
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402


def agree(ref_out, orc_out, what):
    """The reference's output, after checking the oracle's equals it to the bit."""
    a, b = np.asarray(ref_out), np.asarray(orc_out)
    if not (a.shape == b.shape and np.all((a == b) | (np.isnan(a) & np.isnan(b)))):
        raise SystemExit(f"oracle and reference differ on {what}")
    return a


def ref_kl(basis, posfunc, tol, coef_blocks, comps, x):
    """FastGaussianReverseKLObjective::CommonEval<EvalGrad> per component
    (src/MapObjective.cpp:185-234) from the reference's own calls:
    loss = mean(0.5 T^2 - logdet), grad = mean(T dT/dc - dlogdet/dc)."""
    loss, grad = [], []
    for c, cc in zip(comps, coef_blocks):
        r = R.RefMap(c.input_dim, starts=c.starts, dims=c.dims, orders=c.orders, basis=basis, posfunc=posfunc,
                     abs_tol=tol, rel_tol=tol)
        r.set_coeffs(cc)
        pts = np.ascontiguousarray(x[:c.input_dim])
        T = r.evaluate(pts)[0]
        ld = r.logdet(pts)
        n = pts.shape[1]
        l = 0.0
        for j in range(n):
            l += 0.5 * T[j] * T[j] - ld[j]
        loss.append(l / n)
        grad.append((r.coeff_grad(pts, T[None, :]) - r.logdet_coeff_grad(pts)).sum(axis=1) / n)
    return np.array(loss), np.concatenate(grad)


def oracle_kl(tm, coef, x):
    loss, grad = [], []
    for i, c in enumerate(tm.comps):
        l, g = O.fast_gaussian_reverse_kl(c, tm.split(coef)[i], x[:c.input_dim])
        loss.append(l)
        grad.append(g)
    return np.array(loss), np.concatenate(grad)


def banana(n, seed):
    rng = np.random.default_rng(seed)
    x1 = rng.standard_normal(n)
    x2 = x1 ** 2 + 0.5 * rng.standard_normal(n)
    xs = [x1, x2]
    for _ in range(4):
        xs.append(0.8 * xs[-1] + 0.6 * rng.standard_normal(n))
    return np.stack(xs)


def make_c1(n=500):
    tm = O.OracleTriangularMap(2, 2, 3)
    ref = R.RefMap(2, 2, 3)
    coef = np.random.default_rng(0).normal(0.0, 0.1, tm.num_coeffs)
    ref.set_coeffs(coef)
    x = np.random.default_rng(1).standard_normal((2, n))
    sens = np.random.default_rng(7).standard_normal((2, n))
    r = agree(ref.evaluate(x), tm.evaluate(coef, x), "c1 evaluate")
    loss, grad = ref_kl("ProbabilistHermite", "SoftPlus", 1e-6, tm.split(coef), tm.comps, x)
    oloss, ograd = oracle_kl(tm, coef, x)
    return dict(coef=coef, x=x, sens=sens, evaluate=r,
                logdet=agree(ref.logdet(x), tm.logdet(coef, x), "c1 logdet"),
                inverse_warm=agree(ref.inverse(x, r), tm.inverse(coef, x, r), "c1 inverse (warm)"),
                inverse_cold=agree(ref.inverse(np.zeros((0, n)), r), tm.inverse(coef, np.zeros((0, n)), r),
                                   "c1 inverse (cold)"),
                coeff_grad=agree(ref.coeff_grad(x, sens), tm.coeff_grad(coef, x, sens), "c1 coeff_grad"),
                logdet_coeff_grad=agree(ref.logdet_coeff_grad(x), tm.logdet_coeff_grad(coef, x),
                                        "c1 logdet_coeff_grad"),
                gradient=agree(ref.gradient(x, sens), tm.gradient(coef, x, sens), "c1 gradient"),
                logdet_input_grad=agree(ref.logdet_input_grad(x), tm.logdet_input_grad(coef, x),
                                        "c1 logdet_input_grad"),
                kl_loss=agree(loss, oloss, "c1 kl loss"), kl_grad=agree(grad, ograd, "c1 kl grad"))


def make_c2(n=200):
    s, d, o = O.total_order(8, 4)
    c = O.OracleComponent(8, s, d, o)
    ref = R.RefMap(8, starts=s, dims=d, orders=o)
    coef = np.random.default_rng(0).normal(0.0, 0.05, c.num_terms)
    ref.set_coeffs(coef)
    x = np.random.default_rng(1).standard_normal((8, n))
    sens = np.random.default_rng(2).standard_normal(n)
    ev, nev, _ = c.evaluate(coef, x, return_evals=True)
    return dict(coef=coef, x=x, sens=sens, evaluate=agree(ref.evaluate(x)[0], ev, "c2 evaluate"), nevals=nev,
                logdet=agree(ref.logdet(x), c.logdet(coef, x), "c2 logdet"),
                coeff_grad_sum=agree(ref.coeff_grad(x, sens[None, :]), c.coeff_grad(coef, x, sens),
                                     "c2 coeff_grad").sum(axis=1),
                logdet_coeff_grad_sum=agree(ref.logdet_coeff_grad(x), c.logdet_coeff_grad(coef, x),
                                            "c2 logdet_coeff_grad").sum(axis=1))


def make_c3(n=300):
    tm = O.OracleTriangularMap(6, 6, 5, basis=O.BASIS_HERMITE_FUNCTIONS, posfunc=O.POS_EXP, abs_tol=1e-7,
                               rel_tol=1e-7)
    ref = R.RefMap(6, 6, 5, basis="HermiteFunctions", posfunc="Exp", abs_tol=1e-7, rel_tol=1e-7)
    coef = np.random.default_rng(3).normal(0.0, 0.01, tm.num_coeffs)
    ref.set_coeffs(coef)
    x = banana(n, 11)
    loss, grad = ref_kl("HermiteFunctions", "Exp", 1e-7, tm.split(coef), tm.comps, x)
    oloss, ograd = oracle_kl(tm, coef, x)
    return dict(coef=coef, x=x, evaluate=agree(ref.evaluate(x), tm.evaluate(coef, x), "c3 evaluate"),
                logdet=agree(ref.logdet(x), tm.logdet(coef, x), "c3 logdet"),
                kl_loss=agree(loss, oloss, "c3 kl loss"), kl_grad=agree(grad, ograd, "c3 kl grad"))


def make_c5(n=64):
    tm = O.OracleTriangularMap(16, 16, 3, abs_tol=1e-8, rel_tol=1e-8)
    ref = R.RefMap(16, 16, 3, abs_tol=1e-8, rel_tol=1e-8)
    coef = np.random.default_rng(0).normal(0.0, 0.03, tm.num_coeffs)
    ref.set_coeffs(coef)
    r = np.random.default_rng(1).standard_normal((16, n))
    return dict(coef=coef, r=r, inverse=agree(ref.inverse(np.zeros((0, n)), r, 1e-10, 1e-10),
                                              tm.inverse(coef, np.zeros((0, n)), r, xtol=1e-10, ytol=1e-10),
                                              "c5 inverse"))


def make_sig(n=200):
    """Sigmoid expansions: a 3-D sigmoid triangular map of total order 2,
    three Linear sigmoid terms per component (CreateSigmoidTriangular),
    HermiteFunctions + SoftPlus; non-negative coefficients on the terms with
    a last-input factor."""
    cen = np.array([-3.0, 3.0, 0.0, -1.5, 1.5, -2.0, 0.0, 2.0])
    centers = np.column_stack([cen, cen * 0.8, cen * 1.2])
    tm = O.sigmoid_triangular(3, 3, 2, centers, 1.5, O.SUM_LINEAR, O.POS_SOFTPLUS)
    rng = np.random.default_rng(5)
    coef = rng.normal(0.0, 0.2, tm.num_coeffs)
    diag = []  # the CoeffBounds lower bounds: terms with a last-input factor
    for c in tm.comps:
        s, d = c.starts, c.dims
        for t in range(len(s) - 1):
            diag.append(s[t + 1] > s[t] and d[s[t + 1] - 1] == c.input_dim - 1)
    diag = np.array(diag)
    coef[diag] = np.abs(coef[diag]) + 0.05
    x = rng.standard_normal((3, n))
    sens = rng.standard_normal((3, n))
    r = tm.evaluate(coef, x)
    return dict(centers=centers, coef=coef, x=x, sens=sens, evaluate=r, logdet=tm.logdet(coef, x),
                coeff_grad=tm.coeff_grad(coef, x, sens), logdet_coeff_grad=tm.logdet_coeff_grad(coef, x),
                gradient=tm.gradient(coef, x, sens), logdet_input_grad=tm.logdet_input_grad(coef, x),
                inverse_cold=tm.inverse(coef, np.zeros((0, n)), r))


# build: "triangular" (MapFactory::CreateTriangular, then SetCoeffs),
# "component" (CreateComponent on the total-order set, then SetCoeffs),
# "moved" (TriangularMap(components, moveCoeffs=true) of CreateComponent
# components with coefficients), "wrapped" (CreateTriangular, then WrapCoeffs
# on caller memory).  ops run in order on x (and sens) after an Evaluate.
# The reference's fixed ClenshawCurtis rule keeps a one-double internal
# workspace, so its operations that integrate more than one function
# (CoeffGrad, Gradient, the discrete-derivative log-determinant) fail its
# assertion fdim <= maxDim (Quadrature.h:174-183); its cases run Evaluate and
# Inverse only.
ARCHIVE_CASES = [
    dict(name="tri_ph_softplus_acc", build="triangular", in_dim=3, out_dim=2, order=3,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis"), ops=[]),
    dict(name="tri_hf_exp_acc_coeffgrad", build="triangular", in_dim=4, out_dim=2, order=2,
         opts=dict(basis="HermiteFunctions", posfunc="Exp", quad="AdaptiveClenshawCurtis", abs_tol=1e-7,
                   rel_tol=1e-7, max_sub=20, quad_pts=9), ops=["coeff_grad"]),
    dict(name="tri_ph_exp_cc_unnormalised", build="triangular", in_dim=2, out_dim=2, order=4,
         opts=dict(basis="ProbabilistHermite", posfunc="Exp", quad="ClenshawCurtis", quad_pts=6, normalize=False),
         ops=["evaluate", "inverse"]),
    dict(name="tri_ph_softplus_as_discrete_logdet", build="triangular", in_dim=3, out_dim=3, order=2,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveSimpson", cont_deriv=False,
                   nugget=0.05, min_sub=1, max_sub=12), ops=["logdet"]),
    dict(name="tri_hf_softplus_acc_gradient", build="triangular", in_dim=3, out_dim=2, order=3,
         opts=dict(basis="HermiteFunctions", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis"), ops=["gradient"]),
    dict(name="tri_ph_softplus_acc_discrete_ldcg", build="triangular", in_dim=2, out_dim=1, order=3,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis", cont_deriv=False),
         ops=["logdet_coeff_grad"]),
    dict(name="tri_ph_softplus_acc_inverse", build="triangular", in_dim=3, out_dim=2, order=2,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis"),
         ops=["coeff_grad", "inverse"]),
    dict(name="comp_ph_softplus_acc", build="component", in_dim=4, out_dim=1, order=3,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="AdaptiveClenshawCurtis", nugget=0.01),
         ops=["coeff_grad"]),
    dict(name="moved_hf_exp_as", build="moved", in_dim=3, out_dim=2, order=2,
         opts=dict(basis="HermiteFunctions", posfunc="Exp", quad="AdaptiveSimpson"), ops=[]),
    dict(name="wrapped_ph_softplus_cc", build="wrapped", in_dim=2, out_dim=2, order=2,
         opts=dict(basis="ProbabilistHermite", posfunc="SoftPlus", quad="ClenshawCurtis", quad_pts=5), ops=[]),
]


def _ref_archive_map(case, coef):
    """The reference map of an ARCHIVE_CASES entry, its coefficients set
    (the components, kept alive, for the moved case)."""
    o = case["opts"]
    if case["build"] == "component":
        s, d, r = O.total_order(case["in_dim"], case["order"])
        m = R.RefMap(case["in_dim"], starts=s, dims=d, orders=r, **o)
        m.set_coeffs(coef)
        return m
    if case["build"] == "moved":
        extra = case["in_dim"] - case["out_dim"]
        comps, off = [], 0
        for i in range(case["out_dim"]):
            s, d, r = O.total_order(extra + i + 1, case["order"])
            c = R.RefMap(extra + i + 1, starts=s, dims=d, orders=r, **o)
            c.set_coeffs(coef[off:off + c.num_coeffs])
            off += c.num_coeffs
            comps.append(c)
        return R.RefMap.triangular_from(comps)
    m = R.RefMap(case["in_dim"], case["out_dim"], case["order"], **o)
    if case["build"] == "wrapped":
        m.wrap_coeffs(coef)
    else:
        m.set_coeffs(coef)
    return m


def make_archive(n=40):
    import json
    rng = np.random.default_rng(31)
    x = rng.standard_normal((4, n))
    sens = rng.standard_normal((4, n))
    out = dict(x=x, sens=sens, cases=np.array(json.dumps(ARCHIVE_CASES)))
    for case in ARCHIVE_CASES:
        name, ind, outd = case["name"], case["in_dim"], case["out_dim"]
        dims = [ind] if case["build"] == "component" else [ind - outd + i + 1 for i in range(outd)]
        ncoef = sum(len(O.total_order(d, case["order"])[0]) - 1 for d in dims)
        coef = np.random.default_rng(zlib.crc32(name.encode())).normal(0.0, 0.1, ncoef)
        m = _ref_archive_map(case, coef)
        xi = x[:ind]
        ev = m.evaluate(xi)
        for op in case["ops"]:
            if op == "evaluate":
                m.evaluate(xi)
            elif op == "coeff_grad":
                m.coeff_grad(xi, sens[:outd])
            elif op == "gradient":
                m.gradient(xi, sens[:outd])
            elif op == "logdet":
                m.logdet(xi)
            elif op == "logdet_coeff_grad":
                m.logdet_coeff_grad(xi)
            elif op == "inverse":
                m.inverse(xi[:ind - outd], ev)
            else:
                raise ValueError(op)
        out[f"{name}__coef"] = coef
        out[f"{name}__eval"] = ev
        out[f"{name}__bytes"] = np.frombuffer(m.to_bytes(), np.uint8).copy()
        out[f"{name}__serialize"] = np.frombuffer(m.coeff_archive(), np.uint8).copy()
    return out


if __name__ == "__main__":
    O.build()
    makers = (("c1", make_c1), ("c2", make_c2), ("c3", make_c3), ("c5", make_c5), ("sig", make_sig),
              ("archive", make_archive))
    only = set(sys.argv[1:])
    for name, fn in makers:
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fn())
        print("wrote", name)
