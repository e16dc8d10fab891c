"""Generates the golden fixtures in this directory from the CPU oracle.

    python tests/golden/make_golden.py

Inputs come from numpy's default_rng with the seeds below and are stored in
the fixtures next to the outputs, so the fixtures do not depend on the
generator.  Configurations follow the benchmark configurations at reduced
point counts:
  c1  2x2 triangular map, total order 3, ProbabilistHermite + SoftPlus, tol 1e-6
  c2  one component, dim 8, total order 4 (495 terms), tol 1e-6
  c3  6-D triangular map, total order 5, HermiteFunctions + Exp, tol 1e-7, banana samples
  c5  16-D triangular map, total order 3, tol 1e-8, inverse to xtol 1e-10
  sig 3-D sigmoid triangular map, total order 2, three sigmoid terms (SoftPlus)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


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
    coef = np.random.default_rng(0).normal(0.0, 0.1, tm.num_coeffs)
    x = np.random.default_rng(1).standard_normal((2, n))
    sens = np.random.default_rng(7).standard_normal((2, n))
    r = tm.evaluate(coef, x)
    loss, grad = [], []
    for i, c in enumerate(tm.comps):
        l, g = O.fast_gaussian_reverse_kl(c, tm.split(coef)[i], x[:c.input_dim])
        loss.append(l)
        grad.append(g)
    return dict(coef=coef, x=x, sens=sens, evaluate=r, logdet=tm.logdet(coef, x),
                inverse_warm=tm.inverse(coef, x, r), inverse_cold=tm.inverse(coef, np.zeros((0, n)), r),
                coeff_grad=tm.coeff_grad(coef, x, sens), logdet_coeff_grad=tm.logdet_coeff_grad(coef, x),
                gradient=tm.gradient(coef, x, sens), logdet_input_grad=tm.logdet_input_grad(coef, x),
                kl_loss=np.array(loss), kl_grad=np.concatenate(grad))


def make_c2(n=200):
    s, d, o = O.total_order(8, 4)
    c = O.OracleComponent(8, s, d, o)
    coef = np.random.default_rng(0).normal(0.0, 0.05, c.num_terms)
    x = np.random.default_rng(1).standard_normal((8, n))
    sens = np.random.default_rng(2).standard_normal(n)
    ev, nev, _ = c.evaluate(coef, x, return_evals=True)
    return dict(coef=coef, x=x, sens=sens, evaluate=ev, nevals=nev, logdet=c.logdet(coef, x),
                coeff_grad_sum=c.coeff_grad(coef, x, sens).sum(axis=1),
                logdet_coeff_grad_sum=c.logdet_coeff_grad(coef, x).sum(axis=1))


def make_c3(n=300):
    tm = O.OracleTriangularMap(6, 6, 5, basis=O.BASIS_HERMITE_FUNCTIONS, posfunc=O.POS_EXP, abs_tol=1e-7,
                               rel_tol=1e-7)
    coef = np.random.default_rng(3).normal(0.0, 0.01, tm.num_coeffs)
    x = banana(n, 11)
    loss, grad = [], []
    for i, c in enumerate(tm.comps):
        l, g = O.fast_gaussian_reverse_kl(c, tm.split(coef)[i], x[:c.input_dim])
        loss.append(l)
        grad.append(g)
    return dict(coef=coef, x=x, evaluate=tm.evaluate(coef, x), logdet=tm.logdet(coef, x), kl_loss=np.array(loss),
                kl_grad=np.concatenate(grad))


def make_c5(n=64):
    tm = O.OracleTriangularMap(16, 16, 3, abs_tol=1e-8, rel_tol=1e-8)
    coef = np.random.default_rng(0).normal(0.0, 0.03, tm.num_coeffs)
    r = np.random.default_rng(1).standard_normal((16, n))
    return dict(coef=coef, r=r, inverse=tm.inverse(coef, np.zeros((0, n)), r, xtol=1e-10, ytol=1e-10))


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


if __name__ == "__main__":
    O.build()
    for name, fn in (("c1", make_c1), ("c2", make_c2), ("c3", make_c3), ("c5", make_c5), ("sig", make_sig)):
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fn())
        print("wrote", name)
