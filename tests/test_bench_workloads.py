"""The benchmark's workload definitions (bench.py) against the configurations
they restate: sizes, distributions and seeds, and the FLOP model that the
roofline fraction divides by.  CPU only."""
import math

import numpy as np
import pytest

import bench


def test_c2_workload_and_flop_model():
    assert (bench.DIM, bench.ORDER, bench.NPTS, bench.TOL, bench.MAXSUB) == (8, 4, 1_000_000, 1e-6, 30)
    x, s = bench.synth(1000)
    assert x.shape == (8, 1000) and s.shape == (1, 1000)
    np.testing.assert_array_equal(x, bench.synth(1000)[0])  # seeded
    c = bench.coeffs(495)
    assert abs(c.std() - 0.05) < 0.01
    pytest.importorskip("mpart_gb300")
    nodes, T, nB, sc = bench.prefix_stats()
    assert T == 495 and nB == 28  # C(12, 4) terms; 7 leading inputs x order 4
    assert nodes == math.comb(11, 4) == 330  # distinct leading multi-indices (total order <= 4 over 7 inputs)
    assert sc == 511
    assert math.isclose(bench.flops_per_point(9.0308), 3449.0992, rel_tol=1e-12)
    # the model is linear in the evaluations per point
    f9, f12 = bench.flops_per_point(9.0), bench.flops_per_point(12.0)
    assert f12 > f9 > 2 * T
    assert math.isclose(bench.flops_per_point(10.5), 0.5 * (f9 + f12))


def test_kl_workload_banana():
    assert (bench.KL_DIM, bench.KL_ORDER, bench.KL_N, bench.KL_TOL) == (6, 5, 200_000, 1e-7)
    assert bench.KL_TRAIN["precondition"] and bench.KL_TRAIN["algorithm"] == "LD_LBFGS" and bench.KL_FTOL_REL > 0
    x = bench.banana(200_000)
    assert x.shape == (6, 200_000)
    assert abs(x[0].mean()) < 0.01 and abs(x[0].std() - 1.0) < 0.01
    r = x[1] - x[0] ** 2  # x2 = x1^2 + 0.5 N(0, 1)
    assert abs(r.std() - 0.5) < 0.01
    for k in range(2, 6):  # x_k = 0.8 x_{k-1} + 0.6 N(0, 1)
        e = x[k] - 0.8 * x[k - 1]
        assert abs(e.std() - 0.6) < 0.01


def test_batch_workload_ranges():
    specs = bench.batch_specs()
    assert len(specs) == 64
    dims, orders, npts = zip(*specs)
    assert min(dims) >= 2 and max(dims) <= 16
    assert min(orders) >= 2 and max(orders) <= 6
    assert min(npts) >= 1000 and max(npts) <= 200_000
    assert specs == bench.batch_specs()  # seeded


def test_inverse_and_sigmoid_workloads():
    assert (bench.INV_DIM, bench.INV_ORDER, bench.INV_N, bench.INV_TOL, bench.INV_XTOL) == (16, 3, 4_000_000, 1e-8,
                                                                                             1e-10)
    assert math.comb(16 + 3, 3) == 969  # terms of the last component
    assert (bench.SIG_DIM, bench.SIG_ORDER, bench.SIG_NSIG, bench.SIG_N) == (8, 3, 5, 1_000_000)
    c = bench.sigmoid_centers(5)
    assert len(c) == 2 + 15 and np.all(np.isfinite(c))  # two edge terms, then 1 + 2 + ... + 5 centers


def test_reference_flop_model():
    """The reference-algorithm count: dim 8, order 4 has 495 terms, 165 of
    them with x_D; per node 2 sum k_t (x_D terms) + 15 + 20 + 3 * 165."""
    from mpart_gb300 import FixedMultiIndexSet
    ms = FixedMultiIndexSet(bench.DIM, bench.ORDER)
    terms = [ms.IndexToMulti(t) for t in range(ms.Size())]
    kd = sum(sum(1 for v in m if v > 0) for m in terms if m[-1] > 0)
    ks = sum(sum(1 for v in m if v > 0) for m in terms)
    assert sum(1 for m in terms if m[-1] > 0) == 165
    node = 2 * kd + 15 + 20 + 3 * 165
    fixed = 3 * 7 * 5 + 2 * ks + 495
    assert bench.reference_flops_per_point(10.0) == 10 * node + fixed
    assert bench.reference_flops_per_point(10.0) > 5 * bench.flops_per_point(10.0)
