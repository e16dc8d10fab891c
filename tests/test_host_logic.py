"""Host-side logic that needs no GPU: multi-index sets, options, array views."""
import numpy as np
import pytest

import mpart_gb300 as M


def test_total_order_matches_oracle(oracle):
    for dim, order in [(1, 3), (2, 3), (3, 2), (8, 4), (6, 5)]:
        ms = M.FixedMultiIndexSet(dim, order)
        s, d, o = oracle.total_order(dim, order)
        np.testing.assert_array_equal(ms.nzStarts, s)
        np.testing.assert_array_equal(ms.nzDims, d)
        np.testing.assert_array_equal(ms.nzOrders, o)
    assert M.FixedMultiIndexSet(8, 4).Size() == 495
    assert M.FixedMultiIndexSet(16, 3).Size() == 969


def test_from_multis_round_trip():
    multis = np.array([[0, 0], [0, 1], [2, 0]])
    ms = M.FixedMultiIndexSet.from_multis(multis)
    assert ms.Size() == 3
    for i in range(3):
        np.testing.assert_array_equal(ms.IndexToMulti(i), multis[i])


def test_map_options_defaults():
    o = M.MapOptions()
    assert o.quadType == M.QuadTypes.AdaptiveSimpson and o.quadMaxSub == 30 and o.basisNorm
    o = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=1e-8)
    c = o._c()
    assert c.quad_type == 2 and c.quad_abs_tol == 1e-8
    with pytest.raises(AttributeError):
        M.MapOptions(nonsense=1)


def test_matrix_views():
    from mpart_gb300 import _mat
    a = np.arange(12.0).reshape(3, 4)
    m = _mat(a)
    assert (m.rows, m.cols, m.row_stride, m.col_stride) == (3, 4, 4, 1)
    m = _mat(a.T)
    assert (m.rows, m.cols, m.row_stride, m.col_stride) == (4, 3, 1, 4)
    m = _mat(a[1])
    assert (m.rows, m.cols, m.col_stride) == (1, 4, 1)
    import torch
    t = torch.zeros(5, 7, dtype=torch.float64)[:, ::2]
    m = _mat(t)
    assert (m.rows, m.cols, m.row_stride, m.col_stride) == (5, 4, 7, 2)
    with pytest.raises(ValueError):
        _mat(torch.zeros(3, dtype=torch.float32))


def test_sigmoid_parameters_match_oracle(oracle):
    """CreateSigmoid's widths and weights (host code of the C ABI, no GPU)
    equal the oracle's restatement bit for bit; invalid center counts raise."""
    cases = [(np.array([-3.0, 3.0, 0.0, -1.0, 1.0, -2.0, 0.0, 2.0]), 1.5, 0),
             (np.array([-2.0, 2.5, 1.0, -1.5, 0.3, 0.9]), 0.7, 1),
             (np.array([-3.0, 3.0]), 2.0, 0), (np.array([-3.0, 3.0, 0.2]), 2.0, 1),
             (np.linspace(-4, 4, 2 + 15), 1.2, 0)]
    for c, edge, st in cases:
        S = M.Sigmoid1d.FromCenters(c, edge, M.SigmoidSumSizeType(st))
        ref = oracle.sigmoid_from_centers(c, edge, st)
        for a, b in zip((S.centers, S.widths, S.weights, S.startInds), ref):
            np.testing.assert_array_equal(a, b)
        assert S.GetOrder() == len(ref[3]) + 3
    with pytest.raises(ValueError, match="Linear"):
        M.Sigmoid1d.FromCenters(np.zeros(6))  # 2 + 4 centers: not 2 + n(n+1)/2
    with pytest.raises(ValueError):
        M.Sigmoid1d.FromCenters(np.zeros(1))
    with pytest.raises(ValueError, match="maximum"):
        M.Sigmoid1d.FromCenters(np.zeros(2 + 10 * 11 // 2))  # ten sigmoid terms: order 13 > 12


def test_sigmoid_start_indices():
    # Sigmoid1d::ConstructStartInds (MParT/Sigmoid.h:95-130)
    assert M.Sigmoid1d(np.zeros(8), np.ones(8), np.ones(8)).startInds.tolist() == [2, 3, 5]
    assert M.Sigmoid1d(np.zeros(5), np.ones(5), np.ones(5),
                       sumType=M.SigmoidSumSizeType.Constant).startInds.tolist() == [2, 3, 4]
    with pytest.raises(ValueError):
        M.Sigmoid1d(np.zeros(6), np.ones(6), np.ones(6))


def test_torch_wrappers_are_exported_lazily():
    """The package exports the torch wrappers and mpart_has_torch as the
    reference's does, importing torch only when they are asked for."""
    import mpart_gb300 as M
    assert M.mpart_has_torch is True
    assert M.TorchParameterizedFunctionBase.__name__ == "TorchParameterizedFunctionBase"
    assert M.TorchConditionalMapBase.__name__ == "TorchConditionalMapBase"


def test_initialize_and_concurrency():
    """MParT's Initialize(dict) and Concurrency() exist with their meanings:
    options accepted, and the number of threads the execution space runs."""
    import os

    import mpart_gb300 as M
    assert M.Initialize({"kokkos-num-threads": 4}) is None
    n = M.Concurrency()
    assert isinstance(n, int) and n >= 1
    import torch
    if not torch.cuda.is_available():
        assert n == (os.cpu_count() or 1)
