"""Multi-indices, limiters and adaptive multi-index sets (mpart_gb300.multiindex)
against the reference's own MultiIndexSet (src/MultiIndices/MultiIndexSet.cpp,
compiled unchanged into oracle/_ref): every query of the Python binding's
MultiIndexSet, on sets built term by term, by CreateTotalOrder /
CreateTensorProduct and by SetLimiter, under every limiter kind."""
import numpy as np
import pytest

import mpart_gb300 as M


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference checkout not present")
    return ref


def _limiter(kind, dim, u, w):
    L = M
    return {0: lambda: L.NoneLim(), 1: lambda: L.TotalOrder(u[0]), 2: lambda: L.Dimension(u[0], u[1]),
            3: lambda: L.Anisotropic(w[:dim], w[dim]), 4: lambda: L.MaxDegree(u[0], dim),
            5: lambda: L.Separable(), 6: lambda: L.NonzeroDiag(),
            7: lambda: L.And(L.TotalOrder(u[0]), L.MaxDegree(u[1], dim)),
            8: lambda: L.Or(L.Dimension(u[0], u[1]), L.TotalOrder(u[2])),
            9: lambda: L.Xor(L.TotalOrder(u[0]), L.NonzeroDiag())}[kind]()


def _report(dim, terms, mode, order, kind, u, w):
    """The reference driver's report, from the restatement."""
    lim = _limiter(kind, dim, u, w)
    lines = []
    if mode == 1:
        s = M.MultiIndexSet.CreateTotalOrder(dim, order, lim)
    elif mode == 2:
        s = M.MultiIndexSet.CreateTensorProduct(dim, order, lim)
    elif mode == 0:
        s = M.MultiIndexSet(dim, lim)
        for t in terms:
            s += t
    else:
        s = M.MultiIndexSet(dim)
        for t in terms:
            s += t
        try:
            s.SetLimiter(lim)
        except ValueError:
            lines.append("setlimiter rejected")

    def ms(v):
        return ";".join(str(m) for m in v)

    def ints(v):
        return ",".join(str(int(x)) for x in v)

    def terms_of(x):
        return ms([x.IndexToMulti(k) for k in range(x.Size())])

    lines.append(f"size {s.Size()}")
    lines.append(f"terms {terms_of(s)}")
    lines.append(f"maxorders {ints(s.MaxOrders())}")
    lines.append(f"frontier {ints(s.Frontier())}")
    lines.append(f"strict {ints(s.StrictFrontier())}")
    margin = s.Margin()
    lines.append(f"margin {ms(margin)}")
    lines.append(f"rmargin {ms(s.ReducedMargin())}")
    for d in range(dim):
        lines.append(f"rmargin_dim{d} {ms(s.ReducedMarginDim(d))}")
    lines.append(f"expandable {ints(s.IsExpandable(k) for k in range(s.Size()))}")
    lines.append(f"nforward {ints(s.NumForward(k) for k in range(s.Size()))}")
    lines.append(f"nactiveforward {ints(s.NumActiveForward(k) for k in range(s.Size()))}")
    lines.append(f"nzdiag {ints(s.NonzeroDiagonalEntries())}")
    lines.append(f"margin_admissible {ints(s.IsAdmissible(m) for m in margin)}")
    c = s.DeepCopy()
    ix = c.Expand()
    lines.append(f"expand {ints(ix)} | {terms_of(c)}")
    for k in range(s.Size()):
        lines.append(f"expand{k} {ints(s.DeepCopy().Expand(k))}")
    c = s.DeepCopy()
    added = c.union(M.MultiIndexSet.CreateTotalOrder(dim, 1))
    lines.append(f"union {added} | {terms_of(c)}")
    return "\n".join(lines) + "\n"


def _random_terms(rng, dim, n):
    """Terms as a user might list them: mostly a grown downward-closed set, with
    a few gaps and repeats."""
    terms = [tuple([0] * dim)]
    for _ in range(n):
        base = terms[rng.integers(len(terms))]
        d = rng.integers(dim)
        t = list(base)
        t[d] += int(rng.integers(1, 3))
        terms.append(tuple(t))
    order = rng.permutation(len(terms))
    return [terms[i] for i in order[:max(1, len(terms) - int(rng.integers(0, 2)))]]


def _spec(rng, dim):
    kind = int(rng.integers(0, 10))
    u = [int(rng.integers(1, 4)), int(rng.integers(0, 3)) if kind == 8 else int(rng.integers(1, 3)),
         int(rng.integers(1, 4))]
    if kind in (2, 8):
        u[0] = int(rng.integers(0, dim))
        u[1] = int(rng.integers(1, dim - u[0] + 1))
    w = list(rng.uniform(0.2, 1.0, dim)) + [float(rng.uniform(0.05, 0.5))]
    return kind, u, w


def test_multi_index_set_matches_reference():
    ref = _ref()
    rng = np.random.default_rng(11)
    n_cases = 0
    for dim in (1, 2, 3, 4):
        for mode in (0, 1, 2, 3):
            for _ in range(12):
                kind, u, w = _spec(rng, dim)
                terms = _random_terms(rng, dim, int(rng.integers(1, 7)))
                order = int(rng.integers(0, 4)) if mode != 2 else int(rng.integers(0, 3))
                want = ref.mset_report(dim, terms, mode, order, kind, u, w)
                got = _report(dim, terms, mode, order, kind, u, w)
                assert got == want, (dim, mode, kind, u, w, terms, order)
                n_cases += 1
    assert n_cases == 192


def test_multi_index_basics():
    m = M.MultiIndex([0, 2, 1])
    assert (m.tolist(), m.sum(), m.max(), m.count_nonzero(), len(m)) == ([0, 2, 1], 3, 2, 2, 3)
    assert m.HasNonzeroEnd() and not M.MultiIndex([1, 0]).HasNonzeroEnd()
    assert str(m) == "0 2 1"
    assert M.MultiIndex(3, 2).tolist() == [2, 2, 2] and M.MultiIndex(2).tolist() == [0, 0]
    m[0] = 4
    assert m.tolist() == [4, 2, 1]
    # MultiIndex::operator<: length, total order, maximum, then entries
    terms = [M.MultiIndex(t) for t in ([1, 1], [0, 2], [2, 0], [0, 0], [1, 0], [0, 1], [3], [0, 0, 0])]
    assert [t.tolist() for t in sorted(terms)] == [[3], [0, 0], [0, 1], [1, 0], [1, 1], [0, 2], [2, 0], [0, 0, 0]]


def test_sets_from_arrays_and_fix():
    s = M.MultiIndexSet(np.array([[0, 1], [2, 0], [0, 1]]))
    assert s.Size() == 2 and len(s) == 2 and s.MaxOrders() == [2, 1]
    assert s.MultiToIndex([2, 0]) == 1 and s.MultiToIndex([1, 1]) == -1
    f = s.fix(True)
    assert f.Size() == 2 and [list(f.IndexToMulti(i)) for i in range(2)] == [[0, 1], [2, 0]]
    assert list(f.MaxDegrees()) == [2, 1] and f.MultiToIndex([2, 0]) == 1 and f.NonzeroDiagonalEntries() == [0]
    with pytest.raises(IndexError):
        s[5]
    assert [m.tolist() for m in s] == [[0, 1], [2, 0]]
    with pytest.raises(ValueError, match="epsilon"):
        M.Anisotropic([0.5, 0.5], 1.5)
    t = M.MultiIndexSet.CreateTotalOrder(2, 2)
    with pytest.raises(ValueError, match="not valid with the new limiter"):
        t.SetLimiter(M.TotalOrder(1))
    with pytest.raises(ValueError, match="length must be positive"):
        M.MultiIndexSet.CreateTotalOrder(0, 2)
    with pytest.raises(TypeError):
        M.MultiIndexSet()


def test_fixed_set_constructors_of_the_binding():
    """FixedMultiIndexSet(dim, orders) with every term's orders in turn,
    (dim, nzStarts, nzDims, nzOrders) positionally, and (dim, maxOrder)
    (bindings/python/src/MultiIndex.cpp:195-222)."""
    a = M.FixedMultiIndexSet(2, np.array([0, 0, 1, 0, 0, 2, 1, 1], np.uint32))
    assert [list(a.IndexToMulti(i)) for i in range(a.Size())] == [[0, 0], [1, 0], [0, 2], [1, 1]]
    b = M.FixedMultiIndexSet(3, np.array([0, 0, 1, 2]), np.array([0, 1]), np.array([2, 1]))
    assert [list(b.IndexToMulti(i)) for i in range(b.Size())] == [[0, 0, 0], [2, 0, 0], [0, 1, 0]]
    assert M.FixedMultiIndexSet(2, 2).Size() == 6
    assert M.MultiIndexSet.CreateTotalOrder(2, 2).fix(True).ToBytes() == M.FixedMultiIndexSet(2, 2).ToBytes()


def test_multi_index_order_and_diagonal_entries_match_reference():
    """MultiIndex::operator< (length, total order, maximum, then entries) and
    FixedMultiIndexSet::NonzeroDiagonalEntries against the reference's."""
    ref = _ref()
    rng = np.random.default_rng(3)
    for dim in (1, 2, 3, 5):
        terms = [tuple(int(v) for v in rng.integers(0, 3, dim)) for _ in range(25)]
        less, nzdiag = ref.multi_order(terms)
        ms = [M.MultiIndex(t) for t in terms]
        got = np.array([[a < b for b in ms] for a in ms])
        np.testing.assert_array_equal(got, less)
        s = M.MultiIndexSet(dim)
        for t in terms:
            s += t
        assert s.fix(True).NonzeroDiagonalEntries() == nzdiag
        assert s.NonzeroDiagonalEntries() == nzdiag
