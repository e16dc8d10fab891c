"""Archives: the reference's cereal binary layouts for the coefficient archive
(ParameterizedFunctionBase.Serialize / DeserializeMap), MapOptions and
FixedMultiIndexSet, byte for byte, and the whole-map archive behind
ToBytes / FromBytes / pickle.  The expected bytes are assembled here from the
layout itself -- cereal's binary archive writes values back to back in native
(little-endian) order, strings as a uint64 length and their bytes, and Kokkos
views as (label, uint32 extent, elements) (MParT/Utilities/Serialization.h) --
and, where the reference checkout is present, taken from the reference's own
save functions (oracle/_ref with the cereal stand-in)."""
import pickle
import struct

import numpy as np
import pytest


def _str(s):
    b = s.encode()
    return struct.pack("<Q", len(b)) + b


def _view(label, arr, fmt):
    arr = list(arr)
    return _str(label) + struct.pack("<I", len(arr)) + struct.pack("<%d%s" % (len(arr), fmt), *arr)


def _options_bytes(basis, pos, quad, abs_tol, rel_tol, max_sub, min_sub, pts, cont, norm, nugget,
                   lb=-np.inf, ub=np.inf):
    # MParT/MapOptions.h:126-130
    return struct.pack("<iddiiddIIIBBd", basis, lb, ub, pos, quad, abs_tol, rel_tol, max_sub, min_sub, pts,
                       int(cont), int(norm), nugget)


@pytest.fixture(scope="module")
def M():
    import mpart_gb300
    mpart_gb300.load()
    return mpart_gb300


def test_map_options_archive_layout_and_round_trip(M, tmp_path):
    o = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes.Exp,
                     quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=1e-7, quadRelTol=2e-7, quadMaxSub=25,
                     quadMinSub=1, quadPts=9, contDeriv=True, basisNorm=False, nugget=0.25)
    want = _options_bytes(2, 0, 2, 1e-7, 2e-7, 25, 1, 9, True, False, 0.25)
    assert o.ToBytes() == want
    o.Serialize(tmp_path / "opts.bin")
    assert (tmp_path / "opts.bin").read_bytes() == want
    back = M.MapOptions().Deserialize(tmp_path / "opts.bin")
    assert back == o
    assert pickle.loads(pickle.dumps(o)) == o
    # defaults (AdaptiveSimpson, SoftPlus, ProbabilistHermite, maxSub 30, quadPts 5)
    assert M.MapOptions().ToBytes() == _options_bytes(0, 1, 1, 1e-6, 1e-6, 30, 0, 5, True, True, 0.0)


def test_map_options_archive_rejects_what_this_path_cannot_honour(M):
    with pytest.raises(ValueError, match="basisLB"):
        M.MapOptions.FromBytes(_options_bytes(0, 1, 2, 1e-6, 1e-6, 30, 0, 5, True, True, 0.0, lb=-3.0, ub=3.0))
    with pytest.raises(ValueError, match="enum"):
        M.MapOptions.FromBytes(_options_bytes(7, 1, 2, 1e-6, 1e-6, 30, 0, 5, True, True, 0.0))
    with pytest.raises(ValueError, match="truncated"):
        M.MapOptions.FromBytes(_options_bytes(0, 1, 2, 1e-6, 1e-6, 30, 0, 5, True, True, 0.0)[:-3])


def test_multi_index_set_archive_layout_and_round_trip(M, tmp_path):
    ms = M.FixedMultiIndexSet(3, 2)
    # total order 2 in 3 dims: maxDegrees (2, 2, 2)
    want = (struct.pack("<IB", 3, 1) + _view("nzStarts", ms.nzStarts, "I") + _view("nzDims", ms.nzDims, "I") +
            _view("nzOrders", ms.nzOrders, "I") + _view("Maximum degrees", [2, 2, 2], "I"))
    assert ms.ToBytes() == want
    ms.Serialize(tmp_path / "mset.bin")
    back = M.FixedMultiIndexSet(1, 0).Deserialize(tmp_path / "mset.bin")
    for a in ("nzStarts", "nzDims", "nzOrders"):
        np.testing.assert_array_equal(getattr(back, a), getattr(ms, a))
    assert back.Length() == 3
    p = pickle.loads(pickle.dumps(ms))
    assert [list(p.IndexToMulti(i)) for i in range(p.Size())] == [list(ms.IndexToMulti(i)) for i in range(ms.Size())]


def test_multi_index_set_archive_uncompressed_form(M):
    # isCompressed = false stores every dimension of every term; zeros are dropped on load.
    # The reference leaves the last term start unset (0).
    multis = [[0, 0], [1, 0], [0, 2], [1, 1]]
    starts = [2 * k for k in range(len(multis))] + [0]
    dims = [d for _ in multis for d in (0, 1)]
    orders = [o for m in multis for o in m]
    data = (struct.pack("<IB", 2, 0) + _view("nzStarts", starts, "I") + _view("nzDims", dims, "I") +
            _view("nzOrders", orders, "I") + _view("Maximum degrees", [1, 2], "I"))
    ms = M.FixedMultiIndexSet.FromBytes(data)
    assert [list(ms.IndexToMulti(i)) for i in range(ms.Size())] == multis
    np.testing.assert_array_equal(ms.nzStarts, [0, 0, 1, 2, 4])


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference checkout not present")
    return ref


@pytest.mark.parametrize("basis,pos,quad", [("ProbabilistHermite", "SoftPlus", "AdaptiveClenshawCurtis"),
                                            ("HermiteFunctions", "Exp", "AdaptiveSimpson"),
                                            ("ProbabilistHermite", "Exp", "ClenshawCurtis")])
@pytest.mark.parametrize("norm,cont", [(True, True), (False, False)])
def test_map_options_archive_is_the_references(M, basis, pos, quad, norm, cont):
    """Byte for byte against MapOptions::serialize run by the reference
    (oracle/_ref with the cereal stand-in), and read back."""
    ref = _ref()
    kw = dict(abs_tol=3e-7, rel_tol=2e-6, max_sub=17, min_sub=2, quad_pts=9, nugget=0.125)
    want = ref.options_bytes(basis=basis, normalize=norm, posfunc=pos, quad=quad, cont_deriv=cont, **kw)
    q = {"AdaptiveClenshawCurtis": M.QuadTypes.AdaptiveClenshawCurtis, "ClenshawCurtis": M.QuadTypes.ClenshawCurtis,
         "AdaptiveSimpson": M.QuadTypes.AdaptiveSimpson}[quad]
    o = M.MapOptions(basisType=getattr(M.BasisTypes, basis), posFuncType=getattr(M.PosFuncTypes, pos), quadType=q,
                     quadAbsTol=3e-7, quadRelTol=2e-6, quadMaxSub=17, quadMinSub=2, quadPts=9, contDeriv=cont,
                     basisNorm=norm, nugget=0.125)
    assert o.ToBytes() == want
    assert M.MapOptions.FromBytes(want) == o


def test_multi_index_set_archive_is_the_references(M, oracle):
    """Byte for byte against FixedMultiIndexSet::save run by the reference, for
    total-order sets and a set with unsorted nonzeros; the reference's
    uncompressed form reads back as the same set."""
    ref = _ref()
    for dim, order in [(1, 0), (1, 4), (3, 2), (5, 3)]:
        s, d, o = oracle.total_order(dim, order)
        ms = M.FixedMultiIndexSet(dim, order)
        assert ms.ToBytes() == ref.mset_bytes(dim, s, d, o), (dim, order)
    # unsorted nonzeros in a term after the first: the reference's insertion
    # sort (src/MultiIndices/FixedMultiIndexSet.cpp:74-93) steps its unsigned
    # index below zero when the first term's nonzeros are unsorted
    starts, dims, orders = [0, 1, 3, 4, 7], [1, 2, 0, 1, 3, 0, 1], [2, 1, 3, 2, 1, 2, 4]
    ms = M.FixedMultiIndexSet(4, nzStarts=np.array(starts, np.uint32), nzDims=np.array(dims, np.uint32),
                              nzOrders=np.array(orders, np.uint32))
    assert ms.ToBytes() == ref.mset_bytes(4, starts, dims, orders)
    multis = [[0, 0, 0], [1, 0, 2], [0, 3, 0], [2, 1, 1]]
    back = M.FixedMultiIndexSet.FromBytes(ref.mset_bytes(3, dense=multis))
    assert [list(back.IndexToMulti(i)) for i in range(back.Size())] == multis


def test_coefficient_archive_is_the_references(M, tmp_path):
    """DeserializeMap reads the reference's Serialize archive of a map with
    coefficients, and of one without (an empty view)."""
    ref = _ref()
    m = ref.RefMap(3, 2, 2)
    c = np.random.default_rng(4).normal(size=m.num_coeffs)
    m.set_coeffs(c)
    (tmp_path / "map.bin").write_bytes(m.coeff_archive())
    i, o, coeffs = M.DeserializeMap(tmp_path / "map.bin")
    assert (i, o) == (3, 2)
    np.testing.assert_array_equal(coeffs, c)
    comps = [ref.RefMap(d, starts=s, dims=dd, orders=oo) for d, (s, dd, oo) in
             ((1, ([0, 0, 1], [0], [1])), (2, ([0, 0, 1, 2], [0, 1], [1, 1])))]
    for comp in comps:
        comp.set_coeffs(np.ones(comp.num_coeffs))
    moved = ref.RefMap.triangular_from(comps)
    data = moved.coeff_archive()
    assert b"coeffs" in data  # the moved view's label
    (tmp_path / "moved.bin").write_bytes(data)
    i, o, coeffs = M.DeserializeMap(tmp_path / "moved.bin")
    assert (i, o) == (2, 2) and np.all(coeffs == 1.0)


def test_deserialize_map_reads_the_coefficient_archive(M, tmp_path):
    c = np.random.default_rng(0).normal(size=7)
    data = struct.pack("<III", 3, 2, 7) + _view("ParameterizedFunctionBase<MemorySpace> Coefficients", c, "d")
    (tmp_path / "map.bin").write_bytes(data)
    i, o, coeffs = M.DeserializeMap(tmp_path / "map.bin")
    assert (i, o) == (3, 2)
    np.testing.assert_array_equal(coeffs, c)
    (tmp_path / "bad.bin").write_bytes(data[:-5])
    with pytest.raises(ValueError):
        M.DeserializeMap(tmp_path / "bad.bin")


@pytest.mark.gpu
def test_map_serialize_matches_reference_layout(gpu, tmp_path):
    M = gpu
    tm = M.CreateTriangular(3, 2, 2, M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis))
    c = np.random.default_rng(1).normal(0.0, 0.1, tm.numCoeffs)
    tm.SetCoeffs(c)
    tm.Serialize(tmp_path / "map.bin")
    want = struct.pack("<III", 3, 2, tm.numCoeffs) + _view("ParameterizedFunctionBase<MemorySpace> Coefficients", c,
                                                            "d")
    assert (tmp_path / "map.bin").read_bytes() == want
    i, o, coeffs = M.DeserializeMap(tmp_path / "map.bin")
    assert (i, o) == (3, 2)
    np.testing.assert_array_equal(coeffs, c)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["component", "triangular"])
def test_map_bytes_and_pickle_rebuild_the_same_map(gpu, kind):
    import torch
    M = gpu
    opts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes.Exp,
                        quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=1e-7, quadRelTol=1e-7)
    if kind == "component":
        m = M.CreateComponent(M.FixedMultiIndexSet(4, 3), opts)
    else:
        m = M.CreateTriangular(4, 3, 3, opts)
    m.SetCoeffs(np.random.default_rng(2).normal(0.0, 0.05, m.numCoeffs))
    x = torch.as_tensor(np.random.default_rng(3).standard_normal((4, 500)), device="cuda")
    for back in (M.FromBytes(m.ToBytes()), pickle.loads(pickle.dumps(m))):
        assert type(back) is type(m)
        assert (back.inputDim, back.outputDim, back.numCoeffs) == (m.inputDim, m.outputDim, m.numCoeffs)
        np.testing.assert_array_equal(np.asarray(back.CoeffMap()), np.asarray(m.CoeffMap()))
        np.testing.assert_array_equal(back.Evaluate(x).cpu().numpy(), m.Evaluate(x).cpu().numpy())
        np.testing.assert_array_equal(back.LogDeterminant(x).cpu().numpy(), m.LogDeterminant(x).cpu().numpy())
