"""Batch of independent maps in one persistent launch (mpgb_batch_*): every
map's values, log-determinants and reduced coefficient adjoint must equal
those of the map's own fused call, before and after autotuning, within
1e-10 relative (floored at 1e-3 of the largest entry for the gradients, whose
partial sums follow the tiles per item), and the oracle's; repeated batch
calls are bitwise identical."""
import numpy as np
import pytest

from test_gpu_parity import H, T, assert_parity, opts, oracle_tri

pytestmark = pytest.mark.gpu

# (input dim, output dim, total order, points)
SPECS = [(2, 2, 3, 1500), (3, 3, 2, 4000), (5, 2, 4, 700), (4, 4, 3, 2500), (6, 1, 2, 3000), (3, 3, 5, 1200),
         (2, 1, 2, 0), (7, 3, 3, 900)]


def _setup(M):
    rng = np.random.default_rng(5)
    maps, pts, sens = [], [], []
    for d, o, order, n in SPECS:
        tm = M.CreateTriangular(d, o, order, opts(M))
        tm.SetCoeffs(rng.normal(0.0, 0.05, tm.numCoeffs))
        maps.append(tm)
        pts.append(T(rng.standard_normal((d, n))))
        sens.append(T(rng.standard_normal((o, n))))
    return maps, pts, sens


def _zeros(shape):
    import torch
    return torch.zeros(shape, dtype=torch.float64, device="cuda")


def _run_batch(B, maps, pts, sens):
    ev = [_zeros((m.outputDim, p.shape[1])) for m, p in zip(maps, pts)]
    ld = [_zeros((p.shape[1],)) for p in pts]
    cg = [_zeros((m.numCoeffs,)) for m in maps]
    B.FusedForwardAdjoint(pts, sens, 1.0, ev, ld, cg)
    return [H(x) for x in ev], [H(x) for x in ld], [H(x) for x in cg]


def _run_single(maps, pts, sens):
    out = ([], [], [])
    for m, p, s in zip(maps, pts, sens):
        ev, ld, cg = _zeros((m.outputDim, p.shape[1])), _zeros((p.shape[1],)), _zeros((m.numCoeffs,))
        m.FusedForwardAdjointImpl(p, sens=s, logdet_sens_scale=1.0, out_eval=ev, out_logdet=ld, coeff_grad=cg)
        for k, x in enumerate((ev, ld, cg)):
            out[k].append(H(x))
    return out


def test_batch_matches_single_map_calls(gpu):
    M = gpu
    maps, pts, sens = _setup(M)
    B = M.MapBatch(maps)
    ev, ld, cg = _run_batch(B, maps, pts, sens)
    ev1, ld1, cg1 = _run_single(maps, pts, sens)
    for m in range(len(maps)):
        assert_parity(ev[m], ev1[m], what=f"batch Evaluate, map {m}")
        assert_parity(ld[m], ld1[m], what=f"batch LogDeterminant, map {m}")
        assert_parity(cg[m], cg1[m], floor=1e-3, what=f"batch coefficient adjoint, map {m}")
    assert not cg[6].any()  # no points: zero gradient
    # the same after autotuning (and repeated calls are bitwise identical)
    ms = B.Autotune(pts, sens, 1.0, reps=1)
    assert ms > 0
    tpb, tiles = B.Tuning()
    assert tpb in (64, 128)
    assert set(tiles) == {(d, p) for d, p in _buckets(maps)}
    assert all(t in (1, 2, 4, 8, 16) for t in tiles.values())
    a = _run_batch(B, maps, pts, sens)
    b = _run_batch(B, maps, pts, sens)
    for m in range(len(maps)):
        np.testing.assert_array_equal(a[0][m], ev[m])
        np.testing.assert_array_equal(a[1][m], ld[m])
        assert_parity(a[2][m], cg1[m], floor=1e-3, what=f"tuned batch coefficient adjoint, map {m}")
        np.testing.assert_array_equal(a[2][m], b[2][m])


def _buckets(maps):
    out = set()
    for d, o, order, n in SPECS:
        for k in range(o):
            out.add((d - o + k + 1, order))
    return out


def test_batch_matches_oracle(gpu, oracle):
    M, O = gpu, oracle
    maps, pts, sens = _setup(M)
    B = M.MapBatch(maps)
    ev, ld, cg = _run_batch(B, maps, pts, sens)
    for m in (0, 2, 5):
        d, o, order, n = SPECS[m]
        om = oracle_tri(O, d, o, order)
        coef = np.asarray(maps[m].CoeffMap())
        x, s = H(pts[m]), H(sens[m])
        assert_parity(ev[m], om.evaluate(coef, x), what=f"batch Evaluate, map {m}")
        assert_parity(ld[m], om.logdet(coef, x), what=f"batch LogDeterminant, map {m}")
        ref = om.coeff_grad(coef, x, s).sum(axis=1) + om.logdet_coeff_grad(coef, x).sum(axis=1)
        assert_parity(cg[m], ref, floor=1e-3, what=f"batch coefficient adjoint, map {m}")


def test_batch_rejects_host_memory_and_bad_shapes(gpu):
    M = gpu
    maps, pts, sens = _setup(M)
    B = M.MapBatch(maps[:2])
    with pytest.raises(ValueError, match="not device memory"):
        B.FusedForwardAdjoint([H(pts[0]), pts[1]], sens[:2], 1.0)
    with pytest.raises(ValueError, match="rows"):
        B.FusedForwardAdjoint([pts[1], pts[0]], None, 1.0)
    with pytest.raises(ValueError):
        B.SetTuning(96, {})
