"""mpgb_fused_fwd_adj_noalloc: the fused forward + coefficient adjoint for
callers that may not allocate device memory while they run (code running
inside a custom allocator or memory pool, allocation-free real-time loops,
hosts that manage the whole device heap).  Its scratch is a fixed array in
device memory instead of cudaMalloc'd buffers, so it must give the same
results as mpgb_fused_fwd_adj -- checked here through the C ABI on two calls
in a row, within the parity tolerance of the other GPU tests (1e-10 relative,
floored at 1e-3 of the largest entry for the summed gradient).

The results are also checked against the CPU oracle on a small triangular
map, and a call on a freshly created map must change neither the device's
free memory nor torch's caching allocator (the modules of the kernels it
launches are loaded by a warm-up call first, as CUDA's lazy module loading
does for any library's first launch of a kernel).

This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(a, b, rtol=1e-10, floor=1e-6):
    scale = np.max(np.abs(b))
    ok = (a == b) | (np.abs(a - b) <= rtol * np.maximum(np.abs(b), floor * scale))
    assert ok.all(), f"{np.count_nonzero(~ok)} entries differ, max |diff| {np.max(np.abs(a - b))}"


def _noalloc(M, tm, x, sens, ev, ld, cg):
    from mpart_gb300 import _capi, _mat, _ptr, _stream_of
    lib = _capi.load()
    rc = lib.mpgb_fused_fwd_adj_noalloc(tm._h, _mat(x), _mat(sens), _mat(None), 1.0, _mat(ev), _mat(ld), _ptr(cg),
                                        _stream_of(x))
    _capi.check(rc)


def _opts(M):
    return M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis)


def test_noalloc_matches_fused_on_two_calls(gpu):
    import torch
    M = gpu
    comp = M.CreateComponent(M.FixedMultiIndexSet(8, 4), _opts(M))
    comp.SetCoeffs(np.random.default_rng(0).normal(0.0, 0.05, comp.numCoeffs))
    n = 5000
    dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda")
    x = dev(np.random.default_rng(1).standard_normal((8, n)))
    sens = dev(np.random.default_rng(2).standard_normal((1, n)))
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device="cuda")
    ev0, ld0, cg0 = z(1, n), z(n), z(comp.numCoeffs)
    comp.FusedForwardAdjointImpl(x, sens=sens, logdet_sens_scale=1.0, out_eval=ev0, out_logdet=ld0, coeff_grad=cg0)
    for _ in range(2):
        ev, ld, cg = z(1, n), z(n), z(comp.numCoeffs)
        _noalloc(M, comp, x, sens, ev, ld, cg)
        torch.cuda.synchronize()
        _close(ev.cpu().numpy(), ev0.cpu().numpy())
        _close(ld.cpu().numpy(), ld0.cpu().numpy())
        _close(cg.cpu().numpy(), cg0.cpu().numpy(), floor=1e-3)


def test_noalloc_triangular_map_and_size_limit(gpu):
    import torch
    M = gpu
    tm = M.CreateTriangular(2, 2, 3, _opts(M))
    tm.SetCoeffs(np.random.default_rng(0).normal(0.0, 0.1, tm.numCoeffs))
    n = 3000
    dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda")
    x = dev(np.random.default_rng(1).standard_normal((2, n)))
    sens = dev(np.random.default_rng(2).standard_normal((2, n)))
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device="cuda")
    ev0, cg0 = z(2, n), z(tm.numCoeffs)
    tm.FusedForwardAdjointImpl(x, sens=sens, logdet_sens_scale=1.0, out_eval=ev0, coeff_grad=cg0)
    for _ in range(2):
        ev, cg = z(2, n), z(tm.numCoeffs)
        _noalloc(M, tm, x, sens, ev, None, cg)
        torch.cuda.synchronize()
        _close(ev.cpu().numpy(), ev0.cpu().numpy())
        _close(cg.cpu().numpy(), cg0.cpu().numpy(), floor=1e-3)
    # A call whose scratch would exceed the fixed array is refused, not run.
    big = M.CreateComponent(M.FixedMultiIndexSet(16, 6), _opts(M))
    xb = z(16, 100000)
    with pytest.raises(ValueError, match="bytes of scratch"):
        _noalloc(M, big, xb, z(1, 100000), None, None, z(big.numCoeffs))


def test_noalloc_matches_oracle_and_allocates_nothing(gpu, oracle):
    import torch
    M, O = gpu, oracle
    coef = np.random.default_rng(0).normal(0.0, 0.1, 14)
    n = 2000
    xh = np.random.default_rng(1).standard_normal((2, n))
    sh = np.random.default_rng(2).standard_normal((2, n))
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device="cuda")
    # Warm-up on one map: the kernels' modules are loaded by their first launch.
    warm = M.CreateTriangular(2, 2, 3, _opts(M))
    warm.SetCoeffs(coef)
    x, sens = dev(xh), dev(sh)
    _noalloc(M, warm, x, sens, z(2, n), None, z(warm.numCoeffs))
    # A fresh map and fresh outputs, all created before the measurement.
    tm = M.CreateTriangular(2, 2, 3, _opts(M))
    tm.SetCoeffs(coef)
    ev, cg = z(2, n), z(tm.numCoeffs)
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    for _ in range(2):
        _noalloc(M, tm, x, sens, ev, None, cg)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert torch.cuda.memory_reserved() == reserved0
        om = O.OracleTriangularMap(2, 2, 3, normalize=True, posfunc=O.POS_SOFTPLUS, abs_tol=1e-6, rel_tol=1e-6,
                                   max_sub=30)
        _close(ev.cpu().numpy(), om.evaluate(coef, xh))
        ref = om.coeff_grad(coef, xh, sh).sum(axis=1) + om.logdet_coeff_grad(coef, xh).sum(axis=1)
        _close(cg.cpu().numpy(), ref, floor=1e-3)
