"""The C-ABI library loads and exports every symbol include/mpart_gb300.h
declares; argument checking works without a GPU (no compute calls here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from mpart_gb300 import _build, _capi
    _build.build()
    return _capi.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "mpart_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mpgb_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/mpart_gb300.h but not exported"


def test_python_signatures_cover_header(lib):
    from mpart_gb300 import _capi
    assert set(_declared()) == set(_capi.SIGNATURES)


def test_version_and_defaults(lib):
    from mpart_gb300 import _capi
    assert b"sm_103a" in lib.mpgb_version()
    o = _capi.mpgb_map_options()
    assert lib.mpgb_map_options_default(C.byref(o)) == 0
    # MParT/MapOptions.h defaults
    assert (o.basis_type, o.pos_func_type, o.quad_type) == (0, 1, 1)
    assert (o.quad_abs_tol, o.quad_rel_tol, o.quad_max_sub, o.quad_min_sub, o.quad_pts) == (1e-6, 1e-6, 30, 0, 5)
    assert o.cont_deriv == 1 and o.basis_norm == 1 and o.nugget == 0.0


def test_argument_errors_without_gpu(lib):
    from mpart_gb300 import _capi
    assert lib.mpgb_map_options_default(None) == _capi.MPGB_ERR_INVALID_ARGUMENT
    assert b"null" in lib.mpgb_last_error()
    assert lib.mpgb_create_triangular(2, 2, 3, None, None) == _capi.MPGB_ERR_INVALID_ARGUMENT
    assert lib.mpgb_map_dims(None, None, None, None) == _capi.MPGB_ERR_INVALID_ARGUMENT
    m = _capi.mpgb_matrix(None, 0, 0, 0, 0)
    assert lib.mpgb_evaluate(None, m, m, None) == _capi.MPGB_ERR_INVALID_ARGUMENT
