"""ORACLE -- test infrastructure only.

ctypes front end of ``oracle/_ref/libmpart_ref.so``: MParT's own map classes
(``src/ParameterizedFunctionBase.cpp``, ``src/ConditionalMapBase.cpp``,
``src/TriangularMap.cpp``, the component factory registrations
``src/MapFactoryImpl{4..9}.cpp`` and ``src/MultiIndices/*.cpp``, with the
headers they include), compiled unchanged from the reference checkout by
``oracle/ref.mk`` against the Kokkos / Eigen / cereal (save side) stand-ins in
``oracle/ref_shim/``, with the reference's archive support on.

It exists only where the reference checkout does (the development host):
``available()`` says whether it can be built.  The tests use it to pin the
oracle's restatement, and the golden fixtures, to the reference itself.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_ref", "libmpart_ref.so")
REF_DIR = os.environ.get("MPGB_REFERENCE_DIR", "/root/reference")
_lib = None

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint)

# MapOptions enums (MParT/MapOptions.h)
BASIS_PROB_HERMITE, BASIS_HERMITE_FUNCTIONS = 0, 2
POS_EXP, POS_SOFTPLUS = 0, 1
QUAD_CLENSHAW_CURTIS, QUAD_ADAPTIVE_SIMPSON, QUAD_ACC = 0, 1, 2


def available() -> bool:
    """The reference checkout is present (so the library can be built here)."""
    return os.path.isdir(os.path.join(REF_DIR, "MParT")) and os.path.isdir(os.path.join(REF_DIR, "src"))


def build():
    subprocess.run(["make", "-s", "-j8", "-f", os.path.join(_HERE, "ref.mk"), f"REF={REF_DIR}"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        opt = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_uint, C.c_double,
               C.c_int]
        L.ref_triangular.restype = C.c_void_p
        L.ref_triangular.argtypes = [C.c_uint, C.c_uint, C.c_uint] + opt
        L.ref_component.restype = C.c_void_p
        L.ref_component.argtypes = [C.c_uint, C.c_uint, _up, _up, _up] + opt
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_last_error.restype = C.c_char_p
        L.ref_sizes.argtypes = [C.c_void_p, _up, _up, _up]
        L.ref_set_coeffs.argtypes = [C.c_void_p, _dp, C.c_long]
        for f in ("ref_evaluate", "ref_logdet", "ref_logdet_coeff_grad", "ref_logdet_input_grad"):
            getattr(L, f).argtypes = [C.c_void_p, _dp, C.c_long, _dp]
        for f in ("ref_coeff_grad", "ref_gradient"):
            getattr(L, f).argtypes = [C.c_void_p, _dp, _dp, C.c_long, _dp]
        L.ref_inverse.argtypes = [C.c_void_p, _dp, C.c_long, _dp, C.c_long, C.c_double, C.c_double, _dp]
        L.ref_mset.argtypes = [C.c_uint, C.c_uint, _up, C.c_int, C.c_uint, _up, _up, _up, _up]
        L.ref_sigmoid.restype = C.c_void_p
        L.ref_sigmoid.argtypes = [C.c_uint, C.c_uint, _up, _up, _up, _dp, _dp, _dp, C.c_uint, C.c_int, C.c_int]
        L.ref_direct_inverse.argtypes = [C.c_void_p, _dp, C.c_long, _dp, C.c_long, _dp]
        L.ref_to_bytes.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]
        L.ref_wrap_coeffs.argtypes = [C.c_void_p, _dp, C.c_long]
        out = [C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]
        L.ref_options_bytes.argtypes = opt + out
        L.ref_mset_bytes.argtypes = [C.c_uint, C.c_uint, _up, _up, _up] + out
        L.ref_coeff_archive.argtypes = [C.c_void_p] + out
        L.ref_mset_report.argtypes = [C.c_uint, C.c_uint, _up, C.c_int, C.c_uint, C.c_int, _up, _dp] + out
        L.ref_multi_order.argtypes = [C.c_uint, C.c_uint, _up, C.c_void_p, _up, _up]
        L.ref_triangular_from.restype = C.c_void_p
        L.ref_triangular_from.argtypes = [C.POINTER(C.c_void_p), C.c_uint]
        _lib = L
    return _lib


def _bytes(call):
    n = C.c_size_t()
    if call(None, 0, C.byref(n)) != 0:
        raise RuntimeError(lib().ref_last_error().decode())
    buf = C.create_string_buffer(max(1, n.value))
    if call(buf, n.value, C.byref(n)) != 0:
        raise RuntimeError(lib().ref_last_error().decode())
    return buf.raw[:n.value]


def options_bytes(basis="ProbabilistHermite", normalize=True, posfunc="SoftPlus", quad="AdaptiveClenshawCurtis",
                  abs_tol=1e-6, rel_tol=1e-6, max_sub=30, min_sub=0, quad_pts=5, nugget=0.0, cont_deriv=True):
    """MapOptions.Serialize's archive (MapOptions::serialize)."""
    b = {"ProbabilistHermite": BASIS_PROB_HERMITE, "HermiteFunctions": BASIS_HERMITE_FUNCTIONS}[basis]
    p = {"Exp": POS_EXP, "SoftPlus": POS_SOFTPLUS}[posfunc]
    q = {"AdaptiveSimpson": QUAD_ADAPTIVE_SIMPSON, "ClenshawCurtis": QUAD_CLENSHAW_CURTIS,
         "AdaptiveClenshawCurtis": QUAD_ACC}[quad]
    return _bytes(lambda buf, cap, n: lib().ref_options_bytes(b, int(normalize), p, q, abs_tol, rel_tol, max_sub,
                                                              min_sub, quad_pts, nugget, int(cont_deriv), buf,
                                                              cap, n))


def mset_bytes(dim, starts=None, dims=None, orders=None, dense=None):
    """FixedMultiIndexSet.Serialize's archive of the compressed set (starts,
    dims, orders) or of the uncompressed one (dense: terms x dim orders)."""
    if dense is not None:
        d = np.ascontiguousarray(dense, np.uint32)
        return _bytes(lambda buf, cap, n: lib().ref_mset_bytes(dim, d.shape[0], None, None, d.ctypes.data_as(_up),
                                                               buf, cap, n))
    s = np.ascontiguousarray(starts, np.uint32)
    dd = np.ascontiguousarray(dims if len(dims) else [0], np.uint32)
    o = np.ascontiguousarray(orders if len(orders) else [0], np.uint32)
    return _bytes(lambda buf, cap, n: lib().ref_mset_bytes(dim, len(s) - 1, s.ctypes.data_as(_up),
                                                           dd.ctypes.data_as(_up), o.ctypes.data_as(_up), buf,
                                                           cap, n))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class RefMap:
    """A map of the reference: MapFactory::CreateTriangular(inputDim, outputDim,
    totalOrder, options), or (``starts`` given) MapFactory::CreateComponent on
    a compressed multi-index set.  Options as MapOptions (basisNorm true,
    quadPts 5, AdaptiveClenshawCurtis unless given)."""

    def __init__(self, input_dim, output_dim=None, order=None, basis="ProbabilistHermite", normalize=True,
                 posfunc="SoftPlus", quad="AdaptiveClenshawCurtis", abs_tol=1e-6, rel_tol=1e-6, max_sub=30,
                 min_sub=0, quad_pts=5, nugget=0.0, cont_deriv=True, starts=None, dims=None, orders=None):
        b = {"ProbabilistHermite": BASIS_PROB_HERMITE, "HermiteFunctions": BASIS_HERMITE_FUNCTIONS}[basis]
        p = {"Exp": POS_EXP, "SoftPlus": POS_SOFTPLUS}[posfunc]
        q = {"AdaptiveSimpson": QUAD_ADAPTIVE_SIMPSON, "ClenshawCurtis": QUAD_CLENSHAW_CURTIS,
             "AdaptiveClenshawCurtis": QUAD_ACC}[quad]
        opt = (b, int(normalize), p, q, abs_tol, rel_tol, max_sub, min_sub, quad_pts, nugget, int(cont_deriv))
        L = lib()
        if starts is None:
            self._h = L.ref_triangular(input_dim, output_dim, order, *opt)
        else:
            s = np.ascontiguousarray(starts, np.uint32)
            d = np.ascontiguousarray(dims if len(dims) else [0], np.uint32)
            o = np.ascontiguousarray(orders if len(orders) else [0], np.uint32)
            self._keep = (s, d, o)
            self._h = L.ref_component(input_dim, len(s) - 1, s.ctypes.data_as(_up), d.ctypes.data_as(_up),
                                      o.ctypes.data_as(_up), *opt)
        if not self._h:
            raise RuntimeError(L.ref_last_error().decode())
        a, b_, c = C.c_uint(), C.c_uint(), C.c_uint()
        L.ref_sizes(self._h, C.byref(a), C.byref(b_), C.byref(c))
        self.input_dim, self.output_dim, self.num_coeffs = a.value, b_.value, c.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ref_free(self._h)
            self._h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().ref_last_error().decode())

    @classmethod
    def triangular_from(cls, comps):
        """TriangularMap(components, moveCoeffs=true) over RefMap components
        (each with coefficients set); they must outlive the result."""
        L = lib()
        arr = (C.c_void_p * len(comps))(*[c._h for c in comps])
        self = cls.__new__(cls)
        self._comps = list(comps)
        self._h = L.ref_triangular_from(arr, len(comps))
        if not self._h:
            raise RuntimeError(L.ref_last_error().decode())
        a, b_, c = C.c_uint(), C.c_uint(), C.c_uint()
        L.ref_sizes(self._h, C.byref(a), C.byref(b_), C.byref(c))
        self.input_dim, self.output_dim, self.num_coeffs = a.value, b_.value, c.value
        return self

    def coeff_archive(self) -> bytes:
        """ParameterizedFunctionBase.Serialize's archive: inputDim, outputDim,
        numCoeffs and the coefficient view."""
        return _bytes(lambda buf, cap, n: lib().ref_coeff_archive(self._h, buf, cap, n))

    def to_bytes(self) -> bytes:
        """The reference's ToBytes / pickle archive of this map
        (ParameterizedFunctionBase::Save through the cereal stand-in)."""
        n = C.c_size_t()
        self._check(lib().ref_to_bytes(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._check(lib().ref_to_bytes(self._h, buf, n.value, C.byref(n)))
        return buf.raw[:n.value]

    def wrap_coeffs(self, coeffs):
        """WrapCoeffs on this array's memory (kept alive by the map object)."""
        self._wrapped = _c(coeffs).copy()
        assert self._wrapped.size == self.num_coeffs
        self._check(lib().ref_wrap_coeffs(self._h, self._wrapped.ctypes.data_as(_dp), self._wrapped.size))

    def set_coeffs(self, coeffs):
        c = _c(coeffs)
        assert c.size == self.num_coeffs
        self._check(lib().ref_set_coeffs(self._h, c.ctypes.data_as(_dp), c.size))

    def evaluate(self, pts):
        x = _c(pts)
        out = np.zeros((self.output_dim, x.shape[1]))
        self._check(lib().ref_evaluate(self._h, x.ctypes.data_as(_dp), x.shape[1], out.ctypes.data_as(_dp)))
        return out

    def logdet(self, pts):
        x = _c(pts)
        out = np.zeros(x.shape[1])
        self._check(lib().ref_logdet(self._h, x.ctypes.data_as(_dp), x.shape[1], out.ctypes.data_as(_dp)))
        return out

    def coeff_grad(self, pts, sens):
        x, s = _c(pts), _c(np.reshape(sens, (self.output_dim, -1)))
        out = np.zeros((self.num_coeffs, x.shape[1]))
        self._check(lib().ref_coeff_grad(self._h, x.ctypes.data_as(_dp), s.ctypes.data_as(_dp), x.shape[1],
                                         out.ctypes.data_as(_dp)))
        return out

    def gradient(self, pts, sens):
        x, s = _c(pts), _c(np.reshape(sens, (self.output_dim, -1)))
        out = np.zeros((self.input_dim, x.shape[1]))
        self._check(lib().ref_gradient(self._h, x.ctypes.data_as(_dp), s.ctypes.data_as(_dp), x.shape[1],
                                       out.ctypes.data_as(_dp)))
        return out

    def logdet_coeff_grad(self, pts):
        x = _c(pts)
        out = np.zeros((self.num_coeffs, x.shape[1]))
        self._check(lib().ref_logdet_coeff_grad(self._h, x.ctypes.data_as(_dp), x.shape[1], out.ctypes.data_as(_dp)))
        return out

    def logdet_input_grad(self, pts):
        x = _c(pts)
        out = np.zeros((self.input_dim, x.shape[1]))
        self._check(lib().ref_logdet_input_grad(self._h, x.ctypes.data_as(_dp), x.shape[1], out.ctypes.data_as(_dp)))
        return out

    def inverse(self, x1, r, xtol=1e-6, ytol=1e-6):
        """TriangularMap::InverseImpl with the components' xtol / ytol options;
        x1 has up to inputDim rows (the rows past inputDim - outputDim are the
        initial guesses, zero when absent)."""
        r = _c(np.reshape(r, (self.output_dim, -1)))
        n = r.shape[1]
        x1 = _c(x1) if len(x1) else np.zeros((0, n))
        out = np.zeros((self.output_dim, n))
        self._check(lib().ref_inverse(self._h, x1.ctypes.data_as(_dp), x1.shape[0], r.ctypes.data_as(_dp), n,
                                      xtol, ytol, out.ctypes.data_as(_dp)))
        return out


class RefSigmoid(RefMap):
    """A sigmoid expansion of the reference, built as
    MapFactory::CreateSigmoidComponent builds one (Sigmoid1d with SoftPlus
    edges, HermiteFunction off the diagonal, RectifiedMultivariateExpansion,
    or UnivariateExpansion for one input) from the given centers, widths and
    weights and compressed multi-index set."""

    def __init__(self, dim, starts, dims, orders, centers, widths, weights, sum_type="Linear", posfunc="SoftPlus"):
        s = np.ascontiguousarray(starts, np.uint32)
        d = np.ascontiguousarray(dims if len(dims) else [0], np.uint32)
        o = np.ascontiguousarray(orders if len(orders) else [0], np.uint32)
        c, w, wt = _c(centers), _c(widths), _c(weights)
        self._keep = (s, d, o, c, w, wt)
        L = lib()
        self._h = L.ref_sigmoid(dim, len(s) - 1, s.ctypes.data_as(_up), d.ctypes.data_as(_up), o.ctypes.data_as(_up),
                                c.ctypes.data_as(_dp), w.ctypes.data_as(_dp), wt.ctypes.data_as(_dp), c.size,
                                {"Linear": 0, "Constant": 1}[sum_type], {"Exp": POS_EXP, "SoftPlus": POS_SOFTPLUS}[posfunc])
        if not self._h:
            raise RuntimeError(L.ref_last_error().decode())
        a, b_, cc = C.c_uint(), C.c_uint(), C.c_uint()
        L.ref_sizes(self._h, C.byref(a), C.byref(b_), C.byref(cc))
        self.input_dim, self.output_dim, self.num_coeffs = a.value, b_.value, cc.value

    def inverse(self, x1, r):
        r = _c(np.reshape(r, (self.output_dim, -1)))
        n = r.shape[1]
        x1 = _c(x1) if len(x1) else np.zeros((0, n))
        out = np.zeros((self.output_dim, n))
        self._check(lib().ref_direct_inverse(self._h, x1.ctypes.data_as(_dp), x1.shape[0], r.ctypes.data_as(_dp), n,
                                             out.ctypes.data_as(_dp)))
        return out


def _mset_call(terms, mode):
    t = np.ascontiguousarray(np.asarray(terms, dtype=np.uint32).reshape(len(terms), -1))
    dim = t.shape[1]
    cap = 4 * (len(terms) + 1) * (dim + 1) + 64
    out_t = np.zeros((cap, dim), dtype=np.uint32)
    idx = np.zeros(cap, dtype=np.uint32)
    nt, no = C.c_uint(), C.c_uint()
    L = lib()
    rc = L.ref_mset(dim, len(terms), t.ctypes.data_as(_up), mode, cap, out_t.ctypes.data_as(_up), C.byref(nt),
                    idx.ctypes.data_as(_up), C.byref(no))
    if rc != 0:
        raise RuntimeError(L.ref_last_error().decode())
    return out_t, nt.value, idx, no.value


def mset_report(dim, terms=(), mode=0, order=0, lim_kind=0, u=(0, 0, 0), w=()):
    """The text report of the reference's MultiIndexSet (ref_mset_report in
    oracle/ref_driver.cpp): mode 0 += of terms under the limiter, 1
    CreateTotalOrder(dim, order), 2 CreateTensorProduct(dim, order), 3 += of
    terms then SetLimiter; limiter kinds as documented there."""
    t = np.ascontiguousarray(np.asarray(terms, dtype=np.uint32).reshape(-1, dim) if len(terms) else
                             np.zeros((1, dim), np.uint32))
    uu = np.ascontiguousarray(list(u) + [0] * (3 - len(u)), np.uint32)
    ww = np.ascontiguousarray(list(w) if len(w) else [0.0], np.float64)
    n = len(terms)
    return _bytes(lambda buf, cap, sz: lib().ref_mset_report(dim, n, t.ctypes.data_as(_up), mode, order, lim_kind,
                                                             uu.ctypes.data_as(_up), ww.ctypes.data_as(_dp), buf,
                                                             cap, sz)).decode()


def multi_order(terms):
    """(less, nzdiag): less[i, j] = terms[i] < terms[j] by MultiIndex::operator<,
    and NonzeroDiagonalEntries of the FixedMultiIndexSet of the distinct terms
    added in order (MultiIndexSet += then Fix)."""
    t = np.ascontiguousarray(terms, dtype=np.uint32)
    n, dim = t.shape
    less = np.zeros((n, n), np.uint8)
    nz = np.zeros(max(1, n), np.uint32)
    cnt = C.c_uint()
    if lib().ref_multi_order(dim, n, t.ctypes.data_as(_up), less.ctypes.data_as(C.c_void_p), nz.ctypes.data_as(_up),
                             C.byref(cnt)) != 0:
        raise RuntimeError(lib().ref_last_error().decode())
    return less.astype(bool), [int(v) for v in nz[:cnt.value]]


def mset_reduced_margin(terms):
    """MultiIndexSet::ReducedMargin of the set built by += of terms in order."""
    out_t, _, _, no = _mset_call(terms, 0)
    return [tuple(int(v) for v in out_t[k]) for k in range(no)]


def mset_expand(terms):
    """MultiIndexSet::Expand of the set built by += of terms in order: (the
    returned indices, the set's terms afterwards)."""
    out_t, nt, idx, no = _mset_call(terms, 1)
    return [int(v) for v in idx[:no]], [tuple(int(v) for v in out_t[k]) for k in range(nt)]
