"""ORACLE -- test infrastructure only.

Python front end of the CPU restatement in ``oracle/mpart_oracle.cpp`` (loaded
with ctypes).  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import this module; the product never does.

The component routines are the C++ restatement of ``MParT/MonotoneComponent.h``.
This file adds the composition layers that are plain loops in the reference:

* ``OracleTriangularMap`` -- ``src/TriangularMap.cpp:99-310`` (component loop,
  log-determinant accumulation, coefficient row blocks, sequential inverse),
* ``fast_gaussian_reverse_kl`` -- ``src/MapObjective.cpp:93-234``,
* ``kl_objective`` -- ``src/MapObjective.cpp:54-91`` with the identity-covariance
  ``GaussianSamplerDensity`` (``src/Distributions/GaussianSamplerDensity.cpp:21-88``)
  through ``PullbackDensity`` (``src/Distributions/PullbackDensity.cpp:13-37``).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# MPGB_ORACLE_BUILD=timing selects the timing build (default floating-point
# contraction) for CPU-baseline timings; every parity check uses the default,
# strict build.
_LIB_NAME = "liboracle_timing.so" if os.environ.get("MPGB_ORACLE_BUILD") == "timing" else "liboracle.so"
_LIB_PATH = os.path.join(_HERE, "_build", _LIB_NAME)
_lib = None

BASIS_PROB_HERMITE = 0
BASIS_HERMITE_FUNCTIONS = 2
POS_EXP = 0
POS_SOFTPLUS = 1
QUAD_CC, QUAD_SIMPSON, QUAD_ACC = 0, 1, 2  # MapOptions::quadType

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint)
_lp = C.POINTER(C.c_long)
_ip = C.POINTER(C.c_int)


def build():
    """Compile the oracle with its Makefile (no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_total_order_size.argtypes = [C.c_uint, C.c_uint, _up, _up]
        L.orc_total_order_fill.argtypes = [C.c_uint, C.c_uint, _up, _up, _up]
        L.orc_component_new.restype = C.c_void_p
        L.orc_component_new.argtypes = [C.c_uint, C.c_uint, _up, _up, _up, C.c_int, C.c_int, C.c_int,
                                        C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_int]
        L.orc_component_free.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_cache_size.argtypes = [C.c_void_p]
        L.orc_cache_size.restype = C.c_uint
        pts_sig = [C.c_void_p, _dp, _dp, C.c_long, C.c_long, C.c_long]
        L.orc_evaluate.argtypes = pts_sig + [_dp, _lp, _ip]
        L.orc_cont_derivative.argtypes = pts_sig + [_dp]
        L.orc_logdet.argtypes = pts_sig + [_dp]
        L.orc_coeff_jacobian.argtypes = pts_sig + [_dp, _dp, C.c_long, C.c_long, _ip]
        L.orc_coeff_grad.argtypes = pts_sig + [_dp, C.c_long, _dp, C.c_long, C.c_long]
        L.orc_input_jacobian.argtypes = pts_sig + [_dp, _dp, C.c_long, C.c_long]
        L.orc_gradient.argtypes = pts_sig + [_dp, C.c_long, _dp, C.c_long, C.c_long]
        L.orc_cont_mixed_jacobian.argtypes = pts_sig + [_dp, C.c_long, C.c_long]
        L.orc_logdet_coeff_grad.argtypes = pts_sig + [_dp, C.c_long, C.c_long]
        L.orc_cont_mixed_input_jacobian.argtypes = pts_sig + [_dp, C.c_long, C.c_long]
        L.orc_logdet_input_grad.argtypes = pts_sig + [_dp, C.c_long, C.c_long]
        L.orc_inverse.argtypes = [C.c_void_p, _dp, _dp, C.c_long, C.c_long, C.c_long, _dp, C.c_long, C.c_long,
                                  C.c_double, C.c_double, _dp, C.c_long, _ip]
        L.orc_basis.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint, C.c_double, _dp, _dp, _dp]
        L.orc_posfunc.argtypes = [C.c_int, C.c_int, C.c_double]
        L.orc_posfunc.restype = C.c_double
        L.orc_cc_rule.argtypes = [C.c_uint, _dp, _dp]
        L.orc_acc_test.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_uint, C.c_double,
                                   C.c_double, _dp, _lp]
        L.orc_set_cont_deriv.argtypes = [C.c_void_p, C.c_int]
        L.orc_discrete_derivative.argtypes = [C.c_void_p, _dp, _dp, C.c_long, C.c_long, C.c_long, _dp]
        L.orc_quad_test.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_uint,
                                    C.c_double, C.c_double, _dp, _lp]
        L.orc_rootfind_test.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _ip]
        L.orc_rootfind_test.restype = C.c_double
        L.orc_findbracket_test.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double]
        L.orc_integrand.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, _dp]
        L.orc_sigmoid_from_centers.argtypes = [C.c_uint, _dp, C.c_double, C.c_int, _dp, _dp, _dp, _up, _up]
        L.orc_sigmoid_eval.argtypes = [C.c_uint, _dp, _dp, _dp, C.c_uint, _up, C.c_int, C.c_uint, C.c_double, _dp,
                                       _dp, _dp]
        L.orc_rect_new.restype = C.c_void_p
        L.orc_rect_new.argtypes = [C.c_uint, C.c_uint, _up, _up, _up, C.c_int, C.c_int, C.c_int, C.c_uint, _dp, _dp,
                                   _dp, C.c_uint, _up, C.c_int]
        L.orc_rect_free.argtypes = [C.c_void_p]
        L.orc_rect_evaluate.argtypes = pts_sig + [_dp]
        L.orc_rect_gradient.argtypes = pts_sig + [_dp, _dp, C.c_long, C.c_long]
        L.orc_rect_coeff_grad.argtypes = pts_sig + [_dp, _dp]
        L.orc_rect_logdet.argtypes = pts_sig + [_dp]
        L.orc_rect_logdet_input_grad.argtypes = pts_sig + [_dp, C.c_long, C.c_long]
        L.orc_rect_logdet_coeff_grad.argtypes = pts_sig + [_dp]
        L.orc_rect_inverse.argtypes = [C.c_void_p, _dp, _dp, C.c_long, C.c_long, C.c_long, _dp, C.c_long, C.c_long,
                                       C.c_double, C.c_double, _dp, C.c_long, _ip]
        _lib = L
    return _lib


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def total_order(dim: int, order: int):
    """Compressed total-order multi-index set (FixedMultiIndexSet.cpp:208-233)."""
    L = lib()
    nt, nnz = C.c_uint(), C.c_uint()
    L.orc_total_order_size(dim, order, C.byref(nt), C.byref(nnz))
    starts = np.zeros(nt.value + 1, np.uint32)
    dims = np.zeros(max(nnz.value, 1), np.uint32)
    orders = np.zeros(max(nnz.value, 1), np.uint32)
    L.orc_total_order_fill(dim, order, starts.ctypes.data_as(_up), dims.ctypes.data_as(_up),
                           orders.ctypes.data_as(_up))
    return starts, dims[:nnz.value], orders[:nnz.value]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def total_order_min(dim: int, order: int, min_order: int):
    """FixedMultiIndexSet(dim, order, minOrder): the total-order set without the
    terms of total order below minOrder, in the same order."""
    s, d, o = total_order(dim, order)
    keep = [t for t in range(len(s) - 1) if int(o[s[t]:s[t + 1]].sum()) >= min_order]
    starts, dims, orders = [0], [], []
    for t in keep:
        dims.extend(d[s[t]:s[t + 1]])
        orders.extend(o[s[t]:s[t + 1]])
        starts.append(len(dims))
    return np.array(starts, np.uint32), np.array(dims, np.uint32), np.array(orders, np.uint32)


def cartesian(a, a_len, b):
    """FixedMultiIndexSet::Cartesian (src/MultiIndices/FixedMultiIndexSet.cpp:356-397):
    terms (i, j) with i of the first set outermost; dims of the second set
    shifted by the first set's length."""
    sa, da, oa = a
    sb, db, ob = b
    starts, dims, orders = [0], [], []
    for i in range(len(sa) - 1):
        for j in range(len(sb) - 1):
            dims.extend(da[sa[i]:sa[i + 1]])
            orders.extend(oa[sa[i]:sa[i + 1]])
            dims.extend(int(x) + a_len for x in db[sb[j]:sb[j + 1]])
            orders.extend(ob[sb[j]:sb[j + 1]])
            starts.append(len(dims))
    return np.array(starts, np.uint32), np.array(dims, np.uint32), np.array(orders, np.uint32)


def concatenate(a, b):
    """FixedMultiIndexSet::Concatenate (FixedMultiIndexSet.cpp:400-431)."""
    sa, da, oa = a
    sb, db, ob = b
    starts = np.concatenate([np.asarray(sa[:-1], np.int64), len(da) + np.asarray(sb, np.int64)])
    return (starts.astype(np.uint32), np.concatenate([da, db]).astype(np.uint32),
            np.concatenate([oa, ob]).astype(np.uint32))


def sigmoid_mset(input_dim, off_order, cross_order, num_sigmoids):
    """Multi-index set of CreateSigmoidExpansionTemplate (src/MapFactory.cpp:284-318):
    [leading total order x {0}] followed by [leading cross order x {1..n+3}];
    for one input the total order n+3 set."""
    if input_dim == 1:
        return total_order(1, num_sigmoids + 3)
    m1 = cartesian(total_order(input_dim - 1, off_order), input_dim - 1, total_order(1, 0))
    m2 = cartesian(total_order(input_dim - 1, cross_order), input_dim - 1,
                   total_order_min(1, num_sigmoids + 3, 1))
    return concatenate(m1, m2)


SUM_LINEAR, SUM_CONSTANT = 0, 1  # SigmoidSumSizeType


def sigmoid_from_centers(centers, edge_shape=1.5, sum_type=SUM_LINEAR):
    """CreateSigmoid (src/MapFactory.cpp:181-254): (centers, widths, weights, starts)."""
    c = _f64(centers)
    n = len(c)
    oc, ow, owt = np.zeros(n), np.zeros(n), np.zeros(n)
    st = np.zeros(max(n, 1), np.uint32)
    ns = C.c_uint()
    if lib().orc_sigmoid_from_centers(n, _ptr(c), edge_shape, sum_type, _ptr(oc), _ptr(ow), _ptr(owt),
                                      st.ctypes.data_as(_up), C.byref(ns)) != 0:
        raise ValueError("invalid sigmoid centers")
    return oc, ow, owt, st[:ns.value].copy()


def sigmoid_eval(params, x, max_order, which=2):
    """Sigmoid1d EvaluateAll / EvaluateDerivatives / EvaluateSecondDerivatives
    at x: (values, first, second derivatives), each max_order + 1 long."""
    c, w, wt, st = (_f64(params[0]), _f64(params[1]), _f64(params[2]), np.ascontiguousarray(params[3], np.uint32))
    v, d1, d2 = np.zeros(max_order + 1), np.zeros(max_order + 1), np.zeros(max_order + 1)
    st1 = st if len(st) else np.zeros(1, np.uint32)
    rc = lib().orc_sigmoid_eval(len(c), _ptr(c), _ptr(w), _ptr(wt), len(st), st1.ctypes.data_as(_up), which,
                                max_order, float(x), _ptr(v), _ptr(d1), _ptr(d2))
    if rc < 0:
        raise ValueError("invalid sigmoid parameters or order")
    return v, d1, d2


class OracleSigmoidComponent:
    """RectifiedMultivariateExpansion with HermiteFunctions in the leading
    inputs, a Sigmoid1d in the last input and the positive bijector as
    rectifier (MParT/RectifiedMultivariateExpansion.h), or, for one input,
    UnivariateExpansion<Sigmoid1d> (MParT/UnivariateExpansion.h).  params =
    (centers, widths, weights, starts); params None puts the leading basis
    in the last input too (the reference's unrectified test case)."""

    def __init__(self, dim, starts, dims, orders, params, posfunc=POS_SOFTPLUS, rectify=True,
                 basis=BASIS_HERMITE_FUNCTIONS, normalize=True):
        self.dim = int(dim)
        self.starts = np.ascontiguousarray(starts, np.uint32)
        self.dims = np.ascontiguousarray(dims, np.uint32)
        self.orders = np.ascontiguousarray(orders, np.uint32)
        self.num_terms = self.num_coeffs = len(self.starts) - 1
        self.input_dim, self.output_dim = self.dim, 1
        self.nugget = 0.0
        self.univariate = self.dim == 1
        d = self.dims if len(self.dims) else np.zeros(1, np.uint32)
        o = self.orders if len(self.orders) else np.zeros(1, np.uint32)
        if params is None:
            c = w = wt = np.zeros(1)
            st = np.zeros(1, np.uint32)
            nc = ns = 0
        else:
            c, w, wt = _f64(params[0]), _f64(params[1]), _f64(params[2])
            st = np.ascontiguousarray(params[3], np.uint32)
            nc, ns = len(c), len(st)
            if ns == 0:
                st = np.zeros(1, np.uint32)
        self._keep = (c, w, wt, st)
        self._h = lib().orc_rect_new(self.dim, self.num_terms, self.starts.ctypes.data_as(_up),
                                     d.ctypes.data_as(_up), o.ctypes.data_as(_up), basis, int(normalize),
                                     posfunc if rectify else -1, nc, _ptr(c), _ptr(w), _ptr(wt), ns,
                                     st.ctypes.data_as(_up), int(self.univariate))
        if not self._h:
            raise ValueError("invalid sigmoid expansion")

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_rect_free(self._h)
            self._h = None

    def _pts(self, pts):
        pts = np.asarray(pts, dtype=np.float64)
        assert pts.ndim == 2 and pts.shape[0] >= self.dim
        rs, cs = (s // 8 for s in pts.strides)
        return pts, pts.shape[1], rs, cs

    def evaluate(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros(N)
        lib().orc_rect_evaluate(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out))
        return out

    def gradient(self, coeffs, pts, sens):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        sens = _f64(np.asarray(sens).reshape(-1))
        out = np.zeros((self.dim, N))
        lib().orc_rect_gradient(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(sens), _ptr(out), N, 1)
        return out

    def coeff_grad(self, coeffs, pts, sens):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        sens = _f64(np.asarray(sens).reshape(-1))
        out = np.zeros((self.num_terms, N))
        lib().orc_rect_coeff_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(sens), _ptr(out))
        return out

    def logdet(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros(N)
        lib().orc_rect_logdet(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out))
        return out

    def cont_derivative(self, coeffs, pts):
        with np.errstate(over="ignore"):
            return np.exp(self.logdet(coeffs, pts))

    def logdet_input_grad(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros((self.dim, N))
        lib().orc_rect_logdet_input_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out), N, 1)
        return out

    def logdet_coeff_grad(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros((self.num_terms, N))
        lib().orc_rect_logdet_coeff_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out))
        return out

    def inverse(self, coeffs, xs, ys, xtol=1e-6, ytol=1e-6, return_info=False):
        """xs: D x (1 or N) with the initial guess in its last row; ys: N."""
        coeffs = _f64(coeffs)
        xs = np.asarray(xs, dtype=np.float64)
        rs, cs = (s // 8 for s in xs.strides)
        ys = _f64(np.asarray(ys).reshape(-1))
        N = ys.shape[0]
        out = np.zeros(N)
        info = np.zeros(N, np.int32)
        if lib().orc_rect_inverse(self._h, _ptr(coeffs), _ptr(xs), xs.shape[1], rs, cs, _ptr(ys), 1, N, xtol, ytol,
                                  _ptr(out), 1, info.ctypes.data_as(_ip)) != 0:
            raise ValueError("invalid argument sizes given to inverse")
        return (out, info) if return_info else out


def sigmoid_triangular(input_dim, output_dim, order, centers, edge_shape=1.5, sum_type=SUM_LINEAR,
                       posfunc=POS_SOFTPLUS):
    """CreateSigmoidTriangular (src/MapFactory.cpp:389-407): component i has
    input dimension input_dim - output_dim + i + 1 and the centers of column i."""
    comps = []
    centers = np.asarray(centers, dtype=np.float64)
    for i in range(output_dim):
        d = input_dim - output_dim + i + 1
        prm = sigmoid_from_centers(centers[:, i], edge_shape, sum_type)
        nsig = len(prm[3])
        s, dd, o = sigmoid_mset(d, order, order, nsig)
        comps.append(OracleSigmoidComponent(d, s, dd, o, prm, posfunc))
    return OracleTriangularMap(input_dim, output_dim, order, components=comps)


class OracleComponent:
    """One MonotoneComponent (ProbabilistHermite or HermiteFunctions basis,
    SoftPlus or Exp rectifier, AdaptiveClenshawCurtis quadrature)."""

    def __init__(self, dim, starts, dims, orders, basis=BASIS_PROB_HERMITE, normalize=True,
                 posfunc=POS_SOFTPLUS, abs_tol=1e-6, rel_tol=1e-6, max_sub=30, min_sub=0, quad_pts=5,
                 nugget=0.0, quad_type=QUAD_ACC, cont_deriv=True):
        self.dim = int(dim)
        self.starts = np.ascontiguousarray(starts, np.uint32)
        self.dims = np.ascontiguousarray(dims, np.uint32)
        self.orders = np.ascontiguousarray(orders, np.uint32)
        self.num_terms = len(self.starts) - 1
        self.num_coeffs = self.num_terms
        self.input_dim = self.dim
        self.output_dim = 1
        self.nugget = float(nugget)
        self.abs_tol, self.rel_tol = float(abs_tol), float(rel_tol)
        L = lib()
        d = self.dims if len(self.dims) else np.zeros(1, np.uint32)
        o = self.orders if len(self.orders) else np.zeros(1, np.uint32)
        self._h = L.orc_component_new(self.dim, self.num_terms, self.starts.ctypes.data_as(_up),
                                      d.ctypes.data_as(_up), o.ctypes.data_as(_up), basis, int(normalize),
                                      posfunc, abs_tol, rel_tol, max_sub, min_sub, quad_pts, nugget, quad_type)
        self.cont_deriv = bool(cont_deriv)
        L.orc_set_cont_deriv(self._h, int(self.cont_deriv))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_component_free(self._h)
            self._h = None

    @property
    def cache_size(self):
        return lib().orc_cache_size(self._h)

    # All point matrices are D x N (one column per point), any strides.
    def _pts(self, pts):
        pts = np.asarray(pts, dtype=np.float64)
        assert pts.ndim == 2 and pts.shape[0] >= self.dim
        rs, cs = (s // 8 for s in pts.strides)
        return pts, pts.shape[1], rs, cs

    def evaluate(self, coeffs, pts, return_evals=False):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros(N)
        nev = np.zeros(N, np.int64)
        st = np.zeros(N, np.int32)
        lib().orc_evaluate(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out), nev.ctypes.data_as(_lp),
                           st.ctypes.data_as(_ip))
        if return_evals:
            return out, nev, st
        return out

    def cont_derivative(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros(N)
        lib().orc_cont_derivative(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out))
        return out

    def logdet(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros(N)
        lib().orc_logdet(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out))
        return out

    def coeff_jacobian(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        ev = np.zeros(N)
        jac = np.zeros((self.num_terms, N))
        st = np.zeros(N, np.int32)
        lib().orc_coeff_jacobian(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(ev), _ptr(jac), N, 1,
                                 st.ctypes.data_as(_ip))
        return ev, jac

    def coeff_grad(self, coeffs, pts, sens):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        sens = _f64(np.asarray(sens).reshape(-1))
        out = np.zeros((self.num_terms, N))
        lib().orc_coeff_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(sens), 1, _ptr(out), N, 1)
        return out

    def input_jacobian(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        ev = np.zeros(N)
        jac = np.zeros((self.dim, N))
        lib().orc_input_jacobian(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(ev), _ptr(jac), N, 1)
        return ev, jac

    def gradient(self, coeffs, pts, sens):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        sens = _f64(np.asarray(sens).reshape(-1))
        out = np.zeros((self.dim, N))
        lib().orc_gradient(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(sens), 1, _ptr(out), N, 1)
        return out

    def logdet_coeff_grad(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros((self.num_terms, N))
        lib().orc_logdet_coeff_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out), N, 1)
        return out

    def logdet_input_grad(self, coeffs, pts):
        coeffs = _f64(coeffs)
        pts, N, rs, cs = self._pts(pts)
        out = np.zeros((self.dim, N))
        if lib().orc_logdet_input_grad(self._h, _ptr(coeffs), _ptr(pts), N, rs, cs, _ptr(out), N, 1) != 0:
            raise ValueError("Discrete derivative version is not implemented yet (To Do)")
        return out

    def inverse(self, coeffs, xs, ys, xtol=1e-6, ytol=1e-6, return_info=False):
        """xs: D x (1 or N) with the initial guess in its last row; ys: N."""
        coeffs = _f64(coeffs)
        xs = np.asarray(xs, dtype=np.float64)
        rs, cs = (s // 8 for s in xs.strides)
        ys = _f64(np.asarray(ys).reshape(-1))
        N = ys.shape[0]
        out = np.zeros(N)
        info = np.zeros(N, np.int32)
        rc = lib().orc_inverse(self._h, _ptr(coeffs), _ptr(xs), xs.shape[1], rs, cs, _ptr(ys), 1, N, xtol, ytol,
                               _ptr(out), 1, info.ctypes.data_as(_ip))
        if rc != 0:
            raise ValueError("invalid argument sizes given to inverse")
        return (out, info) if return_info else out

    def integrand(self, coeffs, pt, t, mode):
        coeffs = _f64(coeffs)
        pt = _f64(pt)
        n = {0: 1, 1: 2, 2: 1 + self.num_terms, 3: 1 + self.dim}[mode]
        out = np.zeros(n)
        lib().orc_integrand(self._h, _ptr(coeffs), _ptr(pt), float(t), mode, _ptr(out))
        return out


class OracleTriangularMap:
    """Component loop of src/TriangularMap.cpp for the factory's triangular
    layout: component i has input dimension i + extra + 1 (src/MapFactory.cpp:105-124)
    and its coefficients are the i-th block of one vector (:65-97)."""

    def __init__(self, input_dim, output_dim, order, basis=BASIS_PROB_HERMITE, normalize=True,
                 posfunc=POS_SOFTPLUS, abs_tol=1e-6, rel_tol=1e-6, max_sub=30, min_sub=0, quad_pts=5, nugget=0.0,
                 components=None, quad_type=QUAD_ACC, cont_deriv=True):
        if components is None:
            extra = input_dim - output_dim
            components = []
            for i in range(output_dim):
                s, d, o = total_order(i + extra + 1, int(order))
                components.append(OracleComponent(i + extra + 1, s, d, o, basis, normalize, posfunc, abs_tol,
                                                  rel_tol, max_sub, min_sub, quad_pts, nugget, quad_type, cont_deriv))
        self.comps = components
        self.input_dim = components[-1].input_dim
        self.output_dim = len(components)
        self.num_coeffs = sum(c.num_coeffs for c in components)
        self.offsets = np.cumsum([0] + [c.num_coeffs for c in components])

    def split(self, coeffs):
        return [np.asarray(coeffs[self.offsets[i]:self.offsets[i + 1]]) for i in range(len(self.comps))]

    def evaluate(self, coeffs, pts):
        cs = self.split(coeffs)
        return np.stack([c.evaluate(cs[i], pts[:c.input_dim]) for i, c in enumerate(self.comps)])

    def logdet(self, coeffs, pts):
        cs = self.split(coeffs)
        out = self.comps[0].logdet(cs[0], pts[:self.comps[0].input_dim])
        for i in range(1, len(self.comps)):
            out = out + self.comps[i].logdet(cs[i], pts[:self.comps[i].input_dim])
        return out

    def coeff_grad(self, coeffs, pts, sens):
        cs = self.split(coeffs)
        return np.concatenate([c.coeff_grad(cs[i], pts[:c.input_dim], sens[i]) for i, c in enumerate(self.comps)])

    def logdet_coeff_grad(self, coeffs, pts):
        cs = self.split(coeffs)
        return np.concatenate([c.logdet_coeff_grad(cs[i], pts[:c.input_dim]) for i, c in enumerate(self.comps)])

    def gradient(self, coeffs, pts, sens):
        cs = self.split(coeffs)
        out = np.zeros((self.input_dim, pts.shape[1]))
        for i, c in enumerate(self.comps):
            out[:c.input_dim] += c.gradient(cs[i], pts[:c.input_dim], sens[i])
        return out

    def logdet_input_grad(self, coeffs, pts):
        cs = self.split(coeffs)
        out = np.zeros((self.input_dim, pts.shape[1]))
        for i, c in enumerate(self.comps):
            out[:c.input_dim] += c.logdet_input_grad(cs[i], pts[:c.input_dim])
        return out

    def inverse(self, coeffs, x1, r, xtol=1e-6, ytol=1e-6):
        """TriangularMap::InverseImpl / InverseInplace (src/TriangularMap.cpp:146-184)."""
        cs = self.split(coeffs)
        N = r.shape[1]
        full = np.zeros((self.input_dim, N))
        full[:x1.shape[0]] = x1
        extra = self.input_dim - self.output_dim
        for i, c in enumerate(self.comps):
            full[extra + i] = c.inverse(cs[i], full[:c.input_dim], r[i], xtol, ytol)
        return full[extra:]


def fast_gaussian_reverse_kl(comp: OracleComponent, coeffs, pts):
    """FastGaussianReverseKLObjective::CommonEval<EvalGrad> (src/MapObjective.cpp:185-234):
    loss = mean(0.5 T^2 - logdet), grad = mean(T dT/dc - dlogdet/dc)."""
    T = comp.evaluate(coeffs, pts)
    ld = comp.logdet(coeffs, pts)
    N = pts.shape[1]
    loss = 0.0
    for j in range(N):
        loss += 0.5 * T[j] * T[j] - ld[j]
    loss /= N
    g = comp.coeff_grad(coeffs, pts, T)
    lg = comp.logdet_coeff_grad(coeffs, pts)
    grad = (g - lg).sum(axis=1) / N
    return loss, grad


def kl_objective(tmap: OracleTriangularMap, coeffs, pts):
    """KLObjective::ObjectivePlusCoeffGradImpl with a standard-normal density
    (src/MapObjective.cpp:54-91): loss = -mean(log N(T(x)) + logdet)."""
    M = tmap.output_dim
    N = pts.shape[1]
    T = tmap.evaluate(coeffs, pts)
    logtau = math.log(2 * math.pi)
    dens = -0.5 * (M * logtau + 0.0) - 0.5 * (T * T).sum(axis=0)
    dens = dens + tmap.logdet(coeffs, pts)
    loss = -dens.sum() / N
    gx = tmap.coeff_grad(coeffs, pts, -T) + tmap.logdet_coeff_grad(coeffs, pts)
    grad = (-1.0 / N) * gx.sum(axis=1)
    return loss, grad


def inverse_coeff_grad(tmap: OracleTriangularMap, coeffs, pts, w):
    """Implicit-function derivative of TriangularMap::InverseImpl
    (src/TriangularMap.cpp:146-184; the reference itself does not
    differentiate it).  pts = [x1; x] at the solution x = T^{-1}(x1, r), w the
    weights of L = sum w * x.  Solves (dT/dx)^T lambda = w per point, last
    component first: lambda_k = (w_k - sum_{m>k} lambda_m dT_m/dx_k) / dT_k/dx_k
    with dT_k/dx_k = ContinuousDerivative + nugget (MonotoneComponent.h:487-531)
    and the off-diagonal terms from GradientImpl (MonotoneComponent.h:824-874).
    Returns (dL/dc = -sum_i lambda^T dT/dc, [dL/dx1; dL/dr] = [-lambda^T dT/dx1; lambda])."""
    cs = tmap.split(coeffs)
    N = pts.shape[1]
    extra = tmap.input_dim - tmap.output_dim
    acc = np.zeros((tmap.input_dim, N))
    grad = np.zeros(tmap.num_coeffs)
    for k in reversed(range(len(tmap.comps))):
        c = tmap.comps[k]
        D = c.input_dim
        p = np.ascontiguousarray(pts[:D])
        lam = (w[k] - acc[D - 1]) / (c.cont_derivative(cs[k], p) + c.nugget)
        acc[D - 1] = lam
        acc[:D - 1] += c.gradient(cs[k], p, lam)[:D - 1]
        grad[tmap.offsets[k]:tmap.offsets[k + 1]] = -c.coeff_grad(cs[k], p, lam).sum(axis=1)
    acc[:extra] *= -1.0
    return grad, acc
