"""GB300-native monotone transport-map components (the per-point hot path of
MParT) behind MParT's own ConditionalMapBase / TriangularMap interface.

Python mirror of the reference's pybind module (bindings/python/src/*.cpp):
the classes below forward to the C ABI in include/mpart_gb300.h.  Arrays may
be torch tensors (CUDA tensors stay on the device) or numpy arrays (staged
through the device inside the call).  Points are D x N, one column per point,
like the reference's *Impl methods."""
from __future__ import annotations

import ctypes as C
import enum
import math
import os
from typing import Sequence

import numpy as np

from . import _capi
from ._capi import IntegrandError, MpgbError, check, load, mpgb_map_options, mpgb_matrix
from .multiindex import (And, Anisotropic, Dimension, MaxDegree, MultiIndex, MultiIndexSet, NoneLim,  # noqa: F401
                         NonzeroDiag, Or, Separable, TotalOrder, Xor)

__all__ = [
    "BasisTypes", "PosFuncTypes", "QuadTypes", "MapOptions", "FixedMultiIndexSet", "ConditionalMapBase",
    "TriangularMap", "CreateComponent", "CreateTriangular", "IntegrandError", "MpgbError", "load", "DeserializeMap",
    "FromBytes", "MapBatch", "TrainMap", "TrainOptions", "KLObjective", "CreateGaussianKLObjective", "MultiIndexSet",
    "ATMOptions", "TrainMapAdaptive", "SigmoidTypes", "EdgeTypes", "SigmoidSumSizeType", "SigmoidComponent",
    "CreateSigmoidComponent", "CreateSigmoidTriangular", "Sigmoid1d", "MultiIndex", "TotalOrder", "Dimension",
    "Anisotropic", "MaxDegree", "NoneLim", "Separable", "NonzeroDiag", "And", "Or", "Xor", "RewriteMapArchive",
    "Initialize", "Concurrency",
]


class BasisTypes(enum.IntEnum):
    ProbabilistHermite = 0
    PhysicistHermite = 1
    HermiteFunctions = 2


class PosFuncTypes(enum.IntEnum):
    Exp = 0
    SoftPlus = 1


class QuadTypes(enum.IntEnum):
    ClenshawCurtis = 0
    AdaptiveSimpson = 1
    AdaptiveClenshawCurtis = 2


class SigmoidTypes(enum.IntEnum):
    Logistic = 0


class EdgeTypes(enum.IntEnum):
    SoftPlus = 0


class SigmoidSumSizeType(enum.IntEnum):
    """MParT/Sigmoid.h:45-48: term k of a Linear sum has k - 3 sigmoids, of a Constant sum one."""
    Linear = 0
    Constant = 1


class MapOptions:
    """MParT/MapOptions.h:58-123 (same field names and defaults)."""

    def __init__(self, **kw):
        self.basisType = BasisTypes.ProbabilistHermite
        self.posFuncType = PosFuncTypes.SoftPlus
        self.quadType = QuadTypes.AdaptiveSimpson
        self.quadAbsTol = 1e-6
        self.quadRelTol = 1e-6
        self.quadMaxSub = 30
        self.quadMinSub = 0
        self.quadPts = 5
        self.contDeriv = True
        self.basisNorm = True
        self.nugget = 0.0
        self.sigmoidType = SigmoidTypes.Logistic
        self.edgeType = EdgeTypes.SoftPlus
        self.edgeShape = 1.5
        self.sigmoidBasisSumType = SigmoidSumSizeType.Linear
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"MapOptions has no field {k}")
            setattr(self, k, v)

    def _c(self) -> mpgb_map_options:
        return mpgb_map_options(int(self.basisType), int(self.posFuncType), int(self.quadType),
                                float(self.quadAbsTol), float(self.quadRelTol), int(self.quadMaxSub),
                                int(self.quadMinSub), int(self.quadPts), int(bool(self.contDeriv)),
                                int(bool(self.basisNorm)), float(self.nugget), int(self.sigmoidType),
                                int(self.edgeType), float(self.edgeShape), int(self.sigmoidBasisSumType))

    @classmethod
    def _from_c(cls, o: mpgb_map_options) -> "MapOptions":
        return cls(basisType=BasisTypes(o.basis_type), posFuncType=PosFuncTypes(o.pos_func_type),
                   quadType=QuadTypes(o.quad_type), quadAbsTol=o.quad_abs_tol, quadRelTol=o.quad_rel_tol,
                   quadMaxSub=o.quad_max_sub, quadMinSub=o.quad_min_sub, quadPts=o.quad_pts,
                   contDeriv=bool(o.cont_deriv), basisNorm=bool(o.basis_norm), nugget=o.nugget,
                   sigmoidType=SigmoidTypes(o.sigmoid_type), edgeType=EdgeTypes(o.edge_type),
                   edgeShape=o.edge_shape, sigmoidBasisSumType=SigmoidSumSizeType(o.sigmoid_sum_type))

    def ToBytes(self) -> bytes:
        """The reference's cereal archive of MapOptions (MParT/MapOptions.h:126-130)."""
        o = self._c()
        return _archive(lambda buf, cap, size: load().mpgb_options_to_bytes(C.byref(o), buf, cap, size))

    @classmethod
    def FromBytes(cls, data: bytes) -> "MapOptions":
        o = mpgb_map_options()
        check(load().mpgb_options_from_bytes(data, len(data), C.byref(o)))
        return cls._from_c(o)

    def Serialize(self, filename):
        """MapOptions.Serialize (bindings/python/src/MapOptions.cpp:74-78)."""
        with open(filename, "wb") as f:
            f.write(self.ToBytes())

    def Deserialize(self, filename):
        """MapOptions.Deserialize (bindings/python/src/MapOptions.cpp:79-84): fills this object and returns it."""
        with open(filename, "rb") as f:
            other = MapOptions.FromBytes(f.read())
        self.__dict__.update(other.__dict__)
        return self

    def __eq__(self, other):
        return isinstance(other, MapOptions) and self.__dict__ == other.__dict__

    def __reduce__(self):
        # (The cereal archive has no sigmoid fields: pickle every field.)
        return (_options_from_fields, (dict(self.__dict__),))


def _options_from_fields(fields):
    return MapOptions(**fields)


class FixedMultiIndexSet:
    """Compressed multi-index set (MParT/MultiIndices/FixedMultiIndexSet.h),
    with the reference binding's constructors
    (bindings/python/src/MultiIndex.cpp:195-222): ``FixedMultiIndexSet(dim,
    maxOrder)`` is the total-order set in the reference's term order
    (src/MultiIndices/FixedMultiIndexSet.cpp:508-549);
    ``FixedMultiIndexSet(dim, orders)`` takes every term's orders one term
    after another; ``FixedMultiIndexSet(dim, nzStarts, nzDims, nzOrders)`` the
    compressed arrays (also as keywords)."""

    def __init__(self, dim: int, maxOrder=None, *compressed, nzStarts=None, nzDims=None, nzOrders=None):
        self.dim = int(dim)
        if compressed:
            if len(compressed) != 2:
                raise TypeError("FixedMultiIndexSet(dim, nzStarts, nzDims, nzOrders)")
            nzStarts, (nzDims, nzOrders), maxOrder = maxOrder, compressed, None
        elif maxOrder is not None and not isinstance(maxOrder, (int, np.integer)):
            dense = np.asarray(maxOrder, dtype=np.int64).reshape(-1, self.dim)
            other = FixedMultiIndexSet.from_multis(dense)
            nzStarts, nzDims, nzOrders, maxOrder = other.nzStarts, other.nzDims, other.nzOrders, None
        if maxOrder is not None:
            starts, dims, orders = [], [], []
            work = [0] * self.dim

            def rec(d, rem):
                if d < self.dim - 1:
                    for p in range(rem + 1):
                        work[d] = p
                        rec(d + 1, rem - p)
                else:
                    for p in range(rem + 1):
                        work[d] = p
                        starts.append(len(dims))
                        for i in range(self.dim):
                            if work[i] > 0:
                                dims.append(i)
                                orders.append(work[i])
            rec(0, int(maxOrder))
            starts.append(len(dims))
            nzStarts, nzDims, nzOrders = starts, dims, orders
        self.nzStarts = np.ascontiguousarray(nzStarts, dtype=np.uint32)
        self.nzDims = np.ascontiguousarray(nzDims if nzDims is not None else [], dtype=np.uint32)
        self.nzOrders = np.ascontiguousarray(nzOrders if nzOrders is not None else [], dtype=np.uint32)

    @classmethod
    def from_multis(cls, multis):
        """Terms given densely, one row per term."""
        multis = np.asarray(multis, dtype=np.int64)
        starts, dims, orders = [0], [], []
        for row in multis:
            for d, o in enumerate(row):
                if o > 0:
                    dims.append(d)
                    orders.append(int(o))
            starts.append(len(dims))
        return cls(multis.shape[1], nzStarts=starts, nzDims=dims, nzOrders=orders)

    def Size(self):
        return len(self.nzStarts) - 1

    def Length(self):
        return self.dim

    def IndexToMulti(self, i):
        m = np.zeros(self.dim, dtype=np.int64)
        for j in range(self.nzStarts[i], self.nzStarts[i + 1]):
            m[self.nzDims[j]] = self.nzOrders[j]
        return m

    def __len__(self):
        return self.dim

    def MaxDegrees(self):
        """Largest order of each input over the terms (FixedMultiIndexSet::MaxDegrees)."""
        out = np.zeros(self.dim, dtype=np.uint32)
        if self.nzDims.size:
            np.maximum.at(out, self.nzDims, self.nzOrders)
        return out

    def MultiToIndex(self, multi):
        """Index of the term equal to multi, or -1 (FixedMultiIndexSet::MultiToIndex)."""
        want = np.asarray(list(multi), dtype=np.int64)
        if want.size != self.dim:
            return -1
        for i in range(self.Size()):
            if np.array_equal(self.IndexToMulti(i), want):
                return i
        return -1

    def NonzeroDiagonalEntries(self):
        """Terms with a nonzero last entry (FixedMultiIndexSet::NonzeroDiagonalEntries)."""
        return [i for i in range(self.Size())
                if any(self.nzDims[j] == self.dim - 1 for j in range(self.nzStarts[i], self.nzStarts[i + 1]))]

    def ToDevice(self):
        """The set serves host and device alike: itself."""
        return self

    def ToBytes(self) -> bytes:
        """The reference's cereal archive of the set (MParT/MultiIndices/FixedMultiIndexSet.h:115-123)."""
        U = C.POINTER(C.c_uint)
        s, d, o = (a.ctypes.data_as(U) if a.size else None for a in (self.nzStarts, self.nzDims, self.nzOrders))
        return _archive(lambda buf, cap, size: load().mpgb_mset_to_bytes(self.dim, self.Size(), s, d, o, buf, cap,
                                                                         size))

    @classmethod
    def FromBytes(cls, data: bytes) -> "FixedMultiIndexSet":
        dim, nt, nnz = C.c_uint(), C.c_uint(), C.c_uint()
        check(load().mpgb_mset_from_bytes(data, len(data), C.byref(dim), C.byref(nt), C.byref(nnz), None, None,
                                          None))
        s = np.zeros(nt.value + 1, np.uint32)
        d = np.zeros(max(1, nnz.value), np.uint32)
        o = np.zeros(max(1, nnz.value), np.uint32)
        U = C.POINTER(C.c_uint)
        check(load().mpgb_mset_from_bytes(data, len(data), None, None, None, s.ctypes.data_as(U),
                                          d.ctypes.data_as(U), o.ctypes.data_as(U)))
        return cls(dim.value, nzStarts=s, nzDims=d[:nnz.value], nzOrders=o[:nnz.value])

    def Serialize(self, filename):
        """FixedMultiIndexSet.Serialize (bindings/python/src/MultiIndex.cpp:243-248)."""
        with open(filename, "wb") as f:
            f.write(self.ToBytes())

    def Deserialize(self, filename):
        """FixedMultiIndexSet.Deserialize (bindings/python/src/MultiIndex.cpp:249-254): fills this object."""
        with open(filename, "rb") as f:
            other = FixedMultiIndexSet.FromBytes(f.read())
        self.dim, self.nzStarts, self.nzDims, self.nzOrders = other.dim, other.nzStarts, other.nzDims, other.nzOrders
        return self

    def __reduce__(self):
        return (FixedMultiIndexSet.FromBytes, (self.ToBytes(),))


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _archive(call) -> bytes:
    """Two-call archive writer: query the size, then fill a buffer."""
    size = C.c_size_t(0)
    check(call(None, 0, C.byref(size)))
    buf = C.create_string_buffer(max(1, size.value))
    check(call(buf, size.value, C.byref(size)))
    return buf.raw[:size.value]


def DeserializeMap(filename):
    """DeserializeMap (bindings/python/src/Serialization.cpp:20-31): reads a file
    written by ConditionalMapBase.Serialize; returns (inputDim, outputDim, coeffs)."""
    with open(filename, "rb") as f:
        data = f.read()
    i, o, n = C.c_uint(), C.c_uint(), C.c_uint()
    check(load().mpgb_coeff_archive_read(data, len(data), C.byref(i), C.byref(o), C.byref(n), None))
    coeffs = np.zeros(n.value)
    check(load().mpgb_coeff_archive_read(data, len(data), None, None, None, C.c_void_p(coeffs.ctypes.data)))
    return i.value, o.value, coeffs


def _wrap_map(h, keep=()):
    k = C.c_int()
    check(load().mpgb_map_kind(h, C.byref(k)))
    if k.value < 0:
        return TriangularMap(_handle=h)
    return SigmoidComponent(h, keep) if k.value > 0 else ConditionalMapBase(h, keep)


def FromBytes(data: bytes):
    """ParameterizedFunctionBase.FromBytes: rebuilds a component or triangular
    map (with its coefficients) from ConditionalMapBase.ToBytes() or from the
    reference's ToBytes / pickle archive."""
    h = C.c_void_p()
    check(load().mpgb_map_from_bytes(data, len(data), C.byref(h)))
    return _wrap_map(h)


def Initialize(opts=None):
    """MParT's Initialize(dict) (bindings/python/src/CommonPybindUtilities.cpp:15-27)
    hands its options to Kokkos; the CUDA runtime here starts on first use, so
    the options are accepted and have no effect."""
    return None


def Concurrency():
    """Threads the execution space runs at once, as Kokkos'
    DefaultExecutionSpace::concurrency() reports (CommonPybindUtilities.cpp:32):
    on a GPU its SMs times the threads resident per SM, else the host cores."""
    import torch
    if torch.cuda.is_available():
        p = torch.cuda.get_device_properties(torch.cuda.current_device())
        return int(p.multi_processor_count * getattr(p, "max_threads_per_multi_processor", 2048))
    return os.cpu_count() or 1


def RewriteMapArchive(data: bytes) -> bytes:
    """Reads a map archive in the reference's layout and writes it again from
    the map description it holds, on the host (no GPU): checks that this
    library can load it; an archive it loads comes back unchanged."""
    data = bytes(data)
    return _archive(lambda buf, cap, size: load().mpgb_map_archive_rewrite(data, len(data), buf, cap, size))


def __getattr__(name):
    """The torch wrappers and mpart_has_torch, imported on first use (as the
    reference's package exports them when torch is present)."""
    if name in ("TorchConditionalMapBase", "TorchParameterizedFunctionBase"):
        from . import torch as _t
        return getattr(_t, name)
    if name == "mpart_has_torch":
        import importlib.util
        return importlib.util.find_spec("torch") is not None
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")


def _stream_of(*arrs):
    for a in arrs:
        if a is not None and _is_torch(a) and a.is_cuda:
            import torch
            return C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    return C.c_void_p(0)


def _mat(x, allow_none=True) -> mpgb_matrix:
    """A matrix view (pointer, shape, strides in elements) of a 2-D (or 1-D =
    1 x N) float64 torch tensor or numpy array."""
    if x is None:
        if not allow_none:
            raise ValueError("array required")
        return mpgb_matrix(None, 0, 0, 0, 0)
    if _is_torch(x):
        if x.dtype.__repr__() != "torch.float64":
            raise ValueError(f"Currently only tensors with float64 datatype can be converted.  Current dtype is {x.dtype}")
        if x.dim() == 1:
            return mpgb_matrix(C.c_void_p(x.data_ptr()), 1, x.shape[0], x.shape[0] * x.stride(0), x.stride(0))
        if x.dim() != 2:
            raise ValueError("Currently only 1d and 2d tensors can be converted.")
        return mpgb_matrix(C.c_void_p(x.data_ptr()), x.shape[0], x.shape[1], x.stride(0), x.stride(1))
    a = x
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise ValueError("expected a float64 numpy array or torch tensor")
    if a.ndim == 1:
        return mpgb_matrix(C.c_void_p(a.ctypes.data), 1, a.shape[0], a.shape[0] * (a.strides[0] // 8),
                           a.strides[0] // 8)
    return mpgb_matrix(C.c_void_p(a.ctypes.data), a.shape[0], a.shape[1], a.strides[0] // 8, a.strides[1] // 8)


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(x.ctypes.data)


_INVERSE_METHODS = {"Bracket": 0, "Newton": 1}


def _inverse_method(method) -> int:
    """The "Method" option of MonotoneComponent::InverseImpl (MonotoneComponent.h:340-351):
    "Bracket" (the reference's FindBracket + ITP) or "Newton"."""
    if method not in _INVERSE_METHODS:
        raise ValueError(f"Invalid method given to MonotoneComponent::Inverse.  Given \"{method}\", "
                         f"but valid options are {sorted(_INVERSE_METHODS)}.")
    return _INVERSE_METHODS[method]


def _zeros_like_dev(ref, shape):
    if _is_torch(ref):
        import torch
        return torch.zeros(shape, dtype=torch.float64, device=ref.device)
    return np.zeros(shape)


class ConditionalMapBase:
    """Handle on a map (MParT/ConditionalMapBase.h / ParameterizedFunctionBase.h)."""

    def __init__(self, handle: C.c_void_p, keep: Sequence = ()):
        self._h = handle
        self._keep = list(keep)  # objects whose lifetime must cover this one (wrapped coefficients)
        self._wrapped = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.mpgb_map_destroy(h)
            self._h = None

    def _dims(self):
        i, o, n = C.c_uint(), C.c_uint(), C.c_uint()
        check(load().mpgb_map_dims(self._h, C.byref(i), C.byref(o), C.byref(n)))
        return i.value, o.value, n.value

    @property
    def inputDim(self):
        return self._dims()[0]

    @property
    def outputDim(self):
        return self._dims()[1]

    @property
    def numCoeffs(self):
        return self._dims()[2]

    # ---- coefficients -------------------------------------------------
    def SetCoeffs(self, coeffs):
        """Deep copy (src/ParameterizedFunctionBase.cpp:185-207)."""
        if _is_torch(coeffs) and coeffs.is_cuda:
            c = coeffs.detach().contiguous().double()
            check(load().mpgb_set_coeffs(self._h, C.c_void_p(c.data_ptr()), c.numel(), 0, _stream_of(c)))
        else:
            c = np.ascontiguousarray(np.asarray(coeffs.detach().cpu() if _is_torch(coeffs) else coeffs,
                                                dtype=np.float64).reshape(-1))
            check(load().mpgb_set_coeffs(self._h, C.c_void_p(c.ctypes.data), c.size, 1, C.c_void_p(0)))

    def WrapCoeffs(self, coeffs):
        """Aliases a CUDA float64 tensor (src/ParameterizedFunctionBase.cpp:219-228)."""
        if not (_is_torch(coeffs) and coeffs.is_cuda and coeffs.is_contiguous()):
            raise ValueError("WrapCoeffs needs a contiguous CUDA float64 tensor")
        check(load().mpgb_wrap_coeffs(self._h, C.c_void_p(coeffs.data_ptr()), coeffs.numel()))
        self._wrapped = coeffs

    def CoeffMap(self):
        out = np.zeros(self.numCoeffs)
        check(load().mpgb_get_coeffs(self._h, C.c_void_p(out.ctypes.data), out.size))
        return out

    def SetPointOrdering(self, flag: bool):
        """Group points by |x_D| before the quadrature-bearing kernels (default on)."""
        check(load().mpgb_set_point_ordering(self._h, int(bool(flag))))

    def SetAsync(self, flag: bool):
        check(load().mpgb_set_async(self._h, int(bool(flag))))

    def CheckStatus(self, stream=None):
        st = C.c_int(0)
        check(load().mpgb_check_status(self._h, stream if stream is not None else C.c_void_p(0), C.byref(st)))
        return st.value

    # ---- *Impl (caller-allocated outputs) ------------------------------
    def EvaluateImpl(self, pts, out):
        check(load().mpgb_evaluate(self._h, _mat(pts), _mat(out), _stream_of(pts, out)))

    def LogDeterminantImpl(self, pts, out):
        check(load().mpgb_log_determinant(self._h, _mat(pts), _mat(out), _stream_of(pts, out)))

    def InverseImpl(self, x1, r, out, xtol=1e-6, ytol=1e-6, info=None, method="Bracket"):
        """method "Bracket" is the reference's FindBracket + ITP; "Newton" closes
        the same bracket by safeguarded Newton steps (same stopping rules)."""
        check(load().mpgb_inverse_method(self._h, _mat(x1), _mat(r), _mat(out), float(xtol), float(ytol),
                                         _inverse_method(method), _ptr(info), _stream_of(x1, r, out)))

    def CoeffGradImpl(self, pts, sens, out):
        check(load().mpgb_coeff_grad(self._h, _mat(pts), _mat(sens), _mat(out), _stream_of(pts, sens, out)))

    def GradientImpl(self, pts, sens, out):
        check(load().mpgb_gradient(self._h, _mat(pts), _mat(sens), _mat(out), _stream_of(pts, sens, out)))

    def LogDeterminantCoeffGradImpl(self, pts, out):
        check(load().mpgb_log_determinant_coeff_grad(self._h, _mat(pts), _mat(out), _stream_of(pts, out)))

    def LogDeterminantInputGradImpl(self, pts, out):
        check(load().mpgb_log_determinant_input_grad(self._h, _mat(pts), _mat(out), _stream_of(pts, out)))

    def FusedForwardAdjointImpl(self, pts, sens=None, logdet_sens=None, logdet_sens_scale=0.0, out_eval=None,
                                out_logdet=None, coeff_grad=None, input_grad=None):
        check(load().mpgb_fused_fwd_adj(self._h, _mat(pts), _mat(sens), _mat(logdet_sens), float(logdet_sens_scale),
                                        _mat(out_eval), _mat(out_logdet), _ptr(coeff_grad), _mat(input_grad),
                                        _stream_of(pts, sens, out_eval)))

    def InverseCoeffGradImpl(self, pts, w, coeff_grad=None, pts_grad=None):
        """Implicit-function adjoint of Inverse: pts = [x1; x] at the solution,
        w the weights of L = sum w * x; coeff_grad <- dL/dc, pts_grad <- [dL/dx1; dL/dr]."""
        check(load().mpgb_inverse_coeff_grad(self._h, _mat(pts), _mat(w), _ptr(coeff_grad), _mat(pts_grad),
                                             _stream_of(pts, w)))

    def InverseCoeffGrad(self, x1, x, w):
        """Returns (dL/dc, dL/dx1, dL/dr) for L = sum w * x with x = Inverse(x1, r)."""
        extra = self.inputDim - self.outputDim
        if not extra:
            pts = x
        elif _is_torch(x):
            import torch
            pts = torch.cat([x1[:extra].expand(extra, x.shape[1]), x], dim=0).contiguous()
        else:
            pts = np.concatenate([np.broadcast_to(x1[:extra], (extra, x.shape[1])), x], axis=0)
        cg = _zeros_like_dev(x, (self.numCoeffs,))
        pg = _zeros_like_dev(x, (self.inputDim, x.shape[1]))
        self.InverseCoeffGradImpl(pts, w, cg, pg)
        return cg, pg[:extra], pg[extra:]

    # ---- allocating versions (the reference's Evaluate(pts) etc.) --------
    def Evaluate(self, pts):
        out = _zeros_like_dev(pts, (self.outputDim, pts.shape[1]))
        self.EvaluateImpl(pts, out)
        return out

    def LogDeterminant(self, pts):
        out = _zeros_like_dev(pts, (pts.shape[1],))
        self.LogDeterminantImpl(pts, out)
        return out

    def Inverse(self, x1, r, xtol=1e-6, ytol=1e-6, method="Bracket"):
        out = _zeros_like_dev(r, (self.outputDim, r.shape[1]))
        self.InverseImpl(x1, r, out, xtol, ytol, method=method)
        return out

    def CoeffGrad(self, pts, sens):
        out = _zeros_like_dev(pts, (self.numCoeffs, pts.shape[1]))
        self.CoeffGradImpl(pts, sens, out)
        return out

    def Gradient(self, pts, sens):
        out = _zeros_like_dev(pts, (self.inputDim, pts.shape[1]))
        self.GradientImpl(pts, sens, out)
        return out

    def LogDeterminantCoeffGrad(self, pts):
        out = _zeros_like_dev(pts, (self.numCoeffs, pts.shape[1]))
        self.LogDeterminantCoeffGradImpl(pts, out)
        return out

    def LogDeterminantInputGrad(self, pts):
        out = _zeros_like_dev(pts, (self.inputDim, pts.shape[1]))
        self.LogDeterminantInputGradImpl(pts, out)
        return out

    def KLObjective(self, pts):
        """Per-component standard-normal reverse KL (FastGaussianReverseKLObjective)
        and its coefficient gradient: returns (loss per component, gradient)."""
        loss = _zeros_like_dev(pts, (self.outputDim,))
        grad = _zeros_like_dev(pts, (self.numCoeffs,))
        check(load().mpgb_kl_objective(self._h, _mat(pts), _ptr(loss), _ptr(grad), _stream_of(pts)))
        return loss, grad

    # ---- archives ----------------------------------------------------------
    def Serialize(self, filename):
        """ParameterizedFunctionBase.Serialize (bindings/python/src/ParameterizedFunctionBase.cpp:51-56):
        inputDim, outputDim, numCoeffs and the coefficients, in the reference's cereal layout."""
        with open(filename, "wb") as f:
            f.write(_archive(lambda buf, cap, size: load().mpgb_map_to_bytes(self._h, 1, buf, cap, size)))

    def ToBytes(self) -> bytes:
        """The whole map, in the reference's ToBytes / pickle layout for monotone
        components and triangular maps of them; FromBytes rebuilds it."""
        return _archive(lambda buf, cap, size: load().mpgb_map_to_bytes(self._h, 0, buf, cap, size))

    FromBytes = staticmethod(lambda data: FromBytes(data))

    def __reduce__(self):
        return (FromBytes, (self.ToBytes(),))

    def CoeffBounds(self):
        """ConditionalMapBase::CoeffBounds (src/ConditionalMapBase.cpp:297-312): (lb, ub)."""
        n = self.numCoeffs
        lb, ub = np.zeros(n), np.zeros(n)
        D = C.POINTER(C.c_double)
        check(load().mpgb_map_coeff_bounds(self._h, lb.ctypes.data_as(D), ub.ctypes.data_as(D)))
        return lb, ub

    def torch(self, store_coeffs=True, return_logdet=False):
        from .torch import TorchConditionalMapBase
        return TorchConditionalMapBase(self, store_coeffs=store_coeffs, return_logdet=return_logdet)


class TriangularMap(ConditionalMapBase):
    """TriangularMap(components, moveCoeffs) (src/TriangularMap.cpp:9-62)."""

    def __init__(self, components: Sequence[ConditionalMapBase] = (), moveCoeffs: bool = False, *, _handle=None):
        if _handle is not None:
            super().__init__(_handle)
            return
        arr = (C.c_void_p * len(components))(*[c._h for c in components])
        h = C.c_void_p()
        check(load().mpgb_create_triangular_from_components(arr, len(components), int(bool(moveCoeffs)),
                                                            C.byref(h)))
        super().__init__(h, keep=list(components))

    def NumComponents(self):
        n = C.c_uint()
        check(load().mpgb_map_num_components(self._h, C.byref(n)))
        return n.value

    def GetComponent(self, i):
        h = C.c_void_p()
        check(load().mpgb_map_get_component(self._h, int(i), C.byref(h)))
        return _wrap_map(h, keep=[self])


def CreateComponent(mset: FixedMultiIndexSet, opts: MapOptions | None = None) -> ConditionalMapBase:
    """MapFactory::CreateComponent (src/MapFactory.cpp:22-27)."""
    opts = opts or MapOptions()
    o = opts._c()
    h = C.c_void_p()
    s = mset.nzStarts
    d = mset.nzDims if mset.nzDims.size else np.zeros(1, np.uint32)
    r = mset.nzOrders if mset.nzOrders.size else np.zeros(1, np.uint32)
    up = C.POINTER(C.c_uint)
    check(load().mpgb_create_component(mset.dim, mset.Size(), s.ctypes.data_as(up), d.ctypes.data_as(up),
                                       r.ctypes.data_as(up), C.byref(o), C.byref(h)))
    return ConditionalMapBase(h)


def CreateTriangular(inputDim: int, outputDim: int, totalOrder: int, opts: MapOptions | None = None) -> TriangularMap:
    """MapFactory::CreateTriangular (src/MapFactory.cpp:105-124)."""
    opts = opts or MapOptions()
    o = opts._c()
    h = C.c_void_p()
    check(load().mpgb_create_triangular(int(inputDim), int(outputDim), int(totalOrder), C.byref(o), C.byref(h)))
    return TriangularMap(_handle=h)


class SigmoidComponent(ConditionalMapBase):
    """A sigmoid expansion (RectifiedMultivariateExpansion for two or more
    inputs, UnivariateExpansion<Sigmoid1d> for one), built by
    CreateSigmoidComponent / CreateSigmoidTriangular."""

    def GetSigmoid(self):
        """(centers, widths, weights, startInds) of the last input's Sigmoid1d basis."""
        n, ns = C.c_uint(), C.c_uint()
        check(load().mpgb_component_sigmoid(self._h, None, None, None, C.byref(n), None, C.byref(ns)))
        c, w, wt = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        st = np.zeros(max(1, ns.value), np.uint32)
        D = C.POINTER(C.c_double)
        check(load().mpgb_component_sigmoid(self._h, c.ctypes.data_as(D), w.ctypes.data_as(D), wt.ctypes.data_as(D),
                                            None, st.ctypes.data_as(C.POINTER(C.c_uint)), None))
        return c, w, wt, st[:ns.value]

    def Sigmoid(self):
        return Sigmoid1d(*self.GetSigmoid())


def _centers(c):
    if _is_torch(c):
        c = c.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(c, dtype=np.float64).reshape(-1))


def CreateSigmoidComponent(*args) -> SigmoidComponent:
    """MapFactory::CreateSigmoidComponent (MParT/MapFactory.h:138-185,
    bindings/python/src/MapFactory.cpp:26-29):
    (inputDim, totalOrder, centers, opts), (inputDim, offDiagOrder, crossOrder,
    centers, opts) or (mset, centers, opts)."""
    D = C.POINTER(C.c_double)
    h = C.c_void_p()
    if isinstance(args[0], FixedMultiIndexSet):
        mset, centers = args[0], _centers(args[1])
        opts = args[2] if len(args) > 2 and args[2] is not None else MapOptions()
        o = opts._c()
        up = C.POINTER(C.c_uint)
        d = mset.nzDims if mset.nzDims.size else np.zeros(1, np.uint32)
        r = mset.nzOrders if mset.nzOrders.size else np.zeros(1, np.uint32)
        check(load().mpgb_create_sigmoid_component_mset(mset.dim, mset.Size(), mset.nzStarts.ctypes.data_as(up),
                                                        d.ctypes.data_as(up), r.ctypes.data_as(up),
                                                        centers.ctypes.data_as(D), len(centers), C.byref(o),
                                                        C.byref(h)))
        return SigmoidComponent(h)
    if len(args) in (3, 4) and not np.isscalar(args[2]):
        inputDim, off, centers = int(args[0]), int(args[1]), _centers(args[2])
        cross = off
        opts = args[3] if len(args) > 3 and args[3] is not None else MapOptions()
    elif len(args) in (4, 5):
        inputDim, off, cross, centers = int(args[0]), int(args[1]), int(args[2]), _centers(args[3])
        opts = args[4] if len(args) > 4 and args[4] is not None else MapOptions()
    else:
        raise TypeError("CreateSigmoidComponent: unsupported arguments")
    o = opts._c()
    check(load().mpgb_create_sigmoid_component(inputDim, off, cross, centers.ctypes.data_as(D), len(centers),
                                               C.byref(o), C.byref(h)))
    return SigmoidComponent(h)


def CreateSigmoidTriangular(inputDim: int, outputDim: int, totalOrder: int, centers,
                            opts: MapOptions | None = None) -> TriangularMap:
    """MapFactory::CreateSigmoidTriangular (MParT/MapFactory.h:186-213): centers
    is (number of centers) x outputDim, column i for component i."""
    opts = opts or MapOptions()
    c = np.asarray(centers.detach().cpu().numpy() if _is_torch(centers) else centers, dtype=np.float64)
    if c.ndim == 1:
        c = c[:, None]
    o = opts._c()
    h = C.c_void_p()
    check(load().mpgb_create_sigmoid_triangular(int(inputDim), int(outputDim), int(totalOrder),
                                                c.ctypes.data_as(C.POINTER(C.c_double)), c.shape[0],
                                                c.strides[0] // 8, c.strides[1] // 8, C.byref(o), C.byref(h)))
    return TriangularMap(_handle=h)


class Sigmoid1d:
    """Sigmoid1d with the Logistic sigmoid and SoftPlus edges (MParT/Sigmoid.h;
    bindings/python/src/Sigmoid.cpp).  Evaluations run on the GPU."""

    def __init__(self, centers, widths, weights, startInds=None, sumType=SigmoidSumSizeType.Linear):
        self.centers = _centers(centers)
        self.widths = _centers(widths)
        self.weights = _centers(weights)
        if startInds is None:
            startInds = _sigmoid_starts(len(self.centers), sumType)
        self.startInds = np.ascontiguousarray(startInds, dtype=np.uint32)

    @classmethod
    def FromCenters(cls, centers, edgeShape=1.5, sumType=SigmoidSumSizeType.Linear):
        """CreateSigmoid (src/MapFactory.cpp:181-254)."""
        c = _centers(centers)
        n = len(c)
        oc, w, wt = np.zeros(n), np.zeros(n), np.zeros(n)
        st = np.zeros(max(1, n), np.uint32)
        ns = C.c_uint()
        D = C.POINTER(C.c_double)
        check(load().mpgb_sigmoid_params(c.ctypes.data_as(D), n, float(edgeShape), int(sumType),
                                         oc.ctypes.data_as(D), w.ctypes.data_as(D), wt.ctypes.data_as(D),
                                         st.ctypes.data_as(C.POINTER(C.c_uint)), C.byref(ns)))
        return cls(oc, w, wt, st[:ns.value])

    def GetOrder(self):
        return len(self.startInds) + 3

    def Evaluate(self, x, maxOrder=None, which=0):
        """Basis values (and derivatives up to `which`) at the points x (a 1-D
        array, evaluated on the GPU): tensors of shape (maxOrder + 1, len(x))."""
        import torch
        maxOrder = self.GetOrder() if maxOrder is None else int(maxOrder)
        xt = torch.as_tensor(np.asarray(x, dtype=np.float64).reshape(-1) if not _is_torch(x) else x,
                             dtype=torch.float64, device="cuda").reshape(-1).contiguous()
        n = xt.shape[0]
        outs = [torch.zeros((maxOrder + 1, n), dtype=torch.float64, device="cuda") for _ in range(which + 1)]
        D = C.POINTER(C.c_double)
        st = self.startInds if self.startInds.size else np.zeros(1, np.uint32)
        check(load().mpgb_sigmoid1d_evaluate(
            self.centers.ctypes.data_as(D), self.widths.ctypes.data_as(D), self.weights.ctypes.data_as(D),
            len(self.centers), st.ctypes.data_as(C.POINTER(C.c_uint)), len(self.startInds), int(which), maxOrder,
            C.c_void_p(xt.data_ptr()), n, 1, C.c_void_p(outs[0].data_ptr()),
            C.c_void_p(outs[1].data_ptr()) if which >= 1 else None,
            C.c_void_p(outs[2].data_ptr()) if which >= 2 else None,
            C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return outs

    # In-place forms of the reference binding: output has maxOrder + 1 entries.
    def EvaluateAll(self, output, x):
        v, = self.Evaluate([x], len(output) - 1, 0)
        output[:] = v[:, 0].cpu().numpy()

    def EvaluateDerivatives(self, output, derivs, x):
        if len(output) != len(derivs):
            raise ValueError("Vector dimensions do not match.")
        v, d = self.Evaluate([x], len(output) - 1, 1)
        output[:] = v[:, 0].cpu().numpy()
        derivs[:] = d[:, 0].cpu().numpy()

    def EvaluateSecondDerivatives(self, output, derivs, derivs2, x):
        if len(output) != len(derivs) or len(derivs) != len(derivs2):
            raise ValueError("Vector dimensions do not match.")
        v, d, d2 = self.Evaluate([x], len(output) - 1, 2)
        output[:] = v[:, 0].cpu().numpy()
        derivs[:] = d[:, 0].cpu().numpy()
        derivs2[:] = d2[:, 0].cpu().numpy()


def _sigmoid_starts(n, sumType):
    """Sigmoid1d::ConstructStartInds (MParT/Sigmoid.h:95-130)."""
    if n <= 2:
        return []
    if int(sumType) == int(SigmoidSumSizeType.Constant):
        return [2 + i for i in range(n - 2)]
    k = int((math.sqrt(1 + 8 * (n - 2)) - 1) / 2)
    if n - 2 != k * (k + 1) // 2:
        raise ValueError("Sigmoid: Could not construct starting indices.  The size of the centers array cannot be "
                         "used with the Linear sum type.")
    out = [2]
    for i in range(1, k):
        out.append(out[-1] + i)
    return out


class TrainOptions:
    """MParT/TrainMap.h:19-58, same field names and defaults.  NLopt is not
    used: opt_alg "LD_SLSQP" (the default) runs this library's restatement of
    SLSQP's iteration for an unconstrained problem (a damped-BFGS quasi-Newton
    method with SLSQP's line search), "LD_LBFGS" its limited-memory BFGS; other
    names raise ValueError.  opt_maxeval bounds the objective evaluations per
    component, the tolerances are NLopt's stopping rules (0 disables one),
    opt_stopval and opt_maxtime are not used."""

    def __init__(self, **kw):
        self.opt_alg = "LD_SLSQP"
        self.opt_stopval = -np.inf
        self.opt_ftol_rel = 1e-3
        self.opt_ftol_abs = 1e-3
        self.opt_xtol_rel = 1e-4
        self.opt_xtol_abs = 1e-4
        self.opt_maxeval = 1000
        self.opt_maxtime = np.inf
        self.verbose = 0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"{type(self).__name__} has no field {k}")
            setattr(self, k, v)

    def _train_c(self, mode=0):
        from ._capi import mpgb_train_options
        o = mpgb_train_options()
        check(load().mpgb_train_options_default(C.byref(o)))
        algs = {"LD_SLSQP": 0, "LD_LBFGS": 1}
        if self.opt_alg not in algs:
            raise ValueError(f"opt_alg {self.opt_alg!r}: this library provides LD_SLSQP and LD_LBFGS")
        o.algorithm = algs[self.opt_alg]
        o.max_iters = o.max_evals = int(self.opt_maxeval)
        o.ftol_rel, o.ftol_abs = float(self.opt_ftol_rel), float(self.opt_ftol_abs)
        o.xtol_rel, o.xtol_abs = float(self.opt_xtol_rel), float(self.opt_xtol_abs)
        o.mode = int(mode)
        return o


class KLObjective:
    """KLObjective with a standard Gaussian reference density
    (src/MapObjective.cpp:54-91, ObjectiveFactory::CreateGaussianKLObjective):
    value = -mean(log N(T(x)) + log det), the per-component reverse-KL sum plus
    (M/2) log 2 pi.  Samples are copied to the device (float64, inputDim x N)."""

    def __init__(self, train, test=None, dim=0):
        import torch
        dev = torch.device("cuda")
        self.train = torch.as_tensor(np.asarray(train) if not _is_torch(train) else train, dtype=torch.float64,
                                     device=dev).contiguous()
        self.test = None if test is None else torch.as_tensor(np.asarray(test) if not _is_torch(test) else test,
                                                              dtype=torch.float64, device=dev).contiguous()
        self.dim = int(dim) or self.train.shape[0]

    def _value(self, tmap, pts):
        loss, _ = tmap.KLObjective(pts[:tmap.inputDim])
        return float(loss.sum().item()) + 0.5 * tmap.outputDim * np.log(2.0 * np.pi)

    def TrainError(self, tmap):
        return self._value(tmap, self.train)

    def TestError(self, tmap):
        if self.test is None:
            raise RuntimeError("No test dataset given!")
        return self._value(tmap, self.test)

    def TrainCoeffGrad(self, tmap):
        return tmap.KLObjective(self.train[:tmap.inputDim])[1]


def CreateGaussianKLObjective(train, test=None, dim=0):
    """ObjectiveFactory::CreateGaussianKLObjective (src/MapObjective.cpp:40-52)."""
    return KLObjective(train, test, dim)


def TrainMap(tmap: ConditionalMapBase, samples, max_iters=100, max_evals=1000, ftol_rel=0.0, ftol_abs=0.0,
             xtol_rel=0.0, xtol_abs=0.0, gtol=0.0, memory=10, mode=0, algorithm="LD_SLSQP", precondition=False):
    """TrainMap(map, objective, options) (src/TrainMap.cpp:166-216) when samples
    is a KLObjective and max_iters a TrainOptions: returns the training objective.

    Otherwise the direct form: TrainMap with a standard-normal KL objective:
    every component minimises its reverse KL with `algorithm` ("LD_SLSQP" or
    "LD_LBFGS", see TrainOptions; with precondition, L-BFGS starts each
    iteration's inverse Hessian from the inverse mean squared per-point
    gradient of every coefficient at the start); samples is a CUDA
    float64 tensor, inputDim x N.  mode 0 replays one batched step from a CUDA
    graph, 1 launches it directly, 2 launches each component separately, 3 runs
    per component the reference objective's call sequence (Evaluate,
    LogDeterminant, CoeffGrad, LogDeterminantCoeffGrad with dense outputs).
    Returns (final loss per component, result dict); the map keeps the result."""
    from ._capi import mpgb_train_options, mpgb_train_result
    if isinstance(samples, KLObjective):
        opts = max_iters if isinstance(max_iters, TrainOptions) else TrainOptions()
        o = opts._train_c(mode)
        loss = np.zeros(tmap.outputDim)
        r = mpgb_train_result()
        pts = samples.train[:tmap.inputDim]
        check(load().mpgb_train_map(tmap._h, _mat(pts), C.byref(o), C.c_void_p(loss.ctypes.data), C.byref(r),
                                    _stream_of(pts)))
        return r.total_loss + 0.5 * tmap.outputDim * np.log(2.0 * np.pi)
    o = mpgb_train_options()
    check(load().mpgb_train_options_default(C.byref(o)))
    o.max_iters, o.max_evals, o.memory, o.mode = int(max_iters), int(max_evals), int(memory), int(mode)
    o.ftol_rel, o.ftol_abs, o.xtol_rel, o.xtol_abs, o.gtol = ftol_rel, ftol_abs, xtol_rel, xtol_abs, gtol
    algs = {"LD_SLSQP": 0, "LD_LBFGS": 1}
    if algorithm not in algs:
        raise ValueError(f"algorithm {algorithm!r}: this library provides LD_SLSQP and LD_LBFGS")
    o.algorithm = algs[algorithm]
    o.precondition = int(bool(precondition))
    loss = np.zeros(tmap.outputDim)
    r = mpgb_train_result()
    check(load().mpgb_train_map(tmap._h, _mat(samples), C.byref(o), C.c_void_p(loss.ctypes.data), C.byref(r),
                                _stream_of(samples)))
    return loss, {"total_loss": r.total_loss, "iterations": r.iterations, "evaluations": r.evaluations,
                  "steps": r.steps, "ms_per_step": r.ms_per_step, "total_ms": r.total_ms,
                  "grad_norm": r.grad_norm}


def KLStepTime(tmap: ConditionalMapBase, samples, mode=0, steps=10, return_values=False):
    """Device milliseconds of one KL objective + gradient step (see TrainMap
    modes); with return_values, also the step's loss per component and gradient."""
    ms = C.c_double(0)
    loss = np.zeros(tmap.outputDim)
    grad = np.zeros(tmap.numCoeffs)
    check(load().mpgb_kl_step_time(tmap._h, _mat(samples), int(mode), int(steps), C.byref(ms),
                                   C.c_void_p(loss.ctypes.data), C.c_void_p(grad.ctypes.data), _stream_of(samples)))
    return (ms.value, loss, grad) if return_values else ms.value


class MapBatch:
    """Many independent maps evaluated together (mpgb_batch_*): forward,
    log-determinant and reduced coefficient adjoint of every map in one
    persistent launch; points per work item from the autotuner.  All arrays
    are CUDA float64 tensors, one per map."""

    def __init__(self, maps: Sequence[ConditionalMapBase]):
        self._maps = list(maps)
        arr = (C.c_void_p * len(self._maps))(*[m._h for m in self._maps])
        h = C.c_void_p()
        check(load().mpgb_batch_create(arr, len(self._maps), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.mpgb_batch_destroy(self._h)
            self._h = None

    def _mats(self, xs):
        n = len(self._maps)
        if xs is None:
            return None
        if len(xs) != n:
            raise ValueError(f"expected {n} arrays, one per map")
        return (_capi.mpgb_matrix * n)(*[_mat(x) for x in xs])

    def FusedForwardAdjoint(self, pts, sens=None, logdet_sens_scale=0.0, out_eval=None, out_logdet=None,
                            coeff_grad=None):
        n = len(self._maps)
        grads = None
        if coeff_grad is not None:
            grads = (C.c_void_p * n)(*[None if g is None else g.data_ptr() for g in coeff_grad])
        check(load().mpgb_batch_fwd_adj(self._h, self._mats(pts), self._mats(sens), float(logdet_sens_scale),
                                        self._mats(out_eval), self._mats(out_logdet), grads, _stream_of(*pts)))

    def Autotune(self, pts, sens=None, logdet_sens_scale=0.0, reps=2):
        """Times the candidate configurations on these inputs and keeps the
        fastest; returns the device ms of one launch with it."""
        ms = C.c_double(0)
        check(load().mpgb_batch_autotune(self._h, self._mats(pts), self._mats(sens), float(logdet_sens_scale),
                                         int(reps), C.byref(ms), _stream_of(*pts)))
        return ms.value

    def Tuning(self):
        """(block size, {(input dim, order): tiles per item})."""
        tpb, nb = C.c_int(0), C.c_int(0)
        check(load().mpgb_batch_tuning(self._h, C.byref(tpb), 0, C.byref(nb), None, None, None))
        d, o, t = (C.c_int * max(1, nb.value))(), (C.c_int * max(1, nb.value))(), (C.c_int * max(1, nb.value))()
        check(load().mpgb_batch_tuning(self._h, C.byref(tpb), nb.value, C.byref(nb), d, o, t))
        return tpb.value, {(d[i], o[i]): t[i] for i in range(nb.value)}

    def SetTuning(self, tpb, tiles):
        items = sorted(tiles.items())
        n = len(items)
        d = (C.c_int * max(1, n))(*[k[0] for k, _ in items])
        o = (C.c_int * max(1, n))(*[k[1] for k, _ in items])
        t = (C.c_int * max(1, n))(*[v for _, v in items])
        check(load().mpgb_batch_set_tuning(self._h, int(tpb), n, d, o, t))


class PlainComponent:
    """Reference-structured GPU comparator (see include/mpart_gb300.h): one
    total-order component evaluated with the reference's per-node term loops
    and full-width quadrature, as separate launches."""

    def __init__(self, dim: int, order: int, opts: MapOptions | None = None):
        o = (opts or MapOptions())._c()
        h = C.c_void_p()
        check(load().mpgb_plain_create(int(dim), int(order), C.byref(o), C.byref(h)))
        self._h = h
        n = C.c_uint()
        check(load().mpgb_plain_num_terms(h, C.byref(n)))
        self.numCoeffs = n.value
        self.dim = int(dim)

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.mpgb_plain_destroy(self._h)
            self._h = None

    def FwdAdj(self, coeffs, pts, sens, out_eval=None, out_logdet=None, coeff_grad=None):
        """All arrays are contiguous CUDA float64 tensors; pts is dim x N."""
        n = pts.shape[1]
        check(load().mpgb_plain_fwd_adj(self._h, _ptr(coeffs), _ptr(pts), n, _ptr(sens), _ptr(out_eval),
                                        _ptr(out_logdet), _ptr(coeff_grad), _stream_of(pts)))


def launch_count():
    """Kernels the library has launched since it was loaded (graph replays
    count their kernel nodes)."""
    return int(load().mpgb_launch_count())


def fp64_probe(blocks=152 * 8, threads=256, iters=4096):
    """DFMA throughput probe; returns (TFLOP/s, ms)."""
    ms = C.c_float(0)
    check(load().mpgb_fp64_probe(blocks, threads, iters, C.c_void_p(0), C.byref(ms)))
    flops = 2.0 * 8 * blocks * threads * iters
    return flops / (ms.value * 1e-3) / 1e12, ms.value


class ATMOptions(MapOptions, TrainOptions):
    """ATMOptions (MParT/TrainMapAdaptive.h:19-47): map options, training
    options and maxPatience, maxSize, maxDegrees (a multi-index of inputDim
    entries, or None)."""

    def __init__(self, **kw):
        MapOptions.__init__(self)
        TrainOptions.__init__(self)
        self.maxPatience = 10
        self.maxSize = 2 ** 31 - 1
        self.maxDegrees = None
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"ATMOptions has no field {k}")
            setattr(self, k, v)


def _component_mset(comp):
    U = C.POINTER(C.c_uint)
    dim, nt, nnz = C.c_uint(), C.c_uint(), C.c_uint()
    check(load().mpgb_component_multi_index(comp._h, C.byref(dim), C.byref(nt), C.byref(nnz), None, None, None))
    s = np.zeros(nt.value + 1, np.uint32)
    d = np.zeros(max(1, nnz.value), np.uint32)
    o = np.zeros(max(1, nnz.value), np.uint32)
    check(load().mpgb_component_multi_index(comp._h, None, None, None, s.ctypes.data_as(U), d.ctypes.data_as(U),
                                            o.ctypes.data_as(U)))
    return FixedMultiIndexSet(dim.value, nzStarts=s, nzDims=d[:nnz.value], nzOrders=o[:nnz.value])


def TrainMapAdaptive(mset0, objective: KLObjective, options: ATMOptions | None = None, mode=0):
    """TrainMapAdaptive (src/TrainMapAdaptive.cpp:44-271): returns the trained
    triangular map; mset0 (a list of MultiIndexSet, one per output) is replaced
    in place by the selected sets, as in the reference."""
    from ._capi import mpgb_atm_options, mpgb_atm_result
    options = options or ATMOptions()
    # The adaptive loop grows each set from its terms in order, without a limiter.
    if any(not isinstance(m.GetLimiter(), NoneLim) for m in mset0):
        raise ValueError("TrainMapAdaptive: limiters on the initial multi-index sets are not supported; bound the "
                         "degrees with ATMOptions.maxDegrees")
    o = mpgb_atm_options()
    check(load().mpgb_atm_options_default(C.byref(o)))
    o.map = options._c()
    o.train = options._train_c(mode)
    o.max_patience = int(options.maxPatience)
    o.max_size = int(min(options.maxSize, 2 ** 32 - 1))
    md = None
    if options.maxDegrees is not None and len(options.maxDegrees):
        md = np.ascontiguousarray(options.maxDegrees, dtype=np.uint32)
        o.max_degrees = md.ctypes.data_as(C.POINTER(C.c_uint))
    o.verbose = int(options.verbose)
    n = len(mset0)
    sizes = np.array([m.Size() for m in mset0], dtype=np.uint32)
    multis = np.ascontiguousarray(np.concatenate([m._dense().reshape(-1) for m in mset0]).astype(np.uint32))
    final = np.zeros(n, dtype=np.uint32)
    res = mpgb_atm_result()
    h = C.c_void_p()
    U = C.POINTER(C.c_uint)
    test = objective.test if objective.test is not None else objective.train
    check(load().mpgb_train_map_adaptive(n, sizes.ctypes.data_as(U), multis.ctypes.data_as(U), _mat(objective.train),
                                         _mat(test), C.byref(o), C.byref(h), C.byref(res), final.ctypes.data_as(U),
                                         _stream_of(objective.train)))
    tmap = TriangularMap(_handle=h)
    for j in range(n):
        fixed = _component_mset(tmap.GetComponent(j))
        mset0[j] = MultiIndexSet(fixed.Length(), [tuple(fixed.IndexToMulti(i)) for i in range(fixed.Size())])
    tmap.atm_result = {"size": res.size, "iterations": res.iterations, "best_test_error": res.best_test_error,
                       "final_train_error": res.final_train_error, "final_test_error": res.final_test_error,
                       "total_ms": res.total_ms}
    return tmap

