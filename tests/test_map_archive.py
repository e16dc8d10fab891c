"""The reference's whole-map archive behind ToBytes / FromBytes / pickle
(ParameterizedFunctionBase::Save / Load, MParT/ParameterizedFunctionBase.h:197-215;
bindings/python/src/ParameterizedFunctionBase.cpp:57-79).

The expected bytes are the reference's own: its map classes compiled unchanged
into oracle/_ref with a save-side stand-in for cereal v1.3.2
(oracle/ref_shim/cereal), where the reference checkout is present, and the
fixture tests/golden/archive.npz made from them (tests/golden/make_golden.py).

CPU: the library's host-only reader and writer (mpgb_map_archive_rewrite)
turn every reference archive back into the same bytes, and a decoder written
here pins what the reference records.  GPU: maps built here archive to the
reference's bytes after the same operations, and the reference's archives
load into maps that evaluate as the reference's did."""
import itertools
import json
import os
import struct

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def M():
    import mpart_gb300
    mpart_gb300.load()
    return mpart_gb300


@pytest.fixture(scope="module")
def fixture():
    z = np.load(os.path.join(HERE, "golden", "archive.npz"))
    return z, json.loads(str(z["cases"]))


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("reference checkout not present")
    return ref


# ---- a decoder written from the layout, independent of the library ---------
class _Dec:
    def __init__(self, b):
        self.b, self.o = b, 0
        self.types, self.objs = {}, {}

    def take(self, fmt):
        v = struct.unpack_from("<" + fmt, self.b, self.o)
        self.o += struct.calcsize("<" + fmt)
        return v[0] if len(v) == 1 else v

    def string(self):
        n = self.take("Q")
        s = self.b[self.o:self.o + n].decode()
        self.o += n
        return s

    def view(self, fmt):
        label, n = self.string(), self.take("I")
        vals = list(struct.unpack_from("<%d%s" % (n, fmt), self.b, self.o))
        self.o += n * struct.calcsize(fmt)
        return label, vals

    def pointer(self):
        tid = self.take("I")
        if tid & 0x80000000:
            self.types[tid & 0x7FFFFFFF] = self.string()
        name = self.types[tid & 0x7FFFFFFF]
        oid = self.take("I")
        if not oid & 0x80000000:
            return self.objs[oid]
        obj = dict(name=name)
        self.objs[oid & 0x7FFFFFFF] = obj
        if name.startswith("mpart::TriangularMap<"):
            n = self.take("Q")
            obj["comps"] = [self.pointer() for _ in range(n)]
            assert self.take("Q") == n  # written a second time, ids only
            obj["again"] = [self.take("II") for _ in range(n)]
            obj["moveCoeffs"] = self.take("B")
            return obj
        obj["dim"] = self.take("I")
        obj["mset"] = (self.take("I"), self.take("B"), [self.view("I") for _ in range(4)])
        obj["normalize"] = self.take("B")
        obj["startPos"] = self.view("I")
        obj["cacheSize"] = self.take("I")
        obj["fdim"], obj["maxDim"], obj["workspace"] = self.take("III")
        obj["internalWork"] = self.view("d")
        if "ClenshawCurtisQuadrature<" in name:
            obj["pts"], obj["wts"], obj["numPts"] = self.view("d"), self.view("d"), self.take("I")
        else:
            obj["maxSub"], obj["minSub"] = self.take("II")
            obj["absTol"], obj["relTol"] = self.take("dd")
            obj["errorMetric"] = self.take("I")
            if "AdaptiveClenshawCurtis<" in name:
                obj["rules"] = [self.view("d") for _ in range(4)]
        obj["contDeriv"], obj["nugget"] = self.take("B"), self.take("d")
        obj["coeffs"] = self.view("d")
        return obj


def _decode(b):
    d = _Dec(b)
    top = d.pointer()
    assert d.o == len(b)
    return top


def _components(top):
    return top["comps"] if "comps" in top else [top]


# ---- CPU ---------------------------------------------------------------------
@pytest.mark.parametrize("basis,pos,quad,norm,cont", list(itertools.product(
    ("ProbabilistHermite", "HermiteFunctions"), ("Exp", "SoftPlus"),
    ("AdaptiveClenshawCurtis", "ClenshawCurtis", "AdaptiveSimpson"), (True, False), (True, False))))
def test_reference_archives_come_back_byte_for_byte(M, basis, pos, quad, norm, cont):
    ref = _ref()
    m = ref.RefMap(3, 2, 3, basis=basis, posfunc=pos, quad=quad, normalize=norm, cont_deriv=cont,
                   quad_pts=6 if quad == "ClenshawCurtis" else 7, nugget=0.1, max_sub=11, min_sub=1,
                   abs_tol=1e-7, rel_tol=3e-7)
    m.set_coeffs(np.random.default_rng(0).normal(size=m.num_coeffs))
    b = m.to_bytes()
    assert M.RewriteMapArchive(b) == b


@pytest.mark.parametrize("ops", [["evaluate"], ["coeff_grad"], ["gradient"], ["logdet"], ["logdet_coeff_grad"],
                                 ["coeff_grad", "inverse"], ["gradient", "logdet_input_grad"]])
@pytest.mark.parametrize("cont", [True, False])
def test_reference_archives_after_operations_come_back_byte_for_byte(M, ops, cont):
    ref = _ref()
    if "logdet_input_grad" in ops and not cont:
        pytest.skip("the reference has no discrete-derivative LogDeterminantInputGrad")
    m = ref.RefMap(3, 2, 2, quad="AdaptiveClenshawCurtis", cont_deriv=cont)
    m.set_coeffs(np.random.default_rng(1).normal(0.0, 0.1, m.num_coeffs))
    rng = np.random.default_rng(2)
    x, sens = rng.standard_normal((3, 30)), rng.standard_normal((2, 30))
    for op in ops:
        if op == "inverse":
            m.inverse(x[:1], m.evaluate(x))
        elif op in ("coeff_grad", "gradient"):
            getattr(m, op)(x, sens)
        else:
            getattr(m, op)(x)
    b = m.to_bytes()
    assert M.RewriteMapArchive(b) == b


def test_reference_component_and_moved_map_archives_come_back_byte_for_byte(M, oracle):
    ref = _ref()
    comps = []
    for d in (2, 3):
        s, dd, o = oracle.total_order(d, 2)
        c = ref.RefMap(d, starts=s, dims=dd, orders=o, quad="AdaptiveSimpson", posfunc="Exp")
        c.set_coeffs(np.linspace(-0.3, 0.4, c.num_coeffs))
        comps.append(c)
        b = c.to_bytes()
        assert M.RewriteMapArchive(b) == b
    tm = ref.RefMap.triangular_from(comps)
    b = tm.to_bytes()
    assert M.RewriteMapArchive(b) == b
    w = ref.RefMap(2, 2, 2)
    w.wrap_coeffs(np.arange(w.num_coeffs) * 0.01)
    b = w.to_bytes()
    assert M.RewriteMapArchive(b) == b


def test_archive_fixture_comes_back_byte_for_byte(M, fixture):
    z, cases = fixture
    for c in cases:
        b = z[c["name"] + "__bytes"].tobytes()
        assert M.RewriteMapArchive(b) == b, c["name"]


def test_archive_fixture_matches_reference(fixture):
    """The fixture is what the reference writes today (reference checkout only)."""
    _ref()
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    z, cases = fixture
    assert cases == mg.ARCHIVE_CASES
    again = mg.make_archive()
    for c in cases:
        assert again[c["name"] + "__bytes"].tobytes() == z[c["name"] + "__bytes"].tobytes(), c["name"]


def test_archive_records_what_the_reference_keeps(fixture):
    """Type names, ids, the quadrature dimension each operation leaves, the
    coefficient view labels of each construction route, and the rules."""
    z, cases = fixture
    want_fdim = {"tri_ph_softplus_acc": lambda c: 1, "tri_hf_exp_acc_coeffgrad": lambda c: c["nterms"] + 1,
                 "tri_ph_exp_cc_unnormalised": lambda c: 1, "tri_ph_softplus_as_discrete_logdet": lambda c: 2,
                 "tri_hf_softplus_acc_gradient": lambda c: c["dim"] + 1,
                 "tri_ph_softplus_acc_discrete_ldcg": lambda c: 2, "tri_ph_softplus_acc_inverse": lambda c: 1,
                 "comp_ph_softplus_acc": lambda c: c["nterms"] + 1, "moved_hf_exp_as": lambda c: 1,
                 "wrapped_ph_softplus_cc": lambda c: 1}
    for case in cases:
        b = z[case["name"] + "__bytes"].tobytes()
        top = _decode(b)
        comps = _components(top)
        coef = z[case["name"] + "__coef"]
        if case["build"] == "component":
            assert top["name"].startswith("mpart::MonotoneComponent<")
        else:
            assert top["name"] == "mpart::TriangularMap<Kokkos::HostSpace>"
            assert top["moveCoeffs"] == 1
            # type 1 is the map; its components share type 2; objects count from 1
            assert top["again"] == [(2, i + 2) for i in range(len(comps))]
        label = {"moved": "coeffs", "wrapped": ""}.get(case["build"],
                                                        "ParameterizedFunctionBase<MemorySpace> Coefficients")
        got = np.concatenate([c["coeffs"][1] for c in comps])
        np.testing.assert_array_equal(got, coef)
        quad = case["opts"]["quad"]
        for c in comps:
            c["nterms"] = len(c["mset"][2][0][1]) - 1
            assert c["coeffs"][0] == label
            assert c["fdim"] == want_fdim[case["name"]](c), case["name"]
            assert c["maxDim"] == 1 and c["dim"] == c["mset"][0]
            assert c["startPos"][0] == "Indices for start of 1d basis evaluations"
            assert c["cacheSize"] == c["startPos"][1][-1]
            ms = c["maxSub"] if "maxSub" in c else 0
            ws = {"AdaptiveClenshawCurtis": (ms + 5) * c["fdim"] + 2 * ms,
                  "AdaptiveSimpson": (2 * ms + 5) * c["fdim"] + 2 * ms, "ClenshawCurtis": c["fdim"]}[quad]
            assert c["workspace"] == ws
            if quad == "ClenshawCurtis":
                assert c["internalWork"] == ("Workspace", [0.0])
                assert c["numPts"] == case["opts"]["quad_pts"] and c["pts"][0] == "Points"
            else:
                assert c["internalWork"] == ("", []) and c["errorMetric"] == 0
            if quad == "AdaptiveClenshawCurtis":
                assert [r[0] for r in c["rules"]] == ["Coarse Pts", "Coarse Wts", "Fine Pts", "Coarse Pts"]
            basis = "HermiteFunction" if case["opts"]["basis"] == "HermiteFunctions" else "ProbabilistHermite"
            assert "BasisEvaluator<BasisHomogeneity::Homogeneous, %s>" % basis in c["name"]
            assert c["normalize"] == (basis == "ProbabilistHermite" and case["opts"].get("normalize", True))


def test_archive_reader_rejects_what_it_cannot_load(M, fixture):
    z, _ = fixture
    b = z["tri_ph_softplus_acc__bytes"].tobytes()
    with pytest.raises(ValueError):
        M.RewriteMapArchive(b[:len(b) // 2])
    # a PhysicistHermite component (registered by the reference, not provided here)
    old = b"BasisHomogeneity::Homogeneous, ProbabilistHermite>"
    new = b"BasisHomogeneity::Homogeneous, PhysicistHermite>"
    i = b.index(old)
    n = struct.unpack_from("<Q", b, i - 8 - len("mpart::MonotoneComponent<mpart::MultivariateExpansionWorker<"
                                                 "mpart::BasisEvaluator<"))[0]
    start = i - len("mpart::MonotoneComponent<mpart::MultivariateExpansionWorker<mpart::BasisEvaluator<")
    name = b[start:start + n].replace(old, new)
    bad = b[:start - 8] + struct.pack("<Q", len(name)) + name + b[start + n:]
    with pytest.raises(ValueError, match="basis not provided"):
        M.RewriteMapArchive(bad)
    # an archive in this library's own layout (sigmoid maps) is not the reference's
    with pytest.raises(ValueError):
        M.RewriteMapArchive(struct.pack("<Q", 3) + b"abc")
    # a triangular map listed as its own component
    name = b"mpart::TriangularMap<Kokkos::HostSpace>"
    loop = struct.pack("<I", 0x80000001) + struct.pack("<Q", len(name)) + name + struct.pack("<I", 0x80000001)
    loop += struct.pack("<Q", 1) + struct.pack("<II", 1, 1) + struct.pack("<B", 0)
    with pytest.raises(ValueError, match="contains itself"):
        M.RewriteMapArchive(loop)
    # triangular maps nested a thousand deep (each holding the next)
    deep = struct.pack("<I", 0x80000001) + struct.pack("<Q", len(name)) + name + struct.pack("<I", 0x80000001)
    for k in range(1000):
        deep += struct.pack("<Q", 1) + struct.pack("<II", 1, 0x80000002 + k)
    with pytest.raises(ValueError, match="nested too deeply"):
        M.RewriteMapArchive(deep)


# ---- GPU ---------------------------------------------------------------------
def _build_case(M, case, coef):
    import torch
    o = case["opts"]
    q = {"AdaptiveClenshawCurtis": M.QuadTypes.AdaptiveClenshawCurtis, "ClenshawCurtis": M.QuadTypes.ClenshawCurtis,
         "AdaptiveSimpson": M.QuadTypes.AdaptiveSimpson}[o["quad"]]
    opts = M.MapOptions(basisType=getattr(M.BasisTypes, o["basis"]), posFuncType=getattr(M.PosFuncTypes, o["posfunc"]),
                        quadType=q, quadAbsTol=o.get("abs_tol", 1e-6), quadRelTol=o.get("rel_tol", 1e-6),
                        quadMaxSub=o.get("max_sub", 30), quadMinSub=o.get("min_sub", 0),
                        quadPts=o.get("quad_pts", 5), contDeriv=o.get("cont_deriv", True),
                        basisNorm=o.get("normalize", True), nugget=o.get("nugget", 0.0))
    ind, outd, order = case["in_dim"], case["out_dim"], case["order"]
    keep = None
    if case["build"] == "component":
        m = M.CreateComponent(M.FixedMultiIndexSet(ind, order), opts)
        m.SetCoeffs(coef)
    elif case["build"] == "moved":
        comps, off = [], 0
        for i in range(outd):
            c = M.CreateComponent(M.FixedMultiIndexSet(ind - outd + i + 1, order), opts)
            c.SetCoeffs(coef[off:off + c.numCoeffs])
            off += c.numCoeffs
            comps.append(c)
        m = M.TriangularMap(comps, True)
    else:
        m = M.CreateTriangular(ind, outd, order, opts)
        if case["build"] == "wrapped":
            keep = torch.as_tensor(coef, device="cuda").clone()
            m.WrapCoeffs(keep)
        else:
            m.SetCoeffs(coef)
    return m, keep


def _run_ops(m, case, x, sens, ev):
    import torch
    ind, outd = case["in_dim"], case["out_dim"]
    for op in case["ops"]:
        if op == "evaluate":
            m.Evaluate(x)
        elif op == "coeff_grad":
            m.CoeffGrad(x, sens[:outd])
        elif op == "gradient":
            m.Gradient(x, sens[:outd])
        elif op == "logdet":
            m.LogDeterminant(x)
        elif op == "logdet_coeff_grad":
            m.LogDeterminantCoeffGrad(x)
        elif op == "inverse":
            m.Inverse(x[:ind - outd], torch.as_tensor(ev, device="cuda"))


@pytest.mark.gpu
def test_maps_archive_to_the_reference_bytes(gpu, fixture, tmp_path):
    import torch
    M = gpu
    z, cases = fixture
    for case in cases:
        name = case["name"]
        coef, ev = z[name + "__coef"], z[name + "__eval"]
        m, keep = _build_case(M, case, coef)
        x = torch.as_tensor(z["x"][:case["in_dim"]], device="cuda")
        sens = torch.as_tensor(z["sens"], device="cuda")
        out = m.Evaluate(x).cpu().numpy()
        np.testing.assert_allclose(out, ev, rtol=1e-10, atol=1e-12, err_msg=name)
        _run_ops(m, case, x, sens, ev)
        assert m.ToBytes() == z[name + "__bytes"].tobytes(), name
        # the binding's Serialize: dimensions and the coefficient view, label included
        path = tmp_path / (name + ".bin")
        m.Serialize(path)
        assert path.read_bytes() == z[name + "__serialize"].tobytes(), name
        del keep


@pytest.mark.gpu
def test_reference_archives_load_and_evaluate_as_the_reference(gpu, fixture):
    import pickle

    import torch
    M = gpu
    z, cases = fixture
    for case in cases:
        name = case["name"]
        b = z[name + "__bytes"].tobytes()
        m = M.FromBytes(b)
        assert (m.inputDim, m.outputDim) == (case["in_dim"], case["out_dim"]), name
        np.testing.assert_array_equal(np.asarray(m.CoeffMap()), z[name + "__coef"])
        x = torch.as_tensor(z["x"][:case["in_dim"]], device="cuda")
        np.testing.assert_allclose(m.Evaluate(x).cpu().numpy(), z[name + "__eval"], rtol=1e-10, atol=1e-12,
                                   err_msg=name)
        back = pickle.loads(pickle.dumps(m))
        np.testing.assert_array_equal(np.asarray(back.CoeffMap()), z[name + "__coef"])
        # what the reference's Load rebuilds: copied component coefficients,
        # a triangular map that moved them into one view ("coeffs")
        comps = _components(_decode(m.ToBytes()))
        labels = {c["coeffs"][0] for c in comps}
        assert labels == ({"ParameterizedFunctionBase<MemorySpace> Coefficients"} if case["build"] == "component"
                          else {"coeffs"}), name
