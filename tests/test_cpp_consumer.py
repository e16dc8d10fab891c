"""A C++ consumer of the boundary: tests/cpp_consumer.cpp, compiled by g++
against include/mpart_gb300.h, include/mpart_gb300.hpp and
libmpart_gb300.so, drives the map through the C++ API (MapFactory,
SetCoeffs, the *Impl methods) and through an adapter of the shape
INTEGRATION.md shows for MParT's ConditionalMapBase<DeviceSpace> over the C
ABI.  On the CPU the program must compile and link; on the GPU both routes
must give the oracle's results (Evaluate, LogDeterminant, CoeffGrad, Inverse)
on the small workload's map, within the parity tolerance of
test_gpu_parity.py."""
import glob
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "mpart_gb300", "lib")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_consumer(out_dir):
    if not os.path.exists(os.path.join(LIB_DIR, "libmpart_gb300.so")):
        pytest.skip("libmpart_gb300.so not built")
    libdirs = [os.path.join(CUDA, "lib64")] + glob.glob(os.path.join(CUDA, "targets", "*", "lib"))
    exe = os.path.join(out_dir, "cpp_consumer")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", os.path.join(ROOT, "tests", "cpp_consumer.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"), "-L", LIB_DIR, "-lmpart_gb300"]
    for d in libdirs:
        cmd += ["-L", d]
    cmd += ["-lcudart", "-Wl,-rpath," + ":".join([LIB_DIR] + libdirs), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_cpp_consumer_compiles_and_links(tmp_path):
    assert os.access(build_consumer(str(tmp_path)), os.X_OK)


@pytest.mark.gpu
def test_cpp_consumer_matches_oracle(tmp_path, oracle):
    from test_gpu_parity import assert_inverse_parity, assert_parity
    O = oracle
    exe = build_consumer(str(tmp_path))
    n = 2000
    om = O.OracleTriangularMap(2, 2, 3)
    coef = np.random.default_rng(0).normal(0.0, 0.1, om.num_coeffs)
    x = np.random.default_rng(1).standard_normal((2, n))
    sens = np.random.default_rng(2).standard_normal((2, n))
    r = om.evaluate(coef, x)
    inp = os.path.join(str(tmp_path), "in.bin")
    out = os.path.join(str(tmp_path), "out.bin")
    with open(inp, "wb") as f:
        f.write(np.int64(n).tobytes())
        for a in (coef, x, sens, r):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    res = subprocess.run([exe, inp, out], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    flat = np.fromfile(out, dtype=np.float64)
    per = 2 * n + n + 14 * n + 2 * n
    assert flat.size == 2 * per + 2 * n
    # Save / Load of route 1's map evaluates bit for bit as the map did
    np.testing.assert_array_equal(flat[2 * per:].reshape(2, n), flat[:2 * n].reshape(2, n))
    flat = flat[:2 * per]
    for route in range(2):
        v = flat[route * per:(route + 1) * per]
        T, v = v[:2 * n].reshape(2, n), v[2 * n:]
        ld, v = v[:n], v[n:]
        cg, v = v[:14 * n].reshape(14, n), v[14 * n:]
        xi = v.reshape(2, n)
        what = ("C++ API", "adapter over the C ABI")[route]
        assert_parity(T, r, what=f"{what}: Evaluate")
        assert_parity(ld, om.logdet(coef, x), what=f"{what}: LogDeterminant")
        assert_parity(cg, om.coeff_grad(coef, x, sens), what=f"{what}: CoeffGrad")
        assert_inverse_parity(om, coef, np.zeros((0, n)), r, xi, 1e-6, 1e-6)


@pytest.mark.gpu
def test_cpp_consumer_train_map(tmp_path, oracle):
    """MParT's training through the C++ API (KLObjective, TrainOptions with
    L-BFGS, TrainMap) on a 2 x 2 order-3 HermiteFunctions + Exp map: the value
    TrainMap returns and KLObjective::TestError equal the oracle's KL objective
    (the components' reverse-KL losses plus log 2 pi) at the coefficients it
    trained, and training lowers it below its value at zero."""
    O = oracle
    exe = build_consumer(str(tmp_path))
    n = 3000
    rng = np.random.default_rng(4)
    x1 = rng.standard_normal(n)
    x = np.stack([x1, x1 ** 2 + 0.5 * rng.standard_normal(n)])
    inp = os.path.join(str(tmp_path), "train_in.bin")
    out = os.path.join(str(tmp_path), "train_out.bin")
    with open(inp, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())
    res = subprocess.run([exe, "train", inp, out], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    v = np.fromfile(out, dtype=np.float64)
    coef, train, test = v[:-2], v[-2], v[-1]
    om = O.OracleTriangularMap(2, 2, 3, basis=O.BASIS_HERMITE_FUNCTIONS, normalize=True, posfunc=O.POS_EXP,
                               abs_tol=1e-7, rel_tol=1e-7)
    assert coef.size == om.num_coeffs
    cs = om.split(coef)
    want = np.log(2.0 * np.pi) + sum(O.fast_gaussian_reverse_kl(c, cs[i], x[:c.input_dim])[0]
                                     for i, c in enumerate(om.comps))
    assert train == pytest.approx(want, rel=1e-10)
    assert test == pytest.approx(want, rel=1e-10)
    zero = np.log(2.0 * np.pi) + sum(O.fast_gaussian_reverse_kl(c, np.zeros(c.num_coeffs), x[:c.input_dim])[0]
                                     for c in om.comps)
    assert train < zero


def test_cpp_consumer_multi_index_sets_match_reference(tmp_path):
    """The C++ API's MultiIndexSet (host only) gives the reference's
    MultiIndexSet report on the random cases tests/test_multi_index.py uses."""
    from oracle import ref
    if not ref.available():
        pytest.skip("reference checkout not present")
    from test_multi_index import _random_terms, _spec
    exe = build_consumer(str(tmp_path))
    rng = np.random.default_rng(11)
    cases, want = [], []
    for dim in (1, 2, 3, 4):
        for mode in (0, 1, 2, 3):
            for _ in range(12):
                kind, u, w = _spec(rng, dim)
                terms = _random_terms(rng, dim, int(rng.integers(1, 7)))
                order = int(rng.integers(0, 4)) if mode != 2 else int(rng.integers(0, 3))
                want.append(ref.mset_report(dim, terms, mode, order, kind, u, w))
                flat = [v for t in terms for v in t]
                cases.append(" ".join(str(v) for v in [dim, mode, order, kind, *u, len(w)]) + " " +
                             " ".join(repr(float(x)) for x in w) + " " +
                             " ".join(str(v) for v in [len(terms), *flat]))
    spec = tmp_path / "specs.txt"
    spec.write_text("\n".join(cases) + "\n")
    rep = tmp_path / "reports.txt"
    res = subprocess.run([exe, "mset", str(spec), str(rep)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    got = rep.read_text().split("====\n")[:-1]
    assert len(got) == len(want) == 192
    for k, (g, w) in enumerate(zip(got, want)):
        assert g == w, (k, cases[k])


@pytest.mark.gpu
def test_cpp_consumer_train_map_adaptive(tmp_path, oracle):
    """MParT's adaptive training through the C++ API (MultiIndexSet,
    ATMOptions, TrainMapAdaptive): the sets come back as the returned map's
    components' sets, no larger than maxSize, and the map's training error
    is the oracle's KL objective at its coefficients."""
    O = oracle
    exe = build_consumer(str(tmp_path))
    n = 2000
    rng = np.random.default_rng(6)
    x1 = rng.standard_normal(n)
    x = np.stack([x1, x1 ** 2 + 0.5 * rng.standard_normal(n)])
    inp = os.path.join(str(tmp_path), "atm_in.bin")
    out = os.path.join(str(tmp_path), "atm_out.bin")
    with open(inp, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())
    res = subprocess.run([exe, "atm", inp, out], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    v = list(np.fromfile(out, dtype=np.float64))
    sets = []
    for j in range(2):
        k = int(v.pop(0))
        sets.append([[int(v.pop(0)) for _ in range(j + 1)] for _ in range(k)])
    coef, train, same = np.array(v[:-2]), v[-2], v[-1]
    assert same == 1.0
    assert sum(len(s) for s in sets) <= 8 and coef.size == sum(len(s) for s in sets)
    comps, off, kl = [], 0, np.log(2.0 * np.pi)
    for j, s in enumerate(sets):
        starts, dims, orders = [0], [], []
        for t in s:
            for d, o in enumerate(t):
                if o:
                    dims.append(d)
                    orders.append(o)
            starts.append(len(dims))
        c = O.OracleComponent(j + 1, np.array(starts, np.uint32), np.array(dims, np.uint32),
                              np.array(orders, np.uint32), basis=O.BASIS_HERMITE_FUNCTIONS, normalize=True,
                              posfunc=O.POS_EXP, abs_tol=1e-7, rel_tol=1e-7)
        kl += O.fast_gaussian_reverse_kl(c, coef[off:off + len(s)], x[:j + 1])[0]
        off += len(s)
    assert train == pytest.approx(kl, rel=1e-10)
