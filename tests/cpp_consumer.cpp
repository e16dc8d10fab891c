// A C++ consumer of the library's boundary, compiled by g++ against the
// installed headers and libmpart_gb300.so (tests/test_cpp_consumer.py):
//
//  * route 1, the C++ API of include/mpart_gb300.hpp, as MParT host code uses
//    its own classes: MapFactory::CreateTriangular, SetCoeffs and the
//    EvaluateImpl / LogDeterminantImpl / CoeffGradImpl / InverseImpl methods
//    (MParT/MapFactory.h, MParT/ConditionalMapBase.h);
//  * route 2, an adapter of the shape INTEGRATION.md shows for MParT's
//    ConditionalMapBase<DeviceSpace>: it keeps an mpgb_map* and forwards
//    each *Impl method to the C ABI of include/mpart_gb300.h.  DView stands
//    in for the reference's StridedMatrix / StridedVector device views; the
//    adapter uses only their data(), extent() and stride_0/1() members.
//
// Usage: cpp_consumer <in.bin> <out.bin>
//   in.bin : int64 N, then 14 coefficients, x (2 x N), sens (2 x N) and
//            r (2 x N, targets), row-major float64
//   out.bin: per route, T (2 x N), log-det (N), CoeffGrad (14 x N) and
//            Inverse(r) (2 x N); then T (2 x N) of route 1's map after
//            Save / Load
// (and the train, mset and atm modes below)
// The map is the 2 x 2 TriangularMap of total order 3, ProbabilistHermite +
// SoftPlus, AdaptiveClenshawCurtis with tolerances 1e-6.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpart_gb300.h"
#include "mpart_gb300.hpp"

namespace {

void cuda(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

struct Dev {
    double* p = nullptr;
    size_t n = 0;
    explicit Dev(size_t count) : n(count) { cuda(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(double))); }
    Dev(const std::vector<double>& h) : Dev(h.size()) {
        cuda(cudaMemcpy(p, h.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    }
    ~Dev() { cudaFree(p); }
    std::vector<double> host() const {
        std::vector<double> h(n);
        cuda(cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
        return h;
    }
};

// Stand-in for a Kokkos LayoutStride device view.
struct DView {
    double* p;
    int64_t e0, e1, s0, s1;
    double* data() const { return p; }
    int64_t extent(int i) const { return i == 0 ? e0 : e1; }
    int64_t stride_0() const { return s0; }
    int64_t stride_1() const { return s1; }
};

// The adapter of INTEGRATION.md (section 1), over the C ABI.
class GB300Map {
    mpgb_map* h_ = nullptr;
    static mpgb_matrix M(DView const& v) { return {v.data(), v.extent(0), v.extent(1), v.stride_0(), v.stride_1()}; }
    static void ok(int rc) {
        if (rc == MPGB_ERR_INVALID_ARGUMENT) throw std::invalid_argument(mpgb_last_error());
        if (rc != MPGB_OK) throw std::runtime_error(mpgb_last_error());
    }

public:
    GB300Map(unsigned in, unsigned out, unsigned order, mpgb::MapOptions const& o) {
        mpgb_map_options c;
        ok(mpgb_map_options_default(&c));
        c.basis_type = (int)o.basisType;
        c.pos_func_type = (int)o.posFuncType;
        c.quad_type = (int)o.quadType;
        c.quad_abs_tol = o.quadAbsTol;
        c.quad_rel_tol = o.quadRelTol;
        c.quad_max_sub = o.quadMaxSub;
        c.quad_min_sub = o.quadMinSub;
        c.quad_pts = o.quadPts;
        c.basis_norm = o.basisNorm;
        c.nugget = o.nugget;
        ok(mpgb_create_triangular(in, out, order, &c, &h_));
    }
    ~GB300Map() { mpgb_map_destroy(h_); }
    void SetCoeffs(DView const& c) { ok(mpgb_set_coeffs(h_, c.data(), (unsigned)c.extent(0), 0, nullptr)); }
    void EvaluateImpl(DView const& pts, DView const& out) { ok(mpgb_evaluate(h_, M(pts), M(out), nullptr)); }
    void LogDeterminantImpl(DView const& pts, DView const& out) {
        mpgb_matrix o{out.data(), 1, out.extent(0), out.extent(0), out.stride_0()};
        ok(mpgb_log_determinant(h_, M(pts), o, nullptr));
    }
    void CoeffGradImpl(DView const& pts, DView const& sens, DView const& out) {
        ok(mpgb_coeff_grad(h_, M(pts), M(sens), M(out), nullptr));
    }
    void InverseImpl(DView const& x1, DView const& r, DView const& out) {
        ok(mpgb_inverse(h_, M(x1), M(r), M(out), 1e-6, 1e-6, nullptr, nullptr));
    }
};

}  // namespace

// cpp_consumer train <in.bin> <out.bin>
//   in.bin : int64 N, then samples (2 x N) row-major float64
//   out.bin: the 14 trained coefficients, TrainMap's return value and
//            KLObjective::TestError on the same samples
// MParT's training through the C++ API (MParT/TrainMap.h, MParT/MapObjective.h):
// KLObjective over device samples, TrainOptions with L-BFGS, TrainMap.
static int trainMain(const char* in, const char* outPath) {
    FILE* f = std::fopen(in, "rb");
    if (!f) throw std::runtime_error("cannot open input");
    int64_t N = 0;
    if (std::fread(&N, sizeof N, 1, f) != 1) throw std::runtime_error("bad input");
    std::vector<double> x(2 * N);
    const bool good = std::fread(x.data(), 8, 2 * N, f) == (size_t)(2 * N);
    std::fclose(f);
    if (!good) throw std::runtime_error("short input");
    mpgb::MapOptions o;
    o.basisType = mpgb::BasisTypes::HermiteFunctions;
    o.posFuncType = mpgb::PosFuncTypes::Exp;
    o.quadType = mpgb::QuadTypes::AdaptiveClenshawCurtis;
    o.quadAbsTol = o.quadRelTol = 1e-7;
    Dev dx(x);
    auto map = mpgb::MapFactory::CreateTriangular(2, 2, 3, o);
    std::vector<double> zero(map->numCoeffs, 0.0);
    Dev dc(zero);
    map->SetCoeffs(dc.p, map->numCoeffs);
    const auto S = mpgb::StridedMatrix::RowMajor(dx.p, 2, N);
    mpgb::KLObjective obj(S, S);
    mpgb::TrainOptions t;
    t.opt_alg = "LD_LBFGS";
    t.opt_maxeval = 30;
    const double train = mpgb::TrainMap(map, obj, t);
    const double test = obj.TestError(map);
    std::vector<double> out(map->numCoeffs);
    cuda(cudaMemcpy(out.data(), map->Coeffs(), out.size() * sizeof(double), cudaMemcpyDeviceToHost));
    out.push_back(train);
    out.push_back(test);
    FILE* g = std::fopen(outPath, "wb");
    if (!g || std::fwrite(out.data(), 8, out.size(), g) != out.size()) throw std::runtime_error("cannot write output");
    std::fclose(g);
    return 0;
}

// cpp_consumer mset <specs.txt> <reports.txt>   (host only)
//   specs: one case per line, "dim mode order kind u0 u1 u2 nw w[nw] nt
//   t[nt * dim]"; reports: for each case the report of the MultiIndexSet of
//   the C++ API, in the format of the reference driver's ref_mset_report
//   (oracle/ref_driver.cpp), cases separated by "====" lines.  mode 0 adds the
//   terms under the limiter, 1 CreateTotalOrder, 2 CreateTensorProduct, 3 adds
//   them and calls SetLimiter; limiter kinds as in ref_mset_report.
static std::string msetReport(unsigned dim, int mode, unsigned order, int kind, const unsigned* u,
                              std::vector<double> const& w, std::vector<unsigned> const& t) {
    namespace L = mpgb::MultiIndexLimiter;
    using mpgb::MultiIndex;
    using mpgb::MultiIndexSet;
    mpgb::LimiterType lim;
    switch (kind) {
        case 0: lim = L::None(); break;
        case 1: lim = L::TotalOrder(u[0]); break;
        case 2: lim = L::Dimension(u[0], u[1]); break;
        case 3: lim = L::Anisotropic(std::vector<double>(w.begin(), w.begin() + dim), w[dim]); break;
        case 4: lim = L::MaxDegree(u[0], dim); break;
        case 5: lim = L::Separable(); break;
        case 6: lim = L::NonzeroDiag(); break;
        case 7: lim = L::And(L::TotalOrder(u[0]), L::MaxDegree(u[1], dim)); break;
        case 8: lim = L::Or(L::Dimension(u[0], u[1]), L::TotalOrder(u[2])); break;
        case 9: lim = L::Xor(L::TotalOrder(u[0]), L::NonzeroDiag()); break;
        default: throw std::invalid_argument("unknown limiter kind");
    }
    const size_t nt = t.size() / dim;
    auto term = [&](size_t k) { return MultiIndex(std::vector<unsigned>(t.begin() + k * dim, t.begin() + (k + 1) * dim)); };
    std::ostringstream os;
    MultiIndexSet s(dim);
    if (mode == 1) {
        s = MultiIndexSet::CreateTotalOrder(dim, order, lim);
    } else if (mode == 2) {
        s = MultiIndexSet::CreateTensorProduct(dim, order, lim);
    } else if (mode == 0) {
        s = MultiIndexSet(dim, lim);
        for (size_t k = 0; k < nt; ++k) s += term(k);
    } else {
        for (size_t k = 0; k < nt; ++k) s += term(k);
        try {
            s.SetLimiter(lim);
        } catch (std::invalid_argument const&) {
            os << "setlimiter rejected\n";
        }
    }
    auto multis = [](std::vector<MultiIndex> const& v) {
        std::string r;
        for (size_t k = 0; k < v.size(); ++k) r += (k ? ";" : "") + v[k].String();
        return r;
    };
    auto ints = [](std::vector<unsigned> const& v) {
        std::string r;
        for (size_t k = 0; k < v.size(); ++k) r += (k ? "," : "") + std::to_string(v[k]);
        return r;
    };
    auto termsOf = [&](MultiIndexSet const& x) {
        std::vector<MultiIndex> v;
        for (unsigned k = 0; k < x.Size(); ++k) v.push_back(x.IndexToMulti(k));
        return multis(v);
    };
    os << "size " << s.Size() << "\n";
    os << "terms " << termsOf(s) << "\n";
    os << "maxorders " << ints(s.MaxOrders()) << "\n";
    os << "frontier " << ints(s.Frontier()) << "\n";
    os << "strict " << ints(s.StrictFrontier()) << "\n";
    const auto margin = s.Margin();
    os << "margin " << multis(margin) << "\n";
    os << "rmargin " << multis(s.ReducedMargin()) << "\n";
    for (unsigned d = 0; d < dim; ++d) os << "rmargin_dim" << d << " " << multis(s.ReducedMarginDim(d)) << "\n";
    std::vector<unsigned> ex, nf, na, adm;
    for (unsigned k = 0; k < s.Size(); ++k) {
        ex.push_back(s.IsExpandable(k));
        nf.push_back(s.NumForward(k));
        na.push_back(s.NumActiveForward(k));
    }
    os << "expandable " << ints(ex) << "\n";
    os << "nforward " << ints(nf) << "\n";
    os << "nactiveforward " << ints(na) << "\n";
    os << "nzdiag " << ints(s.NonzeroDiagonalEntries()) << "\n";
    for (auto const& m : margin) adm.push_back(s.IsAdmissible(m));
    os << "margin_admissible " << ints(adm) << "\n";
    {
        MultiIndexSet c = s;
        const auto ix = c.Expand();
        os << "expand " << ints(ix) << " | " << termsOf(c) << "\n";
    }
    for (unsigned k = 0; k < s.Size(); ++k) {
        MultiIndexSet c = s;
        os << "expand" << k << " " << ints(c.Expand(k)) << "\n";
    }
    {
        MultiIndexSet c = s;
        const unsigned added = c.Union(MultiIndexSet::CreateTotalOrder(dim, 1));
        os << "union " << added << " | " << termsOf(c) << "\n";
    }
    return os.str();
}

static int msetMain(const char* in, const char* outPath) {
    std::ifstream f(in);
    std::ofstream g(outPath);
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty()) continue;
        std::istringstream ls(line);
        unsigned dim, order, u[3], nw, nt;
        int mode, kind;
        ls >> dim >> mode >> order >> kind >> u[0] >> u[1] >> u[2] >> nw;
        std::vector<double> w(nw);
        for (auto& x : w) ls >> x;
        ls >> nt;
        std::vector<unsigned> t((size_t)nt * dim);
        for (auto& x : t) ls >> x;
        if (!ls) throw std::runtime_error("bad spec line");
        g << msetReport(dim, mode, order, kind, u, w, t) << "====\n";
    }
    return g ? 0 : 1;
}

// cpp_consumer atm <in.bin> <out.bin>
//   in.bin : int64 N, then samples (2 x N) row-major float64
//   out.bin: per output j, the number of terms and the terms (dim j+1 each),
//            as float64, then the trained coefficients, KLObjective::TrainError
//            of the returned map, and 1 when mset0 came back equal to the
//            components' multi-index sets (else 0)
// MParT's adaptive training through the C++ API (MParT/TrainMapAdaptive.h):
// total-order-1 starting sets, HermiteFunctions + Exp, L-BFGS, maxSize 8.
static int atmMain(const char* in, const char* outPath) {
    FILE* f = std::fopen(in, "rb");
    if (!f) throw std::runtime_error("cannot open input");
    int64_t N = 0;
    if (std::fread(&N, sizeof N, 1, f) != 1) throw std::runtime_error("bad input");
    std::vector<double> x(2 * N);
    const bool good = std::fread(x.data(), 8, 2 * N, f) == (size_t)(2 * N);
    std::fclose(f);
    if (!good) throw std::runtime_error("short input");
    Dev dx(x);
    const auto S = mpgb::StridedMatrix::RowMajor(dx.p, 2, N);
    mpgb::KLObjective obj(S, S);
    std::vector<mpgb::MultiIndexSet> msets;
    for (unsigned d = 0; d < 2; ++d) msets.push_back(mpgb::MultiIndexSet::CreateTotalOrder(d + 1, 1));
    mpgb::ATMOptions o;
    o.basisType = mpgb::BasisTypes::HermiteFunctions;
    o.posFuncType = mpgb::PosFuncTypes::Exp;
    o.quadType = mpgb::QuadTypes::AdaptiveClenshawCurtis;
    o.quadAbsTol = o.quadRelTol = 1e-7;
    o.opt_alg = "LD_LBFGS";
    o.opt_maxeval = 40;
    o.maxSize = 8;
    auto map = mpgb::TrainMapAdaptive(msets, obj, o);
    auto* tm = dynamic_cast<mpgb::TriangularMap*>(map.get());
    if (!tm) throw std::runtime_error("TrainMapAdaptive did not return a TriangularMap");
    std::vector<double> out;
    bool same = true;
    for (unsigned j = 0; j < 2; ++j) {
        const auto& s = msets[j];
        out.push_back(s.Size());
        for (unsigned k = 0; k < s.Size(); ++k)
            for (unsigned v : s.IndexToMulti(k).Vector()) out.push_back(v);
        auto* c = dynamic_cast<mpgb::MonotoneComponent*>(tm->GetComponent(j).get());
        const auto fx = s.Fix();
        same = same && c && c->GetMultiIndexSet().nzStarts == fx.nzStarts && c->GetMultiIndexSet().nzDims == fx.nzDims &&
               c->GetMultiIndexSet().nzOrders == fx.nzOrders;
    }
    std::vector<double> coef(map->numCoeffs);
    cuda(cudaMemcpy(coef.data(), map->Coeffs(), coef.size() * sizeof(double), cudaMemcpyDeviceToHost));
    out.insert(out.end(), coef.begin(), coef.end());
    out.push_back(obj.TrainError(map));
    out.push_back(same ? 1.0 : 0.0);
    FILE* g = std::fopen(outPath, "wb");
    if (!g || std::fwrite(out.data(), 8, out.size(), g) != out.size()) throw std::runtime_error("cannot write output");
    std::fclose(g);
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 4 && (std::string(argv[1]) == "train" || std::string(argv[1]) == "mset" ||
                      std::string(argv[1]) == "atm")) {
        try {
            const std::string m = argv[1];
            return m == "train" ? trainMain(argv[2], argv[3])
                   : m == "mset" ? msetMain(argv[2], argv[3])
                                 : atmMain(argv[2], argv[3]);
        } catch (std::exception const& e) {
            std::fprintf(stderr, "cpp_consumer: %s\n", e.what());
            return 1;
        }
    }
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.bin out.bin | %s train in.bin out.bin\n", argv[0], argv[0]);
        return 2;
    }
    try {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) throw std::runtime_error("cannot open input");
        int64_t N = 0;
        if (std::fread(&N, sizeof N, 1, f) != 1) throw std::runtime_error("bad input");
        const int nc = 14;
        std::vector<double> coef(nc), x(2 * N), sens(2 * N), r(2 * N);
        bool good = std::fread(coef.data(), 8, nc, f) == (size_t)nc && std::fread(x.data(), 8, 2 * N, f) == (size_t)(2 * N) &&
                    std::fread(sens.data(), 8, 2 * N, f) == (size_t)(2 * N) && std::fread(r.data(), 8, 2 * N, f) == (size_t)(2 * N);
        std::fclose(f);
        if (!good) throw std::runtime_error("short input");

        mpgb::MapOptions o;
        o.quadType = mpgb::QuadTypes::AdaptiveClenshawCurtis;
        o.quadAbsTol = o.quadRelTol = 1e-6;
        Dev dc(coef), dx(x), ds(sens), dr(r);
        std::vector<double> out, reloaded;
        auto append = [&](const Dev& d) {
            auto h = d.host();
            out.insert(out.end(), h.begin(), h.end());
        };

        // Route 1: the C++ API.
        {
            auto map = mpgb::MapFactory::CreateTriangular(2, 2, 3, o);
            if (map->numCoeffs != (unsigned)nc) throw std::runtime_error("unexpected number of coefficients");
            map->SetCoeffs(dc.p, nc);
            Dev T(2 * N), ld(N), cg((size_t)nc * N), xi(2 * N);
            const auto P = mpgb::StridedMatrix::RowMajor(dx.p, 2, N);
            map->EvaluateImpl(P, mpgb::StridedMatrix::RowMajor(T.p, 2, N));
            map->LogDeterminantImpl(P, mpgb::StridedMatrix::RowMajor(ld.p, 1, N));
            map->CoeffGradImpl(P, mpgb::StridedMatrix::RowMajor(ds.p, 2, N), mpgb::StridedMatrix::RowMajor(cg.p, nc, N));
            map->InverseImpl(mpgb::StridedMatrix(nullptr, 0, N, N, 1), mpgb::StridedMatrix::RowMajor(dr.p, 2, N),
                             mpgb::StridedMatrix::RowMajor(xi.p, 2, N));
            append(T);
            append(ld);
            append(cg);
            append(xi);
            // ParameterizedFunctionBase::Save / Load: the reloaded map evaluates
            // the same points (appended after both routes).
            std::stringstream ss;
            map->Save(ss);
            auto back = mpgb::ParameterizedFunctionBase::Load(ss);
            Dev T2(2 * N);
            back->EvaluateImpl(P, mpgb::StridedMatrix::RowMajor(T2.p, 2, N));
            reloaded = T2.host();
        }
        // Route 2: the adapter over the C ABI.
        {
            GB300Map map(2, 2, 3, o);
            map.SetCoeffs(DView{dc.p, nc, 1, 1, 1});
            Dev T(2 * N), ld(N), cg((size_t)nc * N), xi(2 * N);
            const DView P{dx.p, 2, N, N, 1};
            map.EvaluateImpl(P, DView{T.p, 2, N, N, 1});
            map.LogDeterminantImpl(P, DView{ld.p, N, 1, 1, 1});
            map.CoeffGradImpl(P, DView{ds.p, 2, N, N, 1}, DView{cg.p, nc, N, N, 1});
            map.InverseImpl(DView{nullptr, 0, N, N, 1}, DView{dr.p, 2, N, N, 1}, DView{xi.p, 2, N, N, 1});
            append(T);
            append(ld);
            append(cg);
            append(xi);
        }
        out.insert(out.end(), reloaded.begin(), reloaded.end());
        FILE* g = std::fopen(argv[2], "wb");
        if (!g || std::fwrite(out.data(), 8, out.size(), g) != out.size()) throw std::runtime_error("cannot write output");
        std::fclose(g);
    } catch (std::exception const& e) {
        std::fprintf(stderr, "cpp_consumer: %s\n", e.what());
        return 1;
    }
    return 0;
}
