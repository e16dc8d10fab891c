// ORACLE -- test infrastructure only.
//
// C entry points over MParT's own map classes, compiled from the reference's
// sources unchanged (oracle/ref.mk builds this file together with
// src/ParameterizedFunctionBase.cpp, src/ConditionalMapBase.cpp,
// src/TriangularMap.cpp, src/MapFactoryImpl{4..9}.cpp, src/MultiIndices/*.cpp
// and src/Utilities/Miscellaneous.cpp against the Kokkos and Eigen stand-ins
// in oracle/ref_shim/).  Everything numeric -- the basis recurrences, the
// expansion worker's caches and term loops, the MonotoneIntegrand, the
// adaptive quadratures, the root finder, the TriangularMap component loops --
// is the reference's code; this file only builds maps the way
// MapFactory::CreateTriangular / CreateComponent do and forwards to the
// maps' *Impl methods.  The tests use it to pin the oracle's C++ restatement
// (and so the GPU) to the reference itself.
//
// Matrices are row-major rows x N arrays (coordinate d of point i at
// d * N + i), the layout the reference's Python binding passes.
#include <cstdio>
#include <cstring>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "MParT/ConditionalMapBase.h"
#include "MParT/HermiteFunction.h"
#include "MParT/MapFactory.h"
#include "MParT/MapOptions.h"
#include "MParT/MonotoneComponent.h"
#include "MParT/MultiIndices/FixedMultiIndexSet.h"
#include "MParT/MultiIndices/MultiIndexLimiter.h"
#include "MParT/MultiIndices/MultiIndexSet.h"
#include "MParT/MultivariateExpansionWorker.h"
#include "MParT/OrthogonalPolynomial.h"
#include "MParT/PositiveBijectors.h"
#include "MParT/Quadrature.h"
#include "MParT/RectifiedMultivariateExpansion.h"
#include "MParT/Sigmoid.h"
#include "MParT/TriangularMap.h"
#include "MParT/UnivariateExpansion.h"

using namespace mpart;
using Host = Kokkos::HostSpace;
using Map = ConditionalMapBase<Host>;

namespace {

thread_local std::string g_err;

struct RefMap {
    std::shared_ptr<Map> map;                 // the object the calls go to
    std::vector<std::shared_ptr<Map>> comps;  // its components (one for a single component)
};

template <class F>
int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (std::exception const& e) {
        g_err = e.what();
        return -1;
    }
}

MapOptions options(int basis, int basisNorm, int pos, int quad, double absTol, double relTol, unsigned maxSub,
                   unsigned minSub, unsigned quadPts, double nugget, int contDeriv) {
    MapOptions o;
    o.basisType = (BasisTypes)basis;
    o.basisNorm = basisNorm != 0;
    o.posFuncType = (PosFuncTypes)pos;
    o.quadType = (QuadTypes)quad;
    o.quadAbsTol = absTol;
    o.quadRelTol = relTol;
    o.quadMaxSub = maxSub;
    o.quadMinSub = minSub;
    o.quadPts = quadPts;
    o.nugget = nugget;
    o.contDeriv = contDeriv != 0;
    return o;
}

StridedMatrix<const double, Host> cmat(const double* p, long rows, long n) {
    return StridedMatrix<const double, Host>(p, Kokkos::LayoutStride(rows, n, n, 1));
}
StridedMatrix<double, Host> mat(double* p, long rows, long n) {
    return StridedMatrix<double, Host>(p, Kokkos::LayoutStride(rows, n, n, 1));
}

// MonotoneComponent::InverseImpl with the "xtol" / "ytol" options
// (MonotoneComponent.h:330-443) for each concrete component type the
// factory registrations in MapFactoryImpl{4..9}.cpp create.
template <class Basis, class Pos, class Quad>
using Comp = MonotoneComponent<MultivariateExpansionWorker<BasisEvaluator<BasisHomogeneity::Homogeneous, Basis>, Host>,
                               Pos, Quad, Host>;

template <class C>
bool tryInverse(Map* m, StridedMatrix<const double, Host> const& x, StridedVector<const double, Host> const& r,
                StridedVector<double, Host> out, std::map<std::string, std::string> const& opts) {
    C* c = dynamic_cast<C*>(m);
    if (!c) return false;
    StridedVector<const double, Host> coeffs = c->Coeffs();
    c->InverseImpl(x, r, coeffs, out, opts);
    return true;
}

template <class... Cs>
void inverseAny(Map* m, StridedMatrix<const double, Host> const& x, StridedVector<const double, Host> const& r,
                StridedVector<double, Host> out, std::map<std::string, std::string> const& opts) {
    if (!(tryInverse<Cs>(m, x, r, out, opts) || ...)) throw std::runtime_error("unsupported component type");
}

void componentInverse(Map* m, StridedMatrix<const double, Host> const& x, StridedVector<const double, Host> const& r,
                      StridedVector<double, Host> out, std::map<std::string, std::string> const& opts) {
    inverseAny<Comp<ProbabilistHermite, SoftPlus, AdaptiveClenshawCurtis<Host>>,
               Comp<ProbabilistHermite, Exp, AdaptiveClenshawCurtis<Host>>,
               Comp<HermiteFunction, SoftPlus, AdaptiveClenshawCurtis<Host>>,
               Comp<HermiteFunction, Exp, AdaptiveClenshawCurtis<Host>>,
               Comp<ProbabilistHermite, SoftPlus, AdaptiveSimpson<Host>>,
               Comp<ProbabilistHermite, Exp, AdaptiveSimpson<Host>>,
               Comp<HermiteFunction, SoftPlus, AdaptiveSimpson<Host>>,
               Comp<HermiteFunction, Exp, AdaptiveSimpson<Host>>,
               Comp<ProbabilistHermite, SoftPlus, ClenshawCurtisQuadrature<Host>>,
               Comp<ProbabilistHermite, Exp, ClenshawCurtisQuadrature<Host>>,
               Comp<HermiteFunction, SoftPlus, ClenshawCurtisQuadrature<Host>>,
               Comp<HermiteFunction, Exp, ClenshawCurtisQuadrature<Host>>>(m, x, r, out, opts);
}

}  // namespace

// A sigmoid expansion as MapFactory::CreateSigmoidComponent builds one
// (CreateSigmoidExpansionTemplate, src/MapFactory.cpp:258-281): Sigmoid1d
// with SoftPlus edges from the given centers, widths and weights (the
// factory's CreateSigmoid computes those; MapFactory.cpp is not compiled
// here), then for one input UnivariateExpansion<Sigmoid1d> with maxOrder =
// numTerms - 1, otherwise RectifiedMultivariateExpansion with
// HermiteFunction off the diagonal and the positive bijector `pos` (Exp 0,
// SoftPlus 1) as rectifier, over the compressed multi-index set.  sumType:
// Linear 0, Constant 1.  Zero coefficients.
template <class Rect>
std::shared_ptr<Map> sigmoidExpansion(unsigned dim, FixedMultiIndexSet<Host> const& mset,
                                      Kokkos::View<double*, Host> c, Kokkos::View<double*, Host> w,
                                      Kokkos::View<double*, Host> wt, SigmoidSumSizeType sumType) {
    using Sig = Sigmoid1d<Host, SigmoidTypeSpace::Logistic, SoftPlus>;
    Sig sigmoid(c, w, wt, sumType);
    if (dim == 1) return std::make_shared<UnivariateExpansion<Host, Sig>>(mset.Size() - 1, sigmoid);
    using Eval = BasisEvaluator<BasisHomogeneity::OffdiagHomogeneous, Kokkos::pair<HermiteFunction, Sig>, Rect>;
    Eval basisEval(dim, HermiteFunction(), sigmoid);
    MultivariateExpansionWorker<Eval, Host> worker(mset, basisEval);
    return std::make_shared<RectifiedMultivariateExpansion<Host, HermiteFunction, Sig, Rect>>(worker);
}


// Runs write on a cereal binary archive in memory; *size receives the archive
// size and buf (cap bytes) the bytes when large enough.
template <class F>
int archiveTo(unsigned char* buf, size_t cap, size_t* size, F&& write) {
    return guard([&] {
        std::stringstream ss;
        {
            cereal::BinaryOutputArchive ar(ss);
            write(ar);
        }
        const std::string b = ss.str();
        *size = b.size();
        if (buf && cap >= b.size()) std::memcpy(buf, b.data(), b.size());
    });
}

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// MapFactory::CreateTriangular (src/MapFactory.cpp:105-124): component i has
// the total-order set of dimension i + extra + 1, made by the registered
// factory function for the options (MapFactory::CreateComponent,
// src/MapFactory.cpp:22-27); zero coefficients.
void* ref_triangular(unsigned inputDim, unsigned outputDim, unsigned totalOrder, int basis, int basisNorm, int pos,
                     int quad, double absTol, double relTol, unsigned maxSub, unsigned minSub, unsigned quadPts,
                     double nugget, int contDeriv) {
    RefMap* out = nullptr;
    guard([&] {
        const MapOptions o = options(basis, basisNorm, pos, quad, absTol, relTol, maxSub, minSub, quadPts, nugget,
                                     contDeriv);
        auto* r = new RefMap;
        const unsigned extra = inputDim - outputDim;
        for (unsigned i = 0; i < outputDim; ++i) {
            FixedMultiIndexSet<Host> mset(i + extra + 1, totalOrder);
            r->comps.push_back(MapFactory::CompFactoryImpl<Host>::GetFactoryFunction(o)(mset, o));
        }
        r->map = std::make_shared<TriangularMap<Host>>(r->comps);
        Kokkos::View<const double*, Host> coeffs = Kokkos::View<double*, Host>("Component Coefficients",
                                                                                 r->map->numCoeffs);
        r->map->SetCoeffs(coeffs);
        out = r;
    });
    return out;
}

// MapFactory::CreateComponent on a compressed multi-index set
// (FixedMultiIndexSet(dim, nzStarts, nzDims, nzOrders)).
void* ref_component(unsigned dim, unsigned numTerms, const unsigned* starts, const unsigned* dims,
                    const unsigned* orders, int basis, int basisNorm, int pos, int quad, double absTol,
                    double relTol, unsigned maxSub, unsigned minSub, unsigned quadPts, double nugget, int contDeriv) {
    RefMap* out = nullptr;
    guard([&] {
        const MapOptions o = options(basis, basisNorm, pos, quad, absTol, relTol, maxSub, minSub, quadPts, nugget,
                                     contDeriv);
        const unsigned nnz = starts[numTerms];
        Kokkos::View<unsigned*, Host> s("nzStarts", numTerms + 1), d("nzDims", nnz), r("nzOrders", nnz);
        for (unsigned i = 0; i <= numTerms; ++i) s(i) = starts[i];
        for (unsigned i = 0; i < nnz; ++i) {
            d(i) = dims[i];
            r(i) = orders[i];
        }
        FixedMultiIndexSet<Host> mset(dim, s, d, r);
        auto* m = new RefMap;
        m->map = MapFactory::CompFactoryImpl<Host>::GetFactoryFunction(o)(mset, o);
        m->comps.push_back(m->map);
        Kokkos::View<const double*, Host> coeffs = Kokkos::View<double*, Host>("Component Coefficients",
                                                                                 m->map->numCoeffs);
        m->map->SetCoeffs(coeffs);
        out = m;
    });
    return out;
}

void* ref_sigmoid(unsigned dim, unsigned numTerms, const unsigned* starts, const unsigned* dims,
                  const unsigned* orders, const double* centers, const double* widths, const double* weights,
                  unsigned nCenters, int sumType, int pos) {
    RefMap* out = nullptr;
    guard([&] {
        const unsigned nnz = starts[numTerms];
        Kokkos::View<unsigned*, Host> s("nzStarts", numTerms + 1), d("nzDims", nnz), r("nzOrders", nnz);
        for (unsigned i = 0; i <= numTerms; ++i) s(i) = starts[i];
        for (unsigned i = 0; i < nnz; ++i) {
            d(i) = dims[i];
            r(i) = orders[i];
        }
        FixedMultiIndexSet<Host> mset(dim, s, d, r);
        Kokkos::View<double*, Host> c("centers", nCenters), w("widths", nCenters), wt("weights", nCenters);
        for (unsigned i = 0; i < nCenters; ++i) {
            c(i) = centers[i];
            w(i) = widths[i];
            wt(i) = weights[i];
        }
        const SigmoidSumSizeType st = sumType ? SigmoidSumSizeType::Constant : SigmoidSumSizeType::Linear;
        auto* m = new RefMap;
        m->map = pos ? sigmoidExpansion<SoftPlus>(dim, mset, c, w, wt, st) : sigmoidExpansion<Exp>(dim, mset, c, w, wt, st);
        m->comps.push_back(m->map);
        Kokkos::View<const double*, Host> coeffs = Kokkos::View<double*, Host>("Component Coefficients",
                                                                                 m->map->numCoeffs);
        m->map->SetCoeffs(coeffs);
        out = m;
    });
    return out;
}

void ref_free(void* h) { delete (RefMap*)h; }

// ParameterizedFunctionBase::Save (ParameterizedFunctionBase.h:197-202), the
// archive of the reference's ToBytes / pickle
// (bindings/python/src/ParameterizedFunctionBase.cpp:57-61), through the
// cereal stand-in.  *size receives the archive's size; the bytes are written
// when cap holds at least that many.
int ref_to_bytes(void* h, unsigned char* buf, size_t cap, size_t* size) {
    return guard([&] {
        std::stringstream ss;
        ((RefMap*)h)->map->Save(ss);
        const std::string b = ss.str();
        *size = b.size();
        if (buf && cap >= b.size()) std::memcpy(buf, b.data(), b.size());
    });
}

// The Python binding's Serialize methods write these archives to a file;
// here the same archive calls go to memory: MapOptions
// (bindings/python/src/MapOptions.cpp:74-78), FixedMultiIndexSet
// (bindings/python/src/MultiIndex.cpp:243-248; compressed from nz arrays, or
// uncompressed from every term's dim orders when dims is null) and the
// coefficient archive (bindings/python/src/ParameterizedFunctionBase.cpp:51-56).
int ref_options_bytes(int basis, int basisNorm, int pos, int quad, double absTol, double relTol, unsigned maxSub,
                      unsigned minSub, unsigned quadPts, double nugget, int contDeriv, unsigned char* buf, size_t cap,
                      size_t* size) {
    return archiveTo(buf, cap, size, [&](cereal::BinaryOutputArchive& ar) {
        const MapOptions o = options(basis, basisNorm, pos, quad, absTol, relTol, maxSub, minSub, quadPts, nugget,
                                     contDeriv);
        ar(o);
    });
}

int ref_mset_bytes(unsigned dim, unsigned numTerms, const unsigned* starts, const unsigned* dims,
                   const unsigned* orders, unsigned char* buf, size_t cap, size_t* size) {
    return archiveTo(buf, cap, size, [&](cereal::BinaryOutputArchive& ar) {
        if (dims) {
            const unsigned nnz = starts[numTerms];
            Kokkos::View<unsigned*, Host> s("nzStarts", numTerms + 1), d("nzDims", nnz), r("nzOrders", nnz);
            for (unsigned i = 0; i <= numTerms; ++i) s(i) = starts[i];
            for (unsigned i = 0; i < nnz; ++i) {
                d(i) = dims[i];
                r(i) = orders[i];
            }
            ar(FixedMultiIndexSet<Host>(dim, s, d, r));
        } else {
            Kokkos::View<unsigned*, Host> r("orders", (size_t)numTerms * dim);
            for (size_t i = 0; i < (size_t)numTerms * dim; ++i) r(i) = orders[i];
            ar(FixedMultiIndexSet<Host>(dim, r));
        }
    });
}

int ref_coeff_archive(void* h, unsigned char* buf, size_t cap, size_t* size) {
    return archiveTo(buf, cap, size, [&](cereal::BinaryOutputArchive& ar) {
        const Map& obj = *((RefMap*)h)->map;
        ar(obj.inputDim, obj.outputDim, obj.numCoeffs);
        ar(obj.Coeffs());
    });
}

// ParameterizedFunctionBase::WrapCoeffs on caller memory, as the Python
// binding's WrapCoeffs does (an unmanaged view of the array, ToKokkos:
// bindings/python/src/ParameterizedFunctionBase.cpp:25-27).  The memory must
// outlive the map.
int ref_wrap_coeffs(void* h, double* c, long n) {
    return guard([&] { ((RefMap*)h)->map->WrapCoeffs(Kokkos::View<double*, Host>(c, (size_t)n)); });
}

// TriangularMap(components, moveCoeffs = true) over the components of maps
// made here (src/TriangularMap.cpp:10-58): the components' coefficients are
// copied into one new view.  The component handles stay owned by their maps.
void* ref_triangular_from(void* const* comps, unsigned n) {
    RefMap* out = nullptr;
    guard([&] {
        auto* r = new RefMap;
        for (unsigned i = 0; i < n; ++i) r->comps.push_back(((RefMap*)comps[i])->map);
        r->map = std::make_shared<TriangularMap<Host>>(r->comps, true);
        out = r;
    });
    return out;
}

// The map's own ConditionalMapBase::InverseImpl (default options): for the
// sigmoid expansions, whose solver is theirs (RectifiedMultivariateExpansion
// and UnivariateExpansion InverseImpl).  x1 has inputDim - outputDim rows.
int ref_direct_inverse(void* h, const double* x1, long x1Rows, const double* r, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        Kokkos::View<double**, Kokkos::LayoutRight, Host> x("x1", (size_t)std::max<long>(x1Rows, 0), (size_t)n);
        for (long k = 0; k < x1Rows; ++k)
            for (long i = 0; i < n; ++i) x(k, i) = x1[k * n + i];
        StridedMatrix<const double, Host> xv = x;
        m.InverseImpl(xv, cmat(r, m.outputDim, n), mat(out, m.outputDim, n));
    });
}

int ref_sizes(void* h, unsigned* inputDim, unsigned* outputDim, unsigned* numCoeffs) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        *inputDim = m.inputDim;
        *outputDim = m.outputDim;
        *numCoeffs = m.numCoeffs;
    });
}

// ParameterizedFunctionBase::SetCoeffs (deep copy, src/ParameterizedFunctionBase.cpp:185-207).
int ref_set_coeffs(void* h, const double* c, long n) {
    return guard([&] {
        Kokkos::View<const double*, Host> v(c, (size_t)n);
        ((RefMap*)h)->map->SetCoeffs(v);
    });
}

int ref_evaluate(void* h, const double* pts, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.EvaluateImpl(cmat(pts, m.inputDim, n), mat(out, m.outputDim, n));
    });
}

int ref_logdet(void* h, const double* pts, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.LogDeterminantImpl(cmat(pts, m.inputDim, n), StridedVector<double, Host>(out, (size_t)n));
    });
}

int ref_coeff_grad(void* h, const double* pts, const double* sens, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.CoeffGradImpl(cmat(pts, m.inputDim, n), cmat(sens, m.outputDim, n), mat(out, m.numCoeffs, n));
    });
}

int ref_gradient(void* h, const double* pts, const double* sens, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.GradientImpl(cmat(pts, m.inputDim, n), cmat(sens, m.outputDim, n), mat(out, m.inputDim, n));
    });
}

int ref_logdet_coeff_grad(void* h, const double* pts, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.LogDeterminantCoeffGradImpl(cmat(pts, m.inputDim, n), mat(out, m.numCoeffs, n));
    });
}

int ref_logdet_input_grad(void* h, const double* pts, long n, double* out) {
    return guard([&] {
        auto& m = *((RefMap*)h)->map;
        m.LogDeterminantInputGradImpl(cmat(pts, m.inputDim, n), mat(out, m.inputDim, n));
    });
}

// TriangularMap::InverseImpl / InverseInplace (src/TriangularMap.cpp:146-184)
// with the components' "xtol" / "ytol" options, which the reference's
// three-argument InverseImpl leaves at their defaults (1e-6).  x1 has x1Rows
// (<= inputDim) rows; fullOut = [x1; 0] is solved in place, component by
// component, and its last outputDim rows are returned.
int ref_inverse(void* h, const double* x1, long x1Rows, const double* r, long n, double xtol, double ytol,
                double* out) {
    return guard([&] {
        RefMap& rm = *(RefMap*)h;
        auto& m = *rm.map;
        const unsigned ipdim = m.inputDim, opdim = m.outputDim, extra = ipdim - opdim;
        Kokkos::View<double**, Host> full("Full Output", ipdim, (size_t)n);
        for (long d = 0; d < x1Rows; ++d)
            for (long i = 0; i < n; ++i) full(d, i) = x1[d * n + i];
        auto R = cmat(r, opdim, n);
        std::map<std::string, std::string> opts;
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g", xtol);
        opts["xtol"] = buf;
        std::snprintf(buf, sizeof buf, "%.17g", ytol);
        opts["ytol"] = buf;
        unsigned start = 0;
        for (auto& c : rm.comps) {
            StridedMatrix<const double, Host> subX =
                Kokkos::subview(full, std::make_pair(0, int(c->inputDim)), Kokkos::ALL());
            StridedVector<const double, Host> subR = Kokkos::subview(R, start, Kokkos::ALL());
            StridedVector<double, Host> subOut = Kokkos::subview(full, extra + start, Kokkos::ALL());
            componentInverse(c.get(), subX, subR, subOut, opts);
            start += c->outputDim;
        }
        for (unsigned k = 0; k < opdim; ++k)
            for (long i = 0; i < n; ++i) out[k * n + i] = full(extra + k, i);
    });
}

// A MultiIndexSet built by += of the given terms in order (n rows of length
// dim), then either its ReducedMargin() (mode 0: the terms, rows of length
// dim, count in *nOut) or its Expand() (mode 1: the returned active indices in
// idx, count in *nOut, and the set's terms after the expansion in terms, count
// in *nTerms).  Outputs hold up to cap rows / entries.
int ref_mset(unsigned dim, unsigned n, const unsigned* multis, int mode, unsigned cap, unsigned* terms,
             unsigned* nTerms, unsigned* idx, unsigned* nOut) {
    return guard([&] {
        mpart::MultiIndexSet s(dim);
        for (unsigned t = 0; t < n; ++t)
            s += mpart::MultiIndex(std::vector<unsigned>(multis + (size_t)t * dim, multis + (size_t)(t + 1) * dim));
        if (mode == 0) {
            auto rm = s.ReducedMargin();
            if (rm.size() > cap) throw std::runtime_error("ref_mset: output too small");
            for (size_t k = 0; k < rm.size(); ++k) {
                auto v = rm[k].Vector();
                for (unsigned d = 0; d < dim; ++d) terms[k * dim + d] = v[d];
            }
            *nOut = (unsigned)rm.size();
        } else {
            auto ix = s.Expand();
            if (ix.size() > cap || s.Size() > cap) throw std::runtime_error("ref_mset: output too small");
            for (size_t k = 0; k < ix.size(); ++k) idx[k] = ix[k];
            *nOut = (unsigned)ix.size();
            for (unsigned k = 0; k < s.Size(); ++k) {
                auto v = s.IndexToMulti(k).Vector();
                for (unsigned d = 0; d < dim; ++d) terms[k * dim + d] = v[d];
            }
            *nTerms = s.Size();
        }
    });
}

// For n multi-indices (rows of length dim): less[i * n + j] = (m_i < m_j) by
// MultiIndex::operator<, and, for the FixedMultiIndexSet of these terms
// (compressed), its NonzeroDiagonalEntries in nzdiag (count in *nNz).
int ref_multi_order(unsigned dim, unsigned n, const unsigned* multis, unsigned char* less, unsigned* nzdiag,
                    unsigned* nNz) {
    return guard([&] {
        std::vector<mpart::MultiIndex> ms;
        for (unsigned t = 0; t < n; ++t)
            ms.emplace_back(std::vector<unsigned>(multis + (size_t)t * dim, multis + (size_t)(t + 1) * dim));
        for (unsigned i = 0; i < n; ++i)
            for (unsigned j = 0; j < n; ++j) less[(size_t)i * n + j] = ms[i] < ms[j];
        mpart::MultiIndexSet s(dim);
        for (auto const& m : ms) s += m;
        const auto nz = s.Fix(true).NonzeroDiagonalEntries();
        for (size_t k = 0; k < nz.size(); ++k) nzdiag[k] = nz[k];
        *nNz = (unsigned)nz.size();
    });
}

// A report of MParT's MultiIndexSet for the set tests: mode 0 builds it by
// += of the n terms (rows of length dim) under the limiter, mode 1 is
// CreateTotalOrder(dim, order), mode 2 CreateTensorProduct(dim, order), mode 3
// builds it by += without a limiter and then calls SetLimiter.  Limiter kinds:
// 0 None, 1 TotalOrder(u0), 2 Dimension(u0, u1), 3 Anisotropic(w[0..dim),
// w[dim]), 4 MaxDegree(u0, dim), 5 Separable, 6 NonzeroDiag,
// 7 And(TotalOrder(u0), MaxDegree(u1, dim)), 8 Or(Dimension(u0, u1),
// TotalOrder(u2)), 9 Xor(TotalOrder(u0), NonzeroDiag).  The report lists the
// set's terms, MaxOrders, Frontier, StrictFrontier, Margin, ReducedMargin,
// ReducedMarginDim for every dimension, IsExpandable / NumForward /
// NumActiveForward of every term, NonzeroDiagonalEntries, IsAdmissible of the
// margin, Expand() and Expand(i) for every term (on copies), and the union
// with the total-order set of order 1.  Written as text into buf (two-call
// convention, as ref_to_bytes).
int ref_mset_report(unsigned dim, unsigned n, const unsigned* multis, int mode, unsigned order, int limKind,
                    const unsigned* u, const double* w, char* buf, size_t cap, size_t* size) {
    return guard([&] {
        using mpart::MultiIndex;
        using mpart::MultiIndexSet;
        namespace L = mpart::MultiIndexLimiter;
        std::function<bool(MultiIndex const&)> lim;
        switch (limKind) {
            case 0: lim = L::None(); break;
            case 1: lim = L::TotalOrder(u[0]); break;
            case 2: lim = L::Dimension(u[0], u[1]); break;
            case 3: lim = L::Anisotropic(std::vector<double>(w, w + dim), w[dim]); break;
            case 4: lim = L::MaxDegree(u[0], dim); break;
            case 5: lim = L::Separable(); break;
            case 6: lim = L::NonzeroDiag(); break;
            case 7: lim = L::And(L::TotalOrder(u[0]), L::MaxDegree(u[1], dim)); break;
            case 8: lim = L::Or(L::Dimension(u[0], u[1]), L::TotalOrder(u[2])); break;
            case 9: lim = L::Xor(L::TotalOrder(u[0]), L::NonzeroDiag()); break;
            default: throw std::invalid_argument("unknown limiter kind");
        }
        auto term = [&](unsigned t) {
            return MultiIndex(std::vector<unsigned>(multis + (size_t)t * dim, multis + (size_t)(t + 1) * dim));
        };
        MultiIndexSet s(dim);
        std::ostringstream os;
        if (mode == 1) {
            s = MultiIndexSet::CreateTotalOrder(dim, order, lim);
        } else if (mode == 2) {
            s = MultiIndexSet::CreateTensorProduct(dim, order, lim);
        } else if (mode == 0) {
            s = MultiIndexSet(dim, lim);
            for (unsigned t = 0; t < n; ++t) s += term(t);
        } else {
            for (unsigned t = 0; t < n; ++t) s += term(t);
            try {
                s.SetLimiter(lim);
            } catch (std::invalid_argument const&) {
                os << "setlimiter rejected\n";
            }
        }
        auto multisOut = [&](std::vector<MultiIndex> const& ms) {
            std::string r;
            for (size_t k = 0; k < ms.size(); ++k) r += (k ? ";" : "") + ms[k].String();
            return r;
        };
        auto ints = [&](auto const& v) {
            std::string r;
            for (size_t k = 0; k < v.size(); ++k) r += (k ? "," : "") + std::to_string(v[k]);
            return r;
        };
        auto termsOf = [&](MultiIndexSet const& x) {
            std::vector<MultiIndex> t;
            for (unsigned k = 0; k < x.Size(); ++k) t.push_back(x.IndexToMulti(k));
            return multisOut(t);
        };
        os << "size " << s.Size() << "\n";
        os << "terms " << termsOf(s) << "\n";
        os << "maxorders " << ints(s.MaxOrders()) << "\n";
        os << "frontier " << ints(s.Frontier()) << "\n";
        os << "strict " << ints(s.StrictFrontier()) << "\n";
        const auto margin = s.Margin();
        os << "margin " << multisOut(margin) << "\n";
        os << "rmargin " << multisOut(s.ReducedMargin()) << "\n";
        for (unsigned d = 0; d < dim; ++d) os << "rmargin_dim" << d << " " << multisOut(s.ReducedMarginDim(d)) << "\n";
        std::vector<unsigned> ex, nf, na;
        for (unsigned k = 0; k < s.Size(); ++k) {
            ex.push_back(s.IsExpandable(k));
            nf.push_back(s.NumForward(k));
            na.push_back(s.NumActiveForward(k));
        }
        os << "expandable " << ints(ex) << "\n";
        os << "nforward " << ints(nf) << "\n";
        os << "nactiveforward " << ints(na) << "\n";
        os << "nzdiag " << ints(s.NonzeroDiagonalEntries()) << "\n";
        std::vector<unsigned> adm;
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
        const std::string r = os.str();
        *size = r.size();
        if (buf && cap >= r.size()) std::memcpy(buf, r.data(), r.size());
    });
}

}  // extern "C"
