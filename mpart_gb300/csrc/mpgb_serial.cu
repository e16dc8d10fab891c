// Archives of maps, map options and multi-index sets (host code).
//
// The reference saves with cereal's binary archive: values back to back in
// native byte order, strings as a 64-bit length and their bytes, Kokkos views
// as (label string, 32-bit extent, raw elements) (MParT/Utilities/Serialization.h:19-56).
// Three of its layouts are reproduced byte for byte:
//   * coefficient archive, ParameterizedFunctionBase.Serialize / DeserializeMap
//     (bindings/python/src/ParameterizedFunctionBase.cpp:51-56,
//     bindings/python/src/Serialization.cpp:20-31): inputDim, outputDim,
//     numCoeffs (uint32 each), then the coefficient view;
//   * MapOptions::serialize (MParT/MapOptions.h:126-130): basisType, basisLB,
//     basisUB, posFuncType, quadType, quadAbsTol, quadRelTol, quadMaxSub,
//     quadMinSub, quadPts, contDeriv, basisNorm, nugget (enums as int32, bools
//     as one byte);
//   * FixedMultiIndexSet::save (MParT/MultiIndices/FixedMultiIndexSet.h:115-123):
//     dim (uint32), isCompressed (byte), then the views nzStarts, nzDims,
//     nzOrders, maxDegrees.
// The whole-map archive of ToBytes / FromBytes / pickle is the reference's own
// (ParameterizedFunctionBase::Save, cereal's polymorphic encoding; see
// RefWriter below) for monotone components and triangular maps of them.
// Sigmoid expansions, which the reference does not archive, have a layout of
// this library's own: a tag, the options, each component's multi-index set and
// Sigmoid1d arrays, then the coefficient archive.
#include <cmath>
#include <cstring>
#include <functional>
#include <istream>
#include <iterator>
#include <ostream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "mpgb_program.h"

namespace mpgb {
namespace {

struct Writer {
    std::vector<unsigned char> b;
    template <class T>
    void pod(const T& v) {
        const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
        b.insert(b.end(), p, p + sizeof(T));
    }
    void bytes(const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        b.insert(b.end(), c, c + n);
    }
    void str(const std::string& s) {
        pod<uint64_t>(s.size());
        bytes(s.data(), s.size());
    }
    template <class T>
    void view(const std::string& label, const T* data, size_t n) {
        str(label);
        pod<uint32_t>((uint32_t)n);
        if (n) bytes(data, n * sizeof(T));
    }
};

struct Reader {
    const unsigned char* p;
    size_t n, off = 0;
    Reader(const unsigned char* d, size_t s) : p(d), n(s) {}
    void need(size_t k) const {
        if (k > n - off || off > n) throw std::invalid_argument("archive is truncated or not of the expected kind");
    }
    template <class T>
    T pod() {
        need(sizeof(T));
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    std::string str() {
        const uint64_t len = pod<uint64_t>();
        need(len);
        std::string s(reinterpret_cast<const char*>(p + off), (size_t)len);
        off += len;
        return s;
    }
    template <class T>
    std::vector<T> view() {
        std::string label;
        return view<T>(label);
    }
    template <class T>
    std::vector<T> view(std::string& label) {
        label = str();
        const uint32_t len = pod<uint32_t>();
        need((size_t)len * sizeof(T));
        std::vector<T> v(len);
        if (len) std::memcpy(v.data(), p + off, (size_t)len * sizeof(T));
        off += (size_t)len * sizeof(T);
        return v;
    }
};

const char kCoeffLabel[] = "ParameterizedFunctionBase<MemorySpace> Coefficients";
const char kMapTag[] = "mpart_gb300 map archive v1";

void writeOptions(Writer& w, const MapOptions& o) {
    w.pod<int32_t>((int32_t)o.basisType);
    w.pod<double>(-std::numeric_limits<double>::infinity());  // basisLB
    w.pod<double>(std::numeric_limits<double>::infinity());   // basisUB
    w.pod<int32_t>((int32_t)o.posFuncType);
    w.pod<int32_t>((int32_t)o.quadType);
    w.pod<double>(o.quadAbsTol);
    w.pod<double>(o.quadRelTol);
    w.pod<uint32_t>(o.quadMaxSub);
    w.pod<uint32_t>(o.quadMinSub);
    w.pod<uint32_t>(o.quadPts);
    w.pod<uint8_t>(o.contDeriv ? 1 : 0);
    w.pod<uint8_t>(o.basisNorm ? 1 : 0);
    w.pod<double>(o.nugget);
}

MapOptions readOptions(Reader& r) {
    MapOptions o;
    const int32_t bt = r.pod<int32_t>();
    const double lb = r.pod<double>(), ub = r.pod<double>();
    const int32_t pf = r.pod<int32_t>(), qt = r.pod<int32_t>();
    if (bt < 0 || bt > 2 || pf < 0 || pf > 1 || qt < 0 || qt > 2)
        throw std::invalid_argument("MapOptions archive: invalid enum value");
    if (!(std::isinf(lb) && lb < 0 && std::isinf(ub) && ub > 0))
        throw std::invalid_argument("MapOptions archive: finite basisLB/basisUB (linearised basis) is not supported");
    o.basisType = (BasisTypes)bt;
    o.posFuncType = (PosFuncTypes)pf;
    o.quadType = (QuadTypes)qt;
    o.quadAbsTol = r.pod<double>();
    o.quadRelTol = r.pod<double>();
    o.quadMaxSub = r.pod<uint32_t>();
    o.quadMinSub = r.pod<uint32_t>();
    o.quadPts = r.pod<uint32_t>();
    o.contDeriv = r.pod<uint8_t>() != 0;
    o.basisNorm = r.pod<uint8_t>() != 0;
    o.nugget = r.pod<double>();
    return o;
}

void writeMset(Writer& w, const FixedMultiIndexSet& m) {
    w.pod<uint32_t>(m.Length());
    w.pod<uint8_t>(1);  // compressed
    w.view<unsigned int>("nzStarts", m.nzStarts.data(), m.nzStarts.size());
    w.view<unsigned int>("nzDims", m.nzDims.data(), m.nzDims.size());
    w.view<unsigned int>("nzOrders", m.nzOrders.data(), m.nzOrders.size());
    w.view<unsigned int>("Maximum degrees", m.maxDegrees.data(), m.maxDegrees.size());
}

// The uncompressed form stores every dimension of every term, term k at
// [k dim, (k + 1) dim); the reference leaves the last of its numTerms + 1
// starts unset (SetupTerms, src/MultiIndices/FixedMultiIndexSet.cpp:141-160),
// so the terms are counted from the orders.  It is converted to the
// compressed form by dropping zero orders.
FixedMultiIndexSet readMset(Reader& r) {
    const uint32_t dim = r.pod<uint32_t>();
    const bool compressed = r.pod<uint8_t>() != 0;
    auto starts = r.view<unsigned int>();
    auto dims = r.view<unsigned int>();
    auto orders = r.view<unsigned int>();
    r.view<unsigned int>();  // maxDegrees: recomputed
    if (starts.empty()) throw std::invalid_argument("multi-index archive: no term starts");
    if (dims.size() != orders.size()) throw std::invalid_argument("multi-index archive: inconsistent sizes");
    if (compressed) {
        if (starts.back() != dims.size()) throw std::invalid_argument("multi-index archive: inconsistent sizes");
        return FixedMultiIndexSet(dim, starts, dims, orders);
    }
    if (dim == 0 || orders.size() % dim != 0 || starts.size() != orders.size() / dim + 1)
        throw std::invalid_argument("multi-index archive: inconsistent sizes");
    std::vector<unsigned> s{0}, d, o;
    for (size_t t = 0; t + 1 < starts.size(); ++t) {
        for (size_t j = t * dim; j < (t + 1) * dim; ++j)
            if (orders[j] != 0) {
                d.push_back(dims[j]);
                o.push_back(orders[j]);
            }
        s.push_back((unsigned)d.size());
    }
    return FixedMultiIndexSet(dim, s, d, o);
}

// The reference's Serialize writes the map's own coefficient view
// (obj.Coeffs()): its label, and no elements when no coefficients are set.
// The sigmoid-map archive of this library (own = true) always carries
// numCoeffs values (zeros when unset) under the default label.
void writeCoeffs(Writer& w, const ConditionalMapBase& m, bool own = false) {
    w.pod<uint32_t>(m.inputDim);
    w.pod<uint32_t>(m.outputDim);
    w.pod<uint32_t>(m.numCoeffs);
    if (m.CheckCoefficients()) {
        const std::vector<double> c = m.CoeffMap();
        w.view<double>(own ? std::string(kCoeffLabel) : m.CoeffLabel(), c.data(), c.size());
    } else if (own) {
        const std::vector<double> z(m.numCoeffs, 0.0);
        w.view<double>(kCoeffLabel, z.data(), z.size());
    } else {
        w.view<double>("", nullptr, 0);
    }
}

struct CoeffArchive {
    uint32_t in, out, n;
    std::vector<double> c;
};

// allowEmpty: the archive of a map without coefficients (DeserializeMap
// returns its empty view, bindings/python/src/Serialization.cpp:22-30).
CoeffArchive readCoeffs(Reader& r, bool allowEmpty = false) {
    CoeffArchive a;
    a.in = r.pod<uint32_t>();
    a.out = r.pod<uint32_t>();
    a.n = r.pod<uint32_t>();
    a.c = r.view<double>();
    if (a.c.size() != a.n && !(allowEmpty && a.c.empty()))
        throw std::invalid_argument("coefficient archive: size does not match numCoeffs");
    return a;
}

// Components of a map in output order (a component, or the components of a
// triangular map, nested maps flattened): monotone components or sigmoid
// expansions (a map holds one kind).
void components(const std::shared_ptr<ConditionalMapBase>& m, std::vector<const MonotoneMapBase*>& out) {
    if (dynamic_cast<const MonotoneComponent*>(m.get()) || dynamic_cast<const SigmoidComponent*>(m.get())) {
        out.push_back(dynamic_cast<const MonotoneMapBase*>(m.get()));
        return;
    }
    if (auto* t = dynamic_cast<TriangularMap*>(m.get())) {
        for (unsigned i = 0; i < t->NumComponents(); ++i) components(t->GetComponent(i), out);
        return;
    }
    throw std::invalid_argument("only monotone components, sigmoid expansions and triangular maps can be archived");
}

// ---------------------------------------------------------------------------
// The reference's map archive: ParameterizedFunctionBase::Save / Load
// (MParT/ParameterizedFunctionBase.h:197-215), behind its ToBytes, FromBytes
// and pickle (bindings/python/src/ParameterizedFunctionBase.cpp:57-79).  It is
// cereal's (v1.3.2) encoding of a shared_ptr to a polymorphic object: a uint32
// type id (top bit set on the type's first use, followed by its registered
// name as a string), then a uint32 object id (top bit set on the object's
// first use, followed by the object's data); both count from 1 in order of
// first use.
//   * TriangularMap<Kokkos::HostSpace> (TriangularMap.h:130-138): its
//     components as a vector of such pointers (uint64 count), the same vector
//     again (ids only: every object has been written), then moveCoeffs, one
//     byte: whether the map holds a coefficient view.
//   * MonotoneComponent (MonotoneComponent.h:1037-1044): its
//     MultivariateExpansionWorker (MultivariateExpansionWorker.h:406-412:
//     input dimension, multi-index set, the 1-D basis's normalisation flag --
//     HermiteFunction's is that of its PhysicistHermite, false -- the cache
//     start positions and size); its quadrature (Quadrature.h:66-90 for
//     every rule: integrand dimension, maximum dimension, workspace size,
//     internal workspace; :422-435 for the adaptive rules: maxSub, minSub,
//     absTol, relTol, error metric; :313-326 for fixed Clenshaw-Curtis:
//     points, weights, count; :970-984 for adaptive Clenshaw-Curtis: the
//     coarse and fine rules, the fine weights under the label "Coarse Pts" as
//     the constructor names them, Quadrature.h:1054-1058); useContDeriv; the
//     nugget; its coefficient view.
// MapFactory builds every quadrature with maximum dimension 1, an external
// workspace (none held) for the adaptive rules and a one-double internal one
// for fixed Clenshaw-Curtis, and error metric QuadError::First
// (src/MapFactoryImpl4.cpp:17-20, Impl5:17, Impl6:17).
// Only the description of the map -- multi-index sets, options, the
// quadrature's integrand dimension, coefficients and their view label -- is
// kept; the writer recomputes the rest, and the reader checks it.
// The reference's TriangularMap loader reads moveCoeffs from the byte after
// the first component vector (the low byte of the second vector's count);
// this reader follows the layout the writer produces.
// ---------------------------------------------------------------------------

constexpr uint32_t kNewId = 0x80000000u;

struct RefComp {
    FixedMultiIndexSet mset{1, 0};
    MapOptions opts;
    unsigned quadDim = 1;
    bool hasCoeffs = false;
    std::string label;
    std::vector<double> coeffs;
};

struct RefNode {
    bool triangular = false;
    RefComp comp;                                     // a component
    std::vector<std::shared_ptr<RefNode>> children;  // a triangular map
    bool moveCoeffs = false;
};

const char* const kSpaces[2] = {"Kokkos::HostSpace", "mpart::DeviceSpace"};
const BasisTypes kArchBases[2] = {BasisTypes::ProbabilistHermite, BasisTypes::HermiteFunctions};
const PosFuncTypes kArchPos[2] = {PosFuncTypes::Exp, PosFuncTypes::SoftPlus};
const QuadTypes kArchQuads[3] = {QuadTypes::AdaptiveClenshawCurtis, QuadTypes::ClenshawCurtis,
                                 QuadTypes::AdaptiveSimpson};

// Registered names: the arguments of CEREAL_REGISTER_TYPE as written
// (src/TriangularMap.cpp:336, MParT/Utilities/Serialization.h:14-15 with the
// arguments of src/MapFactoryImpl4.cpp-9.cpp).
std::string triangularName(int space) { return std::string("mpart::TriangularMap<") + kSpaces[space] + ">"; }

std::string componentName(BasisTypes b, PosFuncTypes p, QuadTypes q, int space) {
    const std::string sp = kSpaces[space];
    const char* basis = b == BasisTypes::HermiteFunctions ? "HermiteFunction" : "ProbabilistHermite";
    const char* pos = p == PosFuncTypes::Exp ? "Exp" : "SoftPlus";
    const char* quad = q == QuadTypes::AdaptiveClenshawCurtis ? "AdaptiveClenshawCurtis"
                       : q == QuadTypes::AdaptiveSimpson     ? "AdaptiveSimpson"
                                                             : "ClenshawCurtisQuadrature";
    return "mpart::MonotoneComponent<mpart::MultivariateExpansionWorker<mpart::BasisEvaluator<"
           "BasisHomogeneity::Homogeneous, " +
           std::string(basis) + ">, " + sp + ">, mpart::" + pos + ", mpart::" + quad + "<" + sp + ">, " + sp + ">";
}

// Start of each 1-D basis block in the expansion's cache: an exclusive scan of
// maxDegrees(i % dim) + 1 over 2 dim entries, then maxDegrees(dim - 1) + 1
// (MultivariateExpansionWorker.h:19-39, :94-106); the cache size is the last.
std::vector<unsigned> startPositions(const FixedMultiIndexSet& m) {
    const unsigned dim = m.Length();
    std::vector<unsigned> sp(2 * dim + 2);
    unsigned run = 0;
    for (unsigned i = 0; i < 2 * dim + 2; ++i) {
        sp[i] = run;
        run += (i < 2 * dim ? m.maxDegrees[i % dim] : m.maxDegrees[dim - 1]) + 1;
    }
    return sp;
}

// Workspace size for an integrand of dimension fdim (GetWorkspaceSize,
// Quadrature.h:172, :520, :786).
uint32_t workspaceSize(QuadTypes q, unsigned maxSub, unsigned fdim) {
    if (q == QuadTypes::AdaptiveClenshawCurtis) return (maxSub + 5) * fdim + 2 * maxSub;
    if (q == QuadTypes::AdaptiveSimpson) return (2 * maxSub + 5) * fdim + 2 * maxSub;
    return fdim;
}

// Level of the adaptive Clenshaw-Curtis rule (src/MapFactoryImpl4.cpp:18).
unsigned accLevel(unsigned quadPts) { return (unsigned)std::log2((double)(quadPts - 2u)); }

class RefWriter {
public:
    Writer w;

    void object(const std::shared_ptr<RefNode>& n) {
        const std::string name =
            n->triangular ? triangularName(0)
                          : componentName(n->comp.opts.basisType, n->comp.opts.posFuncType, n->comp.opts.quadType, 0);
        auto t = types_.find(name);
        if (t == types_.end()) {
            const uint32_t id = (uint32_t)types_.size() + 1;
            types_.emplace(name, id);
            w.pod<uint32_t>(id | kNewId);
            w.str(name);
        } else {
            w.pod<uint32_t>(t->second);
        }
        auto o = objects_.find(n.get());
        if (o != objects_.end()) {
            w.pod<uint32_t>(o->second);
            return;
        }
        const uint32_t id = (uint32_t)objects_.size() + 1;
        objects_.emplace(n.get(), id);
        w.pod<uint32_t>(id | kNewId);
        if (n->triangular)
            triangular(*n);
        else
            component(n->comp);
    }

private:
    void triangular(const RefNode& n) {
        for (int pass = 0; pass < 2; ++pass) {
            w.pod<uint64_t>(n.children.size());
            for (auto& c : n.children) object(c);
        }
        w.pod<uint8_t>(n.moveCoeffs ? 1 : 0);
    }

    void component(const RefComp& c) {
        const FixedMultiIndexSet& m = c.mset;
        const MapOptions& o = c.opts;
        w.pod<uint32_t>(m.Length());
        writeMset(w, m);
        w.pod<uint8_t>(o.basisType != BasisTypes::HermiteFunctions && o.basisNorm ? 1 : 0);
        const std::vector<unsigned> sp = startPositions(m);
        w.view<unsigned int>("Indices for start of 1d basis evaluations", sp.data(), sp.size());
        w.pod<uint32_t>(sp.back());

        const bool fixed = o.quadType == QuadTypes::ClenshawCurtis;
        w.pod<uint32_t>(c.quadDim);
        w.pod<uint32_t>(1u);
        w.pod<uint32_t>(workspaceSize(o.quadType, o.quadMaxSub, c.quadDim));
        const double zero = 0.0;
        if (fixed)
            w.view<double>("Workspace", &zero, 1);
        else
            w.view<double>("", nullptr, 0);
        if (fixed) {
            std::vector<double> pts(o.quadPts), wts(o.quadPts);
            ccRule(o.quadPts, wts.data(), pts.data());
            w.view<double>("Points", pts.data(), pts.size());
            w.view<double>("Weights", wts.data(), wts.size());
            w.pod<uint32_t>(o.quadPts);
        } else {
            w.pod<uint32_t>(o.quadMaxSub);
            w.pod<uint32_t>(o.quadMinSub);
            w.pod<double>(o.quadAbsTol);
            w.pod<double>(o.quadRelTol);
            w.pod<uint32_t>(0u);  // QuadError::First
            if (o.quadType == QuadTypes::AdaptiveClenshawCurtis) {
                const unsigned level = accLevel(o.quadPts);
                const unsigned nc = (1u << level) + 1, nf = (1u << (level + 1)) + 1;
                std::vector<double> cp(nc), cw(nc), fp(nf), fw(nf);
                ccRule(nc, cw.data(), cp.data());
                ccRule(nf, fw.data(), fp.data());
                w.view<double>("Coarse Pts", cp.data(), nc);
                w.view<double>("Coarse Wts", cw.data(), nc);
                w.view<double>("Fine Pts", fp.data(), nf);
                w.view<double>("Coarse Pts", fw.data(), nf);
            }
        }
        w.pod<uint8_t>(o.contDeriv ? 1 : 0);
        w.pod<double>(o.nugget);
        if (c.hasCoeffs)
            w.view<double>(c.label, c.coeffs.data(), c.coeffs.size());
        else
            w.view<double>("", nullptr, 0);
    }

    std::map<std::string, uint32_t> types_;
    std::map<const RefNode*, uint32_t> objects_;
};

class RefReader {
public:
    explicit RefReader(Reader& r) : r_(r) {}

    std::shared_ptr<RefNode> object() {
        const uint32_t tid = r_.pod<uint32_t>();
        if (tid == 0) throw std::invalid_argument("map archive: null map pointer");
        std::string name;
        if (tid & kNewId) {
            name = r_.str();
            types_[tid & ~kNewId] = name;
        } else {
            auto it = types_.find(tid);
            if (it == types_.end()) throw std::invalid_argument("map archive: unknown type id");
            name = it->second;
        }
        const uint32_t oid = r_.pod<uint32_t>();
        if (!(oid & kNewId)) {
            auto it = objects_.find(oid);
            if (it == objects_.end()) throw std::invalid_argument("map archive: unknown object id");
            for (const RefNode* o : open_)
                if (o == it->second.get()) throw std::invalid_argument("map archive: a map contains itself");
            return it->second;
        }
        auto n = std::make_shared<RefNode>();
        objects_[oid & ~kNewId] = n;
        if (name == triangularName(0) || name == triangularName(1)) {
            n->triangular = true;
            if (open_.size() >= kMaxNesting) bad("triangular maps nested too deeply");
            open_.push_back(n.get());
            triangular(*n);
            open_.pop_back();
            return n;
        }
        for (int sp = 0; sp < 2; ++sp)
            for (BasisTypes b : kArchBases)
                for (PosFuncTypes p : kArchPos)
                    for (QuadTypes q : kArchQuads)
                        if (name == componentName(b, p, q, sp)) {
                            n->comp.opts.basisType = b;
                            n->comp.opts.posFuncType = p;
                            n->comp.opts.quadType = q;
                            component(n->comp);
                            return n;
                        }
        if (name.rfind("mpart::MonotoneComponent<", 0) == 0)
            throw std::invalid_argument(
                "map archive: component basis not provided here (ProbabilistHermite and HermiteFunction only): " +
                name);
        throw std::invalid_argument("map archive: map type not provided here: " + name);
    }

private:
    static void bad(const char* what) { throw std::invalid_argument(std::string("map archive: ") + what); }

    void triangular(RefNode& n) {
        const uint64_t count = r_.pod<uint64_t>();
        if (count == 0 || count > r_.n - r_.off) bad("bad component count");
        for (uint64_t i = 0; i < count; ++i) n.children.push_back(object());
        // the component vector written again, ids only
        const size_t mark = r_.off;
        bool again = r_.n - r_.off >= 8 + 8 * count + 1 && r_.pod<uint64_t>() == count;
        for (uint64_t i = 0; again && i < count; ++i) {
            const uint32_t tid = r_.pod<uint32_t>(), oid = r_.pod<uint32_t>();
            auto it = objects_.find(oid);
            again = !(tid & kNewId) && types_.count(tid) && it != objects_.end() && it->second == n.children[i];
        }
        if (!again) r_.off = mark;
        n.moveCoeffs = r_.pod<uint8_t>() != 0;
    }

    void component(RefComp& c) {
        MapOptions& o = c.opts;
        const uint32_t dim = r_.pod<uint32_t>();
        c.mset = readMset(r_);
        if (dim != c.mset.Length()) bad("expansion dimension does not match its multi-index set");
        const uint8_t norm = r_.pod<uint8_t>();
        if (o.basisType == BasisTypes::HermiteFunctions) {
            if (norm != 0) bad("Hermite functions over normalised Hermite polynomials are not provided");
        } else {
            o.basisNorm = norm != 0;
        }
        const std::vector<unsigned> sp = r_.view<unsigned>();
        const uint32_t cacheSize = r_.pod<uint32_t>();
        if (sp != startPositions(c.mset) || cacheSize != sp.back())
            bad("expansion cache layout does not match its multi-index set");

        const bool fixed = o.quadType == QuadTypes::ClenshawCurtis;
        const uint32_t fdim = r_.pod<uint32_t>(), maxDim = r_.pod<uint32_t>(), ws = r_.pod<uint32_t>();
        const std::vector<double> internal = r_.view<double>();
        if (maxDim != 1 || internal.size() != (fixed ? 1u : 0u))
            bad("quadrature workspace not as MapFactory builds it (maximum dimension 1)");
        if (fdim == 0) bad("quadrature of dimension 0");
        if (fixed) {
            const std::vector<double> pts = r_.view<double>(), wts = r_.view<double>();
            const uint32_t numPts = r_.pod<uint32_t>();
            if (pts.size() != numPts || wts.size() != numPts) bad("Clenshaw-Curtis rule sizes disagree");
            o.quadPts = numPts;
        } else {
            o.quadMaxSub = r_.pod<uint32_t>();
            o.quadMinSub = r_.pod<uint32_t>();
            o.quadAbsTol = r_.pod<double>();
            o.quadRelTol = r_.pod<double>();
            if (r_.pod<uint32_t>() != 0) bad("quadrature error metrics other than QuadError::First are not provided");
            if (o.quadType == QuadTypes::AdaptiveClenshawCurtis) {
                const std::vector<double> cp = r_.view<double>(), cw = r_.view<double>();
                const std::vector<double> fp = r_.view<double>(), fw = r_.view<double>();
                unsigned level = 0;
                while (level < 30 && (1u << level) + 1 < cp.size()) ++level;
                if (cp.size() != (1u << level) + 1 || cw.size() != cp.size() ||
                    fp.size() != (1u << (level + 1)) + 1 || fw.size() != fp.size())
                    bad("adaptive Clenshaw-Curtis rule sizes disagree");
                o.quadPts = (1u << (level + 1)) + 1;  // any quadPts of this level
            }
        }
        if (ws != workspaceSize(o.quadType, o.quadMaxSub, fdim)) bad("quadrature workspace size disagrees");
        c.quadDim = fdim;
        o.contDeriv = r_.pod<uint8_t>() != 0;
        o.nugget = r_.pod<double>();
        c.coeffs = r_.view<double>(c.label);
        // MonotoneComponent::load_and_construct (MonotoneComponent.h:1046-1062)
        // keeps coefficients only of the right size.
        c.hasCoeffs = c.coeffs.size() == c.mset.Size() && !c.coeffs.empty();
        if (!c.hasCoeffs) c.coeffs.clear();
    }

    static constexpr size_t kMaxNesting = 256;  // bounds the reader's recursion
    Reader& r_;
    std::map<uint32_t, std::string> types_;
    std::map<uint32_t, std::shared_ptr<RefNode>> objects_;
    std::vector<const RefNode*> open_;  // triangular maps being read
};

// The archive's description of a map of this library, or null when it holds
// a component the reference cannot archive (sigmoid expansions).
std::shared_ptr<RefNode> describe(const ConditionalMapBase* m,
                                  std::map<const ConditionalMapBase*, std::shared_ptr<RefNode>>& memo) {
    auto it = memo.find(m);
    if (it != memo.end()) return it->second;
    auto n = std::make_shared<RefNode>();
    if (auto* t = dynamic_cast<const TriangularMap*>(m)) {
        n->triangular = true;
        auto* tm = const_cast<TriangularMap*>(t);
        for (unsigned i = 0; i < tm->NumComponents(); ++i) {
            auto c = describe(tm->GetComponent(i).get(), memo);
            if (!c) return nullptr;
            n->children.push_back(c);
        }
        n->moveCoeffs = t->CheckCoefficients() && t->numCoeffs > 0;
    } else if (auto* c = dynamic_cast<const MonotoneComponent*>(m)) {
        RefComp& rc = n->comp;
        rc.mset = c->GetMultiIndexSet();
        rc.opts = c->Options();
        rc.quadDim = c->Parts().at(0).prog->quadDim;
        rc.hasCoeffs = c->CheckCoefficients() && c->numCoeffs > 0;
        rc.label = c->CoeffLabel();
        if (rc.hasCoeffs) rc.coeffs = c->CoeffMap();
    } else {
        return nullptr;
    }
    memo[m] = n;
    return n;
}

// The map the reference's Load builds: components constructed with their
// coefficients (copied: MonotoneComponent.h:1057, ParameterizedFunctionBase.h:35),
// triangular maps with their moveCoeffs flag (TriangularMap.h:141-149).
std::shared_ptr<ConditionalMapBase> build(const std::shared_ptr<RefNode>& n,
                                          std::map<const RefNode*, std::shared_ptr<ConditionalMapBase>>& memo) {
    auto it = memo.find(n.get());
    if (it != memo.end()) return it->second;
    std::shared_ptr<ConditionalMapBase> m;
    if (n->triangular) {
        std::vector<std::shared_ptr<ConditionalMapBase>> comps;
        for (auto& c : n->children) comps.push_back(build(c, memo));
        m = std::make_shared<TriangularMap>(comps, n->moveCoeffs);
    } else {
        auto c = std::make_shared<MonotoneComponent>(n->comp.mset, n->comp.opts);
        if (n->comp.hasCoeffs) c->SetCoeffs(n->comp.coeffs.data(), (unsigned)n->comp.coeffs.size(), true);
        c->Parts().at(0).prog->quadDim = n->comp.quadDim;
        m = c;
    }
    memo[n.get()] = m;
    return m;
}

bool isRefArchive(const unsigned char* buf, size_t size) {
    if (size < 4) return false;
    uint32_t first;
    std::memcpy(&first, buf, 4);
    return (first & kNewId) != 0;
}

std::shared_ptr<RefNode> readRefArchive(const unsigned char* buf, size_t size) {
    Reader r(buf, size);
    RefReader rr(r);
    return rr.object();
}

std::vector<unsigned char> writeRefArchive(const std::shared_ptr<RefNode>& root) {
    RefWriter rw;
    rw.object(root);
    return rw.w.b;
}

const char* const kSigLabels[4] = {"Sigmoid centers", "Sigmoid widths", "Sigmoid weights", "Sigmoid starting indices"};

// Map archive: tag, options, kind (0 component, 1 triangular map; +2 for
// sigmoid expansions), component count, per component its multi-index set
// (and, for sigmoid expansions, the Sigmoid1d arrays and edge/sum options),
// then the coefficient archive.
std::vector<unsigned char> mapBytes(const std::shared_ptr<ConditionalMapBase>& m) {
    {
        std::map<const ConditionalMapBase*, std::shared_ptr<RefNode>> memo;
        if (auto root = describe(m.get(), memo)) return writeRefArchive(root);
    }
    auto* mono = dynamic_cast<MonotoneMapBase*>(m.get());
    if (!mono) throw std::invalid_argument("only monotone components, sigmoid expansions and triangular maps can be archived");
    std::vector<const MonotoneMapBase*> comps;
    components(m, comps);
    const bool sig = dynamic_cast<const SigmoidComponent*>(comps[0]) != nullptr;
    for (auto* c : comps)
        if ((dynamic_cast<const SigmoidComponent*>(c) != nullptr) != sig)
            throw std::invalid_argument("map archive: mixed component kinds");
    Writer w;
    w.str(kMapTag);
    writeOptions(w, mono->Options());
    const bool single = dynamic_cast<TriangularMap*>(m.get()) == nullptr;
    w.pod<uint32_t>((single ? 0u : 1u) + (sig ? 2u : 0u));
    w.pod<uint32_t>((uint32_t)comps.size());
    for (auto* c : comps) {
        if (sig) {
            auto* sc = static_cast<const SigmoidComponent*>(c);
            writeMset(w, sc->GetMultiIndexSet());
            const Sigmoid1dParams& p = sc->GetSigmoid();
            w.view<double>(kSigLabels[0], p.centers.data(), p.centers.size());
            w.view<double>(kSigLabels[1], p.widths.data(), p.widths.size());
            w.view<double>(kSigLabels[2], p.weights.data(), p.weights.size());
            w.view<unsigned int>(kSigLabels[3], p.startInds.data(), p.startInds.size());
            w.pod<double>(sc->Options().edgeShape);
            w.pod<int32_t>((int32_t)sc->Options().sigmoidBasisSumType);
        } else {
            writeMset(w, static_cast<const MonotoneComponent*>(c)->GetMultiIndexSet());
        }
    }
    writeCoeffs(w, *m, true);
    return w.b;
}

std::shared_ptr<ConditionalMapBase> mapFromBytes(const unsigned char* buf, size_t size) {
    if (isRefArchive(buf, size)) {
        std::map<const RefNode*, std::shared_ptr<ConditionalMapBase>> memo;
        return build(readRefArchive(buf, size), memo);
    }
    Reader r(buf, size);
    if (r.str() != kMapTag) throw std::invalid_argument("not a map archive written by this library");
    MapOptions o = readOptions(r);
    const uint32_t kind = r.pod<uint32_t>();
    const uint32_t nc = r.pod<uint32_t>();
    const bool single = (kind & 1u) == 0, sig = kind >= 2;
    if (kind > 3 || nc == 0 || (single && nc != 1)) throw std::invalid_argument("map archive: bad structure");
    std::vector<std::shared_ptr<ConditionalMapBase>> comps;
    for (uint32_t i = 0; i < nc; ++i) {
        FixedMultiIndexSet ms = readMset(r);
        if (sig) {
            Sigmoid1dParams p;
            p.centers = r.view<double>();
            p.widths = r.view<double>();
            p.weights = r.view<double>();
            p.startInds = r.view<unsigned int>();
            o.edgeShape = r.pod<double>();
            const int32_t st = r.pod<int32_t>();
            if (st < 0 || st > 1) throw std::invalid_argument("map archive: bad sigmoid sum type");
            o.sigmoidBasisSumType = (SigmoidSumSizeType)st;
            auto c = std::make_shared<SigmoidComponent>(ms, p, o);
            std::vector<double> z(c->numCoeffs, 0.0);
            c->SetCoeffs(z.data(), c->numCoeffs, true);
            comps.push_back(c);
        } else {
            comps.push_back(MapFactory::CreateComponent(ms, o));
        }
    }
    std::shared_ptr<ConditionalMapBase> m =
        single ? comps[0] : std::shared_ptr<ConditionalMapBase>(std::make_shared<TriangularMap>(comps, true));
    const CoeffArchive a = readCoeffs(r);
    if (a.in != m->inputDim || a.out != m->outputDim || a.n != m->numCoeffs)
        throw std::invalid_argument("map archive: coefficient block does not match the map");
    m->SetCoeffs(a.c.data(), a.n, true);
    return m;
}

int serialGuard(const std::function<void()>& f) {
    try {
        f();
        return MPGB_OK;
    } catch (CudaError const& e) {
        setLastError(e.what());
        return MPGB_ERR_CUDA;
    } catch (std::invalid_argument const& e) {
        setLastError(e.what());
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        setLastError(e.what());
        return MPGB_ERR_RUNTIME;
    }
}

// Two-call convention: *size always receives the archive size; the bytes are
// written when buf holds at least that many.
void emit(const std::vector<unsigned char>& b, unsigned char* buf, size_t cap, size_t* size) {
    if (!size) throw std::invalid_argument("null size");
    *size = b.size();
    if (buf) {
        if (cap < b.size()) throw std::invalid_argument("buffer too small for the archive");
        std::memcpy(buf, b.data(), b.size());
    }
}


}  // namespace

void ParameterizedFunctionBase::Save(std::ostream& os) const {
    auto* m = dynamic_cast<const ConditionalMapBase*>(this);
    std::map<const ConditionalMapBase*, std::shared_ptr<RefNode>> memo;
    auto root = m ? describe(m, memo) : nullptr;
    if (!root)
        throw std::invalid_argument("Save: only monotone components and triangular maps of them have the reference's "
                                    "archive.");
    const std::vector<unsigned char> b = writeRefArchive(root);
    os.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
    if (!os) throw std::runtime_error("Save: failed to write to the stream.");
}

std::shared_ptr<ConditionalMapBase> ParameterizedFunctionBase::Load(std::istream& is) {
    std::vector<unsigned char> b((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    if (!isRefArchive(b.data(), b.size())) throw std::invalid_argument("Load: not a map archive in the reference's layout.");
    std::map<const RefNode*, std::shared_ptr<ConditionalMapBase>> memo;
    return build(readRefArchive(b.data(), b.size()), memo);
}

}  // namespace mpgb

using namespace mpgb;

extern "C" {

int mpgb_map_to_bytes(mpgb_map* map, int layout, unsigned char* buf, size_t cap, size_t* size) {
    return serialGuard([&] {
        if (!map || !map->obj) throw std::invalid_argument("null map handle");
        if (layout == MPGB_ARCHIVE_MAP) {
            emit(mapBytes(map->obj), buf, cap, size);
        } else if (layout == MPGB_ARCHIVE_COEFFS) {
            Writer w;
            writeCoeffs(w, *map->obj);
            emit(w.b, buf, cap, size);
        } else {
            throw std::invalid_argument("unknown archive layout");
        }
    });
}

int mpgb_map_archive_rewrite(const unsigned char* in, size_t in_size, unsigned char* buf, size_t cap, size_t* size) {
    return serialGuard([&] {
        if (!in) throw std::invalid_argument("null argument");
        if (!isRefArchive(in, in_size)) throw std::invalid_argument("not a map archive in the reference's layout");
        emit(writeRefArchive(readRefArchive(in, in_size)), buf, cap, size);
    });
}

int mpgb_map_from_bytes(const unsigned char* buf, size_t size, mpgb_map** out) {
    return serialGuard([&] {
        if (!buf || !out) throw std::invalid_argument("null argument");
        *out = new mpgb_map{mapFromBytes(buf, size)};
    });
}

int mpgb_coeff_archive_read(const unsigned char* buf, size_t size, unsigned int* input_dim, unsigned int* output_dim,
                            unsigned int* num_coeffs, double* coeffs) {
    return serialGuard([&] {
        if (!buf) throw std::invalid_argument("null archive");
        Reader r(buf, size);
        const CoeffArchive a = readCoeffs(r, true);
        if (input_dim) *input_dim = a.in;
        if (output_dim) *output_dim = a.out;
        if (num_coeffs) *num_coeffs = a.n;
        if (coeffs && !a.c.empty()) std::memcpy(coeffs, a.c.data(), a.n * sizeof(double));
    });
}

int mpgb_options_to_bytes(const mpgb_map_options* opts, unsigned char* buf, size_t cap, size_t* size) {
    return serialGuard([&] {
        if (!opts) throw std::invalid_argument("null options");
        Writer w;
        writeOptions(w, mapOptionsFromC(opts));
        emit(w.b, buf, cap, size);
    });
}

int mpgb_options_from_bytes(const unsigned char* buf, size_t size, mpgb_map_options* out) {
    return serialGuard([&] {
        if (!buf || !out) throw std::invalid_argument("null argument");
        Reader r(buf, size);
        const MapOptions m = readOptions(r);
        out->basis_type = (int)m.basisType;
        out->pos_func_type = (int)m.posFuncType;
        out->quad_type = (int)m.quadType;
        out->quad_abs_tol = m.quadAbsTol;
        out->quad_rel_tol = m.quadRelTol;
        out->quad_max_sub = m.quadMaxSub;
        out->quad_min_sub = m.quadMinSub;
        out->quad_pts = m.quadPts;
        out->cont_deriv = m.contDeriv ? 1 : 0;
        out->basis_norm = m.basisNorm ? 1 : 0;
        out->nugget = m.nugget;
        // (The archive has no sigmoid fields, MapOptions.h:126-130: defaults.)
        out->sigmoid_type = (int)m.sigmoidType;
        out->edge_type = (int)m.edgeType;
        out->edge_shape = m.edgeShape;
        out->sigmoid_sum_type = (int)m.sigmoidBasisSumType;
    });
}

int mpgb_mset_to_bytes(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                       const unsigned int* nz_dims, const unsigned int* nz_orders, unsigned char* buf, size_t cap,
                       size_t* size) {
    return serialGuard([&] {
        if (!nz_starts) throw std::invalid_argument("null nz_starts");
        std::vector<unsigned> s(nz_starts, nz_starts + num_terms + 1);
        const unsigned nnz = s.back();
        if (nnz && (!nz_dims || !nz_orders)) throw std::invalid_argument("null nonzero arrays");
        std::vector<unsigned> d(nz_dims, nz_dims + nnz), o(nz_orders, nz_orders + nnz);
        Writer w;
        writeMset(w, FixedMultiIndexSet(dim, s, d, o));
        emit(w.b, buf, cap, size);
    });
}

int mpgb_mset_from_bytes(const unsigned char* buf, size_t size, unsigned int* dim, unsigned int* num_terms,
                         unsigned int* nnz, unsigned int* nz_starts, unsigned int* nz_dims, unsigned int* nz_orders) {
    return serialGuard([&] {
        if (!buf) throw std::invalid_argument("null archive");
        Reader r(buf, size);
        const FixedMultiIndexSet m = readMset(r);
        if (dim) *dim = m.Length();
        if (num_terms) *num_terms = m.Size();
        if (nnz) *nnz = (unsigned)m.nzDims.size();
        if (nz_starts) std::memcpy(nz_starts, m.nzStarts.data(), m.nzStarts.size() * sizeof(unsigned));
        if (nz_dims && !m.nzDims.empty()) std::memcpy(nz_dims, m.nzDims.data(), m.nzDims.size() * sizeof(unsigned));
        if (nz_orders && !m.nzOrders.empty())
            std::memcpy(nz_orders, m.nzOrders.data(), m.nzOrders.size() * sizeof(unsigned));
    });
}

}  // extern "C"
