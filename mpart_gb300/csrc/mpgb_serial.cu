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
// The whole-map archive (the reference's polymorphic ToBytes / pickle, which
// depends on cereal's type registry) has a layout of its own: a tag, the
// options, each monotone component's multi-index set, then the coefficient
// archive; it rebuilds the same component or triangular map.
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
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
        str();  // label
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

// The uncompressed form stores every dimension of every term (nzStarts[k] =
// k dim); it is converted to the compressed one by dropping zero orders.
FixedMultiIndexSet readMset(Reader& r) {
    const uint32_t dim = r.pod<uint32_t>();
    const bool compressed = r.pod<uint8_t>() != 0;
    auto starts = r.view<unsigned int>();
    auto dims = r.view<unsigned int>();
    auto orders = r.view<unsigned int>();
    r.view<unsigned int>();  // maxDegrees: recomputed
    if (starts.empty()) throw std::invalid_argument("multi-index archive: no term starts");
    if (dims.size() != orders.size() || starts.back() != dims.size())
        throw std::invalid_argument("multi-index archive: inconsistent sizes");
    if (compressed) return FixedMultiIndexSet(dim, starts, dims, orders);
    std::vector<unsigned> s{0}, d, o;
    for (size_t t = 0; t + 1 < starts.size(); ++t) {
        for (unsigned j = starts[t]; j < starts[t + 1]; ++j)
            if (orders[j] != 0) {
                d.push_back(dims[j]);
                o.push_back(orders[j]);
            }
        s.push_back((unsigned)d.size());
    }
    return FixedMultiIndexSet(dim, s, d, o);
}

void writeCoeffs(Writer& w, const ConditionalMapBase& m) {
    w.pod<uint32_t>(m.inputDim);
    w.pod<uint32_t>(m.outputDim);
    w.pod<uint32_t>(m.numCoeffs);
    const std::vector<double> c = m.CheckCoefficients() ? m.CoeffMap() : std::vector<double>(m.numCoeffs, 0.0);
    w.view<double>(kCoeffLabel, c.data(), c.size());
}

struct CoeffArchive {
    uint32_t in, out, n;
    std::vector<double> c;
};

CoeffArchive readCoeffs(Reader& r) {
    CoeffArchive a;
    a.in = r.pod<uint32_t>();
    a.out = r.pod<uint32_t>();
    a.n = r.pod<uint32_t>();
    a.c = r.view<double>();
    if (a.c.size() != a.n) throw std::invalid_argument("coefficient archive: size does not match numCoeffs");
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

const char* const kSigLabels[4] = {"Sigmoid centers", "Sigmoid widths", "Sigmoid weights", "Sigmoid starting indices"};

// Map archive: tag, options, kind (0 component, 1 triangular map; +2 for
// sigmoid expansions), component count, per component its multi-index set
// (and, for sigmoid expansions, the Sigmoid1d arrays and edge/sum options),
// then the coefficient archive.
std::vector<unsigned char> mapBytes(const std::shared_ptr<ConditionalMapBase>& m) {
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
    writeCoeffs(w, *m);
    return w.b;
}

std::shared_ptr<ConditionalMapBase> mapFromBytes(const unsigned char* buf, size_t size) {
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
        const CoeffArchive a = readCoeffs(r);
        if (input_dim) *input_dim = a.in;
        if (output_dim) *output_dim = a.out;
        if (num_coeffs) *num_coeffs = a.n;
        if (coeffs && a.n) std::memcpy(coeffs, a.c.data(), a.n * sizeof(double));
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
