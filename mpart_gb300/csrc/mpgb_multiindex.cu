// Multi-indices, limiters and adaptive multi-index sets of the C++ API (host
// code): the reference's MultiIndex (src/MultiIndices/MultiIndex.cpp),
// MultiIndexLimiter (MParT/MultiIndices/MultiIndexLimiter.h,
// src/MultiIndices/MultiIndexLimiter.cpp) and MultiIndexSet
// (src/MultiIndices/MultiIndexSet.cpp with the default neighbourhood of
// src/MultiIndices/MultiIndexNeighborhood.cpp).
#include <algorithm>
#include <cmath>
#include <sstream>

#include "../../include/mpart_gb300.hpp"

namespace mpgb {

// ---- MultiIndex --------------------------------------------------------------
unsigned int MultiIndex::Sum() const {
    unsigned int s = 0;
    for (unsigned int v : v_) s += v;
    return s;
}

unsigned int MultiIndex::Max() const {
    unsigned int m = 0;
    for (unsigned int v : v_) m = std::max(m, v);
    return m;
}

unsigned int MultiIndex::NumNz() const {
    unsigned int n = 0;
    for (unsigned int v : v_) n += v != 0;
    return n;
}

unsigned int MultiIndex::Get(unsigned int i) const {
    if (i > v_.size())
        throw std::out_of_range("Tried to access index " + std::to_string(i) + " of a multiindex with only " +
                                std::to_string(v_.size()) + " components.");
    return i < v_.size() ? v_[i] : 0u;
}

bool MultiIndex::Set(unsigned int i, unsigned int val) {
    if (i >= v_.size())
        throw std::out_of_range("Tried to set the value of index " + std::to_string(i) + " on an multiindex with only " +
                                std::to_string(v_.size()) + " components.");
    const bool was = v_[i] != 0;
    v_[i] = val;
    return was;
}

std::string MultiIndex::String() const {
    std::string out;
    for (size_t i = 0; i < v_.size(); ++i) out += (i ? " " : "") + std::to_string(v_[i]);
    return out;
}

bool MultiIndex::operator<(MultiIndex const& b) const {
    if (Length() != b.Length()) return Length() < b.Length();
    if (Sum() != b.Sum()) return Sum() < b.Sum();
    if (Max() != b.Max()) return Max() < b.Max();
    return v_ < b.v_;
}

// ---- limiters ----------------------------------------------------------------
namespace MultiIndexLimiter {

bool Dimension::operator()(MultiIndex const& m) const {
    for (unsigned int i = 0; i < lowerDim; ++i)
        if (m.Get(i) != 0) return false;
    for (unsigned int i = lowerDim + length; i < m.Length(); ++i)
        if (m.Get(i) != 0) return false;
    return true;
}

Anisotropic::Anisotropic(std::vector<double> const& w, double eps) : weights(w), epsilon(eps) {
    for (double x : weights)
        if (x > 1.0 || x < 0.0)
            throw std::invalid_argument("AnisotropicLimiter requires all weights have to be in [0,1]. Got weight " +
                                        std::to_string(x));
    if (epsilon >= 1.0 || epsilon <= 0.0)
        throw std::invalid_argument("AnisotropicLimiter requires epsilon to be in (0,1). Got epsilon = " +
                                    std::to_string(epsilon));
}

bool Anisotropic::operator()(MultiIndex const& m) const {
    if (m.Length() != weights.size()) return false;
    double prod = 1.0;
    for (unsigned int i = 0; i < m.Length(); ++i) prod *= std::pow(weights[i], (int)m.Get(i));
    return prod >= epsilon;
}

bool MaxDegree::operator()(MultiIndex const& m) const {
    if (m.Length() != maxDegrees.size()) return false;
    for (unsigned int i = 0; i < m.Length(); ++i)
        if (m.Get(i) > maxDegrees[i]) return false;
    return true;
}

}  // namespace MultiIndexLimiter

// ---- MultiIndexSet -------------------------------------------------------------
MultiIndexSet::MultiIndexSet(unsigned int length, LimiterType const& limiter)
    : length_(length), limiter_(limiter ? limiter : LimiterType(MultiIndexLimiter::None())), maxOrders_(length, 0) {
    hasLimiter_ = limiter_.target<MultiIndexLimiter::None>() == nullptr;
}

namespace {
// The recursive fills of CreateTotalOrder / CreateTensorProduct
// (MultiIndexSet.cpp:40-115): the last dimension fastest.
void fillSet(MultiIndexSet& out, std::vector<unsigned int>& base, unsigned int dim, unsigned int maxOrder, bool total,
             LimiterType const& limiter) {
    unsigned int cur = 0;
    for (unsigned int i = 0; i < dim; ++i) cur += base[i];
    const unsigned int top = total ? maxOrder - cur : maxOrder;
    for (unsigned int i = 0; i <= top; ++i) {
        if (dim == base.size() - 1) {
            base.back() = i;
            MultiIndex m(base);
            if (limiter(m)) out.AddActive(m);
        } else {
            for (size_t k = dim + 1; k < base.size(); ++k) base[k] = 0;
            base[dim] = i;
            fillSet(out, base, dim + 1, maxOrder, total, limiter);
        }
    }
}
}  // namespace

MultiIndexSet MultiIndexSet::CreateTotalOrder(unsigned int length, unsigned int maxOrder,
                                              LimiterType const& limiter) {
    if (length == 0) throw std::invalid_argument("MultiIndexSet::CreateTotalOrder: length must be positive.");
    MultiIndexSet out(length, limiter);
    const LimiterType lim = out.GetLimiter();
    std::vector<unsigned int> base(length, 0);
    fillSet(out, base, 0, maxOrder, true, lim);
    return out;
}

MultiIndexSet MultiIndexSet::CreateTensorProduct(unsigned int length, unsigned int maxDegree,
                                                 LimiterType const& limiter) {
    if (length == 0) throw std::invalid_argument("MultiIndexSet::CreateTensorProduct: length must be positive.");
    MultiIndexSet out(length, limiter);
    const LimiterType lim = out.GetLimiter();
    std::vector<unsigned int> base(length, 0);
    fillSet(out, base, 0, maxDegree, false, lim);
    return out;
}

FixedMultiIndexSet MultiIndexSet::Fix(bool) const {
    std::vector<unsigned int> s{0}, d, o;
    for (int g : a2g_) {
        const auto& v = all_[g].Vector();
        for (unsigned int e = 0; e < length_; ++e)
            if (v[e]) {
                d.push_back(e);
                o.push_back(v[e]);
            }
        s.push_back((unsigned int)d.size());
    }
    return FixedMultiIndexSet(length_, s, d, o);
}

int MultiIndexSet::MultiToIndex(MultiIndex const& m) const {
    auto it = global_.find(m.Vector());
    return it == global_.end() ? -1 : g2a_[it->second];
}

std::vector<unsigned int> MultiIndexSet::NonzeroDiagonalEntries() const {
    std::vector<unsigned int> out;
    for (size_t a = 0; a < a2g_.size(); ++a)
        if (all_[a2g_[a]].HasNonzeroEnd()) out.push_back((unsigned int)a);
    return out;
}

int MultiIndexSet::addMulti(MultiIndex const& m) {
    all_.push_back(m);
    const int g = (int)all_.size() - 1;
    global_[m.Vector()] = g;
    g2a_.push_back(-1);
    in_.emplace_back();
    out_.emplace_back();
    addForward(g, false);
    addBackward(g, false);
    return g;
}

int MultiIndexSet::addInactive(MultiIndex const& m) {
    auto it = global_.find(m.Vector());
    if (it != global_.end()) return it->second;
    if (limiter_(m)) return addMulti(m);
    return -1;
}

void MultiIndexSet::addForward(int g, bool addInactive) {
    std::vector<unsigned int> v = all_[g].Vector();
    for (unsigned int d = 0; d < length_; ++d) {
        ++v[d];
        MultiIndex f(v);
        --v[d];
        if (!limiter_(f)) continue;
        auto it = global_.find(f.Vector());
        if (it != global_.end()) {
            in_[it->second].insert(g);
            out_[g].insert(it->second);
        } else if (addInactive) {
            this->addInactive(f);
        }
    }
}

void MultiIndexSet::addBackward(int g, bool addInactive) {
    std::vector<unsigned int> v = all_[g].Vector();
    for (unsigned int d = 0; d < length_; ++d) {
        if (v[d] == 0) continue;
        --v[d];
        MultiIndex b(v);
        ++v[d];
        if (!limiter_(b)) continue;
        auto it = global_.find(b.Vector());
        if (it != global_.end()) {
            out_[it->second].insert(g);
            in_[g].insert(it->second);
        } else if (addInactive) {
            this->addInactive(b);
        }
    }
}

void MultiIndexSet::activate(int g) {
    if (g2a_[g] >= 0) return;
    a2g_.push_back(g);
    g2a_[g] = (int)a2g_.size() - 1;
    const auto& v = all_[g].Vector();
    for (unsigned int d = 0; d < length_; ++d) maxOrders_[d] = std::max(maxOrders_[d], v[d]);
    addForward(g, true);
    addBackward(g, true);
}

bool MultiIndexSet::admissible(int g) const {
    if (!limiter_(all_[g])) return false;
    if (active(g)) return true;
    unsigned int n = 0;
    for (int h : in_[g]) n += active(h);
    return n == all_[g].NumNz();
}

int MultiIndexSet::AddActive(MultiIndex const& m) {
    if (m.Length() != length_)
        throw std::invalid_argument("MultiIndexSet: a multi-index of length " + std::to_string(m.Length()) +
                                    " in a set of length " + std::to_string(length_) + ".");
    const int g = addInactive(m);
    if (g < 0) return -1;
    activate(g);
    return g2a_[g];
}

void MultiIndexSet::Activate(MultiIndex const& m) {
    auto it = global_.find(m.Vector());
    if (it == global_.end() || !admissible(it->second))
        throw std::invalid_argument("MultiIndexSet::Activate: the multi-index is not an admissible member of the set.");
    activate(it->second);
}

unsigned int MultiIndexSet::Union(MultiIndexSet const& rhs) {
    const unsigned int old = Size();
    for (size_t g = 0; g < rhs.all_.size(); ++g) {
        MultiIndex const& m = rhs.all_[g];
        if (!limiter_(m)) continue;
        const int h = addInactive(m);
        if (rhs.g2a_[g] >= 0 && h >= 0) activate(h);
    }
    return Size() - old;
}

void MultiIndexSet::SetLimiter(LimiterType const& limiter) {
    limiter_ = limiter ? limiter : LimiterType(MultiIndexLimiter::None());
    hasLimiter_ = limiter_.target<MultiIndexLimiter::None>() == nullptr;
    for (size_t g = 0; g < all_.size(); ++g) {  // all_ may grow: new entries are visited too
        if (active((int)g)) {
            if (!limiter_(all_[g])) {
                std::ostringstream os;
                os << "Invalid limiter passed to MultiIndexSet::SetLimiter.  The active multi-index, ["
                   << all_[g].String() << "], is not valid with the new limiter.";
                throw std::invalid_argument(os.str());
            }
            addForward((int)g, true);
        } else if (!limiter_(all_[g])) {
            for (int h : in_[g]) out_[h].erase((int)g);
            in_[g].clear();
        }
    }
}

bool MultiIndexSet::IsActive(MultiIndex const& m) const {
    auto it = global_.find(m.Vector());
    return it != global_.end() && active(it->second);
}

bool MultiIndexSet::IsAdmissible(MultiIndex const& m) const {
    auto it = global_.find(m.Vector());
    return it != global_.end() && admissible(it->second);
}

bool MultiIndexSet::IsExpandable(unsigned int activeIndex) const {
    for (int h : out_[a2g_.at(activeIndex)])
        if (!active(h) && admissible(h)) return true;
    return false;
}

unsigned int MultiIndexSet::NumActiveForward(unsigned int activeIndex) const {
    unsigned int n = 0;
    for (int h : out_[a2g_.at(activeIndex)]) n += active(h);
    return n;
}

unsigned int MultiIndexSet::NumForward(unsigned int activeIndex) const {
    return (unsigned int)out_[a2g_.at(activeIndex)].size();
}

std::vector<unsigned int> MultiIndexSet::Frontier() const {
    std::vector<unsigned int> out;
    for (unsigned int a = 0; a < Size(); ++a)
        if (IsExpandable(a)) out.push_back(a);
    return out;
}

std::vector<unsigned int> MultiIndexSet::StrictFrontier() const {
    std::vector<unsigned int> out;
    for (unsigned int a : Frontier()) {
        bool strict = true;
        for (int h : out_[a2g_[a]]) strict = strict && !active(h);
        if (strict) out.push_back(a);
    }
    return out;
}

std::vector<MultiIndex> MultiIndexSet::Margin() const {
    std::vector<MultiIndex> out;
    for (size_t g = 0; g < all_.size(); ++g) {
        if (active((int)g)) continue;
        for (int h : in_[g])
            if (active(h)) {
                out.push_back(all_[g]);
                break;
            }
    }
    return out;
}

std::vector<MultiIndex> MultiIndexSet::ReducedMargin() const {
    std::vector<MultiIndex> out;
    for (size_t g = 0; g < all_.size(); ++g) {
        if (active((int)g)) continue;
        bool all = true;
        for (int h : in_[g]) all = all && active(h);
        if (all) out.push_back(all_[g]);
    }
    return out;
}

std::vector<MultiIndex> MultiIndexSet::ReducedMarginDim(unsigned int dim) const {
    std::vector<MultiIndex> out;
    for (size_t g = 0; g < all_.size(); ++g) {
        if (active((int)g)) continue;
        bool all = true, less = false;
        for (int h : in_[g]) {
            all = all && active(h);
            less = less || all_[h].Get(dim) < all_[g].Get(dim);
        }
        if (all && less) out.push_back(all_[g]);
    }
    return out;
}

std::vector<unsigned int> MultiIndexSet::Expand(unsigned int activeIndex) {
    if (activeIndex >= Size()) {
        std::ostringstream os;
        os << "Invalid index passed to MultiIndexSet::Expand.  A value of " << activeIndex
           << " was passed to the function, but only " << Size() << " active components exist in the set.";
        throw std::out_of_range(os.str());
    }
    std::vector<unsigned int> out;
    const std::set<int> next = out_[a2g_[activeIndex]];
    for (int h : next)
        if (admissible(h) && !active(h)) {
            activate(h);
            out.push_back((unsigned int)g2a_[h]);
        }
    return out;
}

std::vector<unsigned int> MultiIndexSet::Expand() {
    std::vector<int> pending;
    for (unsigned int a : Frontier()) {
        const std::set<int> next = out_[a2g_[a]];
        for (int h : next)
            if (admissible(h) && !active(h)) pending.push_back(h);
    }
    std::vector<unsigned int> out;
    for (int h : pending) {
        activate(h);
        out.push_back((unsigned int)g2a_[h]);
    }
    return out;
}

}  // namespace mpgb
