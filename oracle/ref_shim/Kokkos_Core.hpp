// ORACLE -- test infrastructure only.
//
// A minimal, serial stand-in for the part of Kokkos 4.2's API that MParT's
// monotone-component sources use, so that those reference files compile
// unchanged into oracle/_ref (Kokkos itself is not installed here).  Host
// memory only; every parallel dispatch runs in order on the calling thread;
// a TeamPolicy runs its league with one thread per team and hands each call
// fresh per-thread scratch memory.  Views are reference counted (owning) or
// unmanaged, of rank 1 or 2, with LayoutRight (the host default), LayoutLeft
// or LayoutStride.  Owning views are zero-initialised, as Kokkos' are.
#pragma once

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_VERSION 40200
#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]
#define KOKKOS_IF_ON_DEVICE(CODE)
#define KOKKOS_IF_ON_HOST(CODE) \
    { CODE }

namespace Kokkos {

struct Serial;
struct HostSpace {
    using memory_space = HostSpace;
    using execution_space = Serial;
};
struct Serial {
    using memory_space = HostSpace;
    using execution_space = Serial;
    void fence() const {}
};
using DefaultHostExecutionSpace = Serial;
using DefaultExecutionSpace = Serial;

inline void initialize(int = 0, char** = nullptr) {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string&) {}
[[noreturn]] inline void abort(const char* msg) {
    std::fprintf(stderr, "Kokkos::abort: %s\n", msg);
    std::abort();
}

template <class T>
KOKKOS_INLINE_FUNCTION void atomic_max(T* p, T v) {
    if (v > *p) *p = v;
}

using std::exp;
using std::fabs;
using std::log;
using std::pow;
using std::sqrt;
using std::tanh;
namespace Experimental {
using std::exp;
using std::fabs;
using std::log;
using std::pow;
using std::sqrt;
using std::tanh;
}  // namespace Experimental

template <class T1, class T2 = T1>
struct pair {
    T1 first;
    T2 second;
    pair() = default;
    pair(T1 a, T2 b) : first(a), second(b) {}
};
template <class T1, class T2>
pair<T1, T2> make_pair(T1 a, T2 b) {
    return pair<T1, T2>(a, b);
}

struct ALL_t {
    constexpr const ALL_t& operator()() const { return *this; }
};
inline constexpr ALL_t ALL{};
inline constexpr ALL_t All{};

struct LayoutRight {};
struct LayoutLeft {};
struct LayoutStride {
    size_t dimension[2] = {0, 0};
    size_t stride[2] = {0, 0};
    LayoutStride() = default;
    LayoutStride(size_t n0, size_t s0, size_t n1 = 0, size_t s1 = 0) {
        dimension[0] = n0;
        stride[0] = s0;
        dimension[1] = n1;
        stride[1] = s1;
    }
};

enum MemoryTraitsFlags : unsigned { Unmanaged = 1, RandomAccess = 2, Atomic = 4, Restrict = 8 };
template <unsigned Flags>
struct MemoryTraits {};

// Per-thread scratch of a team dispatch: views constructed from it take
// consecutive, 8-byte aligned pieces.
struct ScratchMemorySpace {
    mutable char* cur = nullptr;
    char* end = nullptr;
    void* get_shmem(size_t bytes) const {
        char* p = cur;
        cur += (bytes + 7) & ~size_t(7);
        if (cur > end) throw std::runtime_error("Kokkos shim: thread scratch exhausted");
        return p;
    }
};

namespace Impl {
template <class D>
struct DataTraits;
template <class T>
struct DataTraits<T*> {
    using value = T;
    static constexpr unsigned rank = 1;
    template <class U>
    using rebind = U*;
};
template <class T>
struct DataTraits<T**> {
    using value = T;
    static constexpr unsigned rank = 2;
    template <class U>
    using rebind = U**;
};

template <class... P>
struct LayoutOf {
    using type = LayoutRight;
};
template <class P0, class... P>
struct LayoutOf<P0, P...> {
    using type = std::conditional_t<std::is_same_v<P0, LayoutRight> || std::is_same_v<P0, LayoutLeft> ||
                                        std::is_same_v<P0, LayoutStride>,
                                    P0, typename LayoutOf<P...>::type>;
};
}  // namespace Impl

template <class DataType, class... Props>
class View {
    using Tr = Impl::DataTraits<DataType>;

public:
    using value_type = typename Tr::value;
    using non_const_value_type = std::remove_const_t<value_type>;
    using const_value_type = const non_const_value_type;
    using pointer_type = value_type*;
    using reference_type = value_type&;
    using data_type = DataType;
    using non_const_data_type = typename Tr::template rebind<non_const_value_type>;
    using const_data_type = typename Tr::template rebind<const_value_type>;
    using array_layout = typename Impl::LayoutOf<Props...>::type;
    using memory_space = HostSpace;
    using execution_space = Serial;
    using size_type = size_t;
    using HostMirror = View<non_const_data_type, array_layout, HostSpace>;
    using non_const_type = View<non_const_data_type, array_layout, HostSpace>;
    using const_type = View<const_data_type, array_layout, HostSpace>;
    static constexpr unsigned Rank = Tr::rank;
    static constexpr unsigned rank() { return Tr::rank; }

    View() = default;

    // Owning, zero-initialised.
    explicit View(const std::string& label, size_t n0 = 0, size_t n1 = 0, size_t = 0, size_t = 0, size_t = 0,
                  size_t = 0, size_t = 0, size_t = 0)
        : label_(label) {
        allocate(n0, n1);
    }
    // Unmanaged, on caller memory.
    View(pointer_type p, size_t n0, size_t n1 = 0, size_t = 0, size_t = 0, size_t = 0, size_t = 0, size_t = 0,
         size_t = 0) {
        p_ = p;
        setShape(n0, n1);
    }
    View(pointer_type p, const LayoutStride& ls) {
        p_ = p;
        n_[0] = ls.dimension[0];
        n_[1] = Tr::rank > 1 ? ls.dimension[1] : 1;
        s_[0] = ls.stride[0];
        s_[1] = Tr::rank > 1 ? ls.stride[1] : 0;
    }
    // Thread scratch.
    View(const ScratchMemorySpace& sp, size_t n0, size_t n1 = 0) {
        setShape(n0, n1);
        p_ = (pointer_type)sp.get_shmem(span() * sizeof(value_type));
    }
    // Shallow conversion (adds const, changes layout or memory traits).
    template <class D2, class... P2,
              class = std::enable_if_t<Impl::DataTraits<D2>::rank == Tr::rank &&
                                       std::is_convertible_v<typename Impl::DataTraits<D2>::value*, pointer_type>>>
    View(const View<D2, P2...>& o) : own_(o.own_), p_(o.p_), label_(o.label_) {
        n_[0] = o.n_[0];
        n_[1] = o.n_[1];
        s_[0] = o.s_[0];
        s_[1] = o.s_[1];
    }

    reference_type operator()(size_t i) const { return p_[i * s_[0]]; }
    reference_type operator()(size_t i, size_t j) const { return p_[i * s_[0] + j * s_[1]]; }
    reference_type operator[](size_t i) const { return p_[i * s_[0]]; }

    size_t extent(unsigned r) const { return r < Tr::rank ? n_[r] : 1; }
    int extent_int(unsigned r) const { return (int)extent(r); }
    size_t stride(unsigned r) const { return r < Tr::rank ? (size_t)s_[r] : 0; }
    size_t stride_0() const { return (size_t)s_[0]; }
    size_t stride_1() const { return (size_t)s_[1]; }
    template <class I>
    void stride(I* out) const {
        for (unsigned r = 0; r < Tr::rank; ++r) out[r] = (I)s_[r];
    }
    size_t size() const { return Tr::rank == 1 ? n_[0] : n_[0] * n_[1]; }
    size_t span() const {
        if (size() == 0) return 0;
        if (Tr::rank == 1) return (n_[0] - 1) * (size_t)s_[0] + 1;
        return (n_[0] - 1) * (size_t)s_[0] + (n_[1] - 1) * (size_t)s_[1] + 1;
    }
    pointer_type data() const { return p_; }
    const std::string& label() const { return label_; }
    bool is_allocated() const { return p_ != nullptr; }
    long use_count() const { return own_.use_count(); }
    bool span_is_contiguous() const { return span() == size(); }
    LayoutStride layout() const { return LayoutStride(n_[0], s_[0], n_[1], s_[1]); }
    static size_t shmem_size(size_t n0, size_t n1 = 1) { return n0 * (n1 ? n1 : 1) * sizeof(value_type) + 64; }

    // (used by Kokkos::resize)
    void allocate(size_t n0, size_t n1) {
        setShape(n0, n1);
        const size_t n = std::max<size_t>(size(), 1);
        std::shared_ptr<non_const_value_type> mem(new non_const_value_type[n](),
                                                  std::default_delete<non_const_value_type[]>());
        own_ = mem;
        p_ = mem.get();
    }

    std::shared_ptr<void> own_;
    pointer_type p_ = nullptr;
    size_t n_[2] = {0, 1};
    ptrdiff_t s_[2] = {1, 0};
    std::string label_;

private:
    void setShape(size_t n0, size_t n1) {
        n_[0] = n0;
        n_[1] = Tr::rank > 1 ? n1 : 1;
        if (Tr::rank == 1) {
            s_[0] = 1;
            s_[1] = 0;
        } else if (std::is_same_v<array_layout, LayoutLeft>) {
            s_[0] = 1;
            s_[1] = (ptrdiff_t)n0;
        } else {
            s_[0] = (ptrdiff_t)n1;
            s_[1] = 1;
        }
    }
};

// ---- subviews --------------------------------------------------------------
namespace Impl {
inline size_t first(ALL_t, size_t) { return 0; }
template <class A, class B>
size_t first(const pair<A, B>& p, size_t) {
    return (size_t)p.first;
}
template <class A, class B>
size_t first(const std::pair<A, B>& p, size_t) {
    return (size_t)p.first;
}
inline size_t count(ALL_t, size_t n) { return n; }
template <class A, class B>
size_t count(const pair<A, B>& p, size_t) {
    return (size_t)(p.second - p.first);
}
template <class A, class B>
size_t count(const std::pair<A, B>& p, size_t) {
    return (size_t)(p.second - p.first);
}
template <class T>
constexpr bool isRange = std::is_same_v<std::decay_t<T>, ALL_t>;
template <class A, class B>
constexpr bool isRangeP(const pair<A, B>*) {
    return true;
}
template <class A, class B>
constexpr bool isRangeP(const std::pair<A, B>*) {
    return true;
}
constexpr bool isRangeP(const void*) { return false; }
template <class T>
constexpr bool range_v = isRange<T> || isRangeP((const std::decay_t<T>*)nullptr);
}  // namespace Impl

template <class D, class... P, class R>
auto subview(const View<D, P...>& v, R r) {
    static_assert(View<D, P...>::Rank == 1, "rank-1 subview of a rank-1 view");
    using T = typename View<D, P...>::value_type;
    View<T*, LayoutStride, HostSpace> o(v);
    const size_t a = Impl::first(r, v.n_[0]);
    o.p_ = v.p_ + a * v.s_[0];
    o.n_[0] = Impl::count(r, v.n_[0]);
    return o;
}

template <class D, class... P, class R0, class R1>
auto subview(const View<D, P...>& v, R0 r0, R1 r1) {
    static_assert(View<D, P...>::Rank == 2, "subview of a rank-2 view");
    using T = typename View<D, P...>::value_type;
    constexpr bool a = Impl::range_v<R0>, b = Impl::range_v<R1>;
    if constexpr (a && b) {
        View<T**, LayoutStride, HostSpace> o;
        o.own_ = v.own_;
        o.p_ = v.p_ + Impl::first(r0, v.n_[0]) * v.s_[0] + Impl::first(r1, v.n_[1]) * v.s_[1];
        o.n_[0] = Impl::count(r0, v.n_[0]);
        o.n_[1] = Impl::count(r1, v.n_[1]);
        o.s_[0] = v.s_[0];
        o.s_[1] = v.s_[1];
        return o;
    } else if constexpr (a) {
        View<T*, LayoutStride, HostSpace> o;
        o.own_ = v.own_;
        o.p_ = v.p_ + Impl::first(r0, v.n_[0]) * v.s_[0] + (size_t)r1 * v.s_[1];
        o.n_[0] = Impl::count(r0, v.n_[0]);
        o.s_[0] = v.s_[0];
        return o;
    } else if constexpr (b) {
        View<T*, LayoutStride, HostSpace> o;
        o.own_ = v.own_;
        o.p_ = v.p_ + (size_t)r0 * v.s_[0] + Impl::first(r1, v.n_[1]) * v.s_[1];
        o.n_[0] = Impl::count(r1, v.n_[1]);
        o.s_[0] = v.s_[1];
        return o;
    } else {
        return v(r0, r1);
    }
}

// ---- copies ----------------------------------------------------------------
template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
    if (dst.extent(0) != src.extent(0) || dst.extent(1) != src.extent(1))
        throw std::runtime_error("Kokkos shim: deep_copy extents differ");
    if ((const void*)dst.data() == (const void*)src.data()) return;
    if constexpr (View<D1, P1...>::Rank == 1) {
        for (size_t i = 0; i < dst.extent(0); ++i) dst(i) = src(i);
    } else {
        for (size_t i = 0; i < dst.extent(0); ++i)
            for (size_t j = 0; j < dst.extent(1); ++j) dst(i, j) = src(i, j);
    }
}
template <class D1, class... P1, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>
void deep_copy(const View<D1, P1...>& dst, S value) {
    if constexpr (View<D1, P1...>::Rank == 1) {
        for (size_t i = 0; i < dst.extent(0); ++i) dst(i) = value;
    } else {
        for (size_t i = 0; i < dst.extent(0); ++i)
            for (size_t j = 0; j < dst.extent(1); ++j) dst(i, j) = value;
    }
}
template <class Space, class D1, class... P1, class D2, class... P2>
void deep_copy(const Space&, const View<D1, P1...>& dst, const View<D2, P2...>& src) {
    deep_copy(dst, src);
}

template <class D, class... P>
typename View<D, P...>::HostMirror create_mirror_view(const View<D, P...>& v) {
    typename View<D, P...>::HostMirror m;
    m.own_ = v.own_;
    m.p_ = const_cast<typename View<D, P...>::non_const_value_type*>(v.p_);
    m.n_[0] = v.n_[0];
    m.n_[1] = v.n_[1];
    m.s_[0] = v.s_[0];
    m.s_[1] = v.s_[1];
    m.label_ = v.label_;
    return m;
}
template <class Space, class D, class... P>
typename View<D, P...>::HostMirror create_mirror_view(const Space&, const View<D, P...>& v) {
    return create_mirror_view(v);
}
template <class Space, class D, class... P>
typename View<D, P...>::HostMirror create_mirror_view_and_copy(const Space&, const View<D, P...>& v) {
    return create_mirror_view(v);
}

template <class D, class... P>
void resize(View<D, P...>& v, size_t n0, size_t n1 = 0) {
    View<D, P...> old = v;
    v.allocate(n0, n1);
    if constexpr (View<D, P...>::Rank == 1) {
        for (size_t i = 0; i < std::min(n0, old.extent(0)); ++i) v(i) = old(i);
    } else {
        for (size_t i = 0; i < std::min(n0, old.extent(0)); ++i)
            for (size_t j = 0; j < std::min(n1, old.extent(1)); ++j) v(i, j) = old(i, j);
    }
}

// ---- dispatch ----------------------------------------------------------------
struct ParallelForTag {};
struct AUTO_t {};
inline constexpr AUTO_t AUTO{};

template <class ExecSpace = Serial, class... P>
class RangePolicy {
public:
    RangePolicy() = default;
    template <class B, class E>
    RangePolicy(B b, E e) : b_((long long)b), e_((long long)e) {}
    template <class B, class E>
    RangePolicy(const ExecSpace&, B b, E e) : b_((long long)b), e_((long long)e) {}
    long long begin() const { return b_; }
    long long end() const { return e_; }

private:
    long long b_ = 0, e_ = 0;
};

struct PerTeamValue {
    size_t v;
};
struct PerThreadValue {
    size_t v;
};
inline PerTeamValue PerTeam(size_t v) { return {v}; }
inline PerThreadValue PerThread(size_t v) { return {v}; }

template <class ExecSpace = Serial, class... P>
class TeamPolicy {
public:
    class member_type {
    public:
        member_type(int league, int team, int rank, const ScratchMemorySpace* s)
            : league_(league), team_(team), rank_(rank), s_(s) {}
        int league_rank() const { return league_; }
        int team_size() const { return team_; }
        int team_rank() const { return rank_; }
        const ScratchMemorySpace& thread_scratch(int) const { return *s_; }
        const ScratchMemorySpace& team_scratch(int) const { return *s_; }
        void team_barrier() const {}

    private:
        int league_, team_, rank_;
        const ScratchMemorySpace* s_;
    };

    TeamPolicy() = default;
    TeamPolicy(int league, int team) : league_(league), team_(team) {}
    TeamPolicy(int league, AUTO_t) : league_(league), team_(1) {}
    TeamPolicy& set_scratch_size(int, PerTeamValue t, PerThreadValue th) {
        perTeam_ = t.v;
        perThread_ = th.v;
        return *this;
    }
    TeamPolicy& set_scratch_size(int, PerThreadValue th) {
        perThread_ = th.v;
        return *this;
    }
    TeamPolicy& set_scratch_size(int, PerTeamValue t) {
        perTeam_ = t.v;
        return *this;
    }
    template <class F>
    int team_size_recommended(const F&, ParallelForTag) const {
        return 1;
    }
    template <class F>
    int team_size_max(const F&, ParallelForTag) const {
        return 1;
    }
    int league_size() const { return league_; }
    int team_size() const { return team_; }
    size_t scratch_bytes() const { return perTeam_ + perThread_; }

private:
    int league_ = 0, team_ = 1;
    size_t perTeam_ = 0, perThread_ = 0;
};

template <unsigned N>
struct Rank {};
struct Index2 {
    long long v[2];
};
template <class R, class ExecSpace = Serial>
class MDRangePolicy {
public:
    // {{a, b}} bounds
    MDRangePolicy(const Index2& b, const Index2& e) : b_{b.v[0], b.v[1]}, e_{e.v[0], e.v[1]} {}
    // {a, b} bounds of any integral types
    template <class LT, class UT>
    MDRangePolicy(const LT (&b)[2], const UT (&e)[2])
        : b_{(long long)b[0], (long long)b[1]}, e_{(long long)e[0], (long long)e[1]} {}
    long long b_[2] = {0, 0}, e_[2] = {0, 0};
};
template <class R, class E, class F>
void parallel_for(const MDRangePolicy<R, E>& p, const F& f) {
    for (long long i = p.b_[0]; i < p.e_[0]; ++i)
        for (long long j = p.b_[1]; j < p.e_[1]; ++j) f((int)i, (int)j);
}

template <class E, class... P, class F>
void parallel_for(const RangePolicy<E, P...>& p, const F& f) {
    for (long long i = p.begin(); i < p.end(); ++i) f(i);
}
template <class E, class... P, class F>
void parallel_for(const TeamPolicy<E, P...>& p, const F& f) {
    std::vector<double> buf((p.scratch_bytes() + 64) / sizeof(double) + 1);
    for (int l = 0; l < p.league_size(); ++l)
        for (int r = 0; r < p.team_size(); ++r) {
            ScratchMemorySpace s;
            s.cur = (char*)buf.data();
            s.end = s.cur + buf.size() * sizeof(double);
            typename TeamPolicy<E, P...>::member_type m(l, p.team_size(), r, &s);
            f(m);
        }
}
template <class F>
void parallel_for(size_t n, const F& f) {
    for (size_t i = 0; i < n; ++i) f(i);
}
template <class Pol, class F>
void parallel_for(const std::string&, const Pol& p, const F& f) {
    parallel_for(p, f);
}

namespace Impl {
template <class T>
struct ScanValue;
template <class C, class I, class V>
struct ScanValue<void (C::*)(I, V&, bool) const> {
    using type = V;
};
}  // namespace Impl

template <class E, class... P, class F>
void parallel_scan(const RangePolicy<E, P...>& p, const F& f) {
    typename Impl::ScanValue<decltype(&F::operator())>::type update{};
    for (long long i = p.begin(); i < p.end(); ++i) f(i, update, true);
}

}  // namespace Kokkos
