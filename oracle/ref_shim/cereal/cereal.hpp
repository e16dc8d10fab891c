// ORACLE -- test infrastructure only.
//
// A serial stand-in for the part of cereal v1.3.2 (github.com/USCiLab/cereal,
// the version the reference's CMakeLists.txt:196-201 fetches; not in the
// reference checkout) that the reference's map classes use to save
// themselves: the binary output archive and the polymorphic shared_ptr
// encoding.  Written here from cereal's documented archive format, so that
// the reference's own save functions (MonotoneComponent.h:1035-1044,
// TriangularMap.h:130-138, MultivariateExpansionWorker.h:406-412,
// Quadrature.h:66-90/422-435/678-690/970-984, FixedMultiIndexSet.h:113-123,
// MapOptions.h:125-131, Utilities/Serialization.h:19-88) produce the bytes
// ParameterizedFunctionBase::Save (ParameterizedFunctionBase.h:197-202) writes.
//
// The format:
//   * arithmetic values: their bytes in native order (bool one byte); enums
//     as their underlying type; a size tag as uint64;
//   * std::string: uint64 length, then the characters;
//   * std::vector: uint64 element count, then the elements;
//   * base_class<B>(this): B's own save, nothing else;
//   * std::shared_ptr<T>, T polymorphic: a uint32 polymorphic id -- 0 for a
//     null pointer; for a registered type, the archive's id for the type's
//     registered name (ids from 1, in first-use order), with the top bit set
//     and the name (as a string) following on its first use; 0x40000000 when
//     T is not abstract and the object is exactly a T -- then a uint32
//     pointer id (ids from 1 per distinct object address, first-use order;
//     top bit set on first use, and only then the object's data follows);
//   * a class: its member save(ar) const, member serialize(ar), or free
//     save(ar, t) (found by argument-dependent lookup), whichever it has.
// Loading is not provided: the input archive and cereal::construct exist so
// that the reference's load functions compile, and throw if called.
#pragma once

#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <typeindex>
#include <typeinfo>
#include <unordered_map>
#include <utility>
#include <vector>

namespace cereal {

class BinaryOutputArchive;
class BinaryInputArchive;

template <class T>
struct BinaryData {
    T data;
    uint64_t size;
};

template <class T>
BinaryData<T> binary_data(T&& data, size_t size) {
    return BinaryData<T>{std::forward<T>(data), (uint64_t)size};
}

namespace traits {
template <class T, class Archive>
struct is_output_serializable : std::is_same<Archive, BinaryOutputArchive> {};
template <class T, class Archive>
struct is_input_serializable : std::is_same<Archive, BinaryInputArchive> {};
}  // namespace traits

// base_class<B>(this): serialize the B part of the object.
template <class Base>
struct base_class {
    template <class Derived>
    base_class(const Derived* derived) : base_ptr(static_cast<const Base*>(derived)) {}
    const Base* base_ptr;
};

template <class T>
class construct {
public:
    template <class... Args>
    void operator()(Args&&...) {
        throw std::logic_error("cereal stand-in: loading is not provided");
    }
};

// Friend of the classes whose save functions are private.
class access {
public:
    template <class A, class T>
    static auto has_member_save(int) -> decltype(std::declval<const T&>().save(std::declval<A&>()), std::true_type{});
    template <class A, class T>
    static std::false_type has_member_save(...);
    template <class A, class T>
    static auto has_member_serialize(int)
        -> decltype(std::declval<T&>().serialize(std::declval<A&>()), std::true_type{});
    template <class A, class T>
    static std::false_type has_member_serialize(...);

    template <class A, class T>
    static void member_save(A& ar, const T& t) {
        t.save(ar);
    }
    template <class A, class T>
    static void member_serialize(A& ar, const T& t) {
        const_cast<T&>(t).serialize(ar);
    }
};

namespace detail {

constexpr uint32_t msb_32bit = 0x80000000u;
constexpr uint32_t msb2_32bit = 0x40000000u;

// The registered name of a polymorphic type (CEREAL_REGISTER_TYPE).
template <class T>
struct binding_name {};

struct OutputBinding {
    const char* name;
    // Saves the object whose most-derived address is given.
    void (*save)(BinaryOutputArchive&, const void*);
};

inline std::unordered_map<std::type_index, OutputBinding>& outputBindings() {
    static std::unordered_map<std::type_index, OutputBinding> m;
    return m;
}

template <class T>
struct is_vector : std::false_type {};
template <class T, class A>
struct is_vector<std::vector<T, A>> : std::true_type {};
template <class T>
struct is_shared_ptr : std::false_type {};
template <class T>
struct is_shared_ptr<std::shared_ptr<T>> : std::true_type {};
template <class T>
struct is_base_class : std::false_type {};
template <class T>
struct is_base_class<base_class<T>> : std::true_type {};
template <class T>
struct is_binary_data : std::false_type {};
template <class T>
struct is_binary_data<BinaryData<T>> : std::true_type {};

template <class A, class T>
auto has_free_save(int) -> decltype(save(std::declval<A&>(), std::declval<const T&>()), std::true_type{});
template <class A, class T>
std::false_type has_free_save(...);

}  // namespace detail

class BinaryOutputArchive {
public:
    explicit BinaryOutputArchive(std::ostream& os) : os_(os) {}

    template <class... Ts>
    BinaryOutputArchive& operator()(Ts&&... ts) {
        (process(ts), ...);
        return *this;
    }

    void saveBinary(const void* data, size_t n) {
        os_.write(static_cast<const char*>(data), (std::streamsize)n);
        if (!os_) throw std::runtime_error("cereal stand-in: failed to write to the stream");
    }

    uint32_t registerPolymorphicType(const char* name) {
        auto it = typeIds_.find(name);
        if (it != typeIds_.end()) return it->second;
        const uint32_t id = nextTypeId_++;
        typeIds_.emplace(name, id);
        return id | detail::msb_32bit;
    }

    uint32_t registerSharedPointer(const void* addr) {
        if (addr == nullptr) return 0;
        auto it = ptrIds_.find(addr);
        if (it != ptrIds_.end()) return it->second;
        const uint32_t id = nextPtrId_++;
        ptrIds_.emplace(addr, id);
        return id | detail::msb_32bit;
    }

    template <class T>
    void process(const T& t) {
        using U = std::decay_t<T>;
        if constexpr (std::is_arithmetic_v<U>) {
            saveBinary(&t, sizeof(U));
        } else if constexpr (std::is_enum_v<U>) {
            const std::underlying_type_t<U> v = static_cast<std::underlying_type_t<U>>(t);
            saveBinary(&v, sizeof(v));
        } else if constexpr (std::is_same_v<U, std::string>) {
            const uint64_t n = t.size();
            saveBinary(&n, sizeof(n));
            saveBinary(t.data(), t.size());
        } else if constexpr (detail::is_binary_data<U>::value) {
            saveBinary(t.data, (size_t)t.size);
        } else if constexpr (detail::is_vector<U>::value) {
            const uint64_t n = t.size();
            saveBinary(&n, sizeof(n));
            for (const auto& e : t) process(e);
        } else if constexpr (detail::is_base_class<U>::value) {
            processClass(*t.base_ptr);
        } else if constexpr (detail::is_shared_ptr<U>::value) {
            saveShared(t);
        } else {
            processClass(t);
        }
    }

private:
    template <class T>
    void processClass(const T& t) {
        constexpr bool mSave = decltype(access::has_member_save<BinaryOutputArchive, T>(0))::value;
        constexpr bool mSer = decltype(access::has_member_serialize<BinaryOutputArchive, T>(0))::value;
        constexpr bool fSave = decltype(detail::has_free_save<BinaryOutputArchive, T>(0))::value;
        static_assert(mSave || mSer || fSave, "cereal stand-in: type has no save or serialize function");
        if constexpr (mSave)
            access::member_save(*this, t);
        else if constexpr (mSer)
            access::member_serialize(*this, t);
        else
            save(*this, t);
    }

    template <class T>
    void saveShared(const std::shared_ptr<T>& ptr) {
        using B = std::remove_const_t<T>;
        if constexpr (std::is_polymorphic_v<B>) {
            if (!ptr) {
                const uint32_t zero = 0;
                saveBinary(&zero, 4);
                return;
            }
            if constexpr (!std::is_abstract_v<B>) {
                if (typeid(*ptr) == typeid(B)) {
                    const uint32_t id = detail::msb2_32bit;
                    saveBinary(&id, 4);
                    saveObject(static_cast<const void*>(ptr.get()), *ptr);
                    return;
                }
            }
            auto& m = detail::outputBindings();
            auto it = m.find(std::type_index(typeid(*ptr)));
            if (it == m.end())
                throw std::runtime_error(std::string("cereal stand-in: unregistered polymorphic type ") +
                                         typeid(*ptr).name());
            const uint32_t tid = registerPolymorphicType(it->second.name);
            saveBinary(&tid, 4);
            if (tid & detail::msb_32bit) process(std::string(it->second.name));
            const void* most = dynamic_cast<const void*>(ptr.get());
            const uint32_t pid = registerSharedPointer(most);
            saveBinary(&pid, 4);
            if (pid & detail::msb_32bit) it->second.save(*this, most);
        } else {
            saveObject(static_cast<const void*>(ptr.get()), *ptr);
        }
    }

    template <class T>
    void saveObject(const void* addr, const T& obj) {
        const uint32_t pid = registerSharedPointer(addr);
        saveBinary(&pid, 4);
        if (pid & detail::msb_32bit) processClass(obj);
    }

    std::ostream& os_;
    std::map<std::string, uint32_t> typeIds_;
    uint32_t nextTypeId_ = 1;
    std::map<const void*, uint32_t> ptrIds_;
    uint32_t nextPtrId_ = 1;
};

class BinaryInputArchive {
public:
    template <class Stream>
    explicit BinaryInputArchive(Stream&) {}
    template <class... Ts>
    BinaryInputArchive& operator()(Ts&&...) {
        throw std::logic_error("cereal stand-in: loading is not provided");
    }
};

namespace detail {
template <class T>
struct Registrar {
    Registrar() {
        outputBindings()[std::type_index(typeid(T))] = OutputBinding{
            binding_name<T>::name(),
            [](BinaryOutputArchive& ar, const void* p) { ar(*static_cast<const T*>(p)); }};
    }
};
}  // namespace detail

}  // namespace cereal

#define CEREAL_SHIM_CAT2(a, b) a##b
#define CEREAL_SHIM_CAT(a, b) CEREAL_SHIM_CAT2(a, b)

// The registered name is the macro argument as written, as in cereal.
#define CEREAL_REGISTER_TYPE(...)                                                      \
    namespace cereal {                                                                 \
    namespace detail {                                                                 \
    template <>                                                                        \
    struct binding_name<__VA_ARGS__> {                                                 \
        static constexpr const char* name() { return #__VA_ARGS__; }                   \
    };                                                                                 \
    }                                                                                  \
    }                                                                                  \
    namespace {                                                                        \
    const ::cereal::detail::Registrar<__VA_ARGS__> CEREAL_SHIM_CAT(cerealShimReg, __COUNTER__); \
    }

// One shared library holds every registration here, so the dynamic-init
// hooks have nothing to do.
#define CEREAL_REGISTER_DYNAMIC_INIT(LibName)
#define CEREAL_FORCE_DYNAMIC_INIT(LibName)
