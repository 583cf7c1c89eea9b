// Header-only C++ front end with the reference's einsum / permute call shape:
//
//   einsum(C_prefactor, Indices{i, j}, &C, AB_prefactor, Indices{i, k}, A, Indices{k, j}, B, &choice);
//   einsum(Indices{i, j}, &C, Indices{i, k}, A, Indices{k, j}, B);          // prefactors 0 and 1
//   einsum(..., &C_list, ..., A_list, ..., B_list, &choice);                  // std::vector batches
//   permute(C_prefactor, Indices{j, i}, &C, A_prefactor, Indices{i, j}, A);
//
// mirroring libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/TensorAlgebra.hpp:41-137,
// Backends/Dispatch.hpp:1264-1286 and Permute.hpp:330-339.  The pattern analysis
// (classify.hpp) runs at compile time on the index tags, as the reference's
// template dispatch does; the call then goes through the C ABI
// (einsums_gb300.h) to the sm_103a kernels, which also apply the reference's
// runtime stride vetoes and report the final AlgorithmChoice.  Operands are
// DeviceTensor / DeviceTensorView (row-major FP64 device storage).
// Errors surface as exceptions named like the reference's (rank_error,
// dimension_error; Errors/Error.hpp:90-190).
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../einsums_gb300.h"
#include "classify.hpp"

namespace einsums {

// ------------------------------------------------------------- errors ----
struct einsums_error : std::runtime_error {
    eg_status status;
    einsums_error(eg_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};
struct rank_error : einsums_error {
    using einsums_error::einsums_error;
};
struct dimension_error : einsums_error {
    using einsums_error::einsums_error;
};
struct not_supported_error : einsums_error {
    using einsums_error::einsums_error;
};

namespace detail {
inline void check(eg_status s) {
    if (s == EG_SUCCESS) return;
    std::string msg = std::string(eg_status_string(s)) + ": " + eg_last_error();
    if (s == EG_ERROR_RANK) throw rank_error(s, msg);
    if (s == EG_ERROR_DIMENSION) throw dimension_error(s, msg);
    if (s == EG_ERROR_NOT_SUPPORTED) throw not_supported_error(s, msg);
    throw einsums_error(s, msg);
}

// FNV-1a of an index tag's letter, masked to 31 bits (the Python front end
// hashes index names the same way).
constexpr int32_t label_of(const char *s) {
    uint32_t h = 0x811C9DC5u;
    for (; *s; ++s) {
        h ^= (uint8_t)*s;
        h *= 0x01000193u;
    }
    return (int32_t)(h & 0x7FFFFFFFu);
}
} // namespace detail

// ------------------------------------------------------------ indices ----
namespace index {
struct LabelBase {};
} // namespace index

#define EINSUMS_GB300_MAKE_INDEX(x)                                                                                    \
    namespace index {                                                                                                  \
    struct x : public LabelBase {                                                                                      \
        static constexpr const char *letter = #x;                                                                      \
        constexpr x() = default;                                                                                       \
    };                                                                                                                 \
    inline constexpr struct x x {};                                                                                    \
    }

EINSUMS_GB300_MAKE_INDEX(A) EINSUMS_GB300_MAKE_INDEX(a) EINSUMS_GB300_MAKE_INDEX(B) EINSUMS_GB300_MAKE_INDEX(b)
EINSUMS_GB300_MAKE_INDEX(C) EINSUMS_GB300_MAKE_INDEX(c) EINSUMS_GB300_MAKE_INDEX(D) EINSUMS_GB300_MAKE_INDEX(d)
EINSUMS_GB300_MAKE_INDEX(E) EINSUMS_GB300_MAKE_INDEX(e) EINSUMS_GB300_MAKE_INDEX(F) EINSUMS_GB300_MAKE_INDEX(f)
EINSUMS_GB300_MAKE_INDEX(G) EINSUMS_GB300_MAKE_INDEX(g) EINSUMS_GB300_MAKE_INDEX(H) EINSUMS_GB300_MAKE_INDEX(h)
EINSUMS_GB300_MAKE_INDEX(I) EINSUMS_GB300_MAKE_INDEX(i) EINSUMS_GB300_MAKE_INDEX(J) EINSUMS_GB300_MAKE_INDEX(j)
EINSUMS_GB300_MAKE_INDEX(K) EINSUMS_GB300_MAKE_INDEX(k) EINSUMS_GB300_MAKE_INDEX(L) EINSUMS_GB300_MAKE_INDEX(l)
EINSUMS_GB300_MAKE_INDEX(M) EINSUMS_GB300_MAKE_INDEX(m) EINSUMS_GB300_MAKE_INDEX(N) EINSUMS_GB300_MAKE_INDEX(n)
EINSUMS_GB300_MAKE_INDEX(O) EINSUMS_GB300_MAKE_INDEX(o) EINSUMS_GB300_MAKE_INDEX(P) EINSUMS_GB300_MAKE_INDEX(p)
EINSUMS_GB300_MAKE_INDEX(Q) EINSUMS_GB300_MAKE_INDEX(q) EINSUMS_GB300_MAKE_INDEX(R) EINSUMS_GB300_MAKE_INDEX(r)
EINSUMS_GB300_MAKE_INDEX(S) EINSUMS_GB300_MAKE_INDEX(s) EINSUMS_GB300_MAKE_INDEX(T) EINSUMS_GB300_MAKE_INDEX(t)
EINSUMS_GB300_MAKE_INDEX(U) EINSUMS_GB300_MAKE_INDEX(u) EINSUMS_GB300_MAKE_INDEX(V) EINSUMS_GB300_MAKE_INDEX(v)
EINSUMS_GB300_MAKE_INDEX(W) EINSUMS_GB300_MAKE_INDEX(w) EINSUMS_GB300_MAKE_INDEX(X) EINSUMS_GB300_MAKE_INDEX(x)
EINSUMS_GB300_MAKE_INDEX(Y) EINSUMS_GB300_MAKE_INDEX(y) EINSUMS_GB300_MAKE_INDEX(Z) EINSUMS_GB300_MAKE_INDEX(z)
EINSUMS_GB300_MAKE_INDEX(alpha) EINSUMS_GB300_MAKE_INDEX(beta) EINSUMS_GB300_MAKE_INDEX(gamma)
EINSUMS_GB300_MAKE_INDEX(delta) EINSUMS_GB300_MAKE_INDEX(epsilon) EINSUMS_GB300_MAKE_INDEX(zeta)
EINSUMS_GB300_MAKE_INDEX(eta) EINSUMS_GB300_MAKE_INDEX(theta) EINSUMS_GB300_MAKE_INDEX(iota)
EINSUMS_GB300_MAKE_INDEX(kappa) EINSUMS_GB300_MAKE_INDEX(lambda) EINSUMS_GB300_MAKE_INDEX(mu)
EINSUMS_GB300_MAKE_INDEX(nu) EINSUMS_GB300_MAKE_INDEX(xi) EINSUMS_GB300_MAKE_INDEX(omicron)
EINSUMS_GB300_MAKE_INDEX(pi) EINSUMS_GB300_MAKE_INDEX(rho) EINSUMS_GB300_MAKE_INDEX(sigma)
EINSUMS_GB300_MAKE_INDEX(tau) EINSUMS_GB300_MAKE_INDEX(upsilon) EINSUMS_GB300_MAKE_INDEX(phi)
EINSUMS_GB300_MAKE_INDEX(chi) EINSUMS_GB300_MAKE_INDEX(psi) EINSUMS_GB300_MAKE_INDEX(omega)

template <typename... Args>
    requires(std::is_base_of_v<index::LabelBase, Args> && ... && true)
struct Indices : std::tuple<Args...> {
    constexpr Indices(Args... args) : std::tuple<Args...>(args...) {}
};

namespace tensor_algebra::detail {
// Same enumerators and order as the reference's AlgorithmChoice.
enum AlgorithmChoice { GENERIC, DOT, DIRECT, GER, GEMV, GEMM, INDETERMINATE };

template <typename... Ix>
constexpr ::einsums_gb300::detail::Labels labels_of(std::tuple<Ix...> const *) {
    ::einsums_gb300::detail::Labels l;
    (l.push(::einsums::detail::label_of(std::remove_cvref_t<Ix>::letter)), ...);
    return l;
}

// Compile-time choice for a pattern (before the runtime stride vetoes).
template <typename CIdx, typename AIdx, typename BIdx>
constexpr AlgorithmChoice compile_time_choice() {
    constexpr auto c = labels_of((CIdx const *)nullptr);
    constexpr auto a = labels_of((AIdx const *)nullptr);
    constexpr auto b = labels_of((BIdx const *)nullptr);
    return (AlgorithmChoice)::einsums_gb300::detail::classify_cpp(c, a, b);
}
} // namespace tensor_algebra::detail

// ------------------------------------------------------------ storage ----
// Row-major FP64 device tensor; storage from eg_device_alloc (budgeted).
template <typename T, size_t Rank>
class DeviceTensor {
    static_assert(std::is_same_v<T, double>, "einsums_gb300 kernels are FP64");
    static_assert(Rank <= EG_MAX_RANK, "rank above EG_MAX_RANK");

  public:
    using ValueType = T;
    static constexpr size_t rank = Rank;

    template <typename... Dims>
        requires(sizeof...(Dims) == Rank)
    explicit DeviceTensor(std::string name, Dims... dims) : name_(std::move(name)), dims_{(size_t)dims...} {
        size_t s = 1;
        for (size_t d = Rank; d-- > 0;) {
            strides_[d] = s;
            s *= dims_[d];
        }
        size_ = s;
        void *p = nullptr;
        detail::check(eg_device_alloc(size_ * sizeof(T) + (size_ == 0), &p));
        data_ = std::shared_ptr<T>((T *)p, [](T *q) { eg_device_free(q); });
    }

    T *gpu_data() { return data_.get(); }
    const T *gpu_data() const { return data_.get(); }
    size_t dim(int d) const { return dims_[d]; }
    size_t stride(int d) const { return strides_[d]; }
    size_t size() const { return size_; }
    const std::string &name() const { return name_; }

    // Host <-> device transfers (synchronous), like DeviceTensor::read / operator=.
    void write(const std::vector<T> &host) {
        if (host.size() != size_) throw dimension_error(EG_ERROR_DIMENSION, "host buffer size mismatch");
        detail::check(eg_copy_to_device(gpu_data(), host.data(), size_ * sizeof(T), nullptr));
        detail::check(eg_stream_synchronize(nullptr));
    }
    std::vector<T> read() const {
        std::vector<T> host(size_);
        detail::check(eg_copy_to_host(host.data(), gpu_data(), size_ * sizeof(T), nullptr));
        detail::check(eg_stream_synchronize(nullptr));
        return host;
    }

    eg_tensor descriptor() const {
        eg_tensor t{};
        t.data = const_cast<T *>(gpu_data());
        t.rank = (int32_t)Rank;
        for (size_t d = 0; d < Rank; d++) {
            t.extent[d] = (int64_t)dims_[d];
            t.stride[d] = (int64_t)strides_[d];
        }
        return t;
    }

  private:
    std::string name_;
    size_t dims_[Rank > 0 ? Rank : 1]{};
    size_t strides_[Rank > 0 ? Rank : 1]{};
    size_t size_ = 1;
    std::shared_ptr<T> data_;
};

// Non-owning strided view (element strides), e.g. a sub-block of a DeviceTensor.
template <typename T, size_t Rank>
class DeviceTensorView {
  public:
    using ValueType = T;
    static constexpr size_t rank = Rank;
    DeviceTensorView(T *data, const size_t (&dims)[Rank], const size_t (&strides)[Rank]) : data_(data) {
        for (size_t d = 0; d < Rank; d++) {
            dims_[d] = dims[d];
            strides_[d] = strides[d];
        }
    }
    eg_tensor descriptor() const {
        eg_tensor t{};
        t.data = data_;
        t.rank = (int32_t)Rank;
        for (size_t d = 0; d < Rank; d++) {
            t.extent[d] = (int64_t)dims_[d];
            t.stride[d] = (int64_t)strides_[d];
        }
        return t;
    }

  private:
    T *data_;
    size_t dims_[Rank > 0 ? Rank : 1]{};
    size_t strides_[Rank > 0 ? Rank : 1]{};
};

// Options of the GB300 kernels beyond the reference's signature (precision).
struct Options {
    eg_precision precision = EG_PRECISION_FP64;
    int slices = 0;
    void *stream = nullptr;
};
inline Options &default_options() {
    static thread_local Options o;
    return o;
}

// ------------------------------------------------------------- einsum ----
namespace tensor_algebra {

namespace detail {
template <typename... Ix>
std::vector<int32_t> label_vector(std::tuple<Ix...> const &) {
    return {::einsums::detail::label_of(std::remove_cvref_t<Ix>::letter)...};
}
} // namespace detail

template <bool ConjA = false, bool ConjB = false, typename AType, typename BType, typename CType, typename U,
          typename... CIndices, typename... AIndices, typename... BIndices>
void einsum(U const C_prefactor, std::tuple<CIndices...> const &C_indices, CType *C, U const AB_prefactor,
            std::tuple<AIndices...> const &A_indices, AType const &A, std::tuple<BIndices...> const &B_indices,
            BType const &B, detail::AlgorithmChoice *algorithm_choice = nullptr) {
    static_assert(sizeof...(CIndices) == CType::rank, "Rank of C does not match Indices given for C.");
    static_assert(sizeof...(AIndices) == AType::rank, "Rank of A does not match Indices given for A.");
    static_assert(sizeof...(BIndices) == BType::rank, "Rank of B does not match Indices given for B.");
    // The pattern analysis runs here, at compile time, as in the reference.
    [[maybe_unused]] constexpr detail::AlgorithmChoice compile_choice =
        detail::compile_time_choice<std::tuple<CIndices...>, std::tuple<AIndices...>, std::tuple<BIndices...>>();
    const auto cl = detail::label_vector(C_indices), al = detail::label_vector(A_indices),
               bl = detail::label_vector(B_indices);
    const eg_tensor tc = C->descriptor(), ta = A.descriptor(), tb = B.descriptor();
    eg_options opt;
    eg_options_default(&opt);
    opt.precision = default_options().precision;
    opt.slices = default_options().slices;
    int32_t alg = (int32_t)compile_choice;
    ::einsums::detail::check(eg_einsum((double)C_prefactor, cl.data(), &tc, (double)AB_prefactor, al.data(), &ta,
                                       bl.data(), &tb, &opt, default_options().stream, &alg));
    if (algorithm_choice) *algorithm_choice = (detail::AlgorithmChoice)alg;
}

// Default prefactors: C = A * B (Dispatch.hpp's default-prefactor form).
template <bool ConjA = false, bool ConjB = false, typename AType, typename BType, typename CType,
          typename... CIndices, typename... AIndices, typename... BIndices>
void einsum(std::tuple<CIndices...> const &C_indices, CType *C, std::tuple<AIndices...> const &A_indices,
            AType const &A, std::tuple<BIndices...> const &B_indices, BType const &B,
            detail::AlgorithmChoice *algorithm_choice = nullptr) {
    einsum<ConjA, ConjB>(0.0, C_indices, C, 1.0, A_indices, A, B_indices, B, algorithm_choice);
}

// Batched form over equal-length lists (Dispatch.hpp:1264-1286); one grouped call.
template <bool ConjA = false, bool ConjB = false, typename T, size_t CR, size_t AR, size_t BR, typename U,
          typename... CIndices, typename... AIndices, typename... BIndices>
void einsum(U const C_prefactor, std::tuple<CIndices...> const &C_indices, std::vector<DeviceTensor<T, CR>> *C_list,
            U const AB_prefactor, std::tuple<AIndices...> const &A_indices,
            std::vector<DeviceTensor<T, AR>> const &A_list, std::tuple<BIndices...> const &B_indices,
            std::vector<DeviceTensor<T, BR>> const &B_list, detail::AlgorithmChoice *algorithm_choice = nullptr) {
    if (C_list->size() != A_list.size() || C_list->size() != B_list.size())
        throw einsums_error(EG_ERROR_INVALID_ARGUMENT, "Lists passed to batched einsum call do not have the same size!");
    if (C_list->empty()) return;
    std::vector<eg_tensor> tc, ta, tb;
    for (size_t i = 0; i < C_list->size(); i++) {
        tc.push_back((*C_list)[i].descriptor());
        ta.push_back(A_list[i].descriptor());
        tb.push_back(B_list[i].descriptor());
    }
    const auto cl = detail::label_vector(C_indices), al = detail::label_vector(A_indices),
               bl = detail::label_vector(B_indices);
    eg_options opt;
    eg_options_default(&opt);
    opt.precision = default_options().precision;
    opt.slices = default_options().slices;
    int32_t alg = -1;
    ::einsums::detail::check(eg_einsum_batched((double)C_prefactor, cl.data(), tc.data(), (double)AB_prefactor,
                                               al.data(), ta.data(), bl.data(), tb.data(), (int64_t)tc.size(), &opt,
                                               default_options().stream, &alg));
    if (algorithm_choice) *algorithm_choice = (detail::AlgorithmChoice)alg;
}

template <bool ConjA = false, bool ConjB = false, typename T, size_t CR, size_t AR, size_t BR, typename... CIndices,
          typename... AIndices, typename... BIndices>
void einsum(std::tuple<CIndices...> const &C_indices, std::vector<DeviceTensor<T, CR>> *C_list,
            std::tuple<AIndices...> const &A_indices, std::vector<DeviceTensor<T, AR>> const &A_list,
            std::tuple<BIndices...> const &B_indices, std::vector<DeviceTensor<T, BR>> const &B_list,
            detail::AlgorithmChoice *algorithm_choice = nullptr) {
    einsum<ConjA, ConjB>(0.0, C_indices, C_list, 1.0, A_indices, A_list, B_indices, B_list, algorithm_choice);
}

// permute(C_prefactor, Cidx, &C, A_prefactor, Aidx, A) (Permute.hpp:330-407).
template <bool ConjA = false, typename AType, typename CType, typename U, typename... CIndices, typename... AIndices>
void permute(U const C_prefactor, std::tuple<CIndices...> const &C_indices, CType *C, U const A_prefactor,
             std::tuple<AIndices...> const &A_indices, AType const &A) {
    static_assert(sizeof...(CIndices) == sizeof...(AIndices), "permute needs the same number of indices");
    static_assert(sizeof...(CIndices) == CType::rank && sizeof...(AIndices) == AType::rank, "rank mismatch");
    const auto cl = detail::label_vector(C_indices), al = detail::label_vector(A_indices);
    const eg_tensor tc = C->descriptor(), ta = A.descriptor();
    ::einsums::detail::check(
        eg_permute((double)C_prefactor, cl.data(), &tc, (double)A_prefactor, al.data(), &ta, default_options().stream));
}

// compile_permute(beta, Cidx, &C, alpha, Aidx, A) (Permute.hpp:37-171): a reusable plan
// for tensors of C's and A's shapes and strides; permute(&C, A, plan) runs it on new data
// (Permute.hpp:292-297).
class PermutePlan {
  public:
    explicit PermutePlan(eg_permute_plan *p) : p_(p) {}
    PermutePlan(PermutePlan const &) = delete;
    PermutePlan &operator=(PermutePlan const &) = delete;
    PermutePlan(PermutePlan &&o) noexcept : p_(o.p_) { o.p_ = nullptr; }
    ~PermutePlan() {
        if (p_) eg_permute_plan_destroy(p_);
    }
    eg_permute_plan *get() const { return p_; }

  private:
    eg_permute_plan *p_;
};

template <typename AType, typename CType, typename U, typename... CIndices, typename... AIndices>
std::shared_ptr<PermutePlan> compile_permute(U const C_prefactor, std::tuple<CIndices...> const &C_indices, CType *C,
                                             U const A_prefactor, std::tuple<AIndices...> const &A_indices,
                                             AType const &A) {
    static_assert(sizeof...(CIndices) == sizeof...(AIndices), "permute needs the same number of indices");
    static_assert(sizeof...(CIndices) == CType::rank && sizeof...(AIndices) == AType::rank, "rank mismatch");
    const auto cl = detail::label_vector(C_indices), al = detail::label_vector(A_indices);
    const eg_tensor tc = C->descriptor(), ta = A.descriptor();
    eg_permute_plan *p = nullptr;
    ::einsums::detail::check(
        eg_permute_plan_create((double)C_prefactor, cl.data(), &tc, (double)A_prefactor, al.data(), &ta, &p));
    return std::make_shared<PermutePlan>(p);
}

template <typename AType, typename CType>
void permute(CType *C, AType const &A, std::shared_ptr<PermutePlan> const &plan) {
    const eg_tensor tc = C->descriptor(), ta = A.descriptor();
    ::einsums::detail::check(eg_permute_plan_execute(plan->get(), tc.data, ta.data, default_options().stream));
}

} // namespace tensor_algebra

} // namespace einsums
