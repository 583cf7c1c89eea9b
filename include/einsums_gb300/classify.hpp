// Pattern analysis for einsum: which lowering the reference picks for a
// (C, A, B) index pattern.  Everything here is constexpr so that the C++
// front end (einsums_gb300/TensorAlgebra.hpp) evaluates it at compile time,
// exactly where the reference's template machinery runs, while the CUDA
// library evaluates the same functions at run time for callers that pass
// labels as data (the Python binding).
//
// Restated from
//   libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Backends/Dispatch.hpp
//     einsum_is_dot_product      :215-221
//     einsum_is_direct_product   :226-238
//     einsum_is_outer_product    :243-266
//     einsum_is_matrix_vector    :407-439
//     einsum_is_matrix_product   :565-609
//     detail::einsum chain       :893-951
//   libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Detail/Utilities.hpp
//     find_type_with_position :133-136, contiguous_positions :320-327,
//     is_same_ordering :336-345, IntersectT/DifferenceT/UniqueT :600-730
//   libs/EinsumsPy/TensorAlgebra/src/PyTensorAlgebra.cpp:168-554 (string form)
// Labels are plain integers; two modes carry the same index when their labels
// are equal.
#pragma once

#include <cstdint>

namespace einsums_gb300::detail {

inline constexpr int kMaxRank = 8;

// Matches the reference's AlgorithmChoice enumerators and their order.
enum class Algorithm : int32_t { GENERIC = 0, DOT = 1, DIRECT = 2, GER = 3, GEMV = 4, GEMM = 5, INDETERMINATE = 6 };

struct Labels {
    int32_t v[3 * kMaxRank] = {};
    int n = 0;
    constexpr void push(int32_t x) { v[n++] = x; }
    constexpr bool contains(int32_t x) const {
        for (int i = 0; i < n; i++)
            if (v[i] == x) return true;
        return false;
    }
};

// (label, position) pairs as produced by find_type_with_position.
struct Positions {
    int32_t label[3 * kMaxRank * kMaxRank] = {};
    int32_t pos[3 * kMaxRank * kMaxRank] = {};
    int n = 0;
};

constexpr Labels make_labels(const int32_t *x, int n) {
    Labels l;
    for (int i = 0; i < n; i++) l.push(x[i]);
    return l;
}

constexpr Labels intersect(const Labels &x, const Labels &y) {
    Labels o;
    for (int i = 0; i < x.n; i++)
        if (y.contains(x.v[i])) o.push(x.v[i]);
    return o;
}

constexpr Labels difference(const Labels &x, const Labels &y) {
    Labels o;
    for (int i = 0; i < x.n; i++)
        if (!y.contains(x.v[i])) o.push(x.v[i]);
    return o;
}

constexpr Labels unique(const Labels &x) {
    Labels o;
    for (int i = 0; i < x.n; i++)
        if (!o.contains(x.v[i])) o.push(x.v[i]);
    return o;
}

constexpr Positions find_with_pos(const Labels &x, const Labels &y) {
    Positions p;
    for (int i = 0; i < x.n; i++)
        for (int j = 0; j < y.n; j++)
            if (y.v[j] == x.v[i]) {
                p.label[p.n] = x.v[i];
                p.pos[p.n] = j;
                p.n++;
            }
    return p;
}

constexpr bool contiguous(const Positions &p) {
    for (int i = 0; i + 1 < p.n; i++)
        if (p.pos[i] != p.pos[i + 1] - 1) return false;
    return true;
}

constexpr bool same_ordering(const Positions &x, const Positions &y) {
    if (x.n == 0 || y.n == 0 || x.n != y.n) return false;
    for (int i = 0; i < x.n; i++)
        if (x.label[i] != y.label[i]) return false;
    return true;
}

constexpr bool equal(const Labels &x, const Labels &y) {
    if (x.n != y.n) return false;
    for (int i = 0; i < x.n; i++)
        if (x.v[i] != y.v[i]) return false;
    return true;
}

struct Analysis {
    Labels C, A, B, linksAB, links, C_unique, link_unique;
    Positions link_pos_A, link_pos_B, target_pos_A, target_pos_B, A_target_pos_C, B_target_pos_C;
    bool hadamard = false;

    constexpr Analysis(const Labels &c, const Labels &a, const Labels &b) : C(c), A(a), B(b) {
        linksAB = intersect(A, B);
        links = difference(linksAB, C);
        C_unique = unique(C);
        link_unique = unique(links);
        link_pos_A = find_with_pos(link_unique, A);
        link_pos_B = find_with_pos(link_unique, B);
        target_pos_A = find_with_pos(C_unique, A);
        target_pos_B = find_with_pos(C_unique, B);
        A_target_pos_C = find_with_pos(A, C);
        B_target_pos_C = find_with_pos(B, C);
        hadamard = unique(A).n != A.n || unique(B).n != B.n || C_unique.n != C.n;
    }

    constexpr bool is_dot() const { return C.n == 0 && equal(A, B); }
    constexpr bool is_direct() const { return equal(C, A) && equal(C, B); }
    constexpr bool is_outer() const { return linksAB.n == 0 && contiguous(target_pos_A) && contiguous(target_pos_B); }

    // einsum_is_matrix_vector(C, A, B); swapped evaluates it for (C, B, A).
    constexpr bool is_gemv(bool swapped) const {
        const Positions &lpA = swapped ? link_pos_B : link_pos_A;
        const Positions &lpB = swapped ? link_pos_A : link_pos_B;
        const Positions &tpA = swapped ? target_pos_B : target_pos_A;
        const Positions &tpB = swapped ? target_pos_A : target_pos_B;
        const Positions &AtC = swapped ? B_target_pos_C : A_target_pos_C;
        const Positions &BtC = swapped ? A_target_pos_C : B_target_pos_C;
        return contiguous(lpA) && contiguous(lpB) && contiguous(tpA) && same_ordering(lpA, lpB) &&
               same_ordering(tpA, AtC) && !same_ordering(tpB, BtC) && BtC.n == 0;
    }

    constexpr bool is_gemm() const {
        return difference(C, A).n > 0 && difference(C, B).n > 0 && contiguous(link_pos_A) && contiguous(link_pos_B) &&
               contiguous(target_pos_A) && contiguous(target_pos_B) && contiguous(A_target_pos_C) &&
               contiguous(B_target_pos_C) && same_ordering(link_pos_A, link_pos_B) &&
               same_ordering(target_pos_A, A_target_pos_C) && same_ordering(target_pos_B, B_target_pos_C);
    }
};

// Compile-time choice of the C++ einsum (Dispatch.hpp:893-951) for real,
// same-typed basic tensors, before any runtime stride veto.
constexpr Algorithm classify_cpp(const Labels &C, const Labels &A, const Labels &B) {
    Analysis an(C, A, B);
    if (an.hadamard) return Algorithm::GENERIC;
    if (an.is_dot()) return Algorithm::DOT;
    if (an.is_direct()) return Algorithm::DIRECT;
    if (an.is_outer()) return Algorithm::GER;
    if (an.is_gemv(false) || an.is_gemv(true)) return Algorithm::GEMV;
    if (C.n >= 2 && A.n >= 2 && B.n >= 2 && an.is_gemm()) return Algorithm::GEMM;
    return Algorithm::GENERIC;
}

// Plan type of compile_plan (PyTensorAlgebra.cpp:168-554).
constexpr Algorithm classify_py(const Labels &C, const Labels &A, const Labels &B) {
    Analysis an(C, A, B);
    if (an.hadamard) return Algorithm::GENERIC;
    if (C.n == 0 && equal(A, B)) return Algorithm::DOT;
    if (equal(C, A) && equal(C, B)) return Algorithm::DIRECT;
    if (an.is_outer()) return Algorithm::GER;
    if (an.is_gemv(false) || an.is_gemv(true)) return Algorithm::GEMV;
    if (an.is_gemm()) return Algorithm::GEMM;
    return Algorithm::GENERIC;
}

// ---- runtime stride vetoes (Dispatch.hpp) ----------------------------------
// A tensor view: extents and element strides, row-major position order.
struct View {
    int rank = 0;
    int64_t extent[kMaxRank] = {};
    int64_t stride[kMaxRank] = {};
    int64_t size() const {
        int64_t s = 1;
        for (int i = 0; i < rank; i++) s *= extent[i];
        return s;
    }
};

// TensorImpl::is_totally_vectorable (TensorImpl.hpp:756-777).
inline bool totally_vectorable(const View &x) {
    if (x.rank == 0) return false;
    if (x.rank == 1) return true;
    if (x.stride[0] < x.stride[x.rank - 1]) return x.extent[x.rank - 1] * x.stride[x.rank - 1] == x.size() * x.stride[0];
    return x.extent[0] * x.stride[0] == x.size() * x.stride[x.rank - 1];
}

// The row-major two-block stride check repeated in Dispatch.hpp:481-504,
// :664-684, :717-737 and :770-790.
inline bool two_groups_ok(const View &x, int64_t s0, int64_t s1) {
    if (x.rank == 2) return !(x.stride[0] != 1 && x.stride[1] != 1);
    const int64_t cutoff = s0 > s1 ? s0 : s1;
    int64_t check = 1;
    for (int i = x.rank - 1; i >= 0; i--) {
        if (x.stride[i] == cutoff) check = cutoff;
        if (x.stride[i] != check) return false;
        check *= x.extent[i];
    }
    return true;
}

inline int64_t last_stride(const Positions &p, const View &x) { return p.n ? x.stride[p.pos[p.n - 1]] : 0; }

// Applies the runtime vetoes of einsum_do_outer_product (:267-401),
// einsum_do_matrix_vector (:444-560) and einsum_do_matrix_product (:614-837):
// a choice whose views are not BLAS-compatible falls back to GENERIC (:953-955).
inline Algorithm apply_vetoes(Algorithm alg, const Labels &Cl, const View &C, const Labels &Al, const View &A,
                              const Labels &Bl, const View &B) {
    Analysis an(Cl, Al, Bl);
    switch (alg) {
    case Algorithm::GER:
        if (!totally_vectorable(A) || !totally_vectorable(B) ||
            !two_groups_ok(C, last_stride(an.A_target_pos_C, C), last_stride(an.B_target_pos_C, C)))
            return Algorithm::GENERIC;
        return alg;
    case Algorithm::GEMV: {
        const bool swapped = !an.is_gemv(false);
        const View &M = swapped ? B : A;
        const View &V = swapped ? A : B;
        const Positions &tp = swapped ? an.target_pos_B : an.target_pos_A;
        const Positions &lp = swapped ? an.link_pos_B : an.link_pos_A;
        if (!totally_vectorable(V) || !totally_vectorable(C) || !two_groups_ok(M, last_stride(tp, M), last_stride(lp, M)))
            return Algorithm::GENERIC;
        return alg;
    }
    case Algorithm::GEMM:
        if (!two_groups_ok(A, last_stride(an.target_pos_A, A), last_stride(an.link_pos_A, A)) ||
            !two_groups_ok(B, last_stride(an.link_pos_B, B), last_stride(an.target_pos_B, B)) ||
            !two_groups_ok(C, last_stride(an.A_target_pos_C, C), last_stride(an.B_target_pos_C, C)))
            return Algorithm::GENERIC;
        return alg;
    default:
        return alg;
    }
}

} // namespace einsums_gb300::detail
