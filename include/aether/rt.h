// aether/rt.h -- rolled-loop twins of the per-sample reductions and
// contractions (expr/Rt.h).
//
// The static forms (`a[i].get().dot(b[i].get())`, `y[i] = M * v`) unroll
// every element, so a long fold keeps one live value per element: a 144-long
// dot or a 16x144 matrix-vector product runs out of registers. The twins in
// aether::rt walk the element index in a loop that stays rolled and read each
// element when it is needed.
//
// Each twin returns the bits of its static form: the same order (acc = x0,
// then acc = x_k (op) acc for ascending k; products acc = a_k * b_k + acc),
// so wherever the compiler contracts per statement the same products fuse;
// compare on the host with -ffp-contract=off. rNorm is 1 / sqrt (a division),
// cubedNorm s * sqrt(s), as the member forms.
//
// Operands are the per-sample proxies `view[i]` (read through .at(k...)) or
// Items (read through operator()); on the device a runtime-indexed Item lives
// in local memory, so pass the proxy. Shapes are static types; an output
// must not alias an operand.
#pragma once

#include <cstddef>
#include <type_traits>
#include <utility>

#include "aether/item.h"

#if defined(__CUDA_ARCH__)
#define AETHER_RT_ROLLED _Pragma("unroll 1")
#else
#define AETHER_RT_ROLLED
#endif

namespace aether {
namespace rt {
namespace detail {

template <class X>
using plain_t = std::remove_cv_t<std::remove_reference_t<X>>;
template <class X>
using elem_t = std::remove_cv_t<typename plain_t<X>::element_type>;
template <class X>
using ext_t = typename plain_t<X>::element_extents;

template <class X>
struct is_item : std::false_type {};
template <class T, std::size_t... Es>
struct is_item<Item<T, Es...>> : std::true_type {};

/** Element ks... of one sample: x(ks...) on an Item, x.at(ks...) on a
 *  per-sample proxy (view[i]) or a transposed operand. */
template <class X, class... Ks>
AETHER_DEVICEANDHOST() constexpr decltype(auto) at(X&& x, Ks... ks) {
    if constexpr (is_item<plain_t<X>>::value) {
        return x(ks...);
    } else {
        return x.at(ks...);
    }
}

template <class A>
AETHER_DEVICEANDHOST() constexpr std::size_t count() {
    using X = ext_t<A>;
    static_assert(X::Rank == 1, "rt: a rank-1 operand");
    return X::static_extent(0);
}

template <class A, class B>
AETHER_DEVICEANDHOST() constexpr elem_t<A> dot_(const A& a, const B& b) {
    static_assert(std::is_same<ext_t<A>, ext_t<B>>::value, "rt::dot: operands of different shapes");
    using T = elem_t<A>;
    constexpr std::size_t N = count<A>();
    T acc = T(at(a, std::size_t(0)) * at(b, std::size_t(0)));
    AETHER_RT_ROLLED
    for (std::size_t k = 1; k < N; ++k) acc = T(at(a, k) * at(b, k) + acc);
    return acc;
}

// dst = v, dst += v or dst -= v, as the assignment forms store a result.
template <int Op, class Out, class T>
AETHER_DEVICEANDHOST() constexpr void store_(Out&& dst, T v) {
    if constexpr (Op == 0)
        dst = v;
    else if constexpr (Op == 1)
        dst = T(dst + v);
    else
        dst = T(dst - v);
}

// out (op)= the row-by-column products: acc = m(r,0) v(0), then
// acc = m(r,k) v(k) + acc for ascending k (likewise l(i,k) r(k,j) below).
template <int Op, class Out, class M, class V>
AETHER_DEVICEANDHOST() constexpr void matVec_(Out& out, const M& m, const V& v) {
    static_assert(ext_t<M>::Rank == 2 && ext_t<V>::Rank == 1, "rt::matVec: m rank 2, v rank 1");
    static_assert(ext_t<M>::static_extent(1) == ext_t<V>::static_extent(0), "rt::matVec: inner extents differ");
    static_assert(std::is_same<ext_t<Out>, extents<ext_t<M>::static_extent(0)>>::value, "rt::matVec: out has m's rows");
    using T = elem_t<M>;
    constexpr std::size_t Rows = ext_t<M>::static_extent(0), K = ext_t<M>::static_extent(1);
    AETHER_RT_ROLLED
    for (std::size_t r = 0; r < Rows; ++r) {
        T acc = T(at(m, r, std::size_t(0)) * at(v, std::size_t(0)));
        AETHER_RT_ROLLED
        for (std::size_t k = 1; k < K; ++k) acc = T(at(m, r, k) * at(v, k) + acc);
        store_<Op>(at(out, r), acc);
    }
}

template <int Op, class Out, class L, class R>
AETHER_DEVICEANDHOST() constexpr void matMat_(Out& out, const L& l, const R& r) {
    static_assert(ext_t<L>::Rank == 2 && ext_t<R>::Rank == 2, "rt::matMat: rank-2 operands");
    static_assert(ext_t<L>::static_extent(1) == ext_t<R>::static_extent(0), "rt::matMat: inner extents differ");
    static_assert(std::is_same<ext_t<Out>, extents<ext_t<L>::static_extent(0), ext_t<R>::static_extent(1)>>::value,
                  "rt::matMat: out is l's rows x r's columns");
    using T = elem_t<L>;
    constexpr std::size_t Rows = ext_t<L>::static_extent(0), K = ext_t<L>::static_extent(1),
                          Cols = ext_t<R>::static_extent(1);
    AETHER_RT_ROLLED
    for (std::size_t i = 0; i < Rows; ++i) {
        AETHER_RT_ROLLED
        for (std::size_t j = 0; j < Cols; ++j) {
            T acc = T(at(l, i, std::size_t(0)) * at(r, std::size_t(0), j));
            AETHER_RT_ROLLED
            for (std::size_t k = 1; k < K; ++k) acc = T(at(l, i, k) * at(r, k, j) + acc);
            store_<Op>(at(out, i, j), acc);
        }
    }
}

}  // namespace detail

/** Dot product of two rank-1 operands; twin of Expression::dot. */
template <class A, class B>
AETHER_DEVICEANDHOST() constexpr detail::elem_t<A> dot(const A& a, const B& b) {
    return detail::dot_(a, b);
}
/** Sum of the components; twin of Expression::sum. */
template <class A>
AETHER_DEVICEANDHOST() constexpr detail::elem_t<A> sum(const A& a) {
    using T = detail::elem_t<A>;
    T acc = T(detail::at(a, std::size_t(0)));
    AETHER_RT_ROLLED
    for (std::size_t k = 1; k < detail::count<A>(); ++k) acc = T(detail::at(a, k) + acc);
    return acc;
}
template <class A>
AETHER_DEVICEANDHOST() constexpr detail::elem_t<A> squaredNorm(const A& a) {
    return detail::dot_(a, a);
}
template <class A>
AETHER_DEVICEANDHOST() detail::elem_t<A> norm(const A& a) {
    return math::sqrt(squaredNorm(a));
}
/** 1 / norm, a division; twin of Expression::rNorm. */
template <class A>
AETHER_DEVICEANDHOST() detail::elem_t<A> rNorm(const A& a) {
    return detail::elem_t<A>(1) / math::sqrt(squaredNorm(a));
}
template <class A>
AETHER_DEVICEANDHOST() constexpr detail::elem_t<A> rSquaredNorm(const A& a) {
    return detail::elem_t<A>(1) / squaredNorm(a);
}
template <class A>
AETHER_DEVICEANDHOST() detail::elem_t<A> cubedNorm(const A& a) {
    const auto s = squaredNorm(a);
    return s * math::sqrt(s);
}
template <class A>
AETHER_DEVICEANDHOST() detail::elem_t<A> rCubedNorm(const A& a) {
    const auto s = squaredNorm(a);
    return detail::elem_t<A>(1) / (s * math::sqrt(s));
}
/** Largest magnitude; twin of Expression::maxNorm. */
template <class A>
AETHER_DEVICEANDHOST() detail::elem_t<A> maxNorm(const A& a) {
    using T = detail::elem_t<A>;
    T acc = math::abs(T(detail::at(a, std::size_t(0))));
    AETHER_RT_ROLLED
    for (std::size_t k = 1; k < detail::count<A>(); ++k) {
        const T x = math::abs(T(detail::at(a, k)));
        acc = x > acc ? x : acc;
    }
    return acc;
}
/** Every component finite; twin of aether::isFinite. */
template <class A>
AETHER_DEVICEANDHOST() bool isFinite(const A& a) {
    bool ok = true;
    AETHER_RT_ROLLED
    for (std::size_t k = 0; k < detail::count<A>(); ++k) ok = LogicalAndOp{}(math::isfinite(detail::at(a, k)), ok);
    return ok;
}
/** Frobenius inner product of two rank-2 operands, row-major; twin of
 *  Expression::matDot. */
template <class L, class R>
AETHER_DEVICEANDHOST() constexpr detail::elem_t<L> matDot(const L& l, const R& r) {
    static_assert(detail::ext_t<L>::Rank == 2 && std::is_same<detail::ext_t<L>, detail::ext_t<R>>::value,
                  "rt::matDot: rank-2 operands of one shape");
    using T = detail::elem_t<L>;
    constexpr std::size_t Cols = detail::ext_t<L>::static_extent(1), N = detail::ext_t<L>::static_extent(0) * Cols;
    T acc = T(detail::at(l, std::size_t(0), std::size_t(0)) * detail::at(r, std::size_t(0), std::size_t(0)));
    AETHER_RT_ROLLED
    for (std::size_t k = 1; k < N; ++k)
        acc = T(detail::at(l, k / Cols, k % Cols) * detail::at(r, k / Cols, k % Cols) + acc);
    return acc;
}

/** out = m * v; twin of view[i] = M * v. */
template <class Out, class M, class V>
AETHER_DEVICEANDHOST() constexpr void matVec(Out&& out, const M& m, const V& v) {
    detail::matVec_<0>(out, m, v);
}
template <class Out, class M, class V>
AETHER_DEVICEANDHOST() constexpr void matVecAdd(Out&& out, const M& m, const V& v) {
    detail::matVec_<1>(out, m, v);
}
template <class Out, class M, class V>
AETHER_DEVICEANDHOST() constexpr void matVecSub(Out&& out, const M& m, const V& v) {
    detail::matVec_<2>(out, m, v);
}
/** out = l * r; twin of view[i] = L * R. */
template <class Out, class L, class R>
AETHER_DEVICEANDHOST() constexpr void matMat(Out&& out, const L& l, const R& r) {
    detail::matMat_<0>(out, l, r);
}
template <class Out, class L, class R>
AETHER_DEVICEANDHOST() constexpr void matMatAdd(Out&& out, const L& l, const R& r) {
    detail::matMat_<1>(out, l, r);
}
template <class Out, class L, class R>
AETHER_DEVICEANDHOST() constexpr void matMatSub(Out&& out, const L& l, const R& r) {
    detail::matMat_<2>(out, l, r);
}

/** A rank-2 operand read transposed (at(r, c) is x's (c, r)); holds x by
 *  reference, so it lives within the statement that names it. */
template <class X>
class Transposed {
public:
    using element_type = detail::elem_t<X>;
    using element_extents = extents<detail::ext_t<X>::static_extent(1), detail::ext_t<X>::static_extent(0)>;
    AETHER_DEVICEANDHOST() constexpr explicit Transposed(const X& x) : x_(x) {
        static_assert(detail::ext_t<X>::Rank == 2, "rt::transposed: a rank-2 operand");
    }
    AETHER_DEVICEANDHOST() constexpr decltype(auto) at(std::size_t r, std::size_t c) const { return detail::at(x_, c, r); }

private:
    const X& x_;
};
/** x read as its transpose; twin of x.transpose() as a matVec/matMat operand. */
template <class X>
AETHER_DEVICEANDHOST() constexpr Transposed<X> transposed(const X& x) {
    return Transposed<X>(x);
}

/** out = x element by element, rolled; twin of view[i] = x for an Item x. */
template <class Out, class X>
AETHER_DEVICEANDHOST() constexpr void store(Out&& out, const X& x) {
    using XO = detail::ext_t<Out>;
    static_assert(std::is_same<XO, detail::ext_t<X>>::value, "rt::store: operands of different shapes");
    if constexpr (XO::Rank == 1) {
        AETHER_RT_ROLLED
        for (std::size_t k = 0; k < XO::static_extent(0); ++k) detail::at(out, k) = detail::at(x, k);
    } else {
        static_assert(XO::Rank == 2, "rt::store: rank 1 or 2");
        AETHER_RT_ROLLED
        for (std::size_t r = 0; r < XO::static_extent(0); ++r) {
            AETHER_RT_ROLLED
            for (std::size_t c = 0; c < XO::static_extent(1); ++c) detail::at(out, r, c) = detail::at(x, r, c);
        }
    }
}

}  // namespace rt
}  // namespace aether
