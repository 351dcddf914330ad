// aether/expression.h -- typed lazy expressions, evaluated per sample.
//
// The expression protocol of the reference (expr/Expression.h:127-486): every
// node derives from Expression<Derived, T> and exposes
//   element_type       the value type of one component,
//   element_extents    the static component shape (extents<> for a scalar),
//   isLeaf,
//   eval<Is...>(SampleIndex)  component Is... of the node at one sample.
// Building an expression does no work. The same tree is evaluated two ways:
//   * per sample, in a consumer's kernel or host loop: `view[i] = expr`
//     (aether/view.h) unrolls the components and calls eval -- the reference's
//     own evaluation model (expr/Assign.h:124-231);
//   * whole views at once through the engine: `dst.deviceView() = expr` on
//     the host serialises the tree's type to aether-ir/1 (gb300_ir() below)
//     and runs it as one generated sm_103a kernel (aether/eval.h).
// Reductions that the reference defines as members (dot, norm, sum, det,
// trace, ...) return a value computed at sample 0, as the reference's do
// (expr/Expression.h:163-243, :381-428); the per-sample forms are expression
// nodes in aether::per_sample (an addition of this engine).
#pragma once

#include "aether/detail/std.h"

#include "aether/layout.h"
#include "aether/math.h"

namespace aether {

class Expr;   // the engine's type-erased expression (aether/expr.h)

template <class Derived, class T>
class Expression;

namespace detail {

template <class E, class = void>
struct is_expression_impl : std::false_type {};
template <class E>
struct is_expression_impl<E, std::void_t<typename E::element_type, typename E::element_extents>>
    : std::is_base_of<Expression<E, typename E::element_type>, E> {};

}  // namespace detail

/** True for the typed expression nodes (the reference's aether_expression). */
template <class E>
inline constexpr bool aether_expression = detail::is_expression_impl<std::remove_cv_t<std::remove_reference_t<E>>>::value;

namespace detail {

template <class E>
using extents_of = typename E::element_extents;

/** Components of an all-static extents. */
template <class X>
inline constexpr std::size_t size_of = static_size<X>::value;

/** Digit d of row-major flat index k over static extents X. */
template <class X>
AETHER_DEVICEANDHOST() constexpr std::size_t unflat(std::size_t k, std::size_t d) {
    std::size_t stride = 1;
    for (std::size_t j = d + 1; j < X::Rank; ++j) stride *= X::static_extent(j);
    return (k / stride) % X::static_extent(d);
}

template <std::size_t K, class E, std::size_t... D>
AETHER_DEVICEANDHOST() constexpr auto eval_flat_(const E& e, const SampleIndex& i, std::index_sequence<D...>) {
    return e.template eval<unflat<extents_of<E>>(K, D)...>(i);
}
/** Component K (row-major over element_extents) of e at sample i. */
template <std::size_t K, class E>
AETHER_DEVICEANDHOST() constexpr auto evalFlat(const E& e, const SampleIndex& i) {
    return eval_flat_<K>(e, i, std::make_index_sequence<extents_of<E>::Rank>{});
}

/** Row-major flat index of a static multi-index. */
template <class X, std::size_t... Is>
AETHER_DEVICEANDHOST() constexpr std::size_t flat_index() {
    static_assert(sizeof...(Is) == X::Rank, "one index per component extent");
    std::size_t k = 0, d = 0;
    ((k = k * X::static_extent(d++) + Is), ...);
    return k;
}

template <class A, class B>
inline constexpr bool same_shape = std::is_same<extents_of<A>, extents_of<B>>::value;

// Right-nested folds over all components (expr/Reduce.h:149-188): the fold of
// N terms is f(N-1) + (f(N-2) + (... + f(0))), with no zero seed.
template <class E, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr auto fold_sum_(const E& e, const SampleIndex& i, std::index_sequence<K...>) {
    using T = typename E::element_type;
    T acc{};
    bool first = true;
    ((acc = first ? T(evalFlat<K>(e, i)) : T(evalFlat<K>(e, i) + acc), first = false), ...);
    return acc;
}
template <class E>
AETHER_DEVICEANDHOST() constexpr auto fold_sum(const E& e, const SampleIndex& i) {
    return fold_sum_(e, i, std::make_index_sequence<size_of<extents_of<E>>>{});
}
template <class L, class R, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr auto fold_dot_(const L& l, const R& r, const SampleIndex& i, std::index_sequence<K...>) {
    using T = typename L::element_type;
    T acc{};
    bool first = true;
    ((acc = first ? T(evalFlat<K>(l, i) * evalFlat<K>(r, i)) : T(evalFlat<K>(l, i) * evalFlat<K>(r, i) + acc),
      first = false),
     ...);
    return acc;
}
template <class L, class R>
AETHER_DEVICEANDHOST() constexpr auto fold_dot(const L& l, const R& r, const SampleIndex& i) {
    static_assert(same_shape<L, R>, "dot: operands of different shapes");
    return fold_dot_(l, r, i, std::make_index_sequence<size_of<extents_of<L>>>{});
}
template <class E, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr auto fold_maxabs_(const E& e, const SampleIndex& i, std::index_sequence<K...>) {
    using T = typename E::element_type;
    T acc{};
    bool first = true;
    ((acc = first ? math::abs(evalFlat<K>(e, i))
                  : (math::abs(evalFlat<K>(e, i)) > acc ? math::abs(evalFlat<K>(e, i)) : acc),
      first = false),
     ...);
    return acc;
}

// Node templates the member surface refers to (defined in aether/geometry.h).
template <class L, class R>
class Cross;
template <class E>
class UnitVector;
template <class L, class R>
class QuatMul;
template <class E>
class QuatConj;
template <class Q, class V>
class QuatRotate;
template <class E>
class AsPureQuaternion;
template <class E, std::size_t Off, std::size_t Len>
class Segment;
template <class E>
class Transpose;
template <class E, std::size_t R>
class Row;
template <class E, std::size_t C>
class Col;
template <class E, std::size_t R0, std::size_t C0, std::size_t BR, std::size_t BC>
class Block;
template <class L, class R>
class CWiseMul;
template <class E>
class Inverse;
template <class E>
class CWiseScale;

/** 2x2 / 3x3 determinant of e at sample i, in the reference's order
 *  (expr/Expression.h:400-428). */
template <class E>
AETHER_DEVICEANDHOST() constexpr typename E::element_type det_at(const E& m, const SampleIndex& i);

}  // namespace detail

/** CRTP base of every node: the member surface of the reference's
 *  Expression<Derived, T> (expr/Expression.h:145-440). */
template <class Derived, class T>
class Expression {
public:
    AETHER_DEVICEANDHOST() constexpr const Derived& derived() const { return static_cast<const Derived&>(*this); }

    // -- reductions, evaluated at sample 0 -----------------------------------
    template <class E>
    AETHER_DEVICEANDHOST() constexpr T dot(const Expression<E, T>& other) const {
        return detail::fold_dot(derived(), other.derived(), SampleIndex::make(std::size_t(0)));
    }
    AETHER_DEVICEANDHOST() constexpr T squaredNorm() const {
        return detail::fold_dot(derived(), derived(), SampleIndex::make(std::size_t(0)));
    }
    AETHER_DEVICEANDHOST() T norm() const { return math::sqrt(squaredNorm()); }
    AETHER_DEVICEANDHOST() T rNorm() const { return T(1) / math::sqrt(squaredNorm()); }   // 1 / sqrt, not rsqrt (expr/Expression.h:202-205)
    AETHER_DEVICEANDHOST() constexpr T rSquaredNorm() const { return T(1) / squaredNorm(); }
    AETHER_DEVICEANDHOST() T cubedNorm() const { return squaredNorm() * norm(); }
    AETHER_DEVICEANDHOST() T rCubedNorm() const { return T(1) / cubedNorm(); }
    AETHER_DEVICEANDHOST() T maxNorm() const {
        return detail::fold_maxabs_(derived(), SampleIndex::make(std::size_t(0)),
                                    std::make_index_sequence<detail::size_of<detail::extents_of<Derived>>>{});
    }
    AETHER_DEVICEANDHOST() constexpr T sum() const {
        return detail::fold_sum(derived(), SampleIndex::make(std::size_t(0)));
    }
    AETHER_DEVICEANDHOST() constexpr T trace() const {
        using X = detail::extents_of<Derived>;
        static_assert(X::Rank == 2 && X::static_extent(0) == X::static_extent(1), "trace of a square matrix");
        const SampleIndex i0 = SampleIndex::make(std::size_t(0));
        if constexpr (X::static_extent(0) == 2) {
            return derived().template eval<0, 0>(i0) + derived().template eval<1, 1>(i0);
        } else {
            return derived().template eval<0, 0>(i0) + derived().template eval<1, 1>(i0) +
                   derived().template eval<2, 2>(i0);
        }
    }
    AETHER_DEVICEANDHOST() constexpr T det() const { return detail::det_at(derived(), SampleIndex::make(std::size_t(0))); }
    template <class E>
    AETHER_DEVICEANDHOST() constexpr T matDot(const Expression<E, T>& other) const {
        return detail::fold_dot(derived(), other.derived(), SampleIndex::make(std::size_t(0)));
    }

    // -- structural and geometric nodes ---------------------------------------
    template <class E>
    AETHER_DEVICEANDHOST() constexpr auto cross(const Expression<E, T>& o) const {
        return detail::Cross<Derived, E>(derived(), o.derived());
    }
    AETHER_DEVICEANDHOST() constexpr auto unitVector() const { return detail::UnitVector<Derived>(derived()); }
    template <class E>
    AETHER_DEVICEANDHOST() constexpr auto quatMul(const Expression<E, T>& o) const {
        return detail::QuatMul<Derived, E>(derived(), o.derived());
    }
    AETHER_DEVICEANDHOST() constexpr auto quatConj() const { return detail::QuatConj<Derived>(derived()); }
    AETHER_DEVICEANDHOST() constexpr auto quatReciprocal() const {
        return detail::CWiseScale<detail::QuatConj<Derived>>(quatConj(), rSquaredNorm());
    }
    template <class E>
    AETHER_DEVICEANDHOST() constexpr auto quatRotate(const Expression<E, T>& v) const {
        return detail::QuatRotate<Derived, E>(derived(), v.derived());
    }
    AETHER_DEVICEANDHOST() constexpr auto asPureQuaternion() const { return detail::AsPureQuaternion<Derived>(derived()); }
    AETHER_DEVICEANDHOST() constexpr auto asBack3DVector() const { return tail<3>(); }
    template <std::size_t Off, std::size_t Len>
    AETHER_DEVICEANDHOST() constexpr auto segment() const { return detail::Segment<Derived, Off, Len>(derived()); }
    template <std::size_t Len>
    AETHER_DEVICEANDHOST() constexpr auto head() const { return detail::Segment<Derived, 0, Len>(derived()); }
    template <std::size_t Len>
    AETHER_DEVICEANDHOST() constexpr auto tail() const {
        return detail::Segment<Derived, detail::extents_of<Derived>::static_extent(0) - Len, Len>(derived());
    }
    AETHER_DEVICEANDHOST() constexpr auto transpose() const { return detail::Transpose<Derived>(derived()); }
    template <std::size_t R>
    AETHER_DEVICEANDHOST() constexpr auto row() const { return detail::Row<Derived, R>(derived()); }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() constexpr auto col() const { return detail::Col<Derived, C>(derived()); }
    template <std::size_t R0, std::size_t C0, std::size_t BR, std::size_t BC>
    AETHER_DEVICEANDHOST() constexpr auto block() const { return detail::Block<Derived, R0, C0, BR, BC>(derived()); }
    template <class E>
    AETHER_DEVICEANDHOST() constexpr auto cwiseMul(const Expression<E, T>& o) const {
        return detail::CWiseMul<Derived, E>(derived(), o.derived());
    }
    AETHER_DEVICEANDHOST() constexpr auto inverse() const { return detail::Inverse<Derived>(derived()); }
};

/** evalW<Is...>(e, i): the value of component Is... of e at sample i. */
template <std::size_t... Is, class E>
AETHER_DEVICEANDHOST() constexpr auto evalW(const E& e, const SampleIndex& i) {
    return e.template eval<Is...>(i);
}

// The reduction operators by their public names, called as
// `SumOp<T>{}(a, b)` (expr/Reduce.h:53-86).
template <class T>
struct SumOp {
    AETHER_DEVICEANDHOST() constexpr T operator()(T a, T b) const { return a + b; }
};
template <class T>
struct TimesOp {
    AETHER_DEVICEANDHOST() constexpr T operator()(T a, T b) const { return a * b; }
};
template <class T>
struct MaxOp {
    AETHER_DEVICEANDHOST() constexpr T operator()(T a, T b) const { return a > b ? a : b; }
};
struct LogicalAndOp {
    AETHER_DEVICEANDHOST() constexpr bool operator()(bool a, bool b) const { return a && b; }
};

namespace detail {
template <class E, std::size_t... K>
AETHER_DEVICEANDHOST() bool all_finite_(const E& e, const SampleIndex& i, std::index_sequence<K...>) {
    bool ok = true;
    ((ok = LogicalAndOp{}(math::isfinite(e.template eval<K>(i)), ok)), ...);
    return ok;
}
}  // namespace detail

/** True when every component of a rank-1 expression is finite, at sample 0
 *  like the member reductions (expr/Reduce.h:198-211). */
template <class E, class = std::enable_if_t<aether_expression<E>>>
AETHER_DEVICEANDHOST() bool isFinite(const E& e) {
    static_assert(detail::extents_of<E>::Rank == 1, "isFinite: only rank-1 expressions are supported");
    return detail::all_finite_(e, SampleIndex::make(std::size_t(0)),
                               std::make_index_sequence<detail::extents_of<E>::static_extent(0)>{});
}

}  // namespace aether
