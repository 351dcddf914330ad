// aether/nodes.h -- arithmetic, elementwise, select and constant nodes.
//
// The reference's node set of expr/nodes/Arithmetic.h:33-143 (Sum, Product,
// CWiseScale), expr/nodes/Elementwise.h:61-854 (cwise* functions, min/max/
// clamp against a bound or an expression, cwiseDiv, cwisePow, select) and
// expr/nodes/Constant.h:68-150 (constant<Extents>(v)), with the operators of
// expr/Operations.h:25-71: + and - componentwise, * as the Hadamard product
// of two same-shaped expressions, s*e and e*s scaling, e/s = e*(1/s) with the
// reciprocal rounded once. Additions of this engine, none of which changes a
// reference spelling: unary minus, cwiseLog1p/Expm1/Exp2/Log2/Log10/Sinh/
// Cosh/Cbrt/Erf/Floor/Ceil/Trunc/Square, comparisons of an expression with a
// scalar or an expression (bool-valued, for select), and aether::per_sample
// folds (dot, squaredNorm, norm, rNorm, sum, maxNorm, det, trace as per-sample
// nodes).
//
// Each node evaluates per sample (eval) and, in host code, serialises itself
// to the engine's aether-ir/1 (gb300_ir) for the fused whole-view launch.
#pragma once

#include "aether/detail/std.h"

#include "aether/expression.h"

#if !defined(__CUDACC_RTC__)
#define AETHER_GB300_HOST_IR 1
#include "aether/expr.h"
#else
#define AETHER_GB300_HOST_IR 0
#endif

namespace aether {
namespace detail {

#if AETHER_GB300_HOST_IR
/** The type-erased IR of a typed node (host only). */
template <class E>
Expr ir_of(const E& e) {
    return e.gb300_ir();
}
template <class X>
ir::Shape shape_of_extents() {
    return ir::shape_of(X{});
}
#endif

// ---------------------------------------------------------------------------
// Arithmetic (expr/nodes/Arithmetic.h:33-143)
// ---------------------------------------------------------------------------
template <class L, class R, bool Neg>
class Sum : public Expression<Sum<L, R, Neg>, typename L::element_type> {
    static_assert(std::is_same<typename L::element_type, typename R::element_type>::value,
                  "+/-: element types differ");
    static_assert(same_shape<L, R>, "+/-: element extents differ");

public:
    using element_type = typename L::element_type;
    using element_extents = extents_of<L>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr Sum(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        if constexpr (Neg)
            return l_.template eval<Is...>(i) - r_.template eval<Is...>(i);
        else
            return l_.template eval<Is...>(i) + r_.template eval<Is...>(i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return Neg ? ir_of(l_) - ir_of(r_) : ir_of(l_) + ir_of(r_); }
#endif
    L l_;
    R r_;
};

/** The Hadamard product of two same-shaped expressions. */
template <class L, class R>
class Product : public Expression<Product<L, R>, typename L::element_type> {
    static_assert(std::is_same<typename L::element_type, typename R::element_type>::value, "*: element types differ");
    static_assert(same_shape<L, R>, "*: element extents differ (matrix products need rank-2 operands)");

public:
    using element_type = typename L::element_type;
    using element_extents = extents_of<L>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr Product(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return l_.template eval<Is...>(i) * r_.template eval<Is...>(i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(l_) * ir_of(r_); }
#endif
    L l_;
    R r_;
};

/** e scaled by a scalar (s*e, e*s, and e/s with s replaced by 1/s). */
template <class E>
class CWiseScale : public Expression<CWiseScale<E>, typename E::element_type> {
public:
    using element_type = typename E::element_type;
    using element_extents = extents_of<E>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr CWiseScale(const E& e, element_type s) : e_(e), s_(s) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return e_.template eval<Is...>(i) * s_;
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_) * double(s_); }
#endif
    E e_;
    element_type s_;
};

template <class E>
class Negate : public Expression<Negate<E>, typename E::element_type> {
public:
    using element_type = typename E::element_type;
    using element_extents = extents_of<E>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr explicit Negate(const E& e) : e_(e) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return -e_.template eval<Is...>(i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return -ir_of(e_); }
#endif
    E e_;
};

// ---------------------------------------------------------------------------
// Elementwise functions (expr/nodes/Elementwise.h)
// ---------------------------------------------------------------------------
namespace op {
#if AETHER_GB300_HOST_IR
#define AETHER_GB300_OPIR(FN) \
    static Expr ir(const Expr& e) { return ::aether::FN(e); }
#else
#define AETHER_GB300_OPIR(FN)
#endif
#define AETHER_GB300_UOP(NAME, CALL, FN)                                          \
    struct NAME {                                                                  \
        template <class T>                                                         \
        AETHER_DEVICEANDHOST() static T apply(T x) {                                  \
            return CALL;                                                           \
        }                                                                          \
        AETHER_GB300_OPIR(FN)                                                      \
    };
AETHER_GB300_UOP(Sqrt, math::sqrt(x), cwiseSqrt)
AETHER_GB300_UOP(Rsqrt, math::rsqrt(x), cwiseRsqrt)
AETHER_GB300_UOP(Exp, math::exp(x), cwiseExp)
AETHER_GB300_UOP(Log, math::log(x), cwiseLog)
AETHER_GB300_UOP(Sin, math::sin(x), cwiseSin)
AETHER_GB300_UOP(Cos, math::cos(x), cwiseCos)
AETHER_GB300_UOP(Tan, math::tan(x), cwiseTan)
AETHER_GB300_UOP(Asin, math::asin(x), cwiseAsin)
AETHER_GB300_UOP(Acos, math::acos(x), cwiseAcos)
AETHER_GB300_UOP(Atan, math::atan(x), cwiseAtan)
AETHER_GB300_UOP(Tanh, math::tanh(x), cwiseTanh)
AETHER_GB300_UOP(Abs, math::abs(x), cwiseAbs)
AETHER_GB300_UOP(Sign, math::sign(x), cwiseSign)
AETHER_GB300_UOP(Log1p, math::log1p(x), cwiseLog1p)
AETHER_GB300_UOP(Expm1, math::expm1(x), cwiseExpm1)
AETHER_GB300_UOP(Exp2, math::exp2(x), cwiseExp2)
AETHER_GB300_UOP(Log2, math::log2(x), cwiseLog2)
AETHER_GB300_UOP(Log10, math::log10(x), cwiseLog10)
AETHER_GB300_UOP(Sinh, math::sinh(x), cwiseSinh)
AETHER_GB300_UOP(Cosh, math::cosh(x), cwiseCosh)
AETHER_GB300_UOP(Cbrt, math::cbrt(x), cwiseCbrt)
AETHER_GB300_UOP(Erf, math::erf(x), cwiseErf)
AETHER_GB300_UOP(Floor, math::floor(x), cwiseFloor)
AETHER_GB300_UOP(Ceil, math::ceil(x), cwiseCeil)
AETHER_GB300_UOP(Trunc, math::trunc(x), cwiseTrunc)
AETHER_GB300_UOP(Square, x * x, cwiseSquare)
#undef AETHER_GB300_UOP
#undef AETHER_GB300_OPIR
}  // namespace op

template <class E, class Op>
class Unary : public Expression<Unary<E, Op>, typename E::element_type> {
public:
    using element_type = typename E::element_type;
    using element_extents = extents_of<E>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr explicit Unary(const E& e) : e_(e) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() element_type eval(const SampleIndex& i) const {
        return Op::apply(e_.template eval<Is...>(i));
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return Op::ir(ir_of(e_)); }
#endif
    E e_;
};
template <class E> using CWiseSqrt = Unary<E, op::Sqrt>;
template <class E> using CWiseRsqrt = Unary<E, op::Rsqrt>;
template <class E> using CWiseExp = Unary<E, op::Exp>;
template <class E> using CWiseLog = Unary<E, op::Log>;
template <class E> using CWiseSin = Unary<E, op::Sin>;
template <class E> using CWiseCos = Unary<E, op::Cos>;
template <class E> using CWiseTan = Unary<E, op::Tan>;
template <class E> using CWiseAsin = Unary<E, op::Asin>;
template <class E> using CWiseAcos = Unary<E, op::Acos>;
template <class E> using CWiseAtan = Unary<E, op::Atan>;
template <class E> using CWiseTanh = Unary<E, op::Tanh>;
template <class E> using CWiseAbs = Unary<E, op::Abs>;
template <class E> using CWiseSign = Unary<E, op::Sign>;

/** min/max against a scalar bound, clamp, pow with a scalar exponent. */
template <class E, int Kind>
class ScalarBinary : public Expression<ScalarBinary<E, Kind>, typename E::element_type> {
public:
    using element_type = typename E::element_type;
    using element_extents = extents_of<E>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr ScalarBinary(const E& e, element_type a, element_type b = element_type(0))
        : e_(e), a_(a), b_(b) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() element_type eval(const SampleIndex& i) const {
        const element_type x = e_.template eval<Is...>(i);
        if constexpr (Kind == 0) return math::min(x, a_);
        if constexpr (Kind == 1) return math::max(x, a_);
        if constexpr (Kind == 2) return math::min(math::max(x, a_), b_);
        if constexpr (Kind == 3) return math::pow(x, a_);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        if constexpr (Kind == 0) return ::aether::cwiseMin(ir_of(e_), double(a_));
        if constexpr (Kind == 1) return ::aether::cwiseMax(ir_of(e_), double(a_));
        if constexpr (Kind == 2) return ::aether::clamp(ir_of(e_), double(a_), double(b_));
        if constexpr (Kind == 3) return ::aether::cwisePow(ir_of(e_), double(a_));
    }
#endif
    E e_;
    element_type a_, b_;
};
template <class E> using CWiseMin = ScalarBinary<E, 0>;
template <class E> using CWiseMax = ScalarBinary<E, 1>;
template <class E> using CWiseClamp = ScalarBinary<E, 2>;
template <class E> using CWisePow = ScalarBinary<E, 3>;

/** Componentwise division, pow, min and max of two same-shaped expressions. */
template <class L, class R, int Kind>
class ExprBinary : public Expression<ExprBinary<L, R, Kind>, typename L::element_type> {
    static_assert(std::is_same<typename L::element_type, typename R::element_type>::value, "element types differ");
    static_assert(same_shape<L, R>, "element extents differ");

public:
    using element_type = typename L::element_type;
    using element_extents = extents_of<L>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr ExprBinary(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() element_type eval(const SampleIndex& i) const {
        const element_type a = l_.template eval<Is...>(i), b = r_.template eval<Is...>(i);
        if constexpr (Kind == 0) return a / b;
        if constexpr (Kind == 1) return math::pow(a, b);
        if constexpr (Kind == 2) return math::min(a, b);
        if constexpr (Kind == 3) return math::max(a, b);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        if constexpr (Kind == 0) return ::aether::cwiseDiv(ir_of(l_), ir_of(r_));
        if constexpr (Kind == 1) return ::aether::cwisePow(ir_of(l_), ir_of(r_));
        if constexpr (Kind == 2) return ::aether::cwiseMin(ir_of(l_), ir_of(r_));
        if constexpr (Kind == 3) return ::aether::cwiseMax(ir_of(l_), ir_of(r_));
    }
#endif
    L l_;
    R r_;
};
template <class L, class R> using CWiseDiv = ExprBinary<L, R, 0>;
template <class L, class R> using CWisePowExpr = ExprBinary<L, R, 1>;
template <class L, class R> using CWiseMinExpr = ExprBinary<L, R, 2>;
template <class L, class R> using CWiseMaxExpr = ExprBinary<L, R, 3>;

/** A comparison, bool-valued (an addition: the condition of select). Kind:
 *  0 >, 1 <, 2 >=, 3 <=. R is an expression or, with IsScalar, the scalar. */
template <class L, class R, int Kind, bool IsScalar>
class Compare : public Expression<Compare<L, R, Kind, IsScalar>, bool> {
public:
    using element_type = bool;
    using element_extents = extents_of<L>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr Compare(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr bool eval(const SampleIndex& i) const {
        const auto a = l_.template eval<Is...>(i);
        const auto b = rhs_<Is...>(i);
        if constexpr (Kind == 0) return a > b;
        if constexpr (Kind == 1) return a < b;
        if constexpr (Kind == 2) return a >= b;
        if constexpr (Kind == 3) return a <= b;
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        const Expr a = ir_of(l_);
        if constexpr (IsScalar) {
            if constexpr (Kind == 0) return a > double(r_);
            if constexpr (Kind == 1) return a < double(r_);
            if constexpr (Kind == 2) return a >= double(r_);
            if constexpr (Kind == 3) return a <= double(r_);
        } else {
            const Expr b = ir_of(r_);
            if constexpr (Kind == 0) return a > b;
            if constexpr (Kind == 1) return a < b;
            if constexpr (Kind == 2) return a >= b;
            if constexpr (Kind == 3) return a <= b;
        }
    }
#endif
    L l_;
    R r_;

private:
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr auto rhs_(const SampleIndex& i) const {
        if constexpr (IsScalar)
            return r_;
        else
            return r_.template eval<Is...>(i);
    }
};

/** select(cond, a, b) (expr/nodes/Elementwise.h:809-854): cond is bool-valued,
 *  rank 0 (one choice per sample) or shaped like a and b. */
template <class C, class A, class B>
class Select : public Expression<Select<C, A, B>, typename A::element_type> {
    static_assert(std::is_same<typename A::element_type, typename B::element_type>::value,
                  "select: a/b element types differ");
    static_assert(same_shape<A, B>, "select: a/b element extents differ");
    static_assert(std::is_same<typename C::element_type, bool>::value, "select: the condition must be bool-valued");
    static_assert(extents_of<C>::Rank == 0 || same_shape<C, A>, "select: condition of rank 0 or shaped like a/b");

public:
    using element_type = typename A::element_type;
    using element_extents = extents_of<A>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr Select(const C& c, const A& a, const B& b) : c_(c), a_(a), b_(b) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        bool pick;
        if constexpr (extents_of<C>::Rank == 0)
            pick = c_.template eval<>(i);
        else
            pick = c_.template eval<Is...>(i);
        return pick ? a_.template eval<Is...>(i) : b_.template eval<Is...>(i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ::aether::select(ir_of(c_), ir_of(a_), ir_of(b_)); }
#endif
    C c_;
    A a_;
    B b_;
};

/** A scalar broadcast over Extents (expr/nodes/Constant.h:68-105). */
template <class T, class X>
class Constant : public Expression<Constant<T, X>, T> {
public:
    using element_type = T;
    using element_extents = X;
    static constexpr bool isLeaf = true;
    AETHER_DEVICEANDHOST() constexpr explicit Constant(T v) : v_(v) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr T eval(const SampleIndex&) const {
        return v_;
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ::aether::constant(double(v_), shape_of_extents<X>()); }
#endif
    T v_;
};

// Per-sample folds (an addition: the reference's dot/norm/... members are
// evaluated at sample 0). Kind: 0 dot, 1 squaredNorm, 2 norm, 3 rNorm, 4 sum,
// 5 maxNorm; the order is the members' right-nested fold.
template <class L, class R, int Kind>
class Fold : public Expression<Fold<L, R, Kind>, typename L::element_type> {
public:
    using element_type = typename L::element_type;
    using element_extents = extents<>;
    static constexpr bool isLeaf = false;
    AETHER_DEVICEANDHOST() constexpr Fold(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() element_type eval(const SampleIndex& i) const {
        static_assert(sizeof...(Is) == 0, "a fold is rank 0");
        if constexpr (Kind == 0) return fold_dot(l_, r_, i);
        if constexpr (Kind == 1) return fold_dot(l_, l_, i);
        if constexpr (Kind == 2) return math::sqrt(fold_dot(l_, l_, i));
        if constexpr (Kind == 3) return element_type(1) / math::sqrt(fold_dot(l_, l_, i));
        if constexpr (Kind == 4) return fold_sum(l_, i);
        if constexpr (Kind == 5)
            return fold_maxabs_(l_, i, std::make_index_sequence<size_of<extents_of<L>>>{});
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        const Expr a = ir_of(l_);
        if constexpr (Kind == 0) return a.dot(ir_of(r_));
        if constexpr (Kind == 1) return a.squaredNorm();
        if constexpr (Kind == 2) return a.norm();
        if constexpr (Kind == 3) return a.rNorm();
        if constexpr (Kind == 4) return a.sum();
        if constexpr (Kind == 5) return a.maxNorm();
    }
#endif
    L l_;
    R r_;
};

}  // namespace detail

// ---------------------------------------------------------------------------
// Operators (expr/Operations.h:25-71)
// ---------------------------------------------------------------------------
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Sum<L, R, false> operator+(const L& l, const R& r) {
    return detail::Sum<L, R, false>(l, r);
}
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Sum<L, R, true> operator-(const L& l, const R& r) {
    return detail::Sum<L, R, true>(l, r);
}
/** Hadamard product; two rank-2 operands, or rank-2 times rank-1, are the
 *  matrix products of aether/geometry.h instead. */
template <class L, class R,
          std::enable_if_t<aether_expression<L> && aether_expression<R> &&
                               !(detail::extents_of<L>::Rank == 2 && detail::extents_of<R>::Rank >= 1),
                           int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Product<L, R> operator*(const L& l, const R& r) {
    return detail::Product<L, R>(l, r);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseScale<E> operator*(const typename E::element_type& s, const E& e) {
    return detail::CWiseScale<E>(e, s);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseScale<E> operator*(const E& e, const typename E::element_type& s) {
    return detail::CWiseScale<E>(e, s);
}
/** e / s is e * (1/s): the reciprocal is rounded once, here. */
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseScale<E> operator/(const E& e, const typename E::element_type& s) {
    return detail::CWiseScale<E>(e, typename E::element_type(1) / s);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Negate<E> operator-(const E& e) {
    return detail::Negate<E>(e);
}

#define AETHER_GB300_CMP_OP(OPER, KIND)                                                                      \
    template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>   \
    AETHER_DEVICEANDHOST() constexpr detail::Compare<L, R, KIND, false> operator OPER(const L& l, const R& r) { \
        return detail::Compare<L, R, KIND, false>(l, r);                                                     \
    }                                                                                                        \
    template <class L, std::enable_if_t<aether_expression<L>, int> = 0>                                     \
    AETHER_DEVICEANDHOST() constexpr detail::Compare<L, typename L::element_type, KIND, true> operator OPER(   \
        const L& l, const typename L::element_type& s) {                                                     \
        return detail::Compare<L, typename L::element_type, KIND, true>(l, s);                               \
    }
AETHER_GB300_CMP_OP(>, 0)
AETHER_GB300_CMP_OP(<, 1)
AETHER_GB300_CMP_OP(>=, 2)
AETHER_GB300_CMP_OP(<=, 3)
#undef AETHER_GB300_CMP_OP

// ---------------------------------------------------------------------------
// Elementwise functions
// ---------------------------------------------------------------------------
#define AETHER_GB300_CWISE(FN, OP)                                               \
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>         \
    AETHER_DEVICEANDHOST() constexpr detail::Unary<E, detail::op::OP> FN(const E& e) { \
        return detail::Unary<E, detail::op::OP>(e);                              \
    }
AETHER_GB300_CWISE(cwiseSqrt, Sqrt)
AETHER_GB300_CWISE(cwiseRsqrt, Rsqrt)
AETHER_GB300_CWISE(cwiseExp, Exp)
AETHER_GB300_CWISE(cwiseLog, Log)
AETHER_GB300_CWISE(cwiseSin, Sin)
AETHER_GB300_CWISE(cwiseCos, Cos)
AETHER_GB300_CWISE(cwiseTan, Tan)
AETHER_GB300_CWISE(cwiseAsin, Asin)
AETHER_GB300_CWISE(cwiseAcos, Acos)
AETHER_GB300_CWISE(cwiseAtan, Atan)
AETHER_GB300_CWISE(cwiseTanh, Tanh)
AETHER_GB300_CWISE(cwiseAbs, Abs)
AETHER_GB300_CWISE(cwiseSign, Sign)
AETHER_GB300_CWISE(cwiseLog1p, Log1p)
AETHER_GB300_CWISE(cwiseExpm1, Expm1)
AETHER_GB300_CWISE(cwiseExp2, Exp2)
AETHER_GB300_CWISE(cwiseLog2, Log2)
AETHER_GB300_CWISE(cwiseLog10, Log10)
AETHER_GB300_CWISE(cwiseSinh, Sinh)
AETHER_GB300_CWISE(cwiseCosh, Cosh)
AETHER_GB300_CWISE(cwiseCbrt, Cbrt)
AETHER_GB300_CWISE(cwiseErf, Erf)
AETHER_GB300_CWISE(cwiseFloor, Floor)
AETHER_GB300_CWISE(cwiseCeil, Ceil)
AETHER_GB300_CWISE(cwiseTrunc, Trunc)
AETHER_GB300_CWISE(cwiseSquare, Square)
#undef AETHER_GB300_CWISE

template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseMin<E> cwiseMin(const E& e, const typename E::element_type& bound) {
    return detail::CWiseMin<E>(e, bound);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseMax<E> cwiseMax(const E& e, const typename E::element_type& bound) {
    return detail::CWiseMax<E>(e, bound);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseClamp<E> clamp(const E& e, const typename E::element_type& lo,
                                                          const typename E::element_type& hi) {
    return detail::CWiseClamp<E>(e, lo, hi);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWisePow<E> cwisePow(const E& e, const typename E::element_type& p) {
    return detail::CWisePow<E>(e, p);
}
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseDiv<L, R> cwiseDiv(const L& l, const R& r) {
    return detail::CWiseDiv<L, R>(l, r);
}
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWisePowExpr<L, R> cwisePow(const L& l, const R& r) {
    return detail::CWisePowExpr<L, R>(l, r);
}
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseMinExpr<L, R> cwiseMin(const L& l, const R& r) {
    return detail::CWiseMinExpr<L, R>(l, r);
}
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::CWiseMaxExpr<L, R> cwiseMax(const L& l, const R& r) {
    return detail::CWiseMaxExpr<L, R>(l, r);
}
template <class C, class A, class B,
          std::enable_if_t<aether_expression<C> && aether_expression<A> && aether_expression<B>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Select<C, A, B> select(const C& c, const A& a, const B& b) {
    return detail::Select<C, A, B>(c, a, b);
}
/** A scalar v broadcast to Extents (expr/nodes/Constant.h:107). */
template <class X, class T>
AETHER_DEVICEANDHOST() constexpr detail::Constant<T, X> constant(const T& v) {
    return detail::Constant<T, X>(v);
}

namespace per_sample {
template <class L, class R, std::enable_if_t<aether_expression<L> && aether_expression<R>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Fold<L, R, 0> dot(const L& l, const R& r) {
    static_assert(detail::same_shape<L, R>, "dot: operands of different shapes");
    return detail::Fold<L, R, 0>(l, r);
}
#define AETHER_GB300_FOLD(FN, KIND)                                                   \
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>              \
    AETHER_DEVICEANDHOST() constexpr detail::Fold<E, E, KIND> FN(const E& e) {           \
        return detail::Fold<E, E, KIND>(e, e);                                        \
    }
AETHER_GB300_FOLD(squaredNorm, 1)
AETHER_GB300_FOLD(norm, 2)
AETHER_GB300_FOLD(rNorm, 3)
AETHER_GB300_FOLD(sum, 4)
AETHER_GB300_FOLD(maxNorm, 5)
#undef AETHER_GB300_FOLD
}  // namespace per_sample

}  // namespace aether
