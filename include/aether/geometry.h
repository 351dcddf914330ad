// aether/geometry.h -- geometric, quaternion, structural and matrix nodes.
//
// cross and unitVector (expr/nodes/Geometric.h:33-103), quaternion product,
// conjugate, rotation and embedding (expr/nodes/Quaternion.h:36-203),
// segment/head/tail, transpose, row, col and block views of an element
// (expr/nodes/Structural.h), M*v, A*B, outer(u, v) and cwiseMul
// (expr/nodes/Product.h:109-512), inverse and det (expr/nodes/Inverse.h:52-118,
// expr/Expression.h:400-428). Each formula keeps the reference's operand
// order, so with contraction off a result is bit-identical to the
// reference's CPU evaluation. As in the reference, inverse() has no
// determinant guard (compose select(...) for one), unitVector() scales by
// the norm of sample 0, and matrices are 2x2 or 3x3 where a formula needs it.
#pragma once

#include "aether/nodes.h"

namespace aether {
namespace detail {

template <std::size_t I, class E>
AETHER_DEVICEANDHOST() constexpr auto at1(const E& e, const SampleIndex& i) {
    return e.template eval<I>(i);
}
template <std::size_t R, std::size_t C, class E>
AETHER_DEVICEANDHOST() constexpr auto at2(const E& e, const SampleIndex& i) {
    return e.template eval<R, C>(i);
}

#define AETHER_GB300_NODE_HEAD(T, LEAF, ...)       \
public:                                            \
    using element_type = T;                        \
    using element_extents = __VA_ARGS__;           \
    static constexpr bool isLeaf = LEAF;

template <class L, class R>
class Cross : public Expression<Cross<L, R>, typename L::element_type> {
    static_assert(std::is_same<extents_of<L>, extents<3>>::value && std::is_same<extents_of<R>, extents<3>>::value,
                  "cross needs two 3-vectors");
    AETHER_GB300_NODE_HEAD(typename L::element_type, false, extents<3>)
    AETHER_DEVICEANDHOST() constexpr Cross(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        constexpr std::size_t a = (I + 1) % 3, b = (I + 2) % 3;
        return at1<a>(l_, i) * at1<b>(r_, i) - at1<b>(l_, i) * at1<a>(r_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(l_).cross(ir_of(r_)); }
#endif
    L l_;
    R r_;
};

/** e scaled by 1/|e| of sample 0 (Geometric.h:99-103, the reference's rule). */
template <class E>
class UnitVector : public Expression<UnitVector<E>, typename E::element_type> {
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents_of<E>)
    AETHER_DEVICEANDHOST() constexpr explicit UnitVector(const E& e) : e_(e) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() element_type eval(const SampleIndex& i) const {
        return e_.template eval<Is...>(i) * e_.rNorm();
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        const Expr a = ir_of(e_);
        return a * a.rNorm().atSample0();
    }
#endif
    E e_;
};

template <class L, class R>
class QuatMul : public Expression<QuatMul<L, R>, typename L::element_type> {
    static_assert(std::is_same<extents_of<L>, extents<4>>::value && std::is_same<extents_of<R>, extents<4>>::value,
                  "quatMul needs two quaternions");
    AETHER_GB300_NODE_HEAD(typename L::element_type, false, extents<4>)
    AETHER_DEVICEANDHOST() constexpr QuatMul(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        const element_type l0 = at1<0>(l_, i), l1 = at1<1>(l_, i), l2 = at1<2>(l_, i), l3 = at1<3>(l_, i);
        const element_type r0 = at1<0>(r_, i), r1 = at1<1>(r_, i), r2 = at1<2>(r_, i), r3 = at1<3>(r_, i);
        if constexpr (I == 0) return l0 * r0 - l1 * r1 - l2 * r2 - l3 * r3;
        else if constexpr (I == 1) return l0 * r1 + l1 * r0 + l2 * r3 - l3 * r2;
        else if constexpr (I == 2) return l0 * r2 - l1 * r3 + l2 * r0 + l3 * r1;
        else return l0 * r3 + l1 * r2 - l2 * r1 + l3 * r0;
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(l_).quatMul(ir_of(r_)); }
#endif
    L l_;
    R r_;
};

template <class E>
class QuatConj : public Expression<QuatConj<E>, typename E::element_type> {
    static_assert(std::is_same<extents_of<E>, extents<4>>::value, "quatConj needs a quaternion");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<4>)
    AETHER_DEVICEANDHOST() constexpr explicit QuatConj(const E& e) : e_(e) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        if constexpr (I == 0) return at1<0>(e_, i);
        else return -at1<I>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).quatConj(); }
#endif
    E e_;
};

/** v rotated by q: v + q0 t + q_v x t with t = 2 (q_v x v) (Quaternion.h:118-168). */
template <class Q, class V>
class QuatRotate : public Expression<QuatRotate<Q, V>, typename Q::element_type> {
    static_assert(std::is_same<extents_of<Q>, extents<4>>::value && std::is_same<extents_of<V>, extents<3>>::value,
                  "quatRotate needs a quaternion and a 3-vector");
    AETHER_GB300_NODE_HEAD(typename Q::element_type, false, extents<3>)
    AETHER_DEVICEANDHOST() constexpr QuatRotate(const Q& q, const V& v) : q_(q), v_(v) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        const element_type q0 = at1<0>(q_, i), q1 = at1<1>(q_, i), q2 = at1<2>(q_, i), q3 = at1<3>(q_, i);
        const element_type v0 = at1<0>(v_, i), v1 = at1<1>(v_, i), v2 = at1<2>(v_, i);
        const element_type tx = element_type(2) * (q2 * v2 - q3 * v1);
        const element_type ty = element_type(2) * (q3 * v0 - q1 * v2);
        const element_type tz = element_type(2) * (q1 * v1 - q2 * v0);
        if constexpr (I == 0) return (v0 + q0 * tx) + (q2 * tz - q3 * ty);
        else if constexpr (I == 1) return (v1 + q0 * ty) + (q3 * tx - q1 * tz);
        else return (v2 + q0 * tz) + (q1 * ty - q2 * tx);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(q_).quatRotate(ir_of(v_)); }
#endif
    Q q_;
    V v_;
};

template <class E>
class AsPureQuaternion : public Expression<AsPureQuaternion<E>, typename E::element_type> {
    static_assert(std::is_same<extents_of<E>, extents<3>>::value, "asPureQuaternion needs a 3-vector");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<4>)
    AETHER_DEVICEANDHOST() constexpr explicit AsPureQuaternion(const E& e) : e_(e) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        if constexpr (I == 0) return element_type(0);
        else return at1<I - 1>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).asPureQuaternion(); }
#endif
    E e_;
};

template <class E, std::size_t Off, std::size_t Len>
class Segment : public Expression<Segment<E, Off, Len>, typename E::element_type> {
    static_assert(extents_of<E>::Rank == 1 && Off + Len <= extents_of<E>::static_extent(0), "segment out of range");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<Len>)
    AETHER_DEVICEANDHOST() constexpr explicit Segment(const E& e) : e_(e) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at1<Off + I>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).segment(int(Off), int(Len)); }
#endif
    E e_;
};

template <class E>
class Transpose : public Expression<Transpose<E>, typename E::element_type> {
    static_assert(extents_of<E>::Rank == 2, "transpose needs a matrix");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false,
                           extents<extents_of<E>::static_extent(1), extents_of<E>::static_extent(0)>)
    AETHER_DEVICEANDHOST() constexpr explicit Transpose(const E& e) : e_(e) {}
    template <std::size_t R, std::size_t C>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at2<C, R>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).transpose(); }
#endif
    E e_;
};

template <class E, std::size_t Rw>
class Row : public Expression<Row<E, Rw>, typename E::element_type> {
    static_assert(extents_of<E>::Rank == 2 && Rw < extents_of<E>::static_extent(0), "row out of range");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<extents_of<E>::static_extent(1)>)
    AETHER_DEVICEANDHOST() constexpr explicit Row(const E& e) : e_(e) {}
    template <std::size_t C>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at2<Rw, C>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).row(int(Rw)); }
#endif
    E e_;
};

template <class E, std::size_t Cl>
class Col : public Expression<Col<E, Cl>, typename E::element_type> {
    static_assert(extents_of<E>::Rank == 2 && Cl < extents_of<E>::static_extent(1), "col out of range");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<extents_of<E>::static_extent(0)>)
    AETHER_DEVICEANDHOST() constexpr explicit Col(const E& e) : e_(e) {}
    template <std::size_t R>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at2<R, Cl>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).col(int(Cl)); }
#endif
    E e_;
};

template <class E, std::size_t R0, std::size_t C0, std::size_t BR, std::size_t BC>
class Block : public Expression<Block<E, R0, C0, BR, BC>, typename E::element_type> {
    static_assert(extents_of<E>::Rank == 2 && R0 + BR <= extents_of<E>::static_extent(0) &&
                      C0 + BC <= extents_of<E>::static_extent(1),
                  "block out of range");
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<BR, BC>)
    AETHER_DEVICEANDHOST() constexpr explicit Block(const E& e) : e_(e) {}
    template <std::size_t R, std::size_t C>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at2<R0 + R, C0 + C>(e_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).block(int(R0), int(C0), int(BR), int(BC)); }
#endif
    E e_;
};

/** The componentwise product of two same-shaped operands, matrices included. */
template <class L, class R>
class CWiseMul : public Expression<CWiseMul<L, R>, typename L::element_type> {
    static_assert(same_shape<L, R>, "cwiseMul: shapes differ");
    AETHER_GB300_NODE_HEAD(typename L::element_type, false, extents_of<L>)
    AETHER_DEVICEANDHOST() constexpr CWiseMul(const L& l, const R& r) : l_(l), r_(r) {}
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

// sum_k a(Rw, k) b(k[, Cl]) folded right-nested: a0 b0, then a_k b_k + acc.
template <class A, class B, std::size_t Rw, std::size_t Cl, bool Vec, std::size_t k>
AETHER_DEVICEANDHOST() constexpr typename A::element_type row_term_(const A& a, const B& b, const SampleIndex& i) {
    if constexpr (Vec)
        return at2<Rw, k>(a, i) * at1<k>(b, i);
    else
        return at2<Rw, k>(a, i) * at2<k, Cl>(b, i);
}
template <class A, class B, std::size_t Rw, std::size_t Cl, bool Vec, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr auto row_dot_(const A& a, const B& b, const SampleIndex& i, std::index_sequence<K...>) {
    using T = typename A::element_type;
    T acc{};
    bool first = true;
    ((acc = first ? row_term_<A, B, Rw, Cl, Vec, K>(a, b, i) : T(row_term_<A, B, Rw, Cl, Vec, K>(a, b, i) + acc),
      first = false),
     ...);
    return acc;
}

template <class M, class V>
class MatVec : public Expression<MatVec<M, V>, typename M::element_type> {
    static_assert(extents_of<M>::Rank == 2 && extents_of<V>::Rank == 1 &&
                      extents_of<M>::static_extent(1) == extents_of<V>::static_extent(0),
                  "M * v: inner extents differ");
    AETHER_GB300_NODE_HEAD(typename M::element_type, false, extents<extents_of<M>::static_extent(0)>)
    AETHER_DEVICEANDHOST() constexpr MatVec(const M& m, const V& v) : m_(m), v_(v) {}
    template <std::size_t Rw>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return row_dot_<M, V, Rw, 0, true>(m_, v_, i, std::make_index_sequence<extents_of<M>::static_extent(1)>{});
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(m_).matvec(ir_of(v_)); }
#endif
    M m_;
    V v_;
};

template <class L, class R>
class MatMat : public Expression<MatMat<L, R>, typename L::element_type> {
    static_assert(extents_of<L>::Rank == 2 && extents_of<R>::Rank == 2 &&
                      extents_of<L>::static_extent(1) == extents_of<R>::static_extent(0),
                  "A * B: inner extents differ");
    AETHER_GB300_NODE_HEAD(typename L::element_type, false,
                           extents<extents_of<L>::static_extent(0), extents_of<R>::static_extent(1)>)
    AETHER_DEVICEANDHOST() constexpr MatMat(const L& l, const R& r) : l_(l), r_(r) {}
    template <std::size_t Rw, std::size_t Cl>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return row_dot_<L, R, Rw, Cl, false>(l_, r_, i, std::make_index_sequence<extents_of<L>::static_extent(1)>{});
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(l_).matmul(ir_of(r_)); }
#endif
    L l_;
    R r_;
};

template <class U, class V>
class Outer : public Expression<Outer<U, V>, typename U::element_type> {
    static_assert(extents_of<U>::Rank == 1 && extents_of<V>::Rank == 1, "outer needs two vectors");
    AETHER_GB300_NODE_HEAD(typename U::element_type, false,
                           extents<extents_of<U>::static_extent(0), extents_of<V>::static_extent(0)>)
    AETHER_DEVICEANDHOST() constexpr Outer(const U& u, const V& v) : u_(u), v_(v) {}
    template <std::size_t Rw, std::size_t Cl>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        return at1<Rw>(u_, i) * at1<Cl>(v_, i);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(u_).outer(ir_of(v_)); }
#endif
    U u_;
    V v_;
};

template <class E>
AETHER_DEVICEANDHOST() constexpr typename E::element_type det_at(const E& m, const SampleIndex& i) {
    using X = extents_of<E>;
    static_assert(X::Rank == 2 && X::static_extent(0) == X::static_extent(1) &&
                      (X::static_extent(0) == 2 || X::static_extent(0) == 3),
                  "det of a 2x2 or 3x3 matrix");
    if constexpr (X::static_extent(0) == 2) {
        return at2<0, 0>(m, i) * at2<1, 1>(m, i) - at2<0, 1>(m, i) * at2<1, 0>(m, i);
    } else {
        const auto a = at2<0, 0>(m, i), b = at2<0, 1>(m, i), c = at2<0, 2>(m, i);
        const auto d = at2<1, 0>(m, i), e = at2<1, 1>(m, i), f = at2<1, 2>(m, i);
        const auto g = at2<2, 0>(m, i), h = at2<2, 1>(m, i), k = at2<2, 2>(m, i);
        return a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
    }
}

/** The inverse by cofactors over the determinant (Inverse.h:73-118). */
template <class E>
class Inverse : public Expression<Inverse<E>, typename E::element_type> {
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents_of<E>)
    AETHER_DEVICEANDHOST() constexpr explicit Inverse(const E& e) : e_(e) {}
    template <std::size_t R, std::size_t C>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        const element_type det = det_at(e_, i);
        constexpr std::size_t k = R * extents_of<E>::static_extent(1) + C;
        if constexpr (extents_of<E>::static_extent(0) == 2) {
            if constexpr (k == 0) return at2<1, 1>(e_, i) / det;
            else if constexpr (k == 1) return -at2<0, 1>(e_, i) / det;
            else if constexpr (k == 2) return -at2<1, 0>(e_, i) / det;
            else return at2<0, 0>(e_, i) / det;
        } else {
            const element_type a = at2<0, 0>(e_, i), b = at2<0, 1>(e_, i), c = at2<0, 2>(e_, i);
            const element_type d = at2<1, 0>(e_, i), e = at2<1, 1>(e_, i), f = at2<1, 2>(e_, i);
            const element_type g = at2<2, 0>(e_, i), h = at2<2, 1>(e_, i), kk = at2<2, 2>(e_, i);
            if constexpr (k == 0) return (e * kk - f * h) / det;
            else if constexpr (k == 1) return (c * h - b * kk) / det;
            else if constexpr (k == 2) return (b * f - c * e) / det;
            else if constexpr (k == 3) return (f * g - d * kk) / det;
            else if constexpr (k == 4) return (a * kk - c * g) / det;
            else if constexpr (k == 5) return (c * d - a * f) / det;
            else if constexpr (k == 6) return (d * h - e * g) / det;
            else if constexpr (k == 7) return (b * g - a * h) / det;
            else return (a * e - b * d) / det;
        }
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return ir_of(e_).inverse(); }
#endif
    E e_;
};

/** Per-sample determinant and trace (rank-0 nodes, an addition). */
template <class E, bool Trace>
class MatScalar : public Expression<MatScalar<E, Trace>, typename E::element_type> {
    AETHER_GB300_NODE_HEAD(typename E::element_type, false, extents<>)
    AETHER_DEVICEANDHOST() constexpr explicit MatScalar(const E& e) : e_(e) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval(const SampleIndex& i) const {
        if constexpr (Trace) {
            if constexpr (extents_of<E>::static_extent(0) == 2)
                return at2<0, 0>(e_, i) + at2<1, 1>(e_, i);
            else
                return at2<0, 0>(e_, i) + at2<1, 1>(e_, i) + at2<2, 2>(e_, i);
        } else {
            return det_at(e_, i);
        }
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const { return Trace ? ir_of(e_).trace() : ir_of(e_).det(); }
#endif
    E e_;
};

#undef AETHER_GB300_NODE_HEAD

}  // namespace detail

/** M * v and A * B (expr/nodes/Product.h:494-507). */
template <class L, class R,
          std::enable_if_t<aether_expression<L> && aether_expression<R> && detail::extents_of<L>::Rank == 2 &&
                               detail::extents_of<R>::Rank == 1,
                           int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::MatVec<L, R> operator*(const L& l, const R& r) {
    return detail::MatVec<L, R>(l, r);
}
template <class L, class R,
          std::enable_if_t<aether_expression<L> && aether_expression<R> && detail::extents_of<L>::Rank == 2 &&
                               detail::extents_of<R>::Rank == 2,
                           int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::MatMat<L, R> operator*(const L& l, const R& r) {
    return detail::MatMat<L, R>(l, r);
}
template <class U, class V, std::enable_if_t<aether_expression<U> && aether_expression<V>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::Outer<U, V> outer(const U& u, const V& v) {
    return detail::Outer<U, V>(u, v);
}

namespace per_sample {
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::MatScalar<E, false> det(const E& e) {
    return detail::MatScalar<E, false>(e);
}
template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
AETHER_DEVICEANDHOST() constexpr detail::MatScalar<E, true> trace(const E& e) {
    return detail::MatScalar<E, true>(e);
}
}  // namespace per_sample

}  // namespace aether
