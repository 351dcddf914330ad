// aether/item.h -- register-resident tensors and the consumer aliases.
//
// Item<T, Es...> (view/Item.h:73): a small tensor of static extents held in
// registers. It is an expression leaf whose value does not depend on the
// sample, so `view[i] = a + item * b` combines per-sample data with a
// per-thread value. Built from an expression it evaluates that expression at
// sample 0 (expr/Assign.h:420-445): in per-sample code, `Vec3d x = v[i].get();`
// reads sample i of a view, and `Vec3d y = x.cross(z);` evaluates on items.
// The aliases Vec<T,N>, Mat<T,R,C>, Vec3d, Mat33d, ScalarView<T>, VecView<T,N>
// and MatView<T,R,C> are the reference's (aether/aether.h:234-260).
#pragma once

#include "aether/detail/std.h"

#include "aether/view.h"

namespace aether {

template <class T, std::size_t... Es>
class Item : public Expression<Item<T, Es...>, T> {
    static_assert(((Es != dyn) && ...), "Item: every extent is static");

public:
    using element_type = T;
    using element_extents = extents<Es...>;
    static constexpr bool isLeaf = true;
    static constexpr std::size_t Rank = sizeof...(Es);
    static constexpr std::size_t Size = (Es * ... * std::size_t{1});

    Item() = default;

    /** The value of `e` at sample 0. */
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr Item(const E& e) : data_{} {
        assign_(e);
    }
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr Item& operator=(const E& e) {
        assign_(e);
        return *this;
    }
    /** Item<T, Es...>{v0, v1, ...}: exactly Size values, row-major. */
    template <class... Vs, std::enable_if_t<sizeof...(Vs) == Size && (Size >= 2) &&
                                                (std::is_arithmetic<Vs>::value && ...),
                                            int> = 0>
    AETHER_DEVICEANDHOST() constexpr Item(Vs... vs) : data_{static_cast<T>(vs)...} {}
    /** A one-component item from its value. */
    template <class V, std::size_t S = Size,
              std::enable_if_t<S == 1 && std::is_arithmetic<V>::value, int> = 0>
    AETHER_DEVICEANDHOST() constexpr Item(V v) : data_{static_cast<T>(v)} {}

    /** The identity matrix (square rank-2 items). */
    AETHER_DEVICEANDHOST() static constexpr Item identity() {
        static_assert(Rank == 2, "identity of a matrix item");
        constexpr std::size_t n = element_extents::static_extent(0);
        static_assert(n == element_extents::static_extent(1), "identity of a square matrix");
        Item m{};
        for (std::size_t k = 0; k < Size; ++k) m.data_[k] = (k % (n + 1) == 0) ? T(1) : T(0);
        return m;
    }
    // The reference's factory spellings (view/Item.h:195-225).
    AETHER_DEVICEANDHOST() static constexpr Item Identity() { return identity(); }
    AETHER_DEVICEANDHOST() static constexpr Item filled(const T& v) {
        Item m{};
        for (std::size_t k = 0; k < Size; ++k) m.data_[k] = v;
        return m;
    }
    AETHER_DEVICEANDHOST() static constexpr Item Zeros() { return filled(T(0)); }
    AETHER_DEVICEANDHOST() static constexpr Item Ones() { return filled(T(1)); }
    AETHER_DEVICEANDHOST() static constexpr std::size_t size() { return Size; }

    template <class... I>
    AETHER_DEVICEANDHOST() constexpr T& operator()(I... idx) {
        return data_[flat_(static_cast<std::size_t>(idx)...)];
    }
    template <class... I>
    AETHER_DEVICEANDHOST() constexpr const T& operator()(I... idx) const {
        return data_[flat_(static_cast<std::size_t>(idx)...)];
    }
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr T& get() {
        return data_[detail::flat_index<element_extents, Is...>()];
    }
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr const T& get() const {
        return data_[detail::flat_index<element_extents, Is...>()];
    }
    AETHER_DEVICEANDHOST() constexpr T* data() { return data_; }
    AETHER_DEVICEANDHOST() constexpr const T* data() const { return data_; }

    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr T eval(const SampleIndex&) const {
        return data_[detail::flat_index<element_extents, Is...>()];
    }

#if AETHER_GB300_HOST_IR
    /** A per-launch constant: Size runtime scalars stacked into the shape. */
    Expr gb300_ir() const {
        if (Size == 1 && Rank == 0) return Expr(ir::scalar(double(data_[0])));
        std::vector<ir::NodeP> k;
        for (std::size_t c = 0; c < Size; ++c) k.push_back(ir::scalar(double(data_[c])));
        Expr v(ir::op("stack", std::move(k), {int(Size)}));
        if (Rank == 2) v = v.reshape(ir::shape_of(element_extents{}));
        return v;
    }
#endif

private:
    template <class... I>
    AETHER_DEVICEANDHOST() static constexpr std::size_t flat_(I... idx) {
        static_assert(sizeof...(I) == Rank || (Rank == 0 && sizeof...(I) <= 1), "one index per extent");
        std::size_t k = 0, d = 0;
        ((k = k * element_extents::static_extent(d++) + idx), ...);
        return Rank == 0 ? 0 : k;
    }
    template <class E, std::size_t... K>
    AETHER_DEVICEANDHOST() constexpr void assign_seq_(const E& e, const SampleIndex& i0, std::index_sequence<K...>) {
        ((data_[K] = static_cast<T>(detail::evalFlat<K>(e, i0))), ...);
    }
    template <class E>
    AETHER_DEVICEANDHOST() constexpr void assign_(const E& e) {
        static_assert(std::is_same<typename E::element_extents, element_extents>::value,
                      "Item(expr): component extents differ");
        assign_seq_(e, SampleIndex::make(std::size_t(0)), std::make_index_sequence<Size>{});
    }

    T data_[Size ? Size : 1]{};   // a default-constructed Item is zero (view/Item.h:275)
};

namespace detail {
template <class It, class V, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr It read_sample(const V& v, const SampleIndex& i, std::index_sequence<K...>) {
    It r{};
    ((r.data()[K] = evalFlat<K>(v, i)), ...);
    return r;
}
}  // namespace detail

template <class V>
AETHER_DEVICEANDHOST() constexpr typename detail::item_of<typename SampleRef<V>::element_type,
                                                       typename SampleRef<V>::element_extents>::type
SampleRef<V>::get() const {
    using It = typename detail::item_of<element_type, element_extents>::type;
    return detail::read_sample<It>(view_, i_, std::make_index_sequence<detail::size_of<element_extents>>{});
}
template <class V>
AETHER_DEVICEANDHOST() constexpr typename detail::item_of<typename ConstSampleRef<V>::element_type,
                                                       typename ConstSampleRef<V>::element_extents>::type
ConstSampleRef<V>::get() const {
    using It = typename detail::item_of<element_type, element_extents>::type;
    return detail::read_sample<It>(view_, i_, std::make_index_sequence<detail::size_of<element_extents>>{});
}

// -- consumer aliases (aether/aether.h:234-260) -------------------------------
template <class T, std::size_t N>
using Vec = Item<T, N>;
template <class T, std::size_t R, std::size_t C>
using Mat = Item<T, R, C>;
using Vec3d = Vec<double, 3>;
using Vec4d = Vec<double, 4>;
using Vec6d = Vec<double, 6>;
using Mat33d = Mat<double, 3, 3>;
using Mat36d = Mat<double, 3, 6>;

template <class T>
using ScalarView = View<T, extents<dyn>>;
template <class T, std::size_t N>
using VecView = View<T, extents<N, dyn>>;
template <class T, std::size_t R, std::size_t C>
using MatView = View<T, extents<R, C, dyn>>;
using Vec3dView = VecView<double, 3>;
using Mat33dView = MatView<double, 3, 3>;

/** K slots of D components in one Item (view/Tile.h): a plain Item<T, D*K>;
 *  slot<s, D>(tile) is its s-th slot, a segment of the item. */
template <class T, std::size_t D, std::size_t K>
using Tile = Item<T, D * K>;
template <std::size_t s, std::size_t D, class T, std::size_t N>
AETHER_DEVICEANDHOST() constexpr auto slot(const Item<T, N>& tile) {
    static_assert((s + 1) * D <= N, "slot<s, D>(): slot index out of range");
    return tile.template segment<s * D, D>();
}

}  // namespace aether
