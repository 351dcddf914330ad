// aether/bundle.h -- W samples per thread.
//
// BundleIndex<W> (index/BundleIndex.h:55-113): thread t of a 1D grid owns the
// W consecutive samples starting at W * t; mask(n) says which of them exist
// (the tail bundle of a launch sized by bundleLaunchConfig may straddle n).
// view[bi] (backend/cuda/bundle/Assign.h:148-268) assigns an expression to
// every existing sample of the bundle, `view[bi] += / -= expr` likewise, and
// view[bi].get() reads the bundle into registers (DeviceBundle,
// backend/cuda/DeviceBundle.h:71-157), whose lane(k) is an Item. Lanes past
// the view's sample count are neither read nor written.
#pragma once

#include "aether/detail/std.h"
#include "aether/item.h"

namespace aether {

template <std::size_t W>
struct BundleIndex {
    static_assert(W >= 1, "a bundle holds at least one sample");
    static constexpr std::size_t width = W;

    offset_t base_;

    AETHER_DEVICEANDHOST() static constexpr BundleIndex make(offset_t threadIdxx, offset_t blockIdxx, offset_t blockDimx) {
        return BundleIndex{static_cast<offset_t>(W) * (blockIdxx * blockDimx + threadIdxx)};
    }
    AETHER_DEVICEANDHOST() static constexpr BundleIndex make(std::size_t i) {
        return BundleIndex{static_cast<offset_t>(W * i)};
    }
    AETHER_DEVICEANDHOST() constexpr offset_t base() const { return base_; }
    /** Sample k of the bundle (work() is the lane). */
    AETHER_DEVICEANDHOST() constexpr SampleIndex lane(std::size_t k) const {
        return SampleIndex{base_ + static_cast<offset_t>(k), static_cast<offset_t>(k)};
    }

    struct Mask {
        offset_t active_;
        AETHER_DEVICEANDHOST() constexpr bool lane(std::size_t k) const { return static_cast<offset_t>(k) < active_; }
        AETHER_DEVICEANDHOST() constexpr bool full() const { return active_ == static_cast<offset_t>(W); }
    };
    /** The lanes below n. */
    AETHER_DEVICEANDHOST() constexpr Mask mask(offset_t n) const {
        const offset_t rem = base_ < n ? n - base_ : offset_t(0);
        return Mask{rem < static_cast<offset_t>(W) ? rem : static_cast<offset_t>(W)};
    }
};

/** W samples of a T-valued element of extents Es... in registers. */
template <class T, std::size_t W, std::size_t... Es>
struct DeviceBundle {
    using ItemT = Item<T, Es...>;
    static constexpr std::size_t width = W;
    ItemT lanes[W];
    AETHER_DEVICEANDHOST() constexpr ItemT& lane(std::size_t k) { return lanes[k]; }
    AETHER_DEVICEANDHOST() constexpr const ItemT& lane(std::size_t k) const { return lanes[k]; }
};

namespace detail {
template <class T, std::size_t W, class X>
struct bundle_of;
template <class T, std::size_t W, std::size_t... Es>
struct bundle_of<T, W, extents<Es...>> {
    using type = DeviceBundle<T, W, Es...>;
};
}  // namespace detail

/** The assignment target view[bi]. */
template <class V, std::size_t W>
class BundleRef {
public:
    using element_type = typename V::element_type;
    using element_extents = typename V::element_extents;
    using BundleT = typename detail::bundle_of<element_type, W, element_extents>::type;

    AETHER_DEVICEANDHOST() constexpr BundleRef(V& view, const BundleIndex<W>& bi) : view_(view), bi_(bi) {}

    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() BundleRef& operator=(const E& e) {
        return apply_<0>(e);
    }
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() BundleRef& operator+=(const E& e) {
        return apply_<1>(e);
    }
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() BundleRef& operator-=(const E& e) {
        return apply_<2>(e);
    }
    template <class S, std::enable_if_t<!aether_expression<S>, int> = 0>
    AETHER_DEVICEANDHOST() BundleRef& operator=(const S& s) {
        return apply_<0>(detail::Constant<element_type, element_extents>(static_cast<element_type>(s)));
    }
    /** The existing lanes in registers (lanes past the end stay zero). */
    AETHER_DEVICEANDHOST() BundleT get() const {
        BundleT b{};
        const auto m = bi_.mask(view_.samples());
        AETHER_UNROLL
        for (std::size_t k = 0; k < W; ++k)
            if (m.lane(k))
                b.lanes[k] = detail::read_sample<typename BundleT::ItemT>(
                    view_, bi_.lane(k), std::make_index_sequence<detail::size_of<element_extents>>{});
        return b;
    }

private:
    template <int Op, class E>
    AETHER_DEVICEANDHOST() BundleRef& apply_(const E& e) {
        static_assert(std::is_same<typename E::element_extents, element_extents>::value,
                      "assignment: expression and view have different component extents");
        const auto m = bi_.mask(view_.samples());
        if (m.full()) {
            AETHER_UNROLL
            for (std::size_t k = 0; k < W; ++k)
                detail::assign_sample_<Op>(view_, bi_.lane(k), e,
                                           std::make_index_sequence<detail::size_of<element_extents>>{});
        } else {
            for (std::size_t k = 0; k < W; ++k)
                if (m.lane(k))
                    detail::assign_sample_<Op>(view_, bi_.lane(k), e,
                                               std::make_index_sequence<detail::size_of<element_extents>>{});
        }
        return *this;
    }
    V& view_;
    BundleIndex<W> bi_;
};

/** view[bi] (view/View.h:408-418). */
template <class T, class X, class L, bool Vo, bool RO>
template <std::size_t W>
AETHER_DEVICEANDHOST() constexpr BundleRef<View<T, X, L, Vo, RO>, W> View<T, X, L, Vo, RO>::operator[](
    const BundleIndex<W>& bi) {
    return BundleRef<View<T, X, L, Vo, RO>, W>(*this, bi);
}

}  // namespace aether
