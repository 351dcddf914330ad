// aether/view.h -- typed non-owning views, the leaves of expressions.
//
// View<T, Extents, Layout, Volatile, ReadOnly> (view/View.h:150-424): a
// pointer, a mapping of (component..., sample) indices to element offsets and
// the device the memory lives on. It never owns memory. It is
//   * an expression leaf: eval<Is...>(i) reads component Is... of sample
//     i.global() (view/View.h:369-377);
//   * element access: v(c..., s) (view/View.h:234-246);
//   * a per-sample assignment target: v[i] = expr, v[i] += expr, v[i] -= expr,
//     v[i] = scalar (SampleRef, expr/Assign.h:251-346); v[i].get() reads the
//     sample into an Item;
//   * in host code, the destination of a whole-view assignment that the
//     engine runs as one generated kernel: `d.deviceView() = expr;`
//     (aether/eval.h; an addition of this engine).
// Array views use layout_stride (components at capacity-sized plane strides,
// samples at stride 1); make_view<T, Es...>(ptr, n) makes compact
// layout_right views. ReadOnly views load through the read-only data path in
// device code (view/View.h:281-286).
#pragma once

#include "aether/detail/std.h"

#include "aether/expression.h"
#include "aether/layout.h"
#include "aether/nodes.h"

namespace aether {

template <class T, class Extents, class Layout = layout_right, bool Volatile = false, bool ReadOnly = false>
class View;
template <class V>
class SampleRef;
template <class V>
class ConstSampleRef;
template <class T, std::size_t... Es>
class Item;
template <std::size_t W>
struct BundleIndex;
template <class V, std::size_t W>
class BundleRef;

#if AETHER_GB300_HOST_IR
// The engine's whole-view assignment (aether/eval.h): dst <op>= e as one kernel.
template <class V, class E>
void gb300_assign_view(const V& dst, const E& e, const char* op);
// The IR leaf of a device view (aether/eval.h).
template <class V>
Expr gb300_view_leaf(const V& v);
#endif

namespace detail {
template <class T, class X>
struct item_of;
template <class T, std::size_t... Es>
struct item_of<T, extents<Es...>> {
    using type = Item<T, Es...>;
};
}  // namespace detail

template <class T, class Extents, class Layout, bool Volatile, bool ReadOnly>
class View : public Expression<View<T, Extents, Layout, Volatile, ReadOnly>, std::remove_cv_t<T>> {
    static_assert(Extents::Rank >= 1, "a batched view has at least the sample mode");

public:
    using value_type = std::remove_cv_t<T>;
    using element_type = value_type;
    using extents_type = Extents;
    using layout_type = Layout;
    using mapping_type = typename Layout::template mapping<Extents>;
    using pointer = std::conditional_t<Volatile, volatile T*, T*>;
    using reference = std::conditional_t<ReadOnly, value_type, std::conditional_t<Volatile, volatile T&, T&>>;
    /** The component shape: every mode but the trailing sample mode. */
    using element_extents = typename element_extents_of<Extents>::type;
    static constexpr bool isLeaf = true;

    View() = default;
    AETHER_DEVICEANDHOST() constexpr View(T* data, const mapping_type& map, Device dev = Device())
        : data_(data), map_(map), dev_(dev) {}

    AETHER_DEVICEANDHOST() constexpr pointer data() const { return data_; }
    AETHER_DEVICEANDHOST() constexpr Device device() const { return dev_; }
    AETHER_DEVICEANDHOST() constexpr offset_t extent(std::size_t k) const { return map_.extents().extent(k); }
    AETHER_DEVICEANDHOST() static constexpr std::size_t rank() { return Extents::Rank; }
    AETHER_DEVICEANDHOST() constexpr offset_t samples() const { return extent(rank() - 1); }
    AETHER_DEVICEANDHOST() constexpr offset_t size() const {
        offset_t s = 1;
        for (std::size_t k = 0; k < Extents::Rank; ++k) s *= extent(k);
        return s;
    }
    AETHER_DEVICEANDHOST() constexpr const mapping_type& mapping() const { return map_; }

    /** Element (c..., s). */
    template <class... I>
    AETHER_DEVICEANDHOST() constexpr reference operator()(I... idx) const {
        static_assert(sizeof...(I) == Extents::Rank, "one index per component extent, then the sample");
        const offset_t off = map_(static_cast<offset_t>(idx)...);
        if constexpr (ReadOnly) {
#if defined(__CUDA_ARCH__)
            return __ldg(const_cast<const value_type*>(data_) + off);
#else
            return data_[off];
#endif
        } else {
            return data_[off];
        }
    }

    AETHER_DEVICEANDHOST() constexpr View<const T, Extents, Layout, Volatile, ReadOnly> as_const() const {
        return View<const T, Extents, Layout, Volatile, ReadOnly>(data_, map_, dev_);
    }
    AETHER_DEVICEANDHOST() constexpr View<T, Extents, Layout, true, ReadOnly> as_volatile() const {
        return View<T, Extents, Layout, true, ReadOnly>(data_, map_, dev_);
    }
    AETHER_DEVICEANDHOST() constexpr View<T, Extents, Layout, Volatile, true> as_readonly() const {
        return View<T, Extents, Layout, Volatile, true>(data_, map_, dev_);
    }

    /** Static component I of a vector view, as a scalar view (view/View.h:315-332). */
    template <std::size_t I>
    AETHER_DEVICEANDHOST() constexpr View<T, extents<dyn>, layout_stride> component() const {
        static_assert(Extents::Rank == 2, "component<I> of a batched vector view");
        static_assert(I < Extents::static_extent(0), "component index out of range");
        using Ext1 = extents<dyn>;
        const offset_t stride[1] = {map_.stride(1)};
        return View<T, Ext1, layout_stride>(data_ + map_.stride(0) * I,
                                             typename layout_stride::template mapping<Ext1>(Ext1(samples()), stride),
                                             dev_);
    }

    /** Component Is... of sample i.global(). */
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr value_type eval(const SampleIndex& i) const {
        return (*this)(Is..., i.global());
    }

    AETHER_DEVICEANDHOST() constexpr SampleRef<View> operator[](const SampleIndex& i) { return SampleRef<View>(*this, i); }
    AETHER_DEVICEANDHOST() constexpr ConstSampleRef<const View> operator[](const SampleIndex& i) const {
        return ConstSampleRef<const View>(*this, i);
    }
    /** W consecutive samples (aether/bundle.h). */
    template <std::size_t W>
    AETHER_DEVICEANDHOST() constexpr BundleRef<View, W> operator[](const BundleIndex<W>& bi);

#if AETHER_GB300_HOST_IR
    /** Host: every sample of this device view <- e, as one engine kernel. */
    template <class E, std::enable_if_t<aether_expression<E> || std::is_same<E, Expr>::value, int> = 0>
    View& operator=(const E& e) {
        gb300_assign_view(*this, e, "set");
        return *this;
    }
    template <class E, std::enable_if_t<aether_expression<E> || std::is_same<E, Expr>::value, int> = 0>
    View& operator+=(const E& e) {
        gb300_assign_view(*this, e, "add");
        return *this;
    }
    template <class E, std::enable_if_t<aether_expression<E> || std::is_same<E, Expr>::value, int> = 0>
    View& operator-=(const E& e) {
        gb300_assign_view(*this, e, "sub");
        return *this;
    }
    View& operator=(const View&) = default;
    View(const View&) = default;
    Expr gb300_ir() const { return gb300_view_leaf(*this); }
#endif

private:
    pointer data_ = nullptr;
    mapping_type map_{};
    Device dev_{};
};

namespace detail {

template <class X, std::size_t K, class V, std::size_t... D>
AETHER_DEVICEANDHOST() constexpr decltype(auto) eval_ref_(const V& v, const SampleIndex& i, std::index_sequence<D...>) {
    return v(unflat<X>(K, D)..., i.global());
}

template <int Op, std::size_t K, class V, class E>
AETHER_DEVICEANDHOST() constexpr void assign_one_(const V& v, const SampleIndex& i, const E& e) {
    using X = typename V::element_extents;
    using T = typename V::value_type;
    auto&& ref = eval_ref_<X, K>(v, i, std::make_index_sequence<X::Rank>{});
    const T val = static_cast<T>(evalFlat<K>(e, i));
    if constexpr (Op == 0) ref = val;
    if constexpr (Op == 1) ref = ref + val;
    if constexpr (Op == 2) ref = ref - val;
}

template <int Op, class V, class E, std::size_t... K>
AETHER_DEVICEANDHOST() constexpr void assign_sample_(const V& v, const SampleIndex& i, const E& e,
                                                     std::index_sequence<K...>) {
    (assign_one_<Op, K>(v, i, e), ...);
}

}  // namespace detail

/** The assignment target v[i] (expr/Assign.h:251-346): every component of
 *  sample i is written, in row-major component order. */
template <class V>
class SampleRef {
public:
    using element_type = typename V::element_type;
    using element_extents = typename V::element_extents;

    AETHER_DEVICEANDHOST() constexpr SampleRef(V& view, const SampleIndex& i) : view_(view), i_(i) {}

    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator=(const E& e) {
        return apply_<0>(e);
    }
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator+=(const E& e) {
        return apply_<1>(e);
    }
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator-=(const E& e) {
        return apply_<2>(e);
    }
    /** Every component of the sample <- s (expr/nodes/Constant.h:118-150). */
    template <class S, std::enable_if_t<!aether_expression<S>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator=(const S& s) {
        return apply_<0>(detail::Constant<element_type, element_extents>(static_cast<element_type>(s)));
    }
    template <class S, std::enable_if_t<!aether_expression<S>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator+=(const S& s) {
        return apply_<1>(detail::Constant<element_type, element_extents>(static_cast<element_type>(s)));
    }
    template <class S, std::enable_if_t<!aether_expression<S>, int> = 0>
    AETHER_DEVICEANDHOST() constexpr SampleRef& operator-=(const S& s) {
        return apply_<2>(detail::Constant<element_type, element_extents>(static_cast<element_type>(s)));
    }
    template <class... K>
    AETHER_DEVICEANDHOST() constexpr decltype(auto) at(K... k) const {
        return view_(k..., i_.global());
    }
    /** The sample as a register Item. */
    AETHER_DEVICEANDHOST() constexpr typename detail::item_of<element_type, element_extents>::type get() const;

private:
    template <int Op, class E>
    AETHER_DEVICEANDHOST() constexpr SampleRef& apply_(const E& e) {
        static_assert(std::is_same<typename E::element_extents, element_extents>::value,
                      "assignment: expression and view have different component extents");
        detail::assign_sample_<Op>(view_, i_, e, std::make_index_sequence<detail::size_of<element_extents>>{});
        return *this;
    }
    V& view_;
    SampleIndex i_;
};

/** The read-only sample v[i] of a const view. */
template <class V>
class ConstSampleRef {
public:
    using element_type = typename V::element_type;
    using element_extents = typename V::element_extents;
    AETHER_DEVICEANDHOST() constexpr ConstSampleRef(V& view, const SampleIndex& i) : view_(view), i_(i) {}
    template <std::size_t... Is>
    AETHER_DEVICEANDHOST() constexpr element_type eval() const {
        return view_.template eval<Is...>(i_);
    }
    template <class... K>
    AETHER_DEVICEANDHOST() constexpr decltype(auto) at(K... k) const {
        return view_(k..., i_.global());
    }
    AETHER_DEVICEANDHOST() constexpr typename detail::item_of<element_type, element_extents>::type get() const;

private:
    V& view_;
    SampleIndex i_;
};

/** A compact (layout_right) view of `ptr`: extents Es..., the dyn ones given
 *  (view/MakeView.h:48-100). */
template <class T, std::size_t... Es, class... D>
AETHER_DEVICEANDHOST() constexpr View<T, extents<Es...>> make_view(T* ptr, Device dev, D... dynVals) {
    using X = extents<Es...>;
    return View<T, X>(ptr, typename layout_right::template mapping<X>(X(dynVals...)), dev);
}
template <class T, std::size_t... Es, class... D,
          std::enable_if_t<(std::is_integral<D>::value && ...), int> = 0>
AETHER_DEVICEANDHOST() constexpr View<T, extents<Es...>> make_view(T* ptr, D... dynVals) {
    return make_view<T, Es...>(ptr, Device(kDLCUDA, 0), dynVals...);
}

/** A view of components Es... over `block_samples` block-local samples in
 *  shared memory (view/WorkView.h): compact, components first, indexed with
 *  SampleIndex::work(). One dynamic shared array can hold several, each
 *  carved at its own byte offset. */
template <class T, std::size_t... Es>
AETHER_DEVICEANDHOST() constexpr View<T, extents<Es..., dyn>> make_work_view(T* shared_ptr, offset_t block_samples) {
    using X = extents<Es..., dyn>;
    return View<T, X>(shared_ptr, typename layout_right::template mapping<X>(X(std::size_t(block_samples))),
                      Device(kDLCUDA));
}

}  // namespace aether
