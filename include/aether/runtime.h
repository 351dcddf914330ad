// aether/runtime.h -- the runtime-typed strided evaluator.
//
// aether::RuntimeView (view/RuntimeView.h:71-150): an untyped descriptor of
// up to six modes with element strides -- the C-ABI's AetherRuntimeView plus
// the device its memory lives on, its element count, and the checked
// promotion as<StaticViewT>() back onto a typed view. fromView() describes a
// typed view (components first, samples last, plane pitch = capacity).
// aether::eval::runtimeEval (eval/Runtime.h:228-300) validates shapes and
// dtypes, throws aether::Error before any launch, and runs one kernel.
#pragma once

#include <cstdint>
#include <string>
#include <type_traits>
#include <utility>

#include "aether/array.h"
#include "aether_gb300.h"

namespace aether {

namespace detail {

/** DLPack's (code, bits) of a view's element type; code 255 for none. */
template <class T>
constexpr std::pair<uint8_t, uint8_t> dlpack_dtype() {
    using U = std::remove_cv_t<T>;
    if (std::is_same<U, bool>::value) return {6, 8};
    if (std::is_floating_point<U>::value) return {2, uint8_t(sizeof(U) * 8)};
    if (std::is_integral<U>::value) return {uint8_t(std::is_signed<U>::value ? 0 : 1), uint8_t(sizeof(U) * 8)};
    return {255, 0};
}

template <class V>
struct view_parts;
template <class T, class X, class L, bool Vo, bool RO>
struct view_parts<View<T, X, L, Vo, RO>> {
    using element = T;
    using ext = X;
    using layout = L;
};

// The mode of the j-th dynamic extent of extents<Es...>.
template <std::size_t... Es>
constexpr std::size_t dyn_mode(std::size_t j) {
    constexpr std::size_t es[] = {Es..., 0};
    for (std::size_t k = 0; k < sizeof...(Es); ++k)
        if (es[k] == dyn && j-- == 0) return k;
    return 0;
}
template <std::size_t... Es, std::size_t... Ds>
extents<Es...> extents_from(const int64_t* e, extents<Es...>*, std::index_sequence<Ds...>) {
    return extents<Es...>(std::size_t(e[dyn_mode<Es...>(Ds)])...);
}
template <class X>
X extents_from(const int64_t* e) {
    if constexpr (X::RankDynamic == 0) {
        (void)e;
        return X();
    } else {
        return extents_from(e, static_cast<X*>(nullptr), std::make_index_sequence<X::RankDynamic>());
    }
}

}  // namespace detail

/** The reference's RuntimeView: the C-ABI descriptor (passed to
 *  aether_runtime_eval as is) plus the device it lives on. */
struct RuntimeView : AetherRuntimeView {
    Device device{};

    /** Element count: the product of the extents (1 for rank 0). */
    int64_t size() const {
        int64_t n = 1;
        for (int k = 0; k < rank; ++k) n *= extents[k];
        return n;
    }

    /** Checked promotion onto a typed view, zero copy (view/RuntimeView.h:
     *  113-150): throws aether::Error unless the element type, the rank,
     *  every static extent, the strides (the compact row-major ones for a
     *  layout_right view; any that the view's 32-bit offsets reach for a
     *  layout_stride view) and the device (host, CUDA or page-locked host
     *  memory) all match. */
    template <class StaticViewT>
    StaticViewT as() const;
};

template <class StaticViewT>
StaticViewT RuntimeView::as() const {
    using P = detail::view_parts<StaticViewT>;
    using X = typename P::ext;
    using T = typename P::element;
    const auto fail = [](const std::string& why) {
        throw Error::memory("aether::RuntimeView::as", "RuntimeView", 0, why);
    };
    constexpr auto dt = detail::dlpack_dtype<T>();
    static_assert(dt.first != 255, "as<>: a view of an arithmetic element type");
    if (dtype_code != dt.first || dtype_bits != dt.second || dtype_lanes != 1) fail("dtype mismatch");
    if (rank != int(X::Rank))
        fail("rank " + std::to_string(rank) + " != the view's " + std::to_string(X::Rank));
    if (!(device.type == kDLCPU || device.type == kDLCUDA || device.type == kDLCUDAHost))
        fail("unknown/unsupported device kind (type=" + std::to_string(device.type) + ")");
    uint64_t span = 1;
    bool empty = false;
    for (std::size_t k = 0; k < X::Rank; ++k) {
        const int64_t e = extents[k], st = strides[k];
        if (X::static_extent(k) != dyn && uint64_t(e) != X::static_extent(k))
            fail("extent " + std::to_string(k) + " is " + std::to_string(e) + ", the view's is " +
                 std::to_string(X::static_extent(k)));
        if (e < 0 || st < 0 || e > int64_t(UINT32_MAX) || st > int64_t(UINT32_MAX))
            fail("extent or stride " + std::to_string(k) + " outside the view's 32-bit offsets");
        empty |= e == 0;
    }
    for (std::size_t k = 0; k < X::Rank && !empty; ++k) {
        span += uint64_t(extents[k] - 1) * uint64_t(strides[k]);
        if (span > uint64_t(UINT32_MAX) + 1u) fail("required span exceeds the view's 32-bit offsets");
    }
    const X ext = detail::extents_from<X>(extents);
    using L = typename P::layout;
    if constexpr (std::is_same<L, layout_right>::value) {
        const typename layout_right::template mapping<X> m(ext);
        for (std::size_t k = 0; k < X::Rank; ++k)
            if (extents[k] > 1 && uint64_t(strides[k]) != uint64_t(m.stride(k)))
                fail("strides are not row-major (layout_right)");
        return StaticViewT(static_cast<T*>(data), m, device);
    } else {
        offset_t st[X::Rank ? X::Rank : 1] = {};
        for (std::size_t k = 0; k < X::Rank; ++k) st[k] = offset_t(strides[k]);
        return StaticViewT(static_cast<T*>(data), typename L::template mapping<X>(ext, st), device);
    }
}

/** The descriptor of a typed view: its modes (components..., samples) with
 *  the view's own element strides and device (view/RuntimeView.h:71-110). */
template <class T, class X, class L, bool Vo, bool RO>
RuntimeView fromView(const View<T, X, L, Vo, RO>& v) {
    static_assert(X::Rank <= AETHER_RT_RANK_CAP, "runtime views have at most six modes");
    using U = std::remove_cv_t<T>;
    constexpr auto dt = detail::dlpack_dtype<U>();
    static_assert(dt.first != 255, "fromView: a view of an arithmetic element type");
    RuntimeView r{};
    r.data = const_cast<U*>(v.data());
    r.dtype_code = dt.first;
    r.dtype_bits = dt.second;
    r.dtype_lanes = 1;
    r.rank = int32_t(X::Rank);
    for (std::size_t k = 0; k < X::Rank; ++k) {
        r.extents[k] = int64_t(v.extent(k));
        r.strides[k] = int64_t(v.mapping().stride(k));
    }
    r.device = v.device();
    return r;
}

namespace eval {

enum class RuntimeOp : int {
    Assign = AETHER_RT_ASSIGN,
    Add = AETHER_RT_ADD,
    Sub = AETHER_RT_SUB,
    Scale = AETHER_RT_SCALE,
    AddScaled = AETHER_RT_ADD_SCALED,
    SubScaled = AETHER_RT_SUB_SCALED,
};

/** out = op(a, b, scalar) elementwise; `b` is read by Add, Sub, AddScaled and
 *  SubScaled only (pass RuntimeView{} otherwise). */
inline void runtimeEval(RuntimeOp op, const RuntimeView& a, const RuntimeView& b, const RuntimeView& out,
                        double scalar = 0.0, Stream s = nullptr) {
    if (aether_runtime_eval(int(op), &a, &b, &out, scalar, s) != AETHER_OK) throw Error(aether::detail::last_error());
}

}  // namespace eval
}  // namespace aether
