// aether/layout.h -- extents, layouts, devices and the 32-bit sample index.
//
// The consumer types of the reference's layout and index layers:
//   extents<Es...> with the dynamic marker `dyn` (layout/Extents.h:30-146):
//     static component extents, then the dynamic sample extent;
//   layout_right and layout_stride mappings (layout/Layout.h:39-199): the
//     element offset of a multi-index, row-major or through explicit strides;
//   offset_t and SampleIndex (index/Offset.h:73-91, index/SampleIndex.h:36-99):
//     device address arithmetic in 32 bits, one sample per thread;
//   Device (device/Device.h:24-83): where a view's memory lives (DLPack codes).
// Every member is usable in device code (AETHER_DEVICEHOST) and in host code.
#pragma once

#include "aether/detail/std.h"

#include "aether/macros.h"

namespace aether {

/** Device address arithmetic is 32-bit (index/Offset.h:73-91); views are
 *  refused on the host when their span does not fit. */
using offset_t = std::uint32_t;

/** The dynamic extent marker (layout/Extents.h:30). */
inline constexpr std::size_t dyn = static_cast<std::size_t>(-1);

/** DLPack device codes of the memory a view points into. */
enum DeviceType : int { kDLCPU = 1, kDLCUDA = 2, kDLCUDAHost = 3 };

struct Device {
    int type = kDLCPU;
    int id = 0;
    constexpr Device() = default;
    AETHER_DEVICEANDHOST() constexpr explicit Device(int t, int i = 0) : type(t), id(i) {}
    AETHER_DEVICEANDHOST() constexpr bool operator==(const Device& o) const { return type == o.type && id == o.id; }
    AETHER_DEVICEANDHOST() constexpr bool operator!=(const Device& o) const { return !(*this == o); }
};

namespace detail {

template <std::size_t... Es>
struct count_dyn : std::integral_constant<std::size_t, ((Es == dyn ? 1 : 0) + ... + 0)> {};

// Compile-time pick of the k-th value of a pack (no array in device memory).
template <std::size_t... Es>
AETHER_DEVICEANDHOST() constexpr std::size_t pick(std::size_t k) {
    std::size_t r = 0, j = 0;
    ((r = (j++ == k ? Es : r)), ...);
    return r;
}

// Position among the dynamic extents of extent k.
template <std::size_t... Es>
AETHER_DEVICEANDHOST() constexpr std::size_t dyn_slot(std::size_t k) {
    std::size_t slot = 0, j = 0;
    ((slot += (j++ < k && Es == dyn) ? 1 : 0), ...);
    return slot;
}

}  // namespace detail

/** Static extents Es...; `dyn` entries are given at construction. */
template <std::size_t... Es>
class extents {
public:
    static constexpr std::size_t Rank = sizeof...(Es);
    static constexpr std::size_t RankDynamic = detail::count_dyn<Es...>::value;

    AETHER_DEVICEANDHOST() static constexpr std::size_t rank() { return Rank; }
    AETHER_DEVICEANDHOST() static constexpr std::size_t rank_dynamic() { return RankDynamic; }
    /** Extent k as spelled (dyn for a dynamic one). */
    AETHER_DEVICEANDHOST() static constexpr std::size_t static_extent(std::size_t k) { return detail::pick<Es...>(k); }

    AETHER_DEVICEANDHOST() constexpr extents() : dyn_{} {}
    template <class... D, class = std::enable_if_t<sizeof...(D) == RankDynamic && (RankDynamic > 0) &&
                                                   (std::is_convertible<D, std::size_t>::value && ...)>>
    AETHER_DEVICEANDHOST() constexpr explicit extents(D... d) : dyn_{static_cast<std::size_t>(d)...} {}

    AETHER_DEVICEANDHOST() constexpr std::size_t extentWide(std::size_t k) const {
        return static_extent(k) == dyn ? dyn_[detail::dyn_slot<Es...>(k)] : static_extent(k);
    }
    AETHER_DEVICEANDHOST() constexpr offset_t extent(std::size_t k) const { return static_cast<offset_t>(extentWide(k)); }

private:
    std::size_t dyn_[RankDynamic ? RankDynamic : 1];
};

/** The component extents of a batched extents<Es..., dyn>: everything but
 *  the trailing sample mode. */
template <class Ext, class Seq = std::make_index_sequence<(Ext::Rank > 0 ? Ext::Rank - 1 : 0)>>
struct element_extents_of;
template <class Ext, std::size_t... Is>
struct element_extents_of<Ext, std::index_sequence<Is...>> {
    using type = extents<Ext::static_extent(Is)...>;
};

/** Product of an all-static extents (the component count of an element). */
template <class Ext>
struct static_size;
template <std::size_t... Es>
struct static_size<extents<Es...>> : std::integral_constant<std::size_t, (Es * ... * std::size_t{1})> {};

/** Row-major mapping: the last index varies fastest (layout/Layout.h:39-98). */
struct layout_right {
    template <class Ext>
    class mapping {
    public:
        using extents_type = Ext;
        constexpr mapping() = default;
        AETHER_DEVICEANDHOST() constexpr explicit mapping(const Ext& e) : ext_(e) {}
        AETHER_DEVICEANDHOST() constexpr const Ext& extents() const { return ext_; }
        AETHER_DEVICEANDHOST() constexpr offset_t stride(std::size_t k) const {
            offset_t s = 1;
            for (std::size_t j = k + 1; j < Ext::Rank; ++j) s *= ext_.extent(j);
            return s;
        }
        template <class... I>
        AETHER_DEVICEANDHOST() constexpr offset_t operator()(I... idx) const {
            static_assert(sizeof...(I) == Ext::Rank, "one index per extent");
            offset_t off = 0;
            std::size_t k = 0;
            ((off = off * ext_.extent(k++) + static_cast<offset_t>(idx)), ...);
            return off;
        }
        AETHER_DEVICEANDHOST() constexpr std::size_t required_span_size() const {
            std::size_t s = 1;
            for (std::size_t k = 0; k < Ext::Rank; ++k) s *= ext_.extentWide(k);
            return s;
        }

    private:
        Ext ext_{};
    };
};

/** Mapping through explicit element strides (layout/Layout.h:100-199). An
 *  Array's views use it: components at capacity-sized plane strides, the
 *  sample mode at stride 1. */
struct layout_stride {
    template <class Ext>
    class mapping {
    public:
        using extents_type = Ext;
        AETHER_DEVICEANDHOST() constexpr mapping() : ext_(), s_{} {}
        template <class S>
        AETHER_DEVICEANDHOST() constexpr mapping(const Ext& e, const S& strides) : ext_(e), s_{} {
            for (std::size_t k = 0; k < Ext::Rank; ++k) s_[k] = static_cast<offset_t>(strides[k]);
        }
        /** From another mapping of the same extents (e.g. layout_right's). */
        template <class M, class = decltype(std::declval<const M&>().stride(0))>
        AETHER_DEVICEANDHOST() constexpr explicit mapping(const M& m) : ext_(m.extents()), s_{} {
            for (std::size_t k = 0; k < Ext::Rank; ++k) s_[k] = m.stride(k);
        }
        AETHER_DEVICEANDHOST() constexpr const Ext& extents() const { return ext_; }
        AETHER_DEVICEANDHOST() constexpr offset_t stride(std::size_t k) const { return s_[k]; }
        template <class... I>
        AETHER_DEVICEANDHOST() constexpr offset_t operator()(I... idx) const {
            static_assert(sizeof...(I) == Ext::Rank, "one index per extent");
            offset_t off = 0;
            std::size_t k = 0;
            ((off += static_cast<offset_t>(idx) * s_[k++]), ...);
            return off;
        }
        AETHER_DEVICEANDHOST() constexpr std::size_t required_span_size() const {
            std::size_t s = 1;
            for (std::size_t k = 0; k < Ext::Rank; ++k) {
                if (ext_.extentWide(k) == 0) return 0;
                s += (ext_.extentWide(k) - 1) * static_cast<std::size_t>(s_[k]);
            }
            return s;
        }

    private:
        Ext ext_;
        offset_t s_[Ext::Rank ? Ext::Rank : 1];
    };
};

/** The thread -> sample mapping of one-sample-per-thread kernels
 *  (index/SampleIndex.h:46-71): global() is the grid-wide sample,
 *  work() the block-local slot. */
struct SampleIndex {
    AETHER_DEVICEANDHOST() static constexpr SampleIndex make(offset_t threadIdxx, offset_t blockIdxx, offset_t blockDimx) {
        return SampleIndex{blockIdxx * blockDimx + threadIdxx, threadIdxx};
    }
    AETHER_DEVICEANDHOST() static constexpr SampleIndex make(std::size_t index) {
        return SampleIndex{static_cast<offset_t>(index), static_cast<offset_t>(index)};
    }
    AETHER_DEVICEANDHOST() constexpr offset_t global() const { return globalIdx_; }
    AETHER_DEVICEANDHOST() constexpr offset_t work() const { return workIdx_; }

    offset_t globalIdx_;
    offset_t workIdx_;
};

}  // namespace aether
