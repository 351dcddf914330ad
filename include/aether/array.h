// aether/array.h -- owning SoA arrays.
//
// Array<T, Es...> (array/Array.h:82-364): samples() samples of a T-valued
// tensor of static extents Es..., stored plane by plane: component c of
// sample s at c * capacity() + s, capacity() a multiple of 32 samples
// (kCapacityAlignment, array/Array.h:80 and :288-304). An Array owns a pinned
// host copy and a device copy (chunk/Chunk.h:111-260), allocated through the
// C-ABI; upload() and download() move the filled samples of every plane,
// blocking or stream-ordered (array/Array.h:250-268).
//
//   hostView()/deviceView()     View<T, extents<Es..., dyn>, layout_stride>
//                               over the filled samples (plane stride =
//                               capacity); const arrays give ConstViewT;
//   hostPacked()/devicePacked() compact layout_right views, only when the
//                               array is exactly full (capacity == samples);
//   hostSpare()/deviceSpare()   the unfilled tail [samples, capacity);
//   reserve/resize/push_back/clear/commit  growth with the capacity rule
//                               kept: reallocation copies every plane's
//                               filled samples, host and device.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>

#include "aether/item.h"
#include "aether_gb300.h"

namespace aether {

/** A raw cudaStream_t; nullptr is the legacy default stream. */
using Stream = void*;

/** Samples rounded up to the 32-sample capacity quantum. */
inline constexpr std::size_t kCapacityAlignment = 32;
inline std::size_t quantized_capacity(std::size_t n) {
    return (n + kCapacityAlignment - 1) / kCapacityAlignment * kCapacityAlignment;
}

namespace detail {

template <class T>
constexpr const char* dtype_name() {
    static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value,
                  "aether arrays hold double or float");
    return std::is_same<T, double>::value ? "f64" : "f32";
}

inline std::string last_error() {
    const char* m = aether_last_error();
    return m ? m : "unknown error";
}

/** One chunk allocated through the C-ABI (chunk/Chunk.h:111-260). */
class Chunk {
public:
    Chunk() = default;
    Chunk(int kind, std::size_t bytes, const char* where) : kind_(kind), bytes_(bytes) {
        if (bytes == 0) return;
        void* h = nullptr;
        void* p = nullptr;
        if (aether_chunk_alloc(kind, 0, bytes, nullptr, &h, &p) != AETHER_OK)
            throw Error::memory("Chunk::allocate", where, bytes, last_error());
        handle_.reset(h);
        ptr_ = p;
    }
    void* get() const { return ptr_; }
    std::size_t bytes() const { return bytes_; }
    int kind() const { return kind_; }

private:
    struct Release {
        void operator()(void* h) const {
            if (h) aether_chunk_release(h);
        }
    };
    std::unique_ptr<void, Release> handle_;
    void* ptr_ = nullptr;
    int kind_ = AETHER_MEM_CPU;
    std::size_t bytes_ = 0;
};

inline void copy(void* dst, int dst_kind, const void* src, int src_kind, std::size_t bytes, Stream s, const char* op) {
    if (bytes == 0) return;
    if (aether_copy(dst_kind, 0, dst, src_kind, 0, src, bytes, s) != AETHER_OK)
        throw Error::memory(op, dst_kind == AETHER_MEM_DEVICE ? "device 0" : "host", bytes, last_error());
}

inline void sync(Stream s) {
    if (aether_stream_sync(0, s) != AETHER_OK) throw Error("stream_sync failed (" + last_error() + ")");
}

/** Row-major strides of extents<Es..., dyn> with the sample mode at stride 1
 *  and planes `pitch` samples apart. */
template <std::size_t... Es>
struct PlaneStrides {
    static constexpr std::size_t rank = sizeof...(Es) + 1;
    offset_t s[rank];
    explicit PlaneStrides(std::size_t pitch) : s{} {
        const std::size_t ext[] = {Es..., 1};
        std::size_t st = pitch;
        s[rank - 1] = 1;
        for (std::size_t k = rank - 1; k-- > 0;) {
            s[k] = static_cast<offset_t>(st);
            st *= ext[k];
        }
    }
    AETHER_DEVICEANDHOST() offset_t operator[](std::size_t k) const { return s[k]; }
};

/** The plane-layout view of `n` samples at `ptr`, planes `pitch` apart. */
template <class T, std::size_t... Es>
View<T, extents<Es..., dyn>, layout_stride> plane_view(T* ptr, std::size_t pitch, std::size_t n,
                                                      Device dev = Device(kDLCUDA, 0)) {
    using X = extents<Es..., dyn>;
    return View<T, X, layout_stride>(ptr, typename layout_stride::template mapping<X>(X(n), PlaneStrides<Es...>(pitch)),
                                     dev);
}

}  // namespace detail

template <class T, std::size_t... Es>
class Array {
public:
    using element_type = T;
    using Extents = extents<Es..., dyn>;
    using ViewT = View<T, Extents, layout_stride>;
    using ConstViewT = View<const T, Extents, layout_stride>;
    using PackedViewT = View<T, Extents, layout_right>;
    using ConstPackedViewT = View<const T, Extents, layout_right>;
    using ItemT = Item<T, Es...>;
    static constexpr std::size_t components = (Es * ... * std::size_t{1});

    explicit Array(std::size_t n_samples)
        : n_(n_samples), cap_(quantized_capacity(n_samples)),
          host_(AETHER_MEM_PINNED, bytes_(cap_), "host (pinned)"), dev_(AETHER_MEM_DEVICE, bytes_(cap_), "device 0") {
        check_span_(cap_);
    }

    std::size_t samples() const { return n_; }
    std::size_t size() const { return components * n_; }
    std::size_t capacity() const { return cap_; }
    std::size_t bytes() const { return bytes_(cap_); }

    /** Room for at least n samples (capacity rounded up to 32). */
    void reserve(std::size_t n) {
        if (n <= cap_) return;
        reallocate_(quantized_capacity(n));
    }
    void resize(std::size_t n) {
        if (n > cap_) reserve(n);
        n_ = n;
    }
    /** Append one sample on the host (upload() to publish it). */
    void push_back(const ItemT& item) {
        if (n_ == cap_) reserve(cap_ == 0 ? kCapacityAlignment : cap_ * 2);
        T* base = static_cast<T*>(host_.get());
        for (std::size_t c = 0; c < components; ++c) base[c * cap_ + n_] = item.data()[c];
        ++n_;
    }
    void clear() { n_ = 0; }
    /** Mark `count` samples written into the spare tail as filled. */
    void commit(std::size_t count) {
        if (count > cap_ - n_)
            throw Error::memory("Array::commit", "host", bytes_(count),
                                "count=" + std::to_string(count) + " exceeds spare capacity (" +
                                    std::to_string(cap_ - n_) + " = capacity()=" + std::to_string(cap_) +
                                    " - samples()=" + std::to_string(n_) + ")");
        n_ += count;
    }

    ViewT hostView() { return strided_<T>(host_, 0, n_, kDLCUDAHost); }
    ConstViewT hostView() const { return strided_<const T>(host_, 0, n_, kDLCUDAHost); }
    ViewT deviceView() { return strided_<T>(dev_, 0, n_, kDLCUDA); }
    ConstViewT deviceView() const { return strided_<const T>(dev_, 0, n_, kDLCUDA); }
    ViewT hostSpare() { return strided_<T>(host_, n_, cap_ - n_, kDLCUDAHost); }
    ViewT deviceSpare() { return strided_<T>(dev_, n_, cap_ - n_, kDLCUDA); }
    PackedViewT hostPacked() { return packed_<T>(host_, kDLCUDAHost); }
    ConstPackedViewT hostPacked() const { return packed_<const T>(host_, kDLCUDAHost); }
    PackedViewT devicePacked() { return packed_<T>(dev_, kDLCUDA); }
    ConstPackedViewT devicePacked() const { return packed_<const T>(dev_, kDLCUDA); }
    ViewT view() { return deviceView(); }

    /** Blocking host -> device copy of every plane. */
    void upload() {
        upload(nullptr);
        detail::sync(nullptr);
    }
    void download() {
        download(nullptr);
        detail::sync(nullptr);
    }
    /** Stream-ordered copies (array/Array.h:266-268). */
    void upload(Stream s) {
        detail::copy(dev_.get(), AETHER_MEM_DEVICE, host_.get(), AETHER_MEM_PINNED, bytes_(cap_), s, "upload");
    }
    void download(Stream s) {
        detail::copy(host_.get(), AETHER_MEM_PINNED, dev_.get(), AETHER_MEM_DEVICE, bytes_(cap_), s, "download");
    }

private:
    static std::size_t bytes_(std::size_t n) { return components * n * sizeof(T); }
    static void check_span_(std::size_t cap) {
        if (components * cap > 0xFFFFFFFFull)
            throw Error::memory("Array", "device 0", bytes_(cap),
                                "span exceeds the 32-bit element offsets of device views");
    }
    template <class U>
    View<U, Extents, layout_stride> strided_(const detail::Chunk& c, std::size_t start, std::size_t count,
                                             int dev) const {
        using Map = typename layout_stride::template mapping<Extents>;
        const detail::PlaneStrides<Es...> st(cap_);
        return View<U, Extents, layout_stride>(static_cast<U*>(c.get()) + start, Map(Extents(count), st),
                                               Device(dev, 0));
    }
    template <class U>
    View<U, Extents, layout_right> packed_(const detail::Chunk& c, int dev) const {
        if (cap_ != n_)
            throw Error::memory("Array::packed", "n/a", bytes_(n_),
                                "capacity()=" + std::to_string(cap_) + " != samples()=" + std::to_string(n_) +
                                    ": packed() requires an exactly-full Array (no reserved headroom)");
        using Map = typename layout_right::template mapping<Extents>;
        return View<U, Extents, layout_right>(static_cast<U*>(c.get()), Map(Extents(n_)), Device(dev, 0));
    }
    void reallocate_(std::size_t cap) {
        check_span_(cap);
        detail::Chunk h(AETHER_MEM_PINNED, bytes_(cap), "host (pinned)");
        detail::Chunk d(AETHER_MEM_DEVICE, bytes_(cap), "device 0");
        for (std::size_t c = 0; c < components; ++c) {
            const std::size_t rb = n_ * sizeof(T);
            detail::copy(static_cast<T*>(h.get()) + c * cap, AETHER_MEM_PINNED, static_cast<T*>(host_.get()) + c * cap_,
                         AETHER_MEM_PINNED, rb, nullptr, "Array::reserve");
            detail::copy(static_cast<T*>(d.get()) + c * cap, AETHER_MEM_DEVICE, static_cast<T*>(dev_.get()) + c * cap_,
                         AETHER_MEM_DEVICE, rb, nullptr, "Array::reserve");
        }
        detail::sync(nullptr);
        host_ = std::move(h);
        dev_ = std::move(d);
        cap_ = cap;
    }

    std::size_t n_, cap_;
    detail::Chunk host_, dev_;
};

}  // namespace aether
