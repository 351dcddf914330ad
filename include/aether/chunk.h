// aether/chunk.h -- owned and borrowed byte ranges on a device
// (chunk/Chunk.h, chunk/Copy.h, chunk/Fill.h), over the C-ABI's chunks.
//
// aether::Chunk is a move-only range of `size()` bytes on a Device: the host
// (kDLCPU), CUDA device memory (kDLCUDA, allocated stream-ordered when a
// stream is given) or page-locked host memory (kDLCUDAHost). allocate() owns
// its bytes and returns them when destroyed (device memory still in use by a
// graph being captured is released after the capture); borrow() wraps bytes
// someone else owns. copy() is a blocking copy between two chunks of equal
// size over any pair but a direct host<->device one (stage through
// page-locked memory); copyAsync() is stream-ordered and takes only pairs the
// copy engines serve asynchronously (device and page-locked memory);
// fill() repeats a value of 1..16 bytes over a chunk. make_view(chunk, n...)
// views a chunk, its size checked. Device memory is released on the stream
// it was allocated on, so a chunk allocated on a stream must be destroyed
// before that stream is. Errors are aether::Error in the
// "<op> failed on <where>, size=<n> bytes (<detail>)" form.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>

#include "aether/array.h"

namespace aether {

class Chunk {
public:
    Chunk() = default;
    Chunk(const Chunk&) = delete;
    Chunk& operator=(const Chunk&) = delete;
    Chunk(Chunk&& o) noexcept { take_(o); }
    Chunk& operator=(Chunk&& o) noexcept {
        if (this != &o) {
            free_();
            take_(o);
        }
        return *this;
    }
    ~Chunk() { free_(); }

    /** `bytes` bytes on `device`, aligned to `alignment` (at most 256). */
    static Chunk allocate(Device device, std::size_t bytes, std::size_t alignment = 256) {
        return allocate_(device, bytes, nullptr, false, alignment);
    }
    /** The same, stream-ordered on `stream` for device memory. */
    static Chunk allocate(Device device, std::size_t bytes, Stream stream, std::size_t alignment = 256) {
        return allocate_(device, bytes, stream, true, alignment);
    }
    /** A non-owning chunk over `bytes` bytes at `ptr` on `device`. */
    static Chunk borrow(void* ptr, std::size_t bytes, Device device, std::size_t alignment = 256) {
        if (bytes && !ptr) throw Error::memory("Chunk::borrow", label(device), bytes, "null pointer");
        if (alignment && reinterpret_cast<std::uintptr_t>(ptr) % alignment)
            throw Error::memory("Chunk::borrow", label(device), bytes,
                                "pointer not aligned to " + std::to_string(alignment) + " bytes");
        Chunk c;
        c.data_ = static_cast<std::byte*>(ptr);
        c.size_ = bytes;
        c.device_ = device;
        c.alignment_ = alignment;
        return c;
    }

    std::byte* data() const { return data_; }
    std::size_t size() const { return size_; }
    Device device() const { return device_; }
    std::size_t alignment() const { return alignment_; }
    bool owns() const { return handle_ != nullptr; }
    bool streamOrdered() const { return streamOrdered_; }
    Stream stream() const { return stream_; }

    /** "cpu", "cuda:<id>", "cuda_host" or "device_type <n>". */
    static std::string label(Device d) {
        switch (d.type) {
        case kDLCPU: return "cpu";
        case kDLCUDA: return "cuda:" + std::to_string(d.id);
        case kDLCUDAHost: return "cuda_host";
        default: return "device_type " + std::to_string(d.type);
        }
    }
    /** The C-ABI memory kind of a device, or -1. */
    static int kind(Device d) {
        return d.type == kDLCPU ? AETHER_MEM_CPU
                                : d.type == kDLCUDA ? AETHER_MEM_DEVICE : d.type == kDLCUDAHost ? AETHER_MEM_PINNED : -1;
    }

private:
    static Chunk allocate_(Device device, std::size_t bytes, Stream stream, bool ordered, std::size_t alignment) {
        const int k = kind(device);
        if (k < 0) throw Error::memory("Chunk::allocate", label(device), bytes, "unsupported device kind");
        if (alignment == 0 || alignment > 256 || (alignment & (alignment - 1)))
            throw Error::memory("Chunk::allocate", label(device), bytes,
                                "alignment must be a power of two up to 256, got " + std::to_string(alignment));
        Chunk c;
        void* h = nullptr;
        void* p = nullptr;
        if (aether_chunk_alloc(k, device.type == kDLCUDA ? device.id : 0, bytes, stream, &h, &p) != AETHER_OK)
            throw Error::memory("Chunk::allocate", label(device), bytes, detail::last_error());
        c.handle_ = h;
        c.data_ = static_cast<std::byte*>(p);
        c.size_ = bytes;
        c.device_ = device;
        c.alignment_ = alignment;
        c.streamOrdered_ = ordered && device.type == kDLCUDA;
        c.stream_ = stream;
        return c;
    }
    void take_(Chunk& o) {
        handle_ = std::exchange(o.handle_, nullptr);
        data_ = std::exchange(o.data_, nullptr);
        size_ = std::exchange(o.size_, 0);
        device_ = o.device_;
        alignment_ = o.alignment_;
        streamOrdered_ = o.streamOrdered_;
        stream_ = o.stream_;
    }
    void free_() {
        if (handle_) aether_chunk_release(handle_);
        handle_ = nullptr;
        data_ = nullptr;
        size_ = 0;
    }

    void* handle_ = nullptr;
    std::byte* data_ = nullptr;
    std::size_t size_ = 0;
    Device device_{};
    std::size_t alignment_ = 256;
    bool streamOrdered_ = false;
    Stream stream_ = nullptr;
};

namespace detail {

inline std::string chunk_path(const ::aether::Chunk& src, const ::aether::Chunk& dst) {
    return ::aether::Chunk::label(src.device()) + " -> " + ::aether::Chunk::label(dst.device());
}
inline bool host_addressable(Device d) { return d.type == kDLCPU || d.type == kDLCUDAHost; }

}  // namespace detail

/** Blocking copy of src's bytes into dst (equal sizes). Host pairs are a
 *  memcpy; pairs with device memory go through the copy engines; a direct
 *  host <-> device pair is refused. The checks come before the empty case. */
inline void copy(Chunk& dst, const Chunk& src) {
    const std::string where = detail::chunk_path(src, dst);
    if (dst.size() != src.size())
        throw Error::memory("copy", where, src.size(), "size mismatch: dst.size()=" + std::to_string(dst.size()));
    const int sk = Chunk::kind(src.device()), dk = Chunk::kind(dst.device());
    if (sk < 0 || dk < 0 || (sk == AETHER_MEM_CPU && dk == AETHER_MEM_DEVICE) ||
        (sk == AETHER_MEM_DEVICE && dk == AETHER_MEM_CPU))
        throw Error::memory("copy", where, src.size(),
                            "illegal device pair (CPU<->CUDA direct is not supported; stage through CUDAHost)");
    if (src.size() == 0) return;
    if (detail::host_addressable(src.device()) && detail::host_addressable(dst.device())) {
        std::memcpy(dst.data(), src.data(), src.size());
        return;
    }
    if (aether_copy(dk, dst.device().type == kDLCUDA ? dst.device().id : 0, dst.data(), sk,
                    src.device().type == kDLCUDA ? src.device().id : 0, src.data(), src.size(), nullptr) != AETHER_OK)
        throw Error::memory("copy", where, src.size(), detail::last_error());
    detail::sync(nullptr);
}

/** Stream-ordered copy (equal sizes) between device or page-locked chunks;
 *  any pair with pageable host memory is refused. */
inline void copyAsync(Chunk& dst, const Chunk& src, Stream stream) {
    const std::string where = detail::chunk_path(src, dst);
    if (dst.size() != src.size())
        throw Error::memory("copyAsync", where, src.size(), "size mismatch: dst.size()=" + std::to_string(dst.size()));
    const int sk = Chunk::kind(src.device()), dk = Chunk::kind(dst.device());
    if (sk != AETHER_MEM_DEVICE && sk != AETHER_MEM_PINNED)
        throw Error::memory("copyAsync", where, src.size(), "not an asynchronous pair (CUDAHost or CUDA on both sides)");
    if (dk != AETHER_MEM_DEVICE && dk != AETHER_MEM_PINNED)
        throw Error::memory("copyAsync", where, src.size(), "not an asynchronous pair (CUDAHost or CUDA on both sides)");
    if (src.size() == 0) return;
    if (aether_copy(dk, dst.device().type == kDLCUDA ? dst.device().id : 0, dst.data(), sk,
                    src.device().type == kDLCUDA ? src.device().id : 0, src.data(), src.size(), stream) != AETHER_OK)
        throw Error::memory("copyAsync", where, src.size(), detail::last_error());
}

/** Repeat the `width`-byte value (1..16 bytes, dividing the size) over dst,
 *  on `stream` for device memory. */
inline void fill(Chunk& dst, const void* value, std::size_t width, Stream stream = nullptr) {
    const std::string where = Chunk::label(dst.device());
    if (width == 0 || width > 16 || dst.size() % width)
        throw Error::memory("fill", where, dst.size(),
                            "value width " + std::to_string(width) + " must be 1..16 bytes and divide the size");
    if (dst.size() == 0) return;
    const int k = Chunk::kind(dst.device());
    if (aether_fill(k, dst.device().type == kDLCUDA ? dst.device().id : 0, dst.data(), dst.size(), value, width,
                    stream) != AETHER_OK)
        throw Error::memory("fill", where, dst.size(), detail::last_error());
}

/** A compact view of `chunk` (view/MakeView.h): extents Es..., the dyn ones
 *  given; the chunk must hold the whole span. */
template <class T, std::size_t... Es, class... D>
View<T, extents<Es...>> make_view(const Chunk& chunk, D... dynVals) {
    using X = extents<Es...>;
    const X ext{static_cast<std::size_t>(dynVals)...};
    const typename layout_right::template mapping<X> map(ext);
    const std::size_t need = std::size_t(map.required_span_size()) * sizeof(T);
    if (need > chunk.size())
        throw Error::memory("make_view", Chunk::label(chunk.device()), need,
                            "the view needs " + std::to_string(need) + " bytes, the chunk holds " +
                                std::to_string(chunk.size()));
    return View<T, X>(reinterpret_cast<T*>(chunk.data()), map, chunk.device());
}

}  // namespace aether
