// aether/view_copy.h -- a stream-ordered copy between two views
// (view/Copy.h).
//
// aether::copyAsync(dst, src, stream) copies the span `src` addresses into
// `dst` on `stream`. Both views have the same extents type and layout and
// element types equal up to const; their runtime extents and every mode's
// stride must also match (two arrays of one shape but different capacities
// pitch their planes differently, and a byte copy between them would
// scramble the samples). The pair must be one the copy engines can run
// asynchronously: CUDA device memory or page-locked host memory on both
// sides; pageable host memory is refused. Errors are aether::Error in the
// "<op> failed on <where>, size=<n> bytes (<detail>)" form.
#pragma once

#include <cstddef>
#include <string>
#include <type_traits>

#include "aether/array.h"

namespace aether {

namespace detail {

inline std::string device_label(Device d) {
    switch (d.type) {
    case kDLCPU: return "cpu";
    case kDLCUDA: return "cuda:" + std::to_string(d.id);
    case kDLCUDAHost: return "cuda_host";
    default: return "device_type " + std::to_string(d.type);
    }
}

// The C-ABI memory kind of a device, or -1 when no asynchronous copy serves it.
inline int async_kind(Device d) {
    return d.type == kDLCUDA ? AETHER_MEM_DEVICE : (d.type == kDLCUDAHost ? AETHER_MEM_PINNED : -1);
}

}  // namespace detail

/** src -> dst on `stream`, never synchronising (view/Copy.h). */
template <class TDst, class TSrc, class X, class L, bool VoD, bool RoD, bool VoS, bool RoS>
void copyAsync(View<TDst, X, L, VoD, RoD> dst, const View<TSrc, X, L, VoS, RoS>& src, Stream stream) {
    static_assert(std::is_same<std::remove_const_t<TSrc>, TDst>::value && !RoD,
                  "copyAsync(View, View, Stream): element types agree up to const, and dst is writable");
    const std::string op = "copyAsync(View)";
    const std::string where = detail::device_label(src.device()) + " -> " + detail::device_label(dst.device());
    const std::size_t bytes = std::size_t(dst.mapping().required_span_size()) * sizeof(TDst);
    for (std::size_t k = 0; k < X::Rank; ++k) {
        if (dst.extent(k) != src.extent(k))
            throw Error::memory(op, where, bytes,
                                "extents mismatch at mode " + std::to_string(k) + ": dst.extent=" +
                                    std::to_string(dst.extent(k)) + " src.extent=" + std::to_string(src.extent(k)));
        if (dst.mapping().stride(k) != src.mapping().stride(k))
            throw Error::memory(op, where, bytes,
                                "strides mismatch at mode " + std::to_string(k) + ": dst.stride=" +
                                    std::to_string(dst.mapping().stride(k)) +
                                    " src.stride=" + std::to_string(src.mapping().stride(k)));
    }
    const int dk = detail::async_kind(dst.device()), sk = detail::async_kind(src.device());
    if (dk < 0 || sk < 0)
        throw Error::memory(op, where, bytes,
                            "no asynchronous copy for this pair: both sides must be CUDA device or page-locked host "
                            "memory");
    if (bytes == 0) return;
    if (aether_copy(dk, dst.device().type == kDLCUDA ? dst.device().id : 0, static_cast<void*>(dst.data()), sk,
                    src.device().type == kDLCUDA ? src.device().id : 0, static_cast<const void*>(src.data()), bytes,
                    stream) != AETHER_OK)
        throw Error::memory(op, where, bytes, detail::last_error());
}

}  // namespace aether
