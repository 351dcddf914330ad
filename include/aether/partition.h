// aether/partition.h -- blocks of the sample mode.
//
// padded_block_samples and partition_view (residency/Partition.h:52-168):
// split a view's trailing sample mode into `parts` blocks whose starts fall
// every ceil(n / parts) samples rounded up to `pad_to`; block r starts at
// sample r * padded and holds min(padded, n - r * padded) real samples (0
// past the end). The block is a view into the same memory with the same
// plane pitch: no allocation, no copy. This is how the sample axis shards
// across devices; on one GPU it also cuts one array into independently
// launched pieces.
#pragma once

#include <cstddef>
#include <string>

#include "aether/array.h"

namespace aether {

struct PartitionSpec {
    std::size_t parts;
    std::size_t pad_to = 32;
};

inline std::size_t padded_block_samples(std::size_t n, std::size_t parts, std::size_t pad_to = 32) {
    if (parts == 0) throw Error::memory("padded_block_samples", "n/a", n, "parts must be > 0");
    if (pad_to == 0) throw Error::memory("padded_block_samples", "n/a", n, "pad_to must be > 0");
    const std::size_t per = (n + parts - 1) / parts;
    return (per + pad_to - 1) / pad_to * pad_to;
}

template <class T, class X, class L, bool Vo, bool RO>
View<T, X, layout_stride, Vo, RO> partition_view(const View<T, X, L, Vo, RO>& v, const PartitionSpec& spec,
                                                  std::size_t r) {
    if (r >= spec.parts)
        throw Error::memory("partition_view", "cuda:0", 0,
                            "block index " + std::to_string(r) + " >= spec.parts=" + std::to_string(spec.parts));
    const std::size_t n = v.samples();
    const std::size_t padded = padded_block_samples(n, spec.parts, spec.pad_to);
    const std::size_t off = r * padded;
    const std::size_t real = off < n ? (padded < n - off ? padded : n - off) : 0;
    // the same strides, the sample extent cut to the block
    using Map = typename layout_stride::template mapping<X>;
    offset_t st[X::Rank];
    for (std::size_t k = 0; k < X::Rank; ++k) st[k] = v.mapping().stride(k);
    const std::size_t start = off < n ? off : n;
    return View<T, X, layout_stride, Vo, RO>(const_cast<T*>(v.data()) + start * st[X::Rank - 1],
                                             Map(X(real), st), v.device());
}

}  // namespace aether
