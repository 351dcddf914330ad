// Host check of the C++ partition algebra (include/aether/partition.h) on
// the reference's cases (tests/test_Partition.cpp): block pitch, offsets,
// real extents of a short last block, unchanged plane pitch, refusals.
#include <aether/aether.h>

#include <cstdio>

#define CHECK(c)                                              \
    do {                                                      \
        if (!(c)) {                                           \
            std::printf("FAILED %s line %d\n", #c, __LINE__); \
            return 1;                                         \
        }                                                     \
    } while (0)

int main() {
    using aether::padded_block_samples;
    CHECK(padded_block_samples(100, 4, 32) == 32);
    CHECK(padded_block_samples(100, 3, 32) == 64);
    CHECK(padded_block_samples(96, 3, 32) == 32);
    CHECK(padded_block_samples(10, 4) == 32);
    CHECK(padded_block_samples(10, 4, 4) == 4);
    CHECK(padded_block_samples(10, 4, 1) == 3);
    bool threw = false;
    try {
        padded_block_samples(100, 0, 32);
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        padded_block_samples(100, 4, 0);
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);

    static double buf[3 * 100];
    auto full = aether::detail::plane_view<double, 3>(buf, 100, 100, aether::Device(aether::kDLCPU));
    const aether::PartitionSpec spec{4, 32};
    const std::size_t off[4] = {0, 32, 64, 96}, real[4] = {32, 32, 32, 4};
    for (std::size_t r = 0; r < 4; ++r) {
        auto b = aether::partition_view(full, spec, r);
        CHECK(b.samples() == real[r]);
        CHECK(b.data() == buf + off[r]);
        CHECK(b.mapping().stride(0) == 100 && b.mapping().stride(1) == 1);
        const auto rt = aether::fromView(b);
        CHECK(rt.extents[0] == 3 && rt.extents[1] == int64_t(real[r]) && rt.strides[0] == 100 && rt.strides[1] == 1);
    }
    auto exact = aether::detail::plane_view<double, 3>(buf, 96, 96, aether::Device(aether::kDLCPU));
    for (std::size_t r = 0; r < 3; ++r) {
        auto b = aether::partition_view(exact, aether::PartitionSpec{3, 32}, r);
        CHECK(b.samples() == 32 && b.data() == buf + r * 32);
    }
    threw = false;
    try {
        aether::partition_view(full, spec, 4);
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    std::printf("partition ok\n");
    return 0;
}
