// Host check of the invariant-divisor division the strided runtime kernels
// use (include/aether/gb300/ag_fastdiv.cuh) against the hardware divide:
// every divisor up to 4096 on edge and random dividends, then random and
// edge divisor/dividend pairs over the whole 32-bit range.
#include <cstdint>
#include <cstdio>
#include <random>

#include "aether/gb300/ag_fastdiv.cuh"

static int check(uint32_t x, uint32_t d) {
    const AgFastDiv f = ag_fastdiv_make(d);
    uint32_t q, r;
    ag_fastdiv_divmod(x, f, q, r);
    if (q != x / d || r != x % d) {
        std::printf("mismatch x=%u d=%u q=%u r=%u\n", x, d, q, r);
        return 1;
    }
    return 0;
}

int main() {
    std::mt19937_64 rng(12345);
    const uint32_t edges[] = {0u, 1u, 2u, 3u, 31u, 32u, 33u, 65535u, 65536u, 65537u, 0x7FFFFFFFu, 0x80000000u,
                              0x80000001u, 0xFFFFFFFEu, 0xFFFFFFFFu};
    int bad = 0;
    for (uint32_t d = 1; d <= 4096 && !bad; ++d) {
        for (uint32_t x : edges) bad |= check(x, d);
        for (int k = 0; k < 64; ++k) bad |= check(uint32_t(rng()), d);
        for (uint32_t m = 1; m < 8; ++m) bad |= check(d * m - 1, d) | check(d * m, d);
    }
    for (int k = 0; k < 4000000 && !bad; ++k) {
        uint32_t d = uint32_t(rng() >> (rng() & 31));
        if (!d) d = 1;
        bad |= check(uint32_t(rng()), d);
        bad |= check(uint32_t(rng() % (uint64_t(d) * 3 + 1)), d);
    }
    for (uint32_t d : edges)
        if (d)
            for (uint32_t x : edges) bad |= check(x, d);
    for (int s = 0; s < 32 && !bad; ++s) {
        const uint32_t p = 1u << s;
        for (uint32_t d : {p - 1, p, p + 1})
            if (d)
                for (uint32_t x : edges) bad |= check(x, d);
    }
    std::printf(bad ? "fastdiv FAILED\n" : "fastdiv ok\n");
    return bad;
}
