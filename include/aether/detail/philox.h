// aether/detail/philox.h -- Philox4x32-10 and its word conversions for
// host and device code of the consumer API.
//
// The generator of random/detail/Philox.h:95-133 in cuRAND's block layout,
// the splitmix64 keying of random/detail/Backend.h:75-82 and the word -> real
// conversions of Backend.h:123-157, written in portable C++ so the same text
// evaluates a random leaf per sample inside a consumer kernel and on the host.
// The 32x32 -> 64-bit products compile to one wide multiply on the device.
// Every conversion is an exact scaling plus at most one rounding, so FMA
// contraction cannot change it: results are bit-identical to the engine's
// generated kernels and to the reference's CPU path.
#pragma once

#include "aether/detail/std.h"

#include "aether/macros.h"

namespace aether {
namespace random {
namespace detail {

struct Words4 {
    std::uint32_t x, y, z, w;
};

AETHER_DEVICEANDHOST() constexpr std::uint64_t splitmix64(std::uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/** Ten rounds on counter c under key (kx, ky). */
AETHER_DEVICEANDHOST() inline Words4 philox4x32_10(Words4 c, std::uint32_t kx, std::uint32_t ky) {
    AETHER_UNROLL
    for (int r = 0; r < 10; ++r) {
        if (r) {
            kx += 0x9E3779B9u;
            ky += 0xBB67AE85u;
        }
        const std::uint64_t p0 = std::uint64_t(0xD2511F53u) * c.x;
        const std::uint64_t p1 = std::uint64_t(0xCD9E8D57u) * c.z;
        c = Words4{std::uint32_t(p1 >> 32) ^ c.y ^ kx, std::uint32_t(p1), std::uint32_t(p0 >> 32) ^ c.w ^ ky,
                   std::uint32_t(p0)};
    }
    return c;
}

/** The block owned by (key, global sample, counter) (Backend.h:136-150). */
AETHER_DEVICEANDHOST() inline Words4 philoxBlock(std::uint64_t key, std::uint32_t global, std::uint64_t counter) {
    return philox4x32_10(Words4{std::uint32_t(counter), std::uint32_t(counter >> 32), global, 0u},
                         std::uint32_t(key), std::uint32_t(key >> 32));
}

/** (0, 1): w 2^-32 + 2^-33 (double) and (2 (w >> 9) + 1) 2^-24 (float). */
AETHER_DEVICEANDHOST() inline double uniformDoubleFromWord(std::uint32_t w) {
    return double(w) * 2.3283064365386963e-10 + 1.1641532182693481e-10;
}
AETHER_DEVICEANDHOST() inline float uniformFloatFromWord(std::uint32_t w) {
    return float(((w >> 9) << 1) | 1u) * 5.9604645e-8f;
}
/** 53-bit uniform from two words: z 2^-53 + 2^-54, z = x ^ (y << 21). */
AETHER_DEVICEANDHOST() inline double uniformDoubleHq(std::uint32_t x, std::uint32_t y) {
    const std::uint64_t z = std::uint64_t(x) ^ (std::uint64_t(y) << 21);
    return double(z) * 1.1102230246251565e-16 + 5.5511151231257827e-17;
}

/** Distribution salts (random/detail/DistributionLeaf.h:117,184,249,313,373). */
constexpr std::uint64_t kSaltUniform = 0x243F6A8885A308D3ull;
constexpr std::uint64_t kSaltNormal = 0x13198A2E03707344ull;
constexpr std::uint64_t kSaltLognormal = 0xA4093822299F31D0ull;
constexpr std::uint64_t kSaltExponential = 0x082EFA98EC4E6C89ull;
constexpr std::uint64_t kSaltBernoulli = 0x452821E638D01377ull;
/** Substream salt (random/Generator.h:78-81). */
constexpr std::uint64_t kSaltSubstream = 0x2545F4914F6CDD1Dull;

}  // namespace detail
}  // namespace random
}  // namespace aether
