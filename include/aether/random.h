// aether/random.h -- Philox streams as expression leaves.
//
// aether::random::Generator (random/Generator.h:56-195): a 64-bit key mixed
// from (seed, stream id) with splitmix64 (:64-67), substreams keyed from the
// parent key (:78-81), and distribution leaves whose sample i, component c
// draws the Philox4x32-10 block at counter (i, c, salt) under the key
// (random/detail/DistributionLeaf.h:79-501). A leaf is an expression: it can
// be assigned (`a.deviceView() = g.substream(0).uniform<double, 3>(-1, 1);`)
// or used inside a larger tree; the kernel regenerates the same numbers.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "aether/expr.h"

namespace aether {
namespace random {

namespace detail {
constexpr std::uint64_t splitmix64(std::uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline Expr leaf(const char* op, std::uint64_t key, int vd, std::vector<double> params) {
    auto n = std::make_shared<ir::RandomNode>();
    n->op = op;
    n->key = key;
    n->shape = {vd};
    // N(0, 1) keeps its parameters as literals: the kernel then skips the
    // affine step 0 + 1 z, which is z bit for bit (a Box-Muller draw is never 0)
    const bool standard = (std::string(op) == "normal" || std::string(op) == "lognormal") && params.size() == 2 &&
                          params[0] == 0.0 && params[1] == 1.0;
    for (double p : params) {
        if (standard) {
            auto l = std::make_shared<ir::LiteralNode>();
            l->v = p;
            n->params.push_back(l);
        } else {
            n->params.push_back(ir::scalar(p));
        }
    }
    return Expr(n);
}
}  // namespace detail

class Generator {
public:
    constexpr explicit Generator(std::uint64_t seed, std::uint64_t streamId = 0)
        : key_(detail::splitmix64(seed ^ detail::splitmix64(streamId))) {}

    constexpr Generator substream(std::uint64_t k) const {
        return fromKey(detail::splitmix64(key_ ^ detail::splitmix64(k ^ kSalt)));
    }
    static constexpr Generator fromKey(std::uint64_t key) {
        Generator g(0);
        g.key_ = key;
        return g;
    }
    constexpr std::uint64_t key() const { return key_; }

    /** U(lo, hi] per component. */
    template <class Real, std::size_t VD>
    Expr uniform(Real lo, Real hi) const { return detail::leaf("uniform", key_, int(VD), {double(lo), double(hi)}); }
    /** N(mean, sd^2) per component (Box-Muller, first normal). */
    template <class Real, std::size_t VD>
    Expr normal(Real mean, Real sd) const { return detail::leaf("normal", key_, int(VD), {double(mean), double(sd)}); }
    /** exp(N(mu, sigma^2)). */
    template <class Real, std::size_t VD>
    Expr lognormal(Real mu, Real sigma) const {
        return detail::leaf("lognormal", key_, int(VD), {double(mu), double(sigma)});
    }
    /** -log(u) / lambda. */
    template <class Real, std::size_t VD>
    Expr exponential(Real lambda) const { return detail::leaf("exponential", key_, int(VD), {double(lambda)}); }
    /** 1 with probability p, else 0. */
    template <class Real, std::size_t VD>
    Expr bernoulli(Real p) const { return detail::leaf("bernoulli", key_, int(VD), {double(p)}); }

private:
    static constexpr std::uint64_t kSalt = 0x2545F4914F6CDD1Dull;
    std::uint64_t key_;
};

}  // namespace random
}  // namespace aether
