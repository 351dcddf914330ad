// aether/random.h -- Philox streams as expression leaves.
//
// aether::random::Generator (random/Generator.h:56-195): a 64-bit key mixed
// from (seed, stream id) with splitmix64 (:64-67), substreams keyed from the
// parent key (:78-81), and distribution leaves (random/detail/
// DistributionLeaf.h:79-501) whose component c at sample i draws the
// Philox4x32-10 block at counter (c, global sample i) under key ^ salt. A leaf
// is a typed expression: inside a consumer kernel `v[i] = g.uniform<double,3>
// (-1, 1)` draws per sample; on the host `a.deviceView() = g.substream(0)
// .uniform<double, 3>(-1.0, 1.0);` runs the engine's generated kernel, which
// regenerates the same numbers.
//
// Per-sample formulas (DistributionLeaf.h:125-131, 192-199, 257-264, 329-333,
// 380-385; Box-Muller from random/detail/Backend.h:209-236, first normal
// only): uniform lo + (hi - lo) u; normal mean + sd z; lognormal exp(mu +
// sigma z); exponential -log(u) / lambda; bernoulli u < p. Double draws take u
// from one word (w 2^-32 + 2^-33) and z from the 53-bit uniforms of two words
// each; float draws use the float conversions.
#pragma once

#include "aether/detail/std.h"

#include "aether/detail/philox.h"
#include "aether/item.h"

namespace aether {
namespace random {

namespace detail {

enum LeafKind { kUniform = 0, kNormal = 1, kLognormal = 2, kExponential = 3, kBernoulli = 4 };

template <class Real>
AETHER_DEVICEANDHOST() inline Real draw01(std::uint64_t key, std::uint32_t g, std::uint32_t c) {
    const Words4 x = philoxBlock(key, g, c);
    if constexpr (sizeof(Real) == 4)
        return uniformFloatFromWord(x.x);
    else
        return uniformDoubleFromWord(x.x);
}

/** One standard normal (Box-Muller, first normal). */
template <class Real>
AETHER_DEVICEANDHOST() inline Real drawNormal(std::uint64_t key, std::uint32_t g, std::uint32_t c) {
    const Words4 x = philoxBlock(key, g, c);
    if constexpr (sizeof(Real) == 4) {
        const float u = uniformFloatFromWord(x.x);
        const float step = 2.3283064e-10f * 6.2831855f;
        const float v = float(x.y) * step + step / 2.0f;
        return math::sqrt(-2.0f * math::log(u)) * math::sin(v);
    } else {
        const double u = uniformDoubleHq(x.x, x.y);
        const std::uint64_t zy = std::uint64_t(x.z) ^ (std::uint64_t(x.w) << 21);
        const double v = double(zy) * 2.2204460492503131e-16 + 1.1102230246251565e-16;
        return math::sqrt(-2.0 * math::log(u)) * math::sin(v * 3.1415926535897932);
    }
}

#if AETHER_GB300_HOST_IR
}  // namespace detail
}  // namespace random
}  // namespace aether
#include <memory>
#include <string>
#include <vector>
namespace aether {
namespace random {
namespace detail {
/** The aether-ir/1 leaf the engine's kernels regenerate. N(0, 1) (and
 *  lognormal(0, 1)) keeps its parameters as literals, so the kernel skips the
 *  affine step 0 + 1 z, which is z bit for bit (a Box-Muller draw is never 0). */
inline Expr ir_leaf(const char* op, std::uint64_t key, int vd, std::vector<double> params) {
    auto n = std::make_shared<ir::RandomNode>();
    n->op = op;
    n->key = key;
    n->shape = {vd};
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
#endif

/** A distribution leaf of VD components. */
template <class Real, std::size_t VD, int Kind>
class Leaf : public Expression<Leaf<Real, VD, Kind>, Real> {
public:
    using element_type = Real;
    using element_extents = extents<VD>;
    static constexpr bool isLeaf = true;
    AETHER_DEVICEANDHOST() constexpr Leaf(std::uint64_t key, Real p0, Real p1) : key_(key), p0_(p0), p1_(p1) {}

    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real eval(const SampleIndex& i) const {
        const std::uint32_t g = i.global();
        if constexpr (Kind == kUniform) {
            return p0_ + (p1_ - p0_) * draw01<Real>(key_ ^ kSaltUniform, g, std::uint32_t(C));
        } else if constexpr (Kind == kNormal) {
            return p0_ + p1_ * drawNormal<Real>(key_ ^ kSaltNormal, g, std::uint32_t(C));
        } else if constexpr (Kind == kLognormal) {
            return math::exp(p0_ + p1_ * drawNormal<Real>(key_ ^ kSaltLognormal, g, std::uint32_t(C)));
        } else if constexpr (Kind == kExponential) {
            return -math::log(draw01<Real>(key_ ^ kSaltExponential, g, std::uint32_t(C))) / p0_;
        } else {
            return draw01<Real>(key_ ^ kSaltBernoulli, g, std::uint32_t(C)) < p0_ ? Real(1) : Real(0);
        }
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        static const char* const names[] = {"uniform", "normal", "lognormal", "exponential", "bernoulli"};
        std::vector<double> params{double(p0_)};
        if (Kind <= kLognormal) params.push_back(double(p1_));
        return ir_leaf(names[Kind], key_, int(VD), params);
    }
#endif
    AETHER_DEVICEANDHOST() constexpr std::uint64_t key() const { return key_; }

private:
    std::uint64_t key_;
    Real p0_, p1_;
};

}  // namespace detail

class Generator {
public:
    AETHER_DEVICEANDHOST() constexpr explicit Generator(std::uint64_t seed, std::uint64_t streamId = 0)
        : key_(detail::splitmix64(seed ^ detail::splitmix64(streamId))) {}

    AETHER_DEVICEANDHOST() constexpr Generator substream(std::uint64_t k) const {
        return fromKey(detail::splitmix64(key_ ^ detail::splitmix64(k ^ detail::kSaltSubstream)));
    }
    AETHER_DEVICEANDHOST() static constexpr Generator fromKey(std::uint64_t key) {
        Generator g(0);
        g.key_ = key;
        return g;
    }
    AETHER_DEVICEANDHOST() constexpr std::uint64_t key() const { return key_; }

    /** U(lo, hi) per component. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kUniform> uniform(Real lo, Real hi) const {
        return {key_, lo, hi};
    }
    /** N(mean, sd^2) per component. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kNormal> normal(Real mean, Real sd) const {
        return {key_, mean, sd};
    }
    /** exp(N(mu, sigma^2)). */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kLognormal> lognormal(Real mu, Real sigma) const {
        return {key_, mu, sigma};
    }
    /** -log(u) / lambda. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kExponential> exponential(Real lambda) const {
        return {key_, lambda, Real(0)};
    }
    /** 1 with probability p, else 0. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kBernoulli> bernoulli(Real p) const {
        return {key_, p, Real(0)};
    }

private:
    std::uint64_t key_;
};

}  // namespace random
}  // namespace aether
