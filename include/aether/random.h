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
// Leaf parameters are scalars or Item<Real, VD> per component; get<I>() without
// an index draws from a separate index-free domain (DistributionLeaf.h:49);
// uniformInt and multivariateNormal (mean + L z, L from cholesky) are
// evaluated per sample only.
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

/** Salt of the index-free draws get<I>() (DistributionLeaf.h:49). */
constexpr std::uint64_t kIndexFreeDomain = 0xD1B54A32D192ED03ull;
constexpr std::uint64_t kSaltUniformInt = 0xBE5466CF34E90C6Cull;
constexpr std::uint64_t kSaltMultivariateNormal = 0xC0AC29B7C97C50DDull;

/** Component C of a parameter at sample i: a scalar broadcasts, an expression
 *  (an Item<Real, VD> in practice) is evaluated per component
 *  (DistributionLeaf.h:58-66). */
template <class Real, std::size_t C, class P>
AETHER_DEVICEANDHOST() constexpr Real param_(const P& p, const SampleIndex& i) {
    if constexpr (aether_expression<P>)
        return static_cast<Real>(p.template eval<C>(i));
    else
        return static_cast<Real>(p);
}

#if AETHER_GB300_HOST_IR
template <class P>
ir::NodeP param_ir_(const P& p) {
    if constexpr (aether_expression<P>)
        return ::aether::Expr(p).node();
    else
        return ir::scalar(double(p));
}
#endif

/** A distribution leaf of VD components; P0 and P1 are its parameters' types,
 *  Real (one value for every component) or Item<Real, VD> (one per component). */
template <class Real, std::size_t VD, int Kind, class P0 = Real, class P1 = Real>
class Leaf : public Expression<Leaf<Real, VD, Kind, P0, P1>, Real> {
public:
    using element_type = Real;
    using element_extents = extents<VD>;
    static constexpr bool isLeaf = true;
    AETHER_DEVICEANDHOST() constexpr Leaf(std::uint64_t key, const P0& p0, const P1& p1) : key_(key), p0_(p0), p1_(p1) {}

    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real eval(const SampleIndex& i) const {
        return draw_<C>(key_, i.global(), i);
    }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real get(const SampleIndex& i) const {
        return draw_<C>(key_, i.global(), i);
    }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real get(offset_t i) const {
        const SampleIndex s = SampleIndex::make(std::size_t(i));
        return draw_<C>(key_, s.global(), s);
    }
    /** The index-free draw: one value per component, the same at every sample,
     *  from a domain apart from every per-sample draw (DistributionLeaf.h:146-156). */
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real get() const {
        return draw_<C>(key_ ^ kIndexFreeDomain, 0u, SampleIndex::make(std::size_t(0)));
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        static const char* const names[] = {"uniform", "normal", "lognormal", "exponential", "bernoulli"};
        if constexpr (!aether_expression<P0> && !aether_expression<P1>) {
            std::vector<double> params{double(p0_)};
            if (Kind <= kLognormal) params.push_back(double(p1_));
            return ir_leaf(names[Kind], key_, int(VD), params);
        } else {
            auto n = std::make_shared<ir::RandomNode>();
            n->op = names[Kind];
            n->key = key_;
            n->shape = {int(VD)};
            n->params.push_back(param_ir_(p0_));
            if (Kind <= kLognormal) n->params.push_back(param_ir_(p1_));
            return Expr(n);
        }
    }
#endif
    AETHER_DEVICEANDHOST() constexpr std::uint64_t key() const { return key_; }

private:
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Real draw_(std::uint64_t key, std::uint32_t g, const SampleIndex& i) const {
        static_assert(C < VD, "leaf component out of range");
        const Real a = param_<Real, C>(p0_, i);
        if constexpr (Kind == kUniform) {
            const Real b = param_<Real, C>(p1_, i);
            return a + (b - a) * draw01<Real>(key ^ kSaltUniform, g, std::uint32_t(C));
        } else if constexpr (Kind == kNormal) {
            const Real b = param_<Real, C>(p1_, i);
            return a + b * drawNormal<Real>(key ^ kSaltNormal, g, std::uint32_t(C));
        } else if constexpr (Kind == kLognormal) {
            const Real b = param_<Real, C>(p1_, i);
            return math::exp(a + b * drawNormal<Real>(key ^ kSaltLognormal, g, std::uint32_t(C)));
        } else if constexpr (Kind == kExponential) {
            return -math::log(draw01<Real>(key ^ kSaltExponential, g, std::uint32_t(C))) / a;
        } else {
            return draw01<Real>(key ^ kSaltBernoulli, g, std::uint32_t(C)) < a ? Real(1) : Real(0);
        }
    }
    std::uint64_t key_;
    P0 p0_;
    P1 p1_;
};

/** Integers uniform over [lo, hi]: lo + (64 random bits) mod (hi - lo + 1),
 *  the bits the first two words of the Philox block (DistributionLeaf.h:440-495).
 *  Evaluated per sample; the engine's whole-view kernels store floating-point
 *  arrays. */
template <class Int, std::size_t VD>
class UniformIntLeaf : public Expression<UniformIntLeaf<Int, VD>, Int> {
    static_assert(std::is_integral<Int>::value, "uniformInt draws an integer type");

public:
    using element_type = Int;
    using element_extents = extents<VD>;
    static constexpr bool isLeaf = true;
    AETHER_DEVICEANDHOST() constexpr UniformIntLeaf(std::uint64_t key, Int lo, Int hi) : key_(key), lo_(lo), hi_(hi) {}
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Int eval(const SampleIndex& i) const {
        return draw_<C>(key_ ^ kSaltUniformInt, i.global());
    }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Int get(const SampleIndex& i) const {
        return draw_<C>(key_ ^ kSaltUniformInt, i.global());
    }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Int get(offset_t i) const {
        return draw_<C>(key_ ^ kSaltUniformInt, std::uint32_t(i));
    }
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Int get() const {
        return draw_<C>(key_ ^ kSaltUniformInt ^ kIndexFreeDomain, 0u);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        throw Error("aether: uniformInt leaves are evaluated per sample (view[i] = leaf); the engine's whole-view "
                    "kernels store floating-point arrays");
    }
#endif

private:
    template <std::size_t C>
    AETHER_DEVICEANDHOST() Int draw_(std::uint64_t key, std::uint32_t g) const {
        static_assert(C < VD, "leaf component out of range");
        const Words4 x = philoxBlock(key, g, C);
        const std::uint64_t bits = (std::uint64_t(x.y) << 32) | std::uint64_t(x.x);
        const std::uint64_t range = std::uint64_t((long long)hi_ - (long long)lo_) + 1u;
        return static_cast<Int>((long long)lo_ + (long long)(bits % range));
    }
    std::uint64_t key_;
    Int lo_, hi_;
};

}  // namespace detail

/** A lower-triangular VD x VD matrix packed by rows, entry (r, c) at
 *  r (r + 1) / 2 + c (random/LowerTriangular.h:36-48). */
template <class Real, std::size_t VD>
struct LowerTriangular {
    static constexpr std::size_t rows = VD;
    static constexpr std::size_t packedSize = VD * (VD + 1) / 2;
    Real data[packedSize];
    AETHER_DEVICEANDHOST() constexpr Real& at(std::size_t r, std::size_t c) { return data[r * (r + 1) / 2 + c]; }
    AETHER_DEVICEANDHOST() constexpr Real at(std::size_t r, std::size_t c) const { return data[r * (r + 1) / 2 + c]; }
};

#if AETHER_GB300_HOST_IR
/** The Cholesky factor L (L L^T = cov) of a symmetric positive-definite
 *  covariance, on the host (random/LowerTriangular.h:58-75); a covariance that
 *  is not positive definite gives NaN entries, as there. */
template <class Real, std::size_t VD>
inline LowerTriangular<Real, VD> cholesky(const Real (&cov)[VD][VD]) {
    LowerTriangular<Real, VD> L{};
    for (std::size_t r = 0; r < VD; ++r)
        for (std::size_t c = 0; c <= r; ++c) {
            Real s = cov[r][c];
            for (std::size_t k = 0; k < c; ++k) s -= L.at(r, k) * L.at(c, k);
            L.at(r, c) = r == c ? std::sqrt(s) : s / L.at(c, c);
        }
    return L;
}
#endif

namespace detail {

/** mean + L z with z_c the standard normal at counter c: component I is
 *  mean[I] + sum over c <= I of L(I, c) z_c, accumulated in c order
 *  (MultivariateNormalLeaf.h:60-120). Evaluated per sample. */
template <class Real, std::size_t VD>
class MultivariateNormalLeaf : public Expression<MultivariateNormalLeaf<Real, VD>, Real> {
public:
    using element_type = Real;
    using element_extents = extents<VD>;
    static constexpr bool isLeaf = true;
    AETHER_DEVICEANDHOST() constexpr MultivariateNormalLeaf(std::uint64_t key, const Item<Real, VD>& mean,
                                                            const LowerTriangular<Real, VD>& L)
        : key_(key), mean_(mean), L_(L) {}
    template <std::size_t I>
    AETHER_DEVICEANDHOST() Real eval(const SampleIndex& i) const {
        return row_<I>(key_ ^ kSaltMultivariateNormal, i.global());
    }
    template <std::size_t I>
    AETHER_DEVICEANDHOST() Real get(const SampleIndex& i) const {
        return row_<I>(key_ ^ kSaltMultivariateNormal, i.global());
    }
    template <std::size_t I>
    AETHER_DEVICEANDHOST() Real get(offset_t i) const {
        return row_<I>(key_ ^ kSaltMultivariateNormal, std::uint32_t(i));
    }
    template <std::size_t I>
    AETHER_DEVICEANDHOST() Real get() const {
        return row_<I>(key_ ^ kSaltMultivariateNormal ^ kIndexFreeDomain, 0u);
    }
#if AETHER_GB300_HOST_IR
    Expr gb300_ir() const {
        throw Error("aether: multivariateNormal leaves are evaluated per sample (view[i] = leaf)");
    }
#endif

private:
    template <std::size_t I>
    AETHER_DEVICEANDHOST() Real row_(std::uint64_t key, std::uint32_t g) const {
        static_assert(I < VD, "leaf component out of range");
        Real acc = mean_.template get<I>();
        for (std::size_t c = 0; c <= I; ++c) acc += L_.at(I, c) * drawNormal<Real>(key, g, std::uint32_t(c));
        return acc;
    }
    std::uint64_t key_;
    Item<Real, VD> mean_;
    LowerTriangular<Real, VD> L_;
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

    template <class Real, std::size_t VD>
    using Per = Item<Real, VD>;

    /** U(lo, hi) per component; lo and hi one value, or an Item of one per component. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kUniform> uniform(Real lo, Real hi) const {
        return {key_, lo, hi};
    }
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kUniform, Per<Real, VD>, Per<Real, VD>> uniform(
        const Per<Real, VD>& lo, const Per<Real, VD>& hi) const {
        return {key_, lo, hi};
    }
    /** N(mean, sd^2) per component. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kNormal> normal(Real mean, Real sd) const {
        return {key_, mean, sd};
    }
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kNormal, Per<Real, VD>, Per<Real, VD>> normal(
        const Per<Real, VD>& mean, const Per<Real, VD>& sd) const {
        return {key_, mean, sd};
    }
    /** exp(N(mu, sigma^2)). */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kLognormal> lognormal(Real mu, Real sigma) const {
        return {key_, mu, sigma};
    }
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kLognormal, Per<Real, VD>, Per<Real, VD>> lognormal(
        const Per<Real, VD>& mu, const Per<Real, VD>& sigma) const {
        return {key_, mu, sigma};
    }
    /** -log(u) / lambda. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kExponential> exponential(Real lambda) const {
        return {key_, lambda, Real(0)};
    }
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kExponential, Per<Real, VD>> exponential(
        const Per<Real, VD>& lambda) const {
        return {key_, lambda, Real(0)};
    }
    /** 1 with probability p, else 0. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kBernoulli> bernoulli(Real p) const {
        return {key_, p, Real(0)};
    }
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::Leaf<Real, VD, detail::kBernoulli, Per<Real, VD>> bernoulli(
        const Per<Real, VD>& p) const {
        return {key_, p, Real(0)};
    }
    /** Integers uniform over [lo, hi]. */
    template <class Int, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::UniformIntLeaf<Int, VD> uniformInt(Int lo, Int hi) const {
        return {key_, lo, hi};
    }
    /** mean + L z per sample, L the Cholesky factor of the covariance. */
    template <class Real, std::size_t VD>
    AETHER_DEVICEANDHOST() constexpr detail::MultivariateNormalLeaf<Real, VD> multivariateNormal(
        const Per<Real, VD>& mean, const LowerTriangular<Real, VD>& L) const {
        return {key_, mean, L};
    }

private:
    std::uint64_t key_;
};

/** The free-function spelling (random/free.h:41-93): the distributions of a
 *  Generator at a fixed seed, and seed(s) naming Generator(s). */
constexpr std::uint64_t DEFAULT_SEED = 0xFE7A5EED0C0FFEE5ull;

AETHER_DEVICEANDHOST() inline Generator seed(std::uint64_t s) { return Generator(s); }

template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto uniform(Real lo, Real hi) {
    return Generator(DEFAULT_SEED).uniform<Real, VD>(lo, hi);
}
template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto normal(Real mean, Real sd) {
    return Generator(DEFAULT_SEED).normal<Real, VD>(mean, sd);
}
template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto lognormal(Real mu, Real sigma) {
    return Generator(DEFAULT_SEED).lognormal<Real, VD>(mu, sigma);
}
template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto exponential(Real lambda) {
    return Generator(DEFAULT_SEED).exponential<Real, VD>(lambda);
}
template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto bernoulli(Real p) {
    return Generator(DEFAULT_SEED).bernoulli<Real, VD>(p);
}
template <class Int, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto uniformInt(Int lo, Int hi) {
    return Generator(DEFAULT_SEED).uniformInt<Int, VD>(lo, hi);
}
template <class Real, std::size_t VD>
AETHER_DEVICEANDHOST() constexpr auto multivariateNormal(const Item<Real, VD>& mean, const LowerTriangular<Real, VD>& L) {
    return Generator(DEFAULT_SEED).multivariateNormal<Real, VD>(mean, L);
}

}  // namespace random
}  // namespace aether
