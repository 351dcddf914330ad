// aether/accum.h -- per-sample compensated accumulation planes.
//
// aether::accum::Plane<VD> (accum/AccumPlane.h:43-502): a value plane and a
// compensation plane per component, both f64, in one array (value planes
// first). `plane += expr` runs one kernel that adds the term to the value and
// the exact residual of that addition to the compensation; add(expr, true)
// does it with atomics so producers on different streams may accumulate into
// one plane at once (the CompensatedAtomic policy). deliver() writes value +
// compensation.
#pragma once

#include <cstddef>

#include "aether/array.h"
#include "aether/eval.h"
#include "aether/expr.h"

namespace aether {
namespace accum {

template <std::size_t VD>
class Plane {
public:
    explicit Plane(std::size_t n) : store_(n) { zero(); }

    using PlaneView = View<double, extents<VD, dyn>, layout_stride>;
    PlaneView value() { return detail::plane_view<double, VD>(store_.deviceView().data(), store_.capacity(), store_.samples()); }
    PlaneView compensation() {
        return detail::plane_view<double, VD>(store_.deviceView().data() + VD * store_.capacity(), store_.capacity(),
                                              store_.samples());
    }
    std::size_t samples() const { return store_.samples(); }

    /** plane += e for every sample (atomic: concurrent producers allowed). */
    void add(const Expr& e, bool atomic = false, Stream s = nullptr) { assign(value(), e, atomic ? "accat" : "acc", s); }
    Plane& operator+=(const Expr& e) {
        add(e);
        return *this;
    }
    /** out = value + compensation. */
    template <class V>
    void deliver(const V& out, Stream s = nullptr) { assign(out, Expr(value() + compensation()), "set", s); }
    void zero(Stream s = nullptr) {
        assign(value(), constant(0.0, ir::Shape{int(VD)}), "set", s);
        assign(compensation(), constant(0.0, ir::Shape{int(VD)}), "set", s);
    }

private:
    Array<double, 2 * VD> store_;
};

}  // namespace accum
}  // namespace aether
