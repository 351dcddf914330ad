// aether/runtime.h -- the runtime-typed strided evaluator.
//
// aether::RuntimeView (view/RuntimeView.h:71-110): an untyped descriptor of
// up to six modes with element strides, here the C-ABI's AetherRuntimeView;
// fromView() describes a device view (components first, samples last, plane
// pitch = capacity). aether::eval::runtimeEval (eval/Runtime.h:228-300)
// validates shapes and dtypes, throws aether::Error before any launch, and
// runs one kernel.
#pragma once

#include <cstdint>

#include "aether/array.h"
#include "aether_gb300.h"

namespace aether {

using RuntimeView = AetherRuntimeView;

/** The descriptor of a device view: its modes (components..., samples) with
 *  the view's own element strides (view/RuntimeView.h:71-110). */
template <class T, class X, class L, bool Vo, bool RO>
RuntimeView fromView(const View<T, X, L, Vo, RO>& v) {
    static_assert(X::Rank <= AETHER_RT_RANK_CAP, "runtime views have at most six modes");
    using U = std::remove_cv_t<T>;
    RuntimeView r{};
    r.data = const_cast<U*>(v.data());
    r.dtype_code = 2;
    r.dtype_bits = uint8_t(sizeof(U) * 8);
    r.dtype_lanes = 1;
    r.rank = int32_t(X::Rank);
    for (std::size_t k = 0; k < X::Rank; ++k) {
        r.extents[k] = int64_t(v.extent(k));
        r.strides[k] = int64_t(v.mapping().stride(k));
    }
    return r;
}

namespace eval {

enum class RuntimeOp : int {
    Assign = AETHER_RT_ASSIGN,
    Add = AETHER_RT_ADD,
    Sub = AETHER_RT_SUB,
    Scale = AETHER_RT_SCALE,
    AddScaled = AETHER_RT_ADD_SCALED,
    SubScaled = AETHER_RT_SUB_SCALED,
};

/** out = op(a, b, scalar) elementwise; `b` is read by Add, Sub, AddScaled and
 *  SubScaled only (pass RuntimeView{} otherwise). */
inline void runtimeEval(RuntimeOp op, const RuntimeView& a, const RuntimeView& b, const RuntimeView& out,
                        double scalar = 0.0, Stream s = nullptr) {
    if (aether_runtime_eval(int(op), &a, &b, &out, scalar, s) != AETHER_OK) throw Error(aether::detail::last_error());
}

}  // namespace eval
}  // namespace aether
