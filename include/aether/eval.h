// aether/eval.h -- assignments: one expression tree, one kernel.
//
// `dst = expr` over every sample (expr/Assign.h:251-346 RecursiveAssign with
// its +=/-= forms, launched as backend/cuda/Launch.h:53-88 does for a
// consumer kernel) becomes: the tree's aether-ir/1 text, a plan compiled once
// per (text, lowering) through aether_plan_create and kept for the process,
// and one aether_plan_launch on the caller's stream. Nothing synchronises;
// errors of the launch throw aether::Error.
#pragma once

#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "aether/array.h"
#include "aether/expr.h"
#include "aether_gb300.h"
#include <cstdint>

namespace aether {
namespace gb300 {

/** Lowering of the kernels this front end compiles. math: 0 FP64 on the FP64
 *  pipe, 1 FP64 emulated on the FP32/INT pipes (double-float, double plans),
 *  2 FP32 storage with float-float arithmetic (float plans), 3 FP64-grade
 *  triple-float on the FP32/INT pipes (double plans), -1 the default for the
 *  destination type (0 for double, 2 for float). contract: 1 FMA contraction,
 *  0 every add and mul rounds, -1 default. Other fields <= 0: tuned default. */
struct Lowering {
    int block = 0, ipt = 0, vec = 0;
    int contract = -1;
    int math = -1;
    int min_blocks = 0;
};

inline Lowering& default_lowering() {
    static Lowering l;
    return l;
}
/** Lowering of every later assignment of this process. */
inline void set_default_lowering(const Lowering& l) { default_lowering() = l; }

namespace detail {

inline std::mutex& plan_mutex() {
    static std::mutex m;
    return m;
}
inline std::map<std::string, void*>& plan_cache() {
    static std::map<std::string, void*> c;
    return c;
}

/** The plan of `text` under `low`, compiled on first use. */
inline void* plan_for(const std::string& text, const std::string& dtype, const Lowering& low) {
    AetherLowering l{low.block, low.ipt, low.vec, low.contract, low.math, low.min_blocks};
    if (l.math < 0) l.math = dtype == "f64" ? 0 : 2;
    const std::string key = text + "|" + std::to_string(l.block) + "/" + std::to_string(l.ipt) + "/" +
                            std::to_string(l.vec) + "/" + std::to_string(l.contract) + "/" + std::to_string(l.math) +
                            "/" + std::to_string(l.min_blocks);
    std::lock_guard<std::mutex> lk(plan_mutex());
    auto it = plan_cache().find(key);
    if (it != plan_cache().end()) return it->second;
    void* p = nullptr;
    if (aether_plan_create(text.c_str(), &l, &p) != AETHER_OK)
        throw Error("plan_create failed (" + aether::detail::last_error() + ")");
    plan_cache().emplace(key, p);
    return p;
}

inline void launch(void* plan, const ir::Context& ctx, std::size_t n, void* dst, std::size_t dst_pitch,
                   double* reduce_out, Stream s) {
    std::vector<AetherOperand> ops;
    for (const ir::OperandSlot& o : ctx.operands) ops.push_back(AetherOperand{o.ptr, o.pitch});
    AetherLaunch a{};
    a.n = n;
    a.dst = dst;
    a.dst_pitch = dst_pitch;
    a.operands = ops.data();
    a.n_operands = uint32_t(ops.size());
    a.scalars = ctx.scalars.data();
    a.n_scalars = uint32_t(ctx.scalars.size());
    a.keys = ctx.keys.data();
    a.n_keys = uint32_t(ctx.keys.size());
    a.reduce_out = reduce_out;
    if (aether_plan_launch(plan, &a, s) != AETHER_OK)
        throw Error("plan_launch failed (" + aether::detail::last_error() + ")");
}

}  // namespace detail
}  // namespace gb300

/** The destination shape of a plan: a rank-0 view takes a 1-vector
 *  expression (a VD = 1 random leaf) as its single component. */
inline ir::Shape dst_shape(const ir::Shape& view_shape, const Expr& e) {
    if (view_shape.empty() && e.shape() == ir::Shape{1}) return e.shape();
    return view_shape;
}

namespace detail {

/** The plane pitch of a view whose components are planes `pitch` elements
 *  apart with samples contiguous (every Array view, every layout_right view):
 *  the only layout the engine's kernels address. Other layouts throw. */
template <class V>
std::uint64_t plane_pitch(const V& v) {
    using X = typename V::extents_type;
    constexpr std::size_t R = X::Rank;
    const auto& m = v.mapping();
    if (m.stride(R - 1) != 1)
        throw Error("aether assign: the engine's kernels need contiguous samples (sample stride " +
                    std::to_string(m.stride(R - 1)) + ")");
    if (R == 1) return v.samples();
    const std::uint64_t pitch = m.stride(R - 2);
    std::uint64_t want = pitch;
    for (std::size_t k = R - 1; k-- > 0;) {
        if (m.stride(k) != want)
            throw Error("aether assign: components must be planes of one pitch in row-major order");
        want *= X::static_extent(k);
    }
    if (pitch < v.samples()) throw Error("aether assign: plane pitch smaller than the sample count");
    return pitch;
}

}  // namespace detail

/** The IR leaf of a device view (operand slot by pointer and pitch). */
template <class V>
Expr gb300_view_leaf(const V& v) {
    using T = typename V::value_type;
    auto n = std::make_shared<ir::Leaf>();
    n->ptr = const_cast<const T*>(v.data());
    n->pitch = detail::plane_pitch(v);
    n->dtype = aether::detail::dtype_name<T>();
    n->shape = ir::shape_of(typename V::element_extents{});
    return Expr(n);
}

/** dst <op>= e for every sample of dst, as one kernel on `s`. op: "set",
 *  "add" or "sub". A rank-0 expression broadcasts over dst's components. */
template <class V>
void assign(const V& dst, const Expr& e, const char* op = "set", Stream s = nullptr,
            const gb300::Lowering& low = gb300::default_lowering()) {
    using T = typename V::value_type;
    const ir::Shape shape = dst_shape(ir::shape_of(typename V::element_extents{}), e);
    Expr ee = e;
    if (e.shape() != shape) {
        if (!e.shape().empty())
            throw Error("aether assign: expression of shape " + ir::shape_text(e.shape()) + " into a view of shape " +
                        ir::shape_text(shape));
        ee = Expr(ir::bcast(e.node(), shape));
    }
    if (dst.samples() == 0) return;
    ir::Context ctx;
    const std::string dtype = aether::detail::dtype_name<T>();
    const std::string text = plan_text(dtype, shape, op, ee, ctx);
    void* plan = gb300::detail::plan_for(text, dtype, low);
    gb300::detail::launch(plan, ctx, dst.samples(), const_cast<T*>(dst.data()), detail::plane_pitch(dst), nullptr, s);
}

template <class V, class E>
void gb300_assign_view(const V& dst, const E& e, const char* op) {
    assign(dst, Expr(e), op);
}

/** Alias of assign (the reference's whole-view evaluation, backend/cpu/Tiled.h:185). */
template <class V>
void packetEval(const V& dst, const Expr& e, Stream s = nullptr) {
    assign(dst, e, "set", s);
}

/** Compensated sum over n samples of a rank-0 expression, reduced in a fixed
 *  order: returns (hi, comp) with hi + comp the sum. Synchronises `s`. The
 *  reference has no grid-level driver for its compensated accumulators
 *  (accum/TwoSum.h:86-155, accum/atomic.h:141-258); this is that driver. */
inline std::pair<double, double> globalSum(const Expr& e, std::size_t n, Stream s = nullptr,
                                           const gb300::Lowering& low = gb300::default_lowering()) {
    if (!e.shape().empty()) throw Error("aether globalSum: the expression must be rank 0");
    ir::Context ctx;
    const std::string text = plan_text("f64", {}, "sum", e, ctx);
    void* plan = gb300::detail::plan_for(text, "f64", low);
    aether::detail::Chunk out(AETHER_MEM_DEVICE, 16, "device 0");
    const double zero[2] = {0.0, 0.0};
    aether::detail::copy(out.get(), AETHER_MEM_DEVICE, zero, AETHER_MEM_CPU, 16, s, "globalSum");
    gb300::detail::launch(plan, ctx, n, nullptr, 0, static_cast<double*>(out.get()), s);
    double r[2];
    aether::detail::copy(r, AETHER_MEM_CPU, out.get(), AETHER_MEM_DEVICE, 16, s, "globalSum");
    aether::detail::sync(s);
    return {r[0], r[1]};
}

}  // namespace aether
