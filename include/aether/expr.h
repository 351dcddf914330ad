// aether/expr.h -- the engine's type-erased expressions (aether-ir/1).
//
// Expr is a handle on an immutable expression tree whose shape is known at
// run time: the form every typed expression (aether/expression.h) is
// serialised to before the engine compiles it, and a builder in its own right
// for trees assembled at run time. It carries the operators of
// expr/Operations.h:25-71 (+, -, Hadamard *, s*e, e*s, e/s = e*(1/s)), the
// elementwise functions of expr/nodes/Elementwise.h:61-854 and the member
// functions of expr/Expression.h:127-486, with one difference from the typed
// layer: dot, squaredNorm, norm, sum, det and trace are per-sample folds
// here. Shapes are checked when the tree is built and a mismatch throws
// aether::Error. An assignment (aether/eval.h) serialises the tree to one
// aether-ir/1 text and runs it as one kernel.
//
// The text is the same one the Python front end (aether_gb300/expr.py) writes
// for the same tree, so a plan compiled from either is shared.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "aether/expression.h"
#include "aether/layout.h"

namespace aether {

/** Errors of the host API (err/Error.h:30-87): "<op> failed on <where>,
 *  size=<bytes> bytes (<detail>)" for memory operations, the plain detail
 *  otherwise. */
class Error : public std::runtime_error {
public:
    explicit Error(const std::string& what) : std::runtime_error(what) {}
    static Error memory(const std::string& op, const std::string& where, std::size_t bytes, const std::string& detail) {
        return Error(op + " failed on " + where + ", size=" + std::to_string(bytes) + " bytes (" + detail + ")");
    }
};

namespace ir {

using Shape = std::vector<int>;

inline std::string shape_text(const Shape& s) {
    std::string t = "[";
    for (std::size_t i = 0; i < s.size(); ++i) {
        if (i) t += ",";
        t += std::to_string(s[i]);
    }
    return t + "]";
}

inline int prod(const Shape& s) {
    int p = 1;
    for (int e : s) p *= e;
    return p;
}

template <std::size_t... Es>
Shape shape_of(extents<Es...>) {
    Shape s;
    for (std::size_t e : {Es...})
        if (e != dyn) s.push_back(int(e));
    return s;
}
inline Shape shape_of(extents<>) { return {}; }

/** Hexadecimal text of a double in the form Python's float.hex() writes. */
inline std::string hex_double(double v) {
    if (std::isnan(v)) return "nan";
    if (std::isinf(v)) return v < 0 ? "-inf" : "inf";
    std::uint64_t b;
    std::memcpy(&b, &v, 8);
    const bool neg = b >> 63;
    const int e = int((b >> 52) & 0x7FF);
    const std::uint64_t m = b & ((std::uint64_t(1) << 52) - 1);
    char buf[64];
    if (e == 0 && m == 0) {
        std::snprintf(buf, sizeof buf, "%s0x0.0p+0", neg ? "-" : "");
    } else if (e == 0) {
        std::snprintf(buf, sizeof buf, "%s0x0.%013llxp-1022", neg ? "-" : "", (unsigned long long)m);
    } else {
        const int ex = e - 1023;
        std::snprintf(buf, sizeof buf, "%s0x1.%013llxp%c%d", neg ? "-" : "", (unsigned long long)m, ex < 0 ? '-' : '+',
                      ex < 0 ? -ex : ex);
    }
    return buf;
}

/** One operand slot: a device SoA array (plane c at ptr + c*pitch elements). */
struct OperandSlot {
    const void* ptr;
    std::uint64_t pitch;
    std::string dtype;
    int comps;
};

/** Slot assignment for one plan: operands by buffer identity, scalars and
 *  generator keys in order of first use. */
struct Context {
    std::vector<OperandSlot> operands;
    std::vector<double> scalars;
    std::vector<std::uint64_t> keys;
    int operand(const void* ptr, std::uint64_t pitch, const std::string& dtype, int comps) {
        for (std::size_t i = 0; i < operands.size(); ++i) {
            const OperandSlot& o = operands[i];
            if (o.ptr == ptr && o.pitch == pitch && o.dtype == dtype && o.comps == comps) return int(i);
        }
        operands.push_back(OperandSlot{ptr, pitch, dtype, comps});
        return int(operands.size()) - 1;
    }
    int scalar(double v) {
        scalars.push_back(v);
        return int(scalars.size()) - 1;
    }
    int key(std::uint64_t k) {
        for (std::size_t i = 0; i < keys.size(); ++i)
            if (keys[i] == k) return int(i);
        keys.push_back(k);
        return int(keys.size()) - 1;
    }
};

struct Node {
    Shape shape;
    bool is_bool = false;
    virtual ~Node() = default;
    virtual std::string text(Context& ctx) const = 0;
};
using NodeP = std::shared_ptr<const Node>;

struct Op : Node {
    std::string op;
    std::vector<NodeP> kids;
    std::vector<int> ints;
    std::string tail;
    std::string text(Context& ctx) const override {
        std::string t = "(" + op;
        for (const NodeP& k : kids) t += " " + k->text(ctx);
        for (int i : ints) t += " " + std::to_string(i);
        if (!tail.empty()) t += " " + tail;
        return t + ")";
    }
};

struct Leaf : Node {
    const void* ptr;
    std::uint64_t pitch;
    std::string dtype;
    std::string text(Context& ctx) const override {
        return "(in " + std::to_string(ctx.operand(ptr, pitch, dtype, prod(shape))) + " " + dtype + " " +
               shape_text(shape) + ")";
    }
};

struct ScalarNode : Node {
    double v;
    // a non-negative value is marked so the plan can drop cancellation-safe sums
    std::string text(Context& ctx) const override {
        return "(sc " + std::to_string(ctx.scalar(v)) + (v >= 0.0 ? " +)" : ")");
    }
};

struct LiteralNode : Node {
    double v;
    std::string text(Context&) const override { return "(lit " + hex_double(v) + ")"; }
};

struct BcastNode : Node {
    NodeP s;
    std::string text(Context& ctx) const override { return "(bcast " + s->text(ctx) + " " + shape_text(shape) + ")"; }
};

struct RandomNode : Node {
    std::string op;
    std::uint64_t key;
    std::vector<NodeP> params;
    std::string text(Context& ctx) const override {
        std::string t = "(" + op + " " + std::to_string(ctx.key(key));
        for (const NodeP& p : params) t += " " + p->text(ctx);
        return t + " " + std::to_string(shape.at(0)) + ")";
    }
};

inline NodeP scalar(double v) {
    auto n = std::make_shared<ScalarNode>();
    n->v = v;
    return n;
}

inline NodeP op(const std::string& name, std::vector<NodeP> kids, Shape shape, bool is_bool = false,
                std::vector<int> ints = {}, std::string tail = {}) {
    auto n = std::make_shared<Op>();
    n->op = name;
    n->kids = std::move(kids);
    n->shape = std::move(shape);
    n->is_bool = is_bool;
    n->ints = std::move(ints);
    n->tail = std::move(tail);
    return n;
}

inline NodeP bcast(NodeP s, const Shape& shape) {
    if (shape.empty()) return s;
    auto n = std::make_shared<BcastNode>();
    n->s = std::move(s);
    n->shape = shape;
    return n;
}

}  // namespace ir

/** A lazy expression: a handle on an immutable tree. Views, random leaves
 *  and constants convert to it. */
class Expr {
public:
    Expr() = default;
    explicit Expr(ir::NodeP n) : node_(std::move(n)) {}
    /** The tree of a typed expression (its type signature, with the operand
     *  pointers, scalars and keys it holds). */
    template <class E, std::enable_if_t<aether_expression<E>, int> = 0>
    Expr(const E& e) : Expr(e.gb300_ir()) {}
    const ir::Shape& shape() const { return node_->shape; }
    bool is_bool() const { return node_->is_bool; }
    const ir::NodeP& node() const { return node_; }
    std::string text(ir::Context& ctx) const { return node_->text(ctx); }

    // -- member surface of Expression<Derived, T> (expr/Expression.h) -----
    Expr dot(const Expr& o) const { return bin_("dot", o, {}, true); }
    Expr squaredNorm() const { return un_("sqnorm", {}); }
    Expr norm() const { return un_("norm", {}); }
    Expr rNorm() const { return un_("rnorm", {}); }
    Expr sum() const { return un_("sum", {}); }
    Expr maxNorm() const { return un_("maxnorm", {}); }
    Expr cross(const Expr& o) const {
        need_(shape() == ir::Shape{3} && o.shape() == ir::Shape{3}, "cross needs two 3-vectors");
        return bin_("cross", o, {3}, false);
    }
    Expr unitVector() const { return un_("unit", shape()); }
    Expr quatMul(const Expr& o) const {
        need_(shape() == ir::Shape{4} && o.shape() == ir::Shape{4}, "quatMul needs two quaternions");
        return bin_("qmul", o, {4}, false);
    }
    Expr quatConj() const {
        need_(shape() == ir::Shape{4}, "quatConj needs a quaternion");
        return un_("qconj", {4});
    }
    Expr quatRotate(const Expr& v) const {
        need_(shape() == ir::Shape{4} && v.shape() == ir::Shape{3}, "quatRotate needs a quaternion and a 3-vector");
        return bin_("qrot", v, {3}, false);
    }
    Expr asPureQuaternion() const {
        need_(shape() == ir::Shape{3}, "asPureQuaternion needs a 3-vector");
        return un_("pureq", {4});
    }
    Expr inverse() const { return un_("inv", shape()); }
    Expr det() const { return un_("det", {}); }
    Expr trace() const { return un_("trace", {}); }
    Expr transpose() const {
        need_(shape().size() == 2, "transpose needs a matrix");
        return un_("transpose", {shape()[1], shape()[0]});
    }
    Expr row(int r) const {
        need_(shape().size() == 2, "row needs a matrix");
        return Expr(ir::op("row", {node_}, {shape()[1]}, false, {r}));
    }
    Expr col(int c) const {
        need_(shape().size() == 2, "col needs a matrix");
        return Expr(ir::op("col", {node_}, {shape()[0]}, false, {c}));
    }
    Expr segment(int off, int len) const { return Expr(ir::op("seg", {node_}, {len}, false, {off, len})); }
    Expr head(int n) const { return segment(0, n); }
    Expr tail(int n) const { return segment(shape().at(0) - n, n); }
    Expr block(int r0, int c0, int br, int bc) const {
        return Expr(ir::op("block", {node_}, {br, bc}, false, {r0, c0, br, bc}));
    }
    Expr component(int k) const { return Expr(ir::op("comp", {node_}, {}, false, {k})); }
    template <std::size_t K>
    Expr component() const { return component(int(K)); }
    Expr matvec(const Expr& v) const { return bin_("matvec", v, {shape().at(0)}, false); }
    Expr matmul(const Expr& o) const { return bin_("matmul", o, {shape().at(0), o.shape().at(1)}, false); }
    Expr outer(const Expr& o) const { return bin_("outer", o, {shape().at(0), o.shape().at(0)}, false); }
    Expr reshape(const ir::Shape& s) const {
        need_(ir::prod(s) == ir::prod(shape()), "reshape changes the component count");
        return Expr(ir::op("reshape", {node_}, s, false, {}, ir::shape_text(s)));
    }
    /** Every sample reads sample 0 (a per-launch constant taken from an array). */
    Expr atSample0() const { return Expr(ir::op("at0", {node_}, shape(), is_bool())); }

private:
    static void need_(bool ok, const char* what) {
        if (!ok) throw Error(std::string("aether expression: ") + what);
    }
    Expr un_(const char* name, ir::Shape s) const { return Expr(ir::op(name, {node_}, std::move(s))); }
    Expr bin_(const char* name, const Expr& o, ir::Shape s, bool scalar_out) const {
        (void)scalar_out;
        return Expr(ir::op(name, {node_, o.node_}, std::move(s)));
    }
    ir::NodeP node_;
};

namespace detail {
inline Expr as_expr(double v, const ir::Shape& shape) { return Expr(ir::bcast(ir::scalar(v), shape)); }
inline Expr as_expr(const Expr& e, const ir::Shape& shape) {
    if (e.shape().empty() && !shape.empty()) return Expr(ir::bcast(e.node(), shape));
    return e;
}
inline void check_same_shape(const Expr& a, const Expr& b, const char* op) {
    if (a.shape() != b.shape())
        throw Error(std::string("aether expression: ") + op + " of shapes " + ir::shape_text(a.shape()) + " and " +
                    ir::shape_text(b.shape()));
}
}  // namespace detail

// -- operators (expr/Operations.h:25-71) -------------------------------------
inline Expr operator+(const Expr& a, const Expr& b) {
    const Expr r = detail::as_expr(b, a.shape());
    const Expr l = detail::as_expr(a, r.shape());
    detail::check_same_shape(l, r, "+");
    return Expr(ir::op("add", {l.node(), r.node()}, l.shape()));
}
inline Expr operator+(const Expr& a, double s) { return Expr(ir::op("add", {a.node(), detail::as_expr(s, a.shape()).node()}, a.shape())); }
inline Expr operator+(double s, const Expr& a) { return Expr(ir::op("add", {detail::as_expr(s, a.shape()).node(), a.node()}, a.shape())); }
inline Expr operator-(const Expr& a, const Expr& b) {
    const Expr r = detail::as_expr(b, a.shape());
    const Expr l = detail::as_expr(a, r.shape());
    detail::check_same_shape(l, r, "-");
    return Expr(ir::op("sub", {l.node(), r.node()}, l.shape()));
}
inline Expr operator-(const Expr& a, double s) { return Expr(ir::op("sub", {a.node(), detail::as_expr(s, a.shape()).node()}, a.shape())); }
inline Expr operator-(double s, const Expr& a) { return Expr(ir::op("sub", {detail::as_expr(s, a.shape()).node(), a.node()}, a.shape())); }
/** Hadamard product; a rank-0 factor scales (CWiseScale). */
inline Expr operator*(const Expr& a, const Expr& b) {
    if (b.shape().empty() && !a.shape().empty()) return Expr(ir::op("scale", {a.node(), b.node()}, a.shape()));
    if (a.shape().empty() && !b.shape().empty()) return Expr(ir::op("mul", {a.node(), b.node()}, a.shape()));
    detail::check_same_shape(a, b, "*");
    return Expr(ir::op("mul", {a.node(), b.node()}, a.shape()));
}
inline Expr operator*(const Expr& a, double s) { return Expr(ir::op("scale", {a.node(), ir::scalar(s)}, a.shape())); }
inline Expr operator*(double s, const Expr& a) { return Expr(ir::op("scale", {a.node(), ir::scalar(s)}, a.shape())); }
/** e / s is e * (1/s), the reciprocal rounded once on the host. */
inline Expr operator/(const Expr& a, double s) { return Expr(ir::op("scale", {a.node(), ir::scalar(1.0 / s)}, a.shape())); }
inline Expr operator/(const Expr& a, const Expr& b) { return Expr(ir::op("div", {a.node(), b.node()}, a.shape())); }
inline Expr operator-(const Expr& a) { return Expr(ir::op("neg", {a.node()}, a.shape())); }

#define AETHER_GB300_CMP(OPER, NAME)                                                                     \
    inline Expr operator OPER(const Expr& a, const Expr& b) {                                          \
        return Expr(ir::op(NAME, {a.node(), detail::as_expr(b, a.shape()).node()}, a.shape(), true)); \
    }                                                                                                  \
    inline Expr operator OPER(const Expr& a, double s) {                                               \
        return Expr(ir::op(NAME, {a.node(), detail::as_expr(s, a.shape()).node()}, a.shape(), true)); \
    }
AETHER_GB300_CMP(>, "gt")
AETHER_GB300_CMP(<, "lt")
AETHER_GB300_CMP(>=, "ge")
AETHER_GB300_CMP(<=, "le")
#undef AETHER_GB300_CMP

// -- elementwise functions (expr/nodes/Elementwise.h) ------------------------
#define AETHER_GB300_UNARY(FN, NAME) \
    inline Expr FN(const Expr& e) { return Expr(ir::op(NAME, {e.node()}, e.shape())); }
AETHER_GB300_UNARY(cwiseSqrt, "sqrt")
AETHER_GB300_UNARY(cwiseRsqrt, "rsqrt")
AETHER_GB300_UNARY(cwiseExp, "exp")
AETHER_GB300_UNARY(cwiseExpm1, "expm1")
AETHER_GB300_UNARY(cwiseLog, "log")
AETHER_GB300_UNARY(cwiseLog1p, "log1p")
AETHER_GB300_UNARY(cwiseLog2, "log2")
AETHER_GB300_UNARY(cwiseLog10, "log10")
AETHER_GB300_UNARY(cwiseExp2, "exp2")
AETHER_GB300_UNARY(cwiseSin, "sin")
AETHER_GB300_UNARY(cwiseCos, "cos")
AETHER_GB300_UNARY(cwiseTan, "tan")
AETHER_GB300_UNARY(cwiseAsin, "asin")
AETHER_GB300_UNARY(cwiseAcos, "acos")
AETHER_GB300_UNARY(cwiseAtan, "atan")
AETHER_GB300_UNARY(cwiseTanh, "tanh")
AETHER_GB300_UNARY(cwiseSinh, "sinh")
AETHER_GB300_UNARY(cwiseCosh, "cosh")
AETHER_GB300_UNARY(cwiseAbs, "abs")
AETHER_GB300_UNARY(cwiseSign, "sign")
AETHER_GB300_UNARY(cwiseSquare, "sq")
AETHER_GB300_UNARY(cwiseFloor, "floor")
AETHER_GB300_UNARY(cwiseCeil, "ceil")
AETHER_GB300_UNARY(cwiseTrunc, "trunc")
AETHER_GB300_UNARY(cwiseCbrt, "cbrt")
AETHER_GB300_UNARY(cwiseErf, "erf")
#undef AETHER_GB300_UNARY

inline Expr cwiseMin(const Expr& e, const Expr& o) {
    if (o.shape() == e.shape()) return Expr(ir::op("min", {e.node(), o.node()}, e.shape()));
    return Expr(ir::op("mins", {e.node(), o.node()}, e.shape()));
}
inline Expr cwiseMin(const Expr& e, double s) { return Expr(ir::op("mins", {e.node(), ir::scalar(s)}, e.shape())); }
inline Expr cwiseMax(const Expr& e, const Expr& o) {
    if (o.shape() == e.shape()) return Expr(ir::op("max", {e.node(), o.node()}, e.shape()));
    return Expr(ir::op("maxs", {e.node(), o.node()}, e.shape()));
}
inline Expr cwiseMax(const Expr& e, double s) { return Expr(ir::op("maxs", {e.node(), ir::scalar(s)}, e.shape())); }
inline Expr clamp(const Expr& e, double lo, double hi) {
    return Expr(ir::op("clamp", {e.node(), ir::scalar(lo), ir::scalar(hi)}, e.shape()));
}
inline Expr cwiseDiv(const Expr& l, const Expr& r) { return Expr(ir::op("div", {l.node(), r.node()}, l.shape())); }
inline Expr cwisePow(const Expr& e, const Expr& p) {
    if (p.shape() == e.shape()) return Expr(ir::op("pow", {e.node(), p.node()}, e.shape()));
    return Expr(ir::op("pows", {e.node(), p.node()}, e.shape()));
}
inline Expr cwisePow(const Expr& e, double p) { return Expr(ir::op("pows", {e.node(), ir::scalar(p)}, e.shape())); }
/** select(cond, a, b) (expr/nodes/Elementwise.h:809). */
inline Expr select(const Expr& c, const Expr& a, const Expr& b) {
    return Expr(ir::op("select", {c.node(), a.node(), b.node()}, a.shape()));
}

/** A scalar broadcast to `Extents` (expr/nodes/Constant.h:98-150): a runtime
 *  scalar, except for 1, -1, 2 and 1/2, which the kernels bake in (a handful of
 *  values, so the plan cache stays small; their magnitude bounds let the
 *  generator drop range tests). */
inline ir::NodeP constant_node(double v) {
    if (v == 1.0 || v == -1.0 || v == 2.0 || v == 0.5) {
        auto n = std::make_shared<ir::LiteralNode>();
        n->v = v;
        return n;
    }
    return ir::scalar(v);
}
inline Expr constant(double v, const ir::Shape& shape) { return Expr(ir::bcast(constant_node(v), shape)); }
/** A scalar baked into the kernel text (compiled once per value). */
inline Expr literal(double v) {
    auto n = std::make_shared<ir::LiteralNode>();
    n->v = v;
    return Expr(n);
}
/** N rank-0 expressions as one N-vector. */
inline Expr stack(std::initializer_list<Expr> items) {
    std::vector<ir::NodeP> k;
    for (const Expr& e : items) k.push_back(e.node());
    const int n = int(k.size());
    return Expr(ir::op("stack", std::move(k), {n}));
}

/** The aether-ir/1 text of `dst <op>= expr` (op: set, add, sub, sum, setsum). */
inline std::string plan_text(const std::string& dtype, const ir::Shape& dst_shape, const std::string& op,
                             const Expr& e, ir::Context& ctx) {
    return "(plan " + dtype + " " + ir::shape_text(dst_shape) + " " + op + " " + e.text(ctx) + ")";
}

}  // namespace aether
