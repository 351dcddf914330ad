// plan.cpp -- aether-ir/1 parser, shape checker and CUDA generator.
//
// The grammar is an S-expression over the node kinds of the reference's
// expression layer (expr/nodes/*.h, expr/Reduce.h, random/detail/
// DistributionLeaf.h). Each generated formula keeps the reference's operand
// order and association, so with contraction off the arithmetic nodes round
// exactly as the reference's `-ffp-contract=off` CPU build does.

#include "plan.h"

#include <cstdio>
#include <cstring>
#include <map>
#include <cmath>
#include <set>
#include <sstream>
#include <stdexcept>

namespace ag {

const char* dtype_name(DType d) {
    switch (d) {
    case DType::F64: return "f64";
    case DType::F32: return "f32";
    case DType::FF: return "ff";
    case DType::I32: return "i32";
    case DType::U8: return "u8";
    }
    return "?";
}
int dtype_size(DType d) {
    switch (d) {
    case DType::F64: return 8;
    case DType::F32: return 4;
    case DType::FF: return 4;
    case DType::I32: return 4;
    case DType::U8: return 1;
    }
    return 8;
}

namespace {

[[noreturn]] void fail(const std::string& m) { throw std::runtime_error("aether-ir: " + m); }

DType parse_dtype(const std::string& t) {
    if (t == "f64") return DType::F64;
    if (t == "f32") return DType::F32;
    if (t == "ff") return DType::FF;
    if (t == "i32") return DType::I32;
    if (t == "u8") return DType::U8;
    fail("unknown dtype '" + t + "'");
}

std::vector<int> parse_shape(const std::string& t) {
    if (t.size() < 2 || t.front() != '[' || t.back() != ']') fail("bad shape '" + t + "'");
    std::vector<int> s;
    const std::string inner = t.substr(1, t.size() - 2);
    size_t i = 0;
    while (i < inner.size()) {
        size_t j = inner.find(',', i);
        if (j == std::string::npos) j = inner.size();
        const int v = std::stoi(inner.substr(i, j - i));
        if (v <= 0 || v > 64) fail("extent out of range in " + t);
        s.push_back(v);
        i = j + 1;
    }
    if (s.size() > 2) fail("rank > 2 element shapes are not supported: " + t);
    return s;
}

int prod(const std::vector<int>& s) {
    int p = 1;
    for (int v : s) p *= v;
    return p;
}

const std::set<std::string>& unary_ops() {
    static const std::set<std::string> s = {"neg", "abs", "sign", "sqrt", "rsqrt", "exp", "expm1", "log", "log1p",
                                            "log2", "log10", "exp2", "sin", "cos", "tan", "asin", "acos", "atan",
                                            "tanh", "sinh", "cosh", "sq", "floor", "ceil", "trunc", "cbrt", "erf"};
    return s;
}
const std::set<std::string>& binary_ops() {
    static const std::set<std::string> s = {"add", "sub", "mul", "div", "pow", "min", "max", "atan2", "hypot"};
    return s;
}
const std::set<std::string>& cmp_ops() {
    static const std::set<std::string> s = {"gt", "lt", "ge", "le", "eq", "ne", "and", "or"};
    return s;
}

struct Parser {
    const char* p;
    const char* begin;
    Plan plan;
    std::map<std::string, int> memo;
    int ctx = 0;   // 0: the lane's own sample; 1: sample 0 (inside at0)
    std::vector<int> node_ctx;

    explicit Parser(const char* s) : p(s), begin(s) {}

    void ws() {
        while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') ++p;
    }
    std::string tok() {
        ws();
        if (!*p) fail("unexpected end of text");
        if (*p == '(' || *p == ')') return std::string(1, *p++);
        const char* s = p;
        if (*p == '[') {
            while (*p && *p != ']') ++p;
            if (*p != ']') fail("unterminated shape");
            ++p;
            return std::string(s, p);
        }
        while (*p && *p != ' ' && *p != '(' && *p != ')' && *p != '\n' && *p != '\t' && *p != '\r') ++p;
        return std::string(s, p);
    }
    std::string peek() {
        const char* save = p;
        std::string t = tok();
        p = save;
        return t;
    }
    void expect(const char* t) {
        const std::string g = tok();
        if (g != t) fail(std::string("expected '") + t + "' but found '" + g + "' at offset " + std::to_string(p - begin));
    }
    int integer() {
        const std::string t = tok();
        char* end = nullptr;
        const long v = std::strtol(t.c_str(), &end, 10);
        if (!end || *end) fail("expected an integer, found '" + t + "'");
        return int(v);
    }
    const Node& N(int i) const { return plan.nodes[size_t(i)]; }

    int expr() {
        const char* start = p;
        expect("(");
        Node n;
        n.op = tok();
        const std::string op = n.op;
        auto kid = [&]() {
            const int c = expr();
            n.kids.push_back(c);
            return c;
        };
        auto same_shape = [&](int a, int b) {
            if (N(a).shape != N(b).shape) fail("operand shapes differ in '" + op + "'");
        };
        auto rank0 = [&](int a) {
            if (!N(a).shape.empty()) fail("'" + op + "' needs a rank-0 operand");
        };
        auto num = [&](int a) {
            if (N(a).is_bool) fail("'" + op + "' needs a numeric operand");
        };
        if (op == "in") {
            n.k = integer();
            if (n.k < 0 || n.k >= 16) fail("operand slot out of range");
            n.dtype = parse_dtype(tok());
            n.shape = parse_shape(tok());
            if (plan.n_operands <= n.k) {
                plan.n_operands = n.k + 1;
                plan.operand_dtype.resize(size_t(n.k) + 1, DType::F64);
                plan.operand_comps.resize(size_t(n.k) + 1, 0);
            }
            if (plan.operand_comps[size_t(n.k)] && (plan.operand_comps[size_t(n.k)] != prod(n.shape) ||
                                                    plan.operand_dtype[size_t(n.k)] != n.dtype))
                fail("operand " + std::to_string(n.k) + " declared twice with different types");
            plan.operand_comps[size_t(n.k)] = prod(n.shape);
            plan.operand_dtype[size_t(n.k)] = n.dtype;
            n.is_bool = n.dtype == DType::U8;
        } else if (op == "sc") {
            n.k = integer();
            if (n.k < 0 || n.k >= 16) fail("scalar slot out of range");
            plan.n_scalars = std::max(plan.n_scalars, n.k + 1);
            if (peek() == "+") {
                tok();
                n.nonneg_hint = true;
                plan.scalar_nonneg.resize(size_t(plan.n_scalars), 0);
                plan.scalar_nonneg[size_t(n.k)] = 1;
            }
        } else if (op == "lit") {
            const std::string t = tok();
            char* end = nullptr;
            n.lit = std::strtod(t.c_str(), &end);
            if (!end || *end) fail("bad literal '" + t + "'");
        } else if (op == "bcast") {
            const int a = kid();
            rank0(a);
            n.shape = parse_shape(tok());
            n.is_bool = N(a).is_bool;
        } else if (op == "at0") {
            const int save = ctx;
            ctx = 1;
            const int a = kid();
            ctx = save;
            n.shape = N(a).shape;
            n.is_bool = N(a).is_bool;
        } else if (unary_ops().count(op)) {
            const int a = kid();
            num(a);
            n.shape = N(a).shape;
        } else if (binary_ops().count(op)) {
            const int a = kid(), b = kid();
            same_shape(a, b);
            num(a);
            num(b);
            n.shape = N(a).shape;
        } else if (op == "scale" || op == "mins" || op == "maxs" || op == "pows") {
            const int a = kid(), s = kid();
            rank0(s);
            n.shape = N(a).shape;
        } else if (op == "clamp") {
            const int a = kid(), lo = kid(), hi = kid();
            rank0(lo);
            rank0(hi);
            n.shape = N(a).shape;
        } else if (cmp_ops().count(op)) {
            const int a = kid(), b = kid();
            same_shape(a, b);
            n.shape = N(a).shape;
            n.is_bool = true;
        } else if (op == "not") {
            const int a = kid();
            n.shape = N(a).shape;
            n.is_bool = true;
        } else if (op == "select") {
            const int c = kid(), a = kid(), b = kid();
            same_shape(a, b);
            if (!N(c).is_bool) fail("select condition must be boolean");
            if (!N(c).shape.empty() && N(c).shape != N(a).shape) fail("select condition shape");
            n.shape = N(a).shape;
            n.is_bool = N(a).is_bool;
        } else if (op == "comp") {
            const int a = kid();
            n.k = integer();
            if (n.k < 0 || n.k >= N(a).comps) fail("comp index out of range");
        } else if (op == "seg") {
            const int a = kid();
            n.k = integer();
            n.ints = {integer()};
            if (N(a).shape.size() != 1 || n.k < 0 || n.ints[0] <= 0 || n.k + n.ints[0] > N(a).comps)
                fail("seg out of range");
            n.shape = {n.ints[0]};
        } else if (op == "row" || op == "col") {
            const int a = kid();
            n.k = integer();
            if (N(a).shape.size() != 2) fail(op + " needs a matrix");
            const int lim = op == "row" ? N(a).shape[0] : N(a).shape[1];
            if (n.k < 0 || n.k >= lim) fail(op + " index out of range");
            n.shape = {op == "row" ? N(a).shape[1] : N(a).shape[0]};
        } else if (op == "transpose") {
            const int a = kid();
            if (N(a).shape.size() != 2) fail("transpose needs a matrix");
            n.shape = {N(a).shape[1], N(a).shape[0]};
        } else if (op == "block") {
            const int a = kid();
            n.ints = {integer(), integer(), integer(), integer()};
            if (N(a).shape.size() != 2 || n.ints[0] + n.ints[2] > N(a).shape[0] || n.ints[1] + n.ints[3] > N(a).shape[1])
                fail("block out of range");
            n.shape = {n.ints[2], n.ints[3]};
        } else if (op == "stack") {
            while (peek() != ")") rank0(kid());
            if (n.kids.empty()) fail("empty stack");
            n.shape = {int(n.kids.size())};
        } else if (op == "reshape") {
            const int a = kid();
            n.shape = parse_shape(tok());
            if (prod(n.shape) != N(a).comps) fail("reshape changes the component count");
        } else if (op == "cross") {
            const int a = kid(), b = kid();
            same_shape(a, b);
            if (N(a).shape != std::vector<int>{3}) fail("cross needs [3] operands");
            n.shape = {3};
        } else if (op == "unit") {
            const int a = kid();
            if (N(a).shape.size() != 1) fail("unit needs a vector");
            n.shape = N(a).shape;
        } else if (op == "qconj") {
            const int a = kid();
            if (N(a).shape != std::vector<int>{4}) fail("qconj needs [4]");
            n.shape = {4};
        } else if (op == "qmul") {
            const int a = kid(), b = kid();
            if (N(a).shape != std::vector<int>{4} || N(b).shape != std::vector<int>{4}) fail("qmul needs [4] operands");
            n.shape = {4};
        } else if (op == "qrot") {
            const int a = kid(), b = kid();
            if (N(a).shape != std::vector<int>{4} || N(b).shape != std::vector<int>{3}) fail("qrot needs [4] and [3]");
            n.shape = {3};
        } else if (op == "pureq") {
            const int a = kid();
            if (N(a).shape != std::vector<int>{3}) fail("pureq needs [3]");
            n.shape = {4};
        } else if (op == "inv" || op == "det" || op == "trace") {
            const int a = kid();
            const auto& s = N(a).shape;
            if (s.size() != 2 || s[0] != s[1] || (s[0] != 2 && s[0] != 3)) fail(op + " needs a 2x2 or 3x3 matrix");
            if (op == "inv") n.shape = s;
        } else if (op == "matvec") {
            const int m = kid(), v = kid();
            if (N(m).shape.size() != 2 || N(v).shape.size() != 1 || N(m).shape[1] != N(v).shape[0]) fail("matvec shapes");
            n.shape = {N(m).shape[0]};
        } else if (op == "matmul") {
            const int a = kid(), b = kid();
            if (N(a).shape.size() != 2 || N(b).shape.size() != 2 || N(a).shape[1] != N(b).shape[0]) fail("matmul shapes");
            n.shape = {N(a).shape[0], N(b).shape[1]};
        } else if (op == "outer") {
            const int a = kid(), b = kid();
            if (N(a).shape.size() != 1 || N(b).shape.size() != 1) fail("outer needs vectors");
            n.shape = {N(a).shape[0], N(b).shape[0]};
        } else if (op == "dot") {
            const int a = kid(), b = kid();
            same_shape(a, b);
            if (N(a).shape.size() != 1) fail("dot needs vectors");
        } else if (op == "sqnorm" || op == "norm" || op == "rnorm" || op == "sum" || op == "maxnorm") {
            const int a = kid();
            if (N(a).shape.size() != 1) fail(op + " needs a vector");
        } else if (op == "uniform" || op == "normal" || op == "lognormal" || op == "exponential" || op == "bernoulli") {
            n.k = integer();
            if (n.k < 0 || n.k >= 8) fail("key slot out of range");
            plan.n_keys = std::max(plan.n_keys, n.k + 1);
            const int p0 = kid();
            const bool two = op == "uniform" || op == "normal" || op == "lognormal";
            const int p1 = two ? kid() : -1;
            const int vd = integer();
            if (vd <= 0 || vd > 64) fail("distribution dimension out of range");
            n.shape = {vd};
            for (int q : {p0, p1}) {
                if (q < 0) continue;
                if (!N(q).shape.empty() && N(q).shape != n.shape) fail(op + " parameter shape");
            }
            plan.has_random = true;
        } else {
            fail("unknown node '" + op + "'");
        }
        expect(")");
        n.comps = prod(n.shape);
        const std::string key = std::to_string(ctx) + std::string(start, p);
        auto it = memo.find(key);
        if (it != memo.end()) return it->second;
        plan.nodes.push_back(std::move(n));
        node_ctx.push_back(ctx);
        const int id = int(plan.nodes.size()) - 1;
        memo.emplace(key, id);
        return id;
    }

    Plan run() {
        expect("(");
        expect("plan");
        plan.dst_dtype = parse_dtype(tok());
        if (plan.dst_dtype != DType::F64 && plan.dst_dtype != DType::F32 && plan.dst_dtype != DType::FF)
            fail("destination dtype must be f64, f32 or ff");
        plan.dst_shape = parse_shape(tok());
        plan.dst_comps = prod(plan.dst_shape);
        plan.op = tok();
        if (plan.op != "set" && plan.op != "add" && plan.op != "sub" && plan.op != "sum" && plan.op != "setsum" &&
            plan.op != "acc" && plan.op != "accat")
            fail("unknown assignment '" + plan.op + "'");
        if (plan.wants_acc() && plan.dst_dtype != DType::F64)
            fail("accumulation planes are f64 (a value and a compensation plane per component)");
        plan.root = expr();
        expect(")");
        ws();
        if (*p) fail("trailing text after the plan");
        if (N(plan.root).shape != plan.dst_shape) fail("expression shape does not match the destination");
        if (N(plan.root).is_bool) fail("a boolean expression cannot be stored");
        if (plan.wants_sum() && plan.dst_comps != 1) fail("sum plans need a rank-0 (or [1]) expression");
        for (int k = 0; k < plan.n_operands; ++k)
            if (!plan.operand_comps[size_t(k)]) fail("operand slot " + std::to_string(k) + " is unused");
        return plan;
    }
};

// ---------------------------------------------------------------------------
// Code generation.
// ---------------------------------------------------------------------------
std::string hexlit(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%a", v);
    return buf;
}

std::string ctype_of(DType d) {
    switch (d) {
    case DType::F64: return "double";
    case DType::I32: return "int";
    case DType::U8: return "unsigned char";
    default: return "float";
    }
}

struct Gen {
    const Plan& P;
    const Lowering& L;
    std::vector<int> ctx;
    std::string W;        // working type
    std::string S;        // destination storage type
    std::vector<std::vector<std::string>> val;
    std::vector<char> done;
    std::ostringstream pro;   // sample-0 prologue (at0 subtrees)
    std::ostringstream body;  // per-lane code
    bool dfm = false;         // double-float working type (emulated FP64)
    bool tfm = false;         // with dfm: triple-float working type (FP64-grade, math 3)
    std::string NS = "ag::e64::";   // namespace of the working type's functions
    std::string pre = "t";    // variable prefix
    bool direct = false;      // leaves load their own sample `s` (per-lane fallback function)
    std::vector<signed char> nn_memo;
    // Double-float magnitude bounds: floor(log2 |v|) of every non-zero value of
    // node id lies in [elo, ehi] (wide open when unknown). A product whose
    // bounds cannot go below 2^-102 needs no range check (ag::e64::ck).
    static constexpr int kOpenLo = -100000, kOpenHi = 100000;
    int kSafeLo = -101;   // products at or above 2^kSafeLo need no check (-80 for triple-float)
    std::vector<int> elo, ehi;
    std::string cur_ok = "ok_";   // the range flag of the node being emitted

    // Conservative sign analysis: true when node `id` can never be negative,
    // which lets emulated sums skip the cancellation-safe form.
    bool nonneg(int id) {
        if (nn_memo.empty()) nn_memo.assign(P.nodes.size(), -1);
        signed char& m = nn_memo[size_t(id)];
        if (m >= 0) return m != 0;
        const Node& n = P.nodes[size_t(id)];
        const std::string& op = n.op;
        bool r = false;
        if (op == "sq" || op == "abs" || op == "sqrt" || op == "rsqrt" || op == "exp" || op == "norm" ||
            op == "sqnorm" || op == "rnorm" || op == "exp2" || op == "cosh")
            r = true;
        else if (op == "lit") r = n.lit >= 0.0;
        else if (op == "sc") r = n.nonneg_hint;
        else if (op == "bcast" || op == "at0") r = nonneg(n.kids[0]);
        else if (op == "mul") r = n.kids[0] == n.kids[1] || (nonneg(n.kids[0]) && nonneg(n.kids[1]));
        else if (op == "add" || op == "scale") r = nonneg(n.kids[0]) && nonneg(n.kids[1]);
        else if (op == "log1p") r = nonneg(n.kids[0]);
        m = r ? 1 : 0;
        return r;
    }

    Gen(const Plan& p, const Lowering& l, const std::vector<int>& c, bool df_mode = false, std::string prefix = "t",
        bool force_double = false, bool tf_mode = false)
        : P(p), L(l), ctx(c), val(p.nodes.size()), done(p.nodes.size(), 0), dfm(df_mode || tf_mode), tfm(tf_mode),
          pre(std::move(prefix)) {
        NS = tfm ? "ag::t64::" : "ag::e64::";
        if (tfm) kSafeLo = -80;
        W = tfm ? "ag::t64::tf" : dfm ? "ag::e64::df" : ((P.dst_dtype == DType::F64 || force_double) ? "double" : "float");
        S = P.dst_dtype == DType::F64 ? "double" : "float";
    }

    // A double-float value that is an exact float (an f32 operand): products
    // of two of them are exact two-products, no double-float multiply.
    bool exact_f32(int id) const {
        const Node& n = P.nodes[size_t(id)];
        return dfm && !tfm && n.op == "in" && n.dtype == DType::F32;
    }
    // `u`: the product is read only by sums and may stay unnormalised. The
    // range check is left out when the factors' bounds keep it above 2^-102.
    std::string mulx(bool u, int ia, int ib, const std::string& a, const std::string& b) {
        const bool safe = lo_of(ia) + lo_of(ib) >= kSafeLo;
        if (exact_f32(ia) && exact_f32(ib)) {
            const std::string p = NS + "two_prod(" + a + ".hi, " + b + ".hi)";
            return checked(p, safe);
        }
        if (dfm && ia == ib && a == b) return checked(sqr(u, a), safe);   // x*x: the square's cheaper form
        return dfm ? checked(NS + "mul(" + a + ", " + b + ")", safe) : mul(a, b);
    }
    int lo_of(int id) const { return elo.empty() ? kOpenLo : elo[size_t(id)]; }
    int hi_of(int id) const { return ehi.empty() ? kOpenHi : ehi[size_t(id)]; }
    std::string checked(const std::string& v, bool safe) const {
        return safe ? v : NS + "ck(" + v + ", " + cur_ok + ")";
    }
    // Nodes read only by sums (add, sub): a square feeding them may stay an
    // unnormalised pair, saving its final Fast2Sum. The root of an emulated
    // FP64 plan is read only by the reassembly into a double, which rounds
    // hi + lo once whether or not the pair is normalised.
    bool root_to_double = false;
    std::vector<signed char> sum_only_memo;
    bool sum_only(int id) {
        if (sum_only_memo.empty()) {
            sum_only_memo.assign(P.nodes.size(), 1);
            sum_only_memo[size_t(P.root)] = root_to_double ? 1 : 0;
            for (const Node& m : P.nodes)
                for (int k : m.kids)
                    if (m.op != "add" && m.op != "sub") sum_only_memo[size_t(k)] = 0;
        }
        return sum_only_memo[size_t(id)] != 0;
    }
    std::string sqr(bool u, const std::string& x) { return (u ? NS + "sqr_u(" : NS + "sqr(") + x + ")"; }

    std::string add(const std::string& a, const std::string& b) const {
        if (dfm) return NS + "add(" + a + ", " + b + ")";
        return L.contract ? "(" + a + " + " + b + ")" : "ag::rn_add(" + a + ", " + b + ")";
    }
    std::string sub(const std::string& a, const std::string& b) const {
        if (dfm) return NS + "sub(" + a + ", " + b + ")";
        return L.contract ? "(" + a + " - " + b + ")" : "ag::rn_sub(" + a + ", " + b + ")";
    }
    // Products and quotients inside composite nodes carry the range check
    // (a product with a literal zero is exact and needs none).
    std::set<std::string> zero_vars;
    // Products of two kid values of the node being emitted, unchecked when
    // the kids' bounds keep every such product above 2^-102.
    bool kids_safe = false;
    std::string mulkk(const std::string& a, const std::string& b) const {
        if (dfm && kids_safe) return NS + "mul(" + a + ", " + b + ")";
        return mul(a, b);
    }
    std::string mul(const std::string& a, const std::string& b) const {
        if (dfm && (zero_vars.count(a) || zero_vars.count(b))) return NS + "mul(" + a + ", " + b + ")";
        if (dfm) return NS + "ck(" + NS + "mul(" + a + ", " + b + "), " + cur_ok + ")";
        return L.contract ? "(" + a + " * " + b + ")" : "ag::rn_mul(" + a + ", " + b + ")";
    }
    std::string div(const std::string& a, const std::string& b) const {
        if (dfm) return NS + "ck(" + NS + "div(" + a + ", " + b + "), " + cur_ok + ")";
        return "ag::rn_div(" + a + ", " + b + ")";
    }
    std::string neg(const std::string& a) const { return dfm ? NS + "neg(" + a + ")" : "(-" + a + ")"; }
    std::string lit(double v) const {
        if (tfm) return tf_literal(v);
        if (dfm) return NS + "dfc(" + hexlit(v) + ")";
        return "((" + W + ")" + hexlit(v) + ")";
    }
    // A literal as three floats split here, exactly for every normal double
    // (no FP64 work in the kernel).
    static std::string fltlit(float f) {
        char b[48];
        std::snprintf(b, sizeof b, "%.9ef", double(f));
        return std::isfinite(f) ? std::string(b) : (f != f ? "__int_as_float(0x7fc00000)" : (f > 0 ? "__int_as_float(0x7f800000)" : "__int_as_float((int)0xff800000)"));
    }
    std::string tf_literal(double v) const {
        const float x = float(v);
        const double r = std::isfinite(x) ? v - double(x) : 0.0;
        const float y = float(r);
        const float z = float(r - double(y));
        return "ag::t64::mk3(" + fltlit(x) + ", " + fltlit(y) + ", " + fltlit(z) + ")";
    }
    std::string okv(int id) const { return ctx[size_t(id)] ? "ok0_" : "ok_"; }
    // |x| of a loaded operand: non-negative and, once the operand passed the
    // double-float range check, below 2^60
    bool abs_of_input(int id) const {
        const Node& n = P.nodes[size_t(id)];
        return n.op == "abs" && P.nodes[size_t(n.kids[0])].op == "in";
    }
    // Function spelling; `id` selects the range flag for functions that set one.
    std::string call(const std::string& name, const std::vector<std::string>& args, int id) const {
        std::string a;
        for (size_t i = 0; i < args.size(); ++i) a += (i ? ", " : "") + args[i];
        if (!dfm) return "ag::f_" + name + "(" + a + ")";
        static const std::set<std::string> own = {"sqrt", "rsqrt", "log", "log1p", "abs", "sign", "min", "max"};
        if (name == "sin" || name == "cos" || name == "exp") return NS + "" + name + "_(" + a + ", " + okv(id) + ")";
        if (name == "log1p" && abs_of_input(P.nodes[size_t(id)].kids[0]))
            return NS + "log1p_nn_(" + a + ")";   // |input| is >= 0 and within the input range check
        if (own.count(name)) return NS + "" + name + "_(" + a + ")";
        return NS + "nat_" + name + "(" + a + ")";
    }
    std::string gtx(const std::string& a, const std::string& b) const {
        return dfm ? NS + "gt(" + a + ", " + b + ")" : "(" + a + " > " + b + ")";
    }

    std::ostringstream& out_for(int id) { return ctx[size_t(id)] ? pro : body; }

    // Declare one variable per component for node `id`.
    void def(int id, const std::vector<std::string>& exprs, bool is_bool = false) {
        std::ostringstream& o = out_for(id);
        std::vector<std::string> names;
        for (size_t c = 0; c < exprs.size(); ++c) {
            const std::string nm = pre + std::to_string(id) + "_" + std::to_string(c);
            o << "        const " << (is_bool ? "bool" : W) << " " << nm << " = " << exprs[c] << ";\n";
            names.push_back(nm);
        }
        val[size_t(id)] = names;
    }

    // Magnitude bounds of node id from its kids' (conservative; open when
    // nothing better is known). Inputs of the double-float path are range
    // checked to [2^-50, 2^60]; exact f32 inputs are not checked.
    static int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
    void bounds(int id) {
        if (!dfm) return;
        if (elo.empty()) {
            elo.assign(P.nodes.size(), kOpenLo);
            ehi.assign(P.nodes.size(), kOpenHi);
        }
        const Node& n = P.nodes[size_t(id)];
        const std::string& op = n.op;
        auto L = [&](int j) { return elo[size_t(n.kids[size_t(j)])]; };
        auto H = [&](int j) { return ehi[size_t(n.kids[size_t(j)])]; };
        auto clampb = [](int v) { return v < kOpenLo ? kOpenLo : (v > kOpenHi ? kOpenHi : v); };
        int lo = kOpenLo, hi = kOpenHi;
        if (op == "in") {
            if (n.dtype == DType::F64) lo = tfm ? -40 : -50, hi = 60;
            else if (n.dtype == DType::F32) lo = -149, hi = 127;
        } else if (op == "lit") {
            if (n.lit != 0.0 && std::isfinite(n.lit)) {
                lo = hi = std::ilogb(n.lit);
            } else if (n.lit == 0.0) {
                lo = kOpenHi, hi = kOpenLo;   // an exact zero: products with it are exact
            }
        } else if (op == "neg" || op == "abs" || op == "bcast" || op == "at0" || op == "comp" || op == "seg" ||
                   op == "row" || op == "col" || op == "transpose" || op == "block" || op == "reshape" ||
                   op == "stack") {
            lo = kOpenHi, hi = kOpenLo;
            for (size_t j = 0; j < n.kids.size(); ++j) {
                lo = std::min(lo, L(int(j)));
                hi = std::max(hi, H(int(j)));
            }
        } else if (op == "sq") {
            lo = clampb(2 * L(0)), hi = clampb(2 * H(0) + 1);
        } else if (op == "mul") {
            lo = clampb(L(0) + L(1)), hi = clampb(H(0) + H(1) + 1);
        } else if (op == "sqrt") {   // 2^L <= x < 2^(H+1): 2^(L/2) <= sqrt x < 2^((H+1)/2)
            lo = L(0) <= kOpenLo ? kOpenLo : floordiv(L(0), 2), hi = H(0) >= kOpenHi ? kOpenHi : floordiv(H(0), 2) + 1;
        } else if (op == "rsqrt") {   // 2^(-(H+1)/2) < 1/sqrt x <= 2^(-L/2)
            lo = H(0) >= kOpenHi ? kOpenLo : floordiv(-(H(0) + 1), 2), hi = L(0) <= kOpenLo ? kOpenHi : floordiv(-L(0), 2);
        } else if (op == "add" && nonneg(n.kids[0]) && nonneg(n.kids[1])) {
            // no cancellation; an exact zero (an empty interval) adds nothing
            const bool z0 = L(0) > H(0), z1 = L(1) > H(1);
            lo = z0 ? L(1) : (z1 ? L(0) : std::max(L(0), L(1)));
            hi = clampb(std::max(H(0), H(1)) + 1);
        } else if (op == "log1p" && nonneg(n.kids[0])) {
            lo = L(0) <= kOpenLo ? kOpenLo : std::min(L(0) - 1, -1);   // log1p(y) >= min(y, 1)/2
            hi = H(0) <= 0 ? H(0) : 7;
        }
        elo[size_t(id)] = lo;
        ehi[size_t(id)] = hi;
    }

    const std::vector<std::string>& emit(int id) {
        if (done[size_t(id)]) return val[size_t(id)];
        const Node& n = P.nodes[size_t(id)];
        for (int k : n.kids) emit(k);
        auto V = [&](int j) -> const std::vector<std::string>& { return val[size_t(n.kids[size_t(j)])]; };
        auto K = [&](int j) -> const Node& { return P.nodes[size_t(n.kids[size_t(j)])]; };
        const std::string& op = n.op;
        const bool c0 = ctx[size_t(id)] != 0;
        cur_ok = okv(id);
        kids_safe = false;
        if (dfm && !n.kids.empty()) {
            int m = kOpenHi;
            for (int k : n.kids) m = std::min(m, lo_of(k));
            kids_safe = m > kOpenLo && 2 * m >= kSafeLo;
        }
        std::vector<std::string> e;
        const std::string gid = c0 ? "g0" : "g";
        const std::string sid = pre + std::to_string(id);

        if (op == "in") {
            const bool pbool = n.dtype == DType::U8;
            for (int c = 0; c < n.comps; ++c) {
                std::string src = c0 ? "x" + std::to_string(n.k) + "_0[" + std::to_string(c) + "]"
                                     : "in" + std::to_string(n.k) + "[" + std::to_string(c) + "][l]";
                if (direct)
                    src = "((const " + ctype_of(n.dtype) + "*)a.ops[" + std::to_string(n.k) + "])[(ag_u64)" +
                          std::to_string(c) + " * a.pitch[" + std::to_string(n.k) + "] + " + (c0 ? "0" : "s") + "]";
                if (pbool) {
                    e.push_back("(" + src + " != 0)");
                } else if (dfm && n.dtype == DType::F32) {
                    e.push_back(tfm ? "ag::t64::mk3((float)" + src + ", 0.0f, 0.0f)"
                                    : NS + "mk((float)" + src + ", 0.0f)");   // exact
                } else if (dfm) {
                    e.push_back(NS + "from_double_ck((double)" + src + ", " + okv(id) + ")");
                } else {
                    e.push_back("(" + W + ")" + src);
                }
            }
            def(id, e, pbool);
        } else if (op == "sc") {
            const std::string s = "a.sc[" + std::to_string(n.k) + "]";
            const std::string k = std::to_string(n.k);
            def(id, {tfm ? "ag::t64::dfc(" + s + ")" : dfm ? NS + "mk(a.sch[" + k + "], a.scl[" + k + "])" : "(" + W + ")" + s});
        } else if (op == "lit") {
            def(id, {lit(n.lit)});
            if (n.lit == 0.0) zero_vars.insert(val[size_t(id)][0]);   // products with it are exact zeros
        } else if (op == "bcast") {
            for (int c = 0; c < n.comps; ++c) e.push_back(V(0)[0]);
            val[size_t(id)] = e;   // aliases: no new variables
        } else if (op == "at0") {
            // Values of the sample-0 subtree are computed in the prologue and
            // are uniform across lanes.
            val[size_t(id)] = V(0);
        } else if (unary_ops().count(op)) {
            for (int c = 0; c < n.comps; ++c) {
                const std::string x = V(0)[size_t(c)];
                if (op == "sq") e.push_back(dfm ? checked(sqr(sum_only(id), x), 2 * lo_of(n.kids[0]) >= kSafeLo) : mul(x, x));
                else if (op == "sqrt" && dfm && nonneg(n.kids[0])) e.push_back(NS + "sqrt_nn_(" + x + ")");
                else if (op == "neg") e.push_back(neg(x));
                else e.push_back(call(op, {x}, id));
            }
            def(id, e);
        } else if (binary_ops().count(op)) {
            for (int c = 0; c < n.comps; ++c) {
                const std::string a = V(0)[size_t(c)], b = V(1)[size_t(c)];
                if (op == "add" && dfm && nonneg(n.kids[0]) && nonneg(n.kids[1]))
                    e.push_back((root_to_double && id == P.root ? NS + "add_fast_u(" : NS + "add_fast(") + a +
                                ", " + b + ")");
                else if (op == "add") e.push_back(add(a, b));
                else if (op == "sub") e.push_back(sub(a, b));
                else if (op == "mul") e.push_back(mulx(sum_only(id), n.kids[0], n.kids[1], a, b));
                else if (op == "div") e.push_back(div(a, b));
                else e.push_back(call(op, {a, b}, id));
            }
            def(id, e);
        } else if (op == "scale") {   // CWiseScale: factor * e (expr/nodes/Arithmetic.h:130-140)
            for (int c = 0; c < n.comps; ++c) e.push_back(mul(V(1)[0], V(0)[size_t(c)]));
            def(id, e);
        } else if (op == "mins" || op == "maxs" || op == "pows") {
            const std::string f = op == "mins" ? "min" : op == "maxs" ? "max" : "pow";
            for (int c = 0; c < n.comps; ++c) e.push_back(call(f, {V(0)[size_t(c)], V(1)[0]}, id));
            def(id, e);
        } else if (op == "clamp") {   // Elementwise.h:138-167
            for (int c = 0; c < n.comps; ++c)
                e.push_back(call("min", {call("max", {V(0)[size_t(c)], V(1)[0]}, id), V(2)[0]}, id));
            def(id, e);
        } else if (cmp_ops().count(op)) {
            static const std::map<std::string, std::string> sym = {{"gt", ">"}, {"lt", "<"}, {"ge", ">="},
                                                                   {"le", "<="}, {"eq", "=="}, {"ne", "!="},
                                                                   {"and", "&&"}, {"or", "||"}};
            const bool logical = op == "and" || op == "or";
            for (int c = 0; c < n.comps; ++c) {
                const std::string a = V(0)[size_t(c)], b = V(1)[size_t(c)];
                if (dfm && !logical && !K(0).is_bool) e.push_back(NS + "" + op + "(" + a + ", " + b + ")");
                else e.push_back("(" + a + " " + sym.at(op) + " " + b + ")");
            }
            def(id, e, true);
        } else if (op == "not") {
            for (int c = 0; c < n.comps; ++c) e.push_back("(!" + V(0)[size_t(c)] + ")");
            def(id, e, true);
        } else if (op == "select") {   // Elementwise.h:809-846
            const bool per_sample = K(0).shape.empty();
            for (int c = 0; c < n.comps; ++c)
                e.push_back("(" + V(0)[per_sample ? 0 : size_t(c)] + " ? " + V(1)[size_t(c)] + " : " + V(2)[size_t(c)] + ")");
            def(id, e, n.is_bool);
        } else if (op == "comp") {
            val[size_t(id)] = {V(0)[size_t(n.k)]};
        } else if (op == "seg") {
            for (int c = 0; c < n.comps; ++c) e.push_back(V(0)[size_t(n.k + c)]);
            val[size_t(id)] = e;
        } else if (op == "row" || op == "col") {
            const int cols = K(0).shape[1];
            for (int c = 0; c < n.comps; ++c)
                e.push_back(V(0)[size_t(op == "row" ? n.k * cols + c : c * cols + n.k)]);
            val[size_t(id)] = e;
        } else if (op == "transpose") {
            const int r0 = K(0).shape[0], c0n = K(0).shape[1];
            for (int r = 0; r < c0n; ++r)
                for (int c = 0; c < r0; ++c) e.push_back(V(0)[size_t(c * c0n + r)]);
            val[size_t(id)] = e;
        } else if (op == "block") {
            const int cols = K(0).shape[1];
            for (int r = 0; r < n.ints[2]; ++r)
                for (int c = 0; c < n.ints[3]; ++c) e.push_back(V(0)[size_t((n.ints[0] + r) * cols + n.ints[1] + c)]);
            val[size_t(id)] = e;
        } else if (op == "stack") {
            for (size_t j = 0; j < n.kids.size(); ++j) e.push_back(V(int(j))[0]);
            val[size_t(id)] = e;
        } else if (op == "reshape") {
            val[size_t(id)] = V(0);
        } else if (op == "cross") {   // expr/nodes/Geometric.h:55-72
            const auto& l = V(0);
            const auto& r = V(1);
            e = {sub(mulkk(l[1], r[2]), mulkk(l[2], r[1])), sub(mulkk(l[2], r[0]), mulkk(l[0], r[2])),
                 sub(mulkk(l[0], r[1]), mulkk(l[1], r[0]))};
            def(id, e);
        } else if (op == "unit") {   // Geometric.h:99-103 on a per-sample (Item) value
            const auto& a = V(0);
            std::string acc = mul(a[0], a[0]);
            for (size_t c = 1; c < a.size(); ++c) acc = add(mul(a[c], a[c]), acc);
            const std::string rn = sid + "r";
            out_for(id) << "        const " << W << " " << rn << " = " << div(lit(1.0), call("sqrt", {acc}, id)) << ";\n";
            for (size_t c = 0; c < a.size(); ++c) e.push_back(mul(a[c], rn));
            def(id, e);
        } else if (op == "qmul") {   // expr/nodes/Quaternion.h:60-79
            const auto& l = V(0);
            const auto& r = V(1);
            e = {sub(sub(sub(mulkk(l[0], r[0]), mulkk(l[1], r[1])), mulkk(l[2], r[2])), mulkk(l[3], r[3])),
                 sub(add(add(mulkk(l[0], r[1]), mulkk(l[1], r[0])), mulkk(l[2], r[3])), mulkk(l[3], r[2])),
                 add(add(sub(mulkk(l[0], r[2]), mulkk(l[1], r[3])), mulkk(l[2], r[0])), mulkk(l[3], r[1])),
                 add(sub(add(mulkk(l[0], r[3]), mulkk(l[1], r[2])), mulkk(l[2], r[1])), mulkk(l[3], r[0]))};
            def(id, e);
        } else if (op == "qconj") {   // Quaternion.h:103-108
            const auto& a = V(0);
            e = {a[0], neg(a[1]), neg(a[2]), neg(a[3])};
            def(id, e);
        } else if (op == "qrot") {   // Quaternion.h:142-168
            const auto& q = V(0);
            const auto& v = V(1);
            const std::string t = sid + "q";
            std::ostringstream& o = out_for(id);
            const std::string two = lit(2.0);
            o << "        const " << W << " " << t << "x = " << mul(two, sub(mulkk(q[2], v[2]), mulkk(q[3], v[1]))) << ";\n";
            o << "        const " << W << " " << t << "y = " << mul(two, sub(mulkk(q[3], v[0]), mulkk(q[1], v[2]))) << ";\n";
            o << "        const " << W << " " << t << "z = " << mul(two, sub(mulkk(q[1], v[1]), mulkk(q[2], v[0]))) << ";\n";
            e = {add(add(v[0], mul(q[0], t + "x")), sub(mul(q[2], t + "z"), mul(q[3], t + "y"))),
                 add(add(v[1], mul(q[0], t + "y")), sub(mul(q[3], t + "x"), mul(q[1], t + "z"))),
                 add(add(v[2], mul(q[0], t + "z")), sub(mul(q[1], t + "y"), mul(q[2], t + "x")))};
            def(id, e);
        } else if (op == "pureq") {   // Quaternion.h:192-203
            const auto& a = V(0);
            e = {lit(0.0), a[0], a[1], a[2]};
            def(id, e);
        } else if (op == "inv" || op == "det") {   // expr/nodes/Inverse.h:73-118, Expression.h:400-428
            const auto& m = V(0);
            const int dim = K(0).shape[0];
            const std::string d = sid + "det";
            std::ostringstream& o = out_for(id);
            // Emulated FP64 divides by the determinant once, as a reciprocal.
            const std::string rd = sid + "rdet";
            auto q = [&](const std::string& num) { return dfm ? mul(num, rd) : div(num, d); };
            if (dim == 2) {
                o << "        const " << W << " " << d << " = " << sub(mulkk(m[0], m[3]), mulkk(m[1], m[2])) << ";\n";
                if (dfm && op == "inv") o << "        const " << W << " " << rd << " = " << NS << "recip(" << d << ");\n";
                if (op == "det") e = {d};
                else e = {q(m[3]), q(neg(m[1])), q(neg(m[2])), q(m[0])};
            } else {
                const std::string &a = m[0], &b = m[1], &c = m[2], &dd = m[3], &ee = m[4], &f = m[5], &g = m[6],
                                  &h = m[7], &k = m[8];
                o << "        const " << W << " " << d << " = "
                  << add(sub(mul(a, sub(mulkk(ee, k), mulkk(f, h))), mul(b, sub(mulkk(dd, k), mulkk(f, g)))),
                         mul(c, sub(mulkk(dd, h), mulkk(ee, g))))
                  << ";\n";
                if (dfm && op == "inv") o << "        const " << W << " " << rd << " = " << NS << "recip(" << d << ");\n";
                if (op == "det") {
                    e = {d};
                } else {
                    e = {q(sub(mulkk(ee, k), mulkk(f, h))), q(sub(mulkk(c, h), mulkk(b, k))), q(sub(mulkk(b, f), mulkk(c, ee))),
                         q(sub(mulkk(f, g), mulkk(dd, k))), q(sub(mulkk(a, k), mulkk(c, g))), q(sub(mulkk(c, dd), mulkk(a, f))),
                         q(sub(mulkk(dd, h), mulkk(ee, g))), q(sub(mulkk(b, g), mulkk(a, h))), q(sub(mulkk(a, ee), mulkk(b, dd)))};
                }
            }
            def(id, e);
        } else if (op == "trace") {   // Expression.h:381-398
            const auto& m = V(0);
            const int dim = K(0).shape[0];
            std::string t = add(m[0], m[size_t(dim + 1)]);
            if (dim == 3) t = add(t, m[8]);
            def(id, {t});
        } else if (op == "matvec" || op == "matmul" || op == "outer") {
            const auto& a = V(0);
            const auto& b = V(1);
            const auto& sa = K(0).shape;
            const auto& sb = K(1).shape;
            if (op == "outer") {
                for (int i = 0; i < sa[0]; ++i)
                    for (int j = 0; j < sb[0]; ++j) e.push_back(mulkk(a[size_t(i)], b[size_t(j)]));
            } else if (op == "matvec") {
                for (int i = 0; i < sa[0]; ++i) {
                    std::string acc = mulkk(a[size_t(i * sa[1])], b[0]);
                    for (int k = 1; k < sa[1]; ++k) acc = add(mulkk(a[size_t(i * sa[1] + k)], b[size_t(k)]), acc);
                    e.push_back(acc);
                }
            } else {
                for (int i = 0; i < sa[0]; ++i)
                    for (int j = 0; j < sb[1]; ++j) {
                        std::string acc = mulkk(a[size_t(i * sa[1])], b[size_t(j)]);
                        for (int k = 1; k < sa[1]; ++k)
                            acc = add(mulkk(a[size_t(i * sa[1] + k)], b[size_t(k * sb[1] + j)]), acc);
                        e.push_back(acc);
                    }
            }
            def(id, e);
        } else if (op == "dot" || op == "sqnorm" || op == "norm" || op == "rnorm" || op == "sum" || op == "maxnorm") {
            // expr/Reduce.h:149-188: acc = f(x0); acc = Reduce(f(x_{k+1}), acc)
            const auto& a = V(0);
            const int m = K(0).comps;
            auto term = [&](int c) -> std::string {
                if (op == "dot") return mulx(false, n.kids[0], n.kids[1], a[size_t(c)], V(1)[size_t(c)]);
                if (op == "sum") return a[size_t(c)];
                if (op == "maxnorm") return call("abs", {a[size_t(c)]}, id);
                return mulkk(a[size_t(c)], a[size_t(c)]);
            };
            std::string acc = term(0);
            for (int c = 1; c < m; ++c) {
                const std::string t = term(c);
                acc = op == "maxnorm" ? "(" + gtx(t, acc) + " ? (" + t + ") : (" + acc + "))" : add(t, acc);
            }
            if (op == "norm") acc = call("sqrt", {acc}, id);
            if (op == "rnorm") acc = div(lit(1.0), call("sqrt", {acc}, id));
            def(id, {acc});
        } else if (op == "uniform" || op == "normal" || op == "lognormal" || op == "exponential" || op == "bernoulli") {
            const std::string key = "a.key[" + std::to_string(n.k) + "]";
            const bool b0 = K(0).shape.empty();
            const bool b1 = n.kids.size() > 1 && K(1).shape.empty();
            const std::string wp = "(" + W + "*)0";
            // N(0, 1) with literal parameters: 0 + 1 z is z bit for bit (z != 0)
            const bool std01 = n.kids.size() > 1 && K(0).op == "lit" && K(0).lit == 0.0 && K(1).op == "lit" &&
                               K(1).lit == 1.0;
            auto u01 = [&](const char* salt, const std::string& cc) {
                return dfm ? NS + "draw01_df(" + key + " ^ " + salt + ", " + gid + ", " + cc + ")"
                           : "ag::draw01(" + wp + ", " + key + " ^ " + salt + ", " + gid + ", " + cc + ")";
            };
            const bool nrm_u = std01 && root_to_double && id == P.root && n.op == "normal";
            auto nrm = [&](const char* salt, const std::string& cc) {
                return dfm ? std::string(nrm_u ? NS + "normal_df<true>(" : NS + "normal_df(") + key + " ^ " +
                                 salt + ", " + gid + ", " + cc + ")"
                           : "ag::drawn(" + wp + ", " + key + " ^ " + salt + ", " + gid + ", " + cc + ")";
            };
            for (int c = 0; c < n.comps; ++c) {
                const std::string x0 = V(0)[b0 ? 0 : size_t(c)];
                const std::string x1 = n.kids.size() > 1 ? V(1)[b1 ? 0 : size_t(c)] : "";
                const std::string cc = std::to_string(c) + "u";
                if (op == "uniform") {   // DistributionLeaf.h:125-131
                    e.push_back(add(x0, mul(sub(x1, x0), u01("AG_SALT_UNIFORM", cc))));
                } else if (op == "normal") {   // DistributionLeaf.h:192-199
                    e.push_back(std01 ? nrm("AG_SALT_NORMAL", cc) : add(x0, mul(x1, nrm("AG_SALT_NORMAL", cc))));
                } else if (op == "lognormal") {   // DistributionLeaf.h:257-264
                    e.push_back(call("exp", {std01 ? nrm("AG_SALT_LOGNORMAL", cc)
                                                   : add(x0, mul(x1, nrm("AG_SALT_LOGNORMAL", cc)))}, id));
                } else if (op == "exponential") {   // DistributionLeaf.h:329-333
                    e.push_back(div(neg(call("log", {u01("AG_SALT_EXPONENTIAL", cc)}, id)), x0));
                } else {   // DistributionLeaf.h:380-385
                    const std::string u = u01("AG_SALT_BERNOULLI", cc);
                    e.push_back("(" + (dfm ? NS + "lt(" + u + ", " + x0 + ")" : "(" + u + " < " + x0 + ")") + " ? " +
                                lit(1.0) + " : " + lit(0.0) + ")");
                }
            }
            def(id, e);
        } else {
            fail("no generator for '" + op + "'");
        }
        bounds(id);
        done[size_t(id)] = 1;
        return val[size_t(id)];
    }
};

std::string ctype(DType d) {
    switch (d) {
    case DType::F64: return "double";
    case DType::F32: return "float";
    case DType::FF: return "float";
    case DType::I32: return "int";
    case DType::U8: return "unsigned char";
    }
    return "double";
}

}  // namespace

Plan parse_plan(const std::string& text) {
    Parser ps(text.c_str());
    return ps.run();
}

int effective_vec(const Plan& plan, const Lowering& low) {
    if (low.vec > 0) return low.vec;
    int widest = dtype_size(plan.dst_dtype);
    for (DType d : plan.operand_dtype) widest = std::max(widest, dtype_size(d));
    return widest >= 8 ? 2 : 4;
}

std::string kernel_base(const Plan& plan, const std::string& text) {
    uint64_t h = 1469598103934665603ULL;
    for (unsigned char c : text) {
        h ^= c;
        h *= 1099511628211ULL;
    }
    char buf[64];
    const char* kind = plan.wants_sum() ? "sum" : (plan.has_random && plan.n_operands == 0) ? "fill" : "expr";
    std::snprintf(buf, sizeof buf, "ag_%s_%08x", kind, unsigned(h ^ (h >> 32)));
    return buf;
}

// FP64-grade plans with trigonometric nodes include the triple-float sine
// and cosine (and their table).
bool uses_trig(const Plan& P) {
    for (const Node& n : P.nodes)
        if (n.op == "sin" || n.op == "cos") return true;
    return false;
}

// Plans with normal or lognormal leaves include the Box-Muller header when
// lowered to double-float.
bool draws_normals(const Plan& P) {
    for (const Node& n : P.nodes)
        if (n.op == "normal" || n.op == "lognormal") return true;
    return false;
}

std::string generate_source(const Plan& plan_in, const Lowering& low, const std::string& base,
                            const std::string& suffix, bool chunk_only) {
    // Re-derive the sample contexts (at0 subtrees) from the node graph: every
    // node reachable only through `at0` belongs to the sample-0 prologue.
    const Plan& P = plan_in;
    std::vector<int> ctx(P.nodes.size(), 1);
    {
        std::vector<int> stack = {P.root};
        std::vector<char> seen(P.nodes.size(), 0);
        while (!stack.empty()) {
            const int id = stack.back();
            stack.pop_back();
            if (seen[size_t(id)]) continue;
            seen[size_t(id)] = 1;
            ctx[size_t(id)] = 0;
            if (P.nodes[size_t(id)].op == "at0") continue;
            for (int k : P.nodes[size_t(id)].kids) stack.push_back(k);
        }
        // A node used both inside and outside at0 would need two copies; the
        // parser keys its memo by context, so such nodes are already distinct.
    }
    // Emulated FP64 (math 1, f64 plans) and the precision form (math 2, f32
    // and ff plans): the tree is generated in double-float (the fast path) and
    // once more on the native FP64 pipe (the per-lane fallback).
    // FP64-grade triple-float (math 3, f64 plans) takes the same frame.
    const bool tfx = low.math == 3 && P.dst_dtype == DType::F64;
    const bool emu = (low.math == 1 && P.dst_dtype == DType::F64) || (low.math == 2 && P.dst_dtype != DType::F64) || tfx;
    const bool prec = emu && P.dst_dtype != DType::F64;   // float storage, float-float working values
    const bool dst_ff = P.dst_dtype == DType::FF;
    if (dst_ff && !prec) fail("ff destinations are written by the precision form (math = 2)");
    Gen g(P, low, ctx, emu, emu ? "d" : "t", false, tfx);
    g.root_to_double = emu && P.dst_dtype == DType::F64;
    const std::vector<std::string> root = g.emit(P.root);
    Lowering nat = low;
    nat.math = 0;
    Gen gn(P, nat, ctx, false, "n", true);
    gn.direct = true;
    std::vector<std::string> nroot;
    if (emu) nroot = gn.emit(P.root);

    const int vec = effective_vec(P, low);
    std::ostringstream o;
    if (!chunk_only) {
        o << "// generated by aether_gb300 from an aether-ir/1 plan\n";
        o << "#include \"ag_device.cuh\"\n";
        if (low.math >= 1) o << "#include \"ag_emu64.cuh\"\n";
        if (tfx) o << "#include \"ag_tf64.cuh\"\n";
        if (tfx && uses_trig(P)) o << "#include \"ag_tf64_trig.cuh\"\n";
        if (low.math >= 1 && draws_normals(P)) o << "#include \"ag_emu64_bm.cuh\"\n";
        o << "#define AG_BLOCK " << low.block << "\n#define AG_IPT " << low.ipt << "\n#define AG_VEC " << vec << "\n";
    }
    const std::string W = g.W, S = g.S;
    const int OC = P.dst_planes();   // stored planes (ff: hi then lo; acc: value then compensation)
    const bool sum = P.wants_sum();
    const bool atomic_acc = P.op == "accat";
    const bool store = P.wants_store() && !atomic_acc;   // atomic accumulation writes in the lane loop
    const bool rw = P.op == "add" || P.op == "sub" || P.op == "acc";
    if ((rw || atomic_acc) && prec)
        fail("+=, -= and accumulation are lowered by the native and emulated-FP64 forms, not the precision form");

    if (emu) {
        // The native FP64 recomputation of one sample, out of line so its
        // registers do not weigh on the double-float fast path. It reloads its
        // own operands at sample `s` (s < n is checked by the caller).
        o << "__device__ __noinline__ void ag_native_lane" << suffix << "(const AgArgs& a, ag_u64 s, double* fv) {\n";
        if (P.has_random) o << "    const ag_u32 g0 = a.offset;\n    const ag_u32 g = a.offset + (ag_u32)s;\n";
        o << gn.pro.str() << gn.body.str();
        for (int c = 0; c < P.dst_comps; ++c) o << "    fv[" << c << "] = " << nroot[size_t(c)] << ";\n";
        o << "}\n";
    }

    // The chunk body: one pass of a CTA over block*ipt*VEC consecutive samples.
    o << "template <int VEC>\n__device__ __forceinline__ void ag_chunk" << suffix << "(const AgArgs& a, ag_u64 chunk";
    if (sum) o << (prec ? ", ag::e64::df& acc" : ", double& acc_h, double& acc_c");
    o << ") {\n";
    o << "    constexpr int L = AG_IPT * VEC;\n";
    o << "    ag_u64 s0[AG_IPT];\n";
    o << "#pragma unroll\n    for (int j = 0; j < AG_IPT; ++j) s0[j] = chunk * (ag_u64)(AG_BLOCK * AG_IPT * VEC) + ((ag_u64)j * AG_BLOCK + threadIdx.x) * VEC;\n";
    // One range check for every lane group of the thread (the last is the furthest).
    o << "    const bool full_ = s0[AG_IPT - 1] + (ag_u64)VEC <= a.n;\n";
    // Loads of every operand used in the lane context.
    std::set<int> lane_ops, zero_ops;
    for (size_t id = 0; id < P.nodes.size(); ++id) {
        const Node& n = P.nodes[id];
        if (n.op != "in") continue;
        if (!g.done[id]) continue;
        (ctx[id] ? zero_ops : lane_ops).insert(n.k);
    }
    for (int k : lane_ops) {
        const std::string T = ctype(P.operand_dtype[size_t(k)]);
        const int C = P.operand_comps[size_t(k)];
        o << "    const " << T << "* __restrict__ p" << k << " = (const " << T << "*)a.ops[" << k << "];\n";
        o << "    " << T << " in" << k << "[" << C << "][L];\n";
        o << "    if (full_) {\n#pragma unroll\n    for (int c = 0; c < " << C << "; ++c)\n#pragma unroll\n        for (int j = 0; j < AG_IPT; ++j) ag::vec_io<VEC, "
          << T << ">::load_full(p" << k << " + c * a.pitch[" << k << "], s0[j], &in" << k << "[c][j * VEC]);\n    } else {\n";
        o << "#pragma unroll\n    for (int c = 0; c < " << C << "; ++c)\n#pragma unroll\n        for (int j = 0; j < AG_IPT; ++j) ag::vec_io<VEC, "
          << T << ">::load(p" << k << " + c * a.pitch[" << k << "], s0[j], a.n, &in" << k << "[c][j * VEC]);\n    }\n";
    }
    if (rw) {
        const int RC = P.op == "acc" ? OC : P.dst_comps;   // accumulation also reads the compensation planes
        o << "    " << S << "* __restrict__ pd = (" << S << "*)a.dst;\n";
        o << "    " << S << " cur[" << RC << "][L];\n";
        o << "#pragma unroll\n    for (int c = 0; c < " << RC << "; ++c)\n#pragma unroll\n        for (int j = 0; j < AG_IPT; ++j) ag::vec_io<VEC, "
          << S << ">::load_rw(pd + c * a.dst_pitch, s0[j], a.n, &cur[c][j * VEC]);\n";
    }
    // Sample-0 prologue (at0 subtrees): loads of sample 0 and their values.
    for (int k : zero_ops) {
        const std::string T = ctype(P.operand_dtype[size_t(k)]);
        const int C = P.operand_comps[size_t(k)];
        o << "    " << T << " x" << k << "_0[" << C << "];\n";
        o << "#pragma unroll\n    for (int c = 0; c < " << C << "; ++c) x" << k << "_0[c] = ((const " << T << "*)a.ops[" << k
          << "])[c * a.pitch[" << k << "]];\n";
    }
    if (P.has_random) o << "    const ag_u32 g0 = a.offset;\n";
    if (emu) o << "    bool ok0_ = true;\n";
    // Plain assignments recompute their out-of-range lanes after the stores,
    // keeping the native call out of the lane loop.
    const bool defer = emu && P.op == "set" && store;
    if (defer) o << "    unsigned bad_ = 0u;\n";
    o << g.pro.str();
    if (store) o << "    " << S << " out[" << OC << "][L];\n";
    o << "#pragma unroll\n    for (int l = 0; l < L; ++l) {\n";
    if (P.has_random) o << "        const ag_u32 g = a.offset + (ag_u32)(s0[l / VEC] + (ag_u64)(l % VEC));\n";
    if (emu) o << "        bool ok_ = ok0_;\n";
    o << g.body.str();
    // Final working values of the output components. The output range test
    // is left out when the magnitude bounds of the root keep every value of a
    // lane that passed its other checks inside [2^-88, 2^126).
    const std::string FW = emu ? "double" : W;
    const bool out_safe = emu && g.lo_of(P.root) >= (tfx ? -80 : -88) && g.hi_of(P.root) <= 125;
    for (int c = 0; c < P.dst_comps; ++c) {
        if (prec) {
            o << "        ag::e64::df fv" << c << " = " << root[size_t(c)] << ";\n";
            if (!out_safe) o << "        ok_ = ok_ && ag::e64::out_ok(fv" << c << ");\n";
        } else if (emu) {
            o << "        double fv" << c << " = " << g.NS << "to_double(" << root[size_t(c)] << ");\n";
            if (!out_safe) o << "        ok_ = ok_ && " << g.NS << "out_ok(" << root[size_t(c)] << ");\n";
        } else {
            o << "        const " << W << " fv" << c << " = " << root[size_t(c)] << ";\n";
        }
    }
    if (defer) {
        o << "        bad_ |= ok_ ? 0u : (1u << l);\n";
    } else if (emu) {
        // Samples outside the double-float range are recomputed natively.
        o << "        const ag_u64 sl_ = s0[l / VEC] + (ag_u64)(l % VEC);\n";
        o << "        if (!ok_ && sl_ < a.n) {\n            double nv_[" << P.dst_comps << "];\n";
        o << "            ag_native_lane" << suffix << "(a, sl_, nv_);\n";
        for (int c = 0; c < P.dst_comps; ++c)
            o << "            fv" << c << " = " << (prec ? "ag::e64::dfc(nv_[" + std::to_string(c) + "])" : "nv_[" + std::to_string(c) + "]") << ";\n";
        o << "        }\n";
    }
    for (int c = 0; c < P.dst_comps; ++c) {
        const std::string v = "fv" + std::to_string(c);
        if (!store) continue;
        if (prec) {
            // float-float value: rounded once to float, or stored as its (hi, lo) planes
            if (dst_ff) {
                o << "        out[" << c << "][l] = " << v << ".hi;\n";
                o << "        out[" << (P.dst_comps + c) << "][l] = " << v << ".lo;\n";
            } else {
                o << "        out[" << c << "][l] = __fadd_rn(" << v << ".hi, " << v << ".lo);\n";
            }
        } else if (P.op == "set" || P.op == "setsum") {
            o << "        out[" << c << "][l] = (" << S << ")" << v << ";\n";
        } else if (P.op == "add") {
            o << "        out[" << c << "][l] = (" << S << ")ag::rn_add((" << FW << ")cur[" << c << "][l], " << v << ");\n";
        } else if (P.op == "acc") {
            // value += term; the exact residual of that sum joins the
            // compensation plane (accum/atomic.h:141-160)
            const std::string cv = "cur[" + std::to_string(c) + "][l]";
            o << "        { const double s_ = ag::rn_add(" << cv << ", " << v << ");\n";
            o << "          out[" << c << "][l] = s_;\n";
            o << "          out[" << (P.dst_comps + c) << "][l] = ag::rn_add(cur[" << (P.dst_comps + c)
              << "][l], ag::two_sum_err(" << cv << ", " << v << ", s_)); }\n";
        } else {
            o << "        out[" << c << "][l] = (" << S << ")ag::rn_sub((" << FW << ")cur[" << c << "][l], " << v << ");\n";
        }
    }
    if (atomic_acc) {
        // concurrent producers: atomicAdd returns the value it added to, so
        // the residual of each addition is exact and goes to the compensation
        // plane (the CompensatedAtomic policy of accum/AccumPlane.h)
        o << "        { const ag_u64 sa_ = s0[l / VEC] + (ag_u64)(l % VEC);\n";
        o << "          if (sa_ < a.n) {\n";
        o << "            double* __restrict__ pv_ = (double*)a.dst;\n";
        for (int c = 0; c < P.dst_comps; ++c) {
            const std::string v = "(double)fv" + std::to_string(c);
            o << "            { const double o_ = atomicAdd(pv_ + " << c << " * a.dst_pitch + sa_, " << v << ");\n";
            o << "              atomicAdd(pv_ + " << (P.dst_comps + c) << " * a.dst_pitch + sa_, ag::two_sum_err(o_, " << v
              << ", ag::rn_add(o_, " << v << "))); }\n";
        }
        o << "          } }\n";
    }
    if (sum) {
        o << "        if (s0[l / VEC] + (ag_u64)(l % VEC) < a.n) ";
        if (prec) o << "acc = ag::e64::add(acc, fv0);\n";   // per-thread float-float sum
        else o << "ag::neumaier_add(acc_h, acc_c, (double)fv0);\n";
    }
    o << "    }\n";
    if (store) {
        o << "    " << S << "* __restrict__ po = (" << S << "*)a.dst;\n";
        o << "    if (full_) {\n#pragma unroll\n    for (int c = 0; c < " << OC << "; ++c)\n#pragma unroll\n        for (int j = 0; j < AG_IPT; ++j) ag::vec_io<VEC, " << S
          << ">::store_full(po + c * a.dst_pitch, s0[j], &out[c][j * VEC]);\n    } else {\n";
        o << "#pragma unroll\n    for (int c = 0; c < " << OC << "; ++c)\n#pragma unroll\n        for (int j = 0; j < AG_IPT; ++j) ag::vec_io<VEC, " << S
          << ">::store(po + c * a.dst_pitch, s0[j], a.n, &out[c][j * VEC]);\n    }\n";
    }
    if (defer) {
        // the native recomputation overwrites the lanes the fast path could not serve
        o << "    if (bad_) {\n        " << S << "* __restrict__ pf_ = (" << S << "*)a.dst;\n";
        o << "        for (int l = 0; l < L; ++l) {\n";
        o << "            const ag_u64 sl_ = s0[l / VEC] + (ag_u64)(l % VEC);\n";
        o << "            if (((bad_ >> l) & 1u) && sl_ < a.n) {\n";
        o << "                double nv_[" << P.dst_comps << "];\n";
        o << "                ag_native_lane" << suffix << "(a, sl_, nv_);\n";
        for (int c = 0; c < P.dst_comps; ++c) {
            const std::string at = "pf_[(ag_u64)" + std::to_string(c) + " * a.dst_pitch + sl_]";
            const std::string nv = "nv_[" + std::to_string(c) + "]";
            if (prec) {
                o << "                { const ag::e64::df f_ = ag::e64::dfc(" << nv << ");\n";
                if (dst_ff)
                    o << "                  " << at << " = f_.hi;\n                  pf_[(ag_u64)" << (P.dst_comps + c)
                      << " * a.dst_pitch + sl_] = f_.lo; }\n";
                else
                    o << "                  " << at << " = __fadd_rn(f_.hi, f_.lo); }\n";
            } else {
                o << "                " << at << " = (" << S << ")" << nv << ";\n";
            }
        }
        o << "            }\n        }\n    }\n";
    }
    o << "}\n";

    if (chunk_only) return o.str();
    std::ostringstream k;
    k << o.str();
    const std::string lb = low.min_blocks > 0 ? "__launch_bounds__(AG_BLOCK, " + std::to_string(low.min_blocks) + ")"
                                              : "__launch_bounds__(AG_BLOCK)";
    for (int variant = 0; variant < 2; ++variant) {
        const std::string name = base + (variant == 0 ? "_v" : "_s");
        const std::string V = variant == 0 ? "AG_VEC" : "1";
        k << "extern \"C\" __global__ void " << lb << " " << name << "(const AgArgs a) {\n";
        k << "    const ag_u64 per = (ag_u64)AG_BLOCK * AG_IPT * " << V << ";\n";
        k << "    const ag_u64 nchunks = (a.n + per - 1) / per;\n";
        k << "    for (ag_u64 ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {\n";
        if (sum && prec) {
            // float-float per thread, FP64 from the warp tree on
            k << "        ag::e64::df acc = ag::e64::mk(0.0f, 0.0f);\n";
            k << "        ag_chunk<" << V << ">(a, ch, acc);\n";
            k << "        ag::sum_chunk_finish<AG_BLOCK>(a, ch, nchunks, ag::e64::f2d(acc.hi), ag::e64::f2d(acc.lo));\n";
        } else if (sum) {
            k << "        double h = 0.0, c = 0.0;\n";
            k << "        ag_chunk<" << V << ">(a, ch, h, c);\n";
            k << "        ag::sum_chunk_finish<AG_BLOCK>(a, ch, nchunks, h, c);\n";
        } else {
            k << "        ag_chunk<" << V << ">(a, ch);\n";
        }
        k << "    }\n}\n";
    }
    return k.str();
}

}  // namespace ag

namespace ag {

std::string generate_batch_source(const std::vector<const Plan*>& plans, const std::vector<Lowering>& lows,
                                  int block, int ipt, const std::string& base, int min_blocks) {
    std::ostringstream o;
    bool emu = false;
    for (const Lowering& l : lows) emu = emu || l.math >= 1;
    o << "// generated by aether_gb300: batch of " << plans.size() << " plans\n";
    o << "#include \"ag_device.cuh\"\n";
    if (emu) o << "#include \"ag_emu64.cuh\"\n";
    bool bm = false;
    for (size_t p = 0; p < plans.size(); ++p) bm = bm || (lows[p].math >= 1 && draws_normals(*plans[p]));
    if (bm) o << "#include \"ag_emu64_bm.cuh\"\n";
    bool tf = false;
    for (size_t p = 0; p < plans.size(); ++p) tf = tf || (lows[p].math == 3 && plans[p]->dst_dtype == DType::F64);
    if (tf) o << "#include \"ag_tf64.cuh\"\n";
    bool tft = false;
    for (size_t p = 0; p < plans.size(); ++p)
        tft = tft || (lows[p].math == 3 && plans[p]->dst_dtype == DType::F64 && uses_trig(*plans[p]));
    if (tft) o << "#include \"ag_tf64_trig.cuh\"\n";
    o << "#define AG_BLOCK " << block << "\n#define AG_IPT " << ipt << "\n";
    std::vector<int> vecs;
    for (size_t p = 0; p < plans.size(); ++p) {
        if (plans[p]->wants_sum()) throw std::runtime_error("aether-ir: sum plans cannot join a batch");
        Lowering l = lows[p];
        l.block = block;
        l.ipt = ipt;
        vecs.push_back(effective_vec(*plans[p], l));
        o << generate_source(*plans[p], l, base, "_p" + std::to_string(p), true);
    }
    // The work list: one argument block per item, the first global tile of the
    // item, and the plan it runs. Items are sorted by tile0.
    o << "struct AgItem {\n    AgArgs a;\n    ag_u64 tile0;\n    int plan;\n    int pad;\n};\n";
    o << "extern \"C\" __global__ void __launch_bounds__(AG_BLOCK"
      << (min_blocks > 0 ? ", " + std::to_string(min_blocks) : std::string()) << ") " << base
      << "(const AgItem* __restrict__ items, int n_items, ag_u64 total_tiles) {\n";
    o << "    __shared__ int s_item;\n";
    o << "    for (ag_u64 t = blockIdx.x; t < total_tiles; t += gridDim.x) {\n";
    o << "        if (threadIdx.x == 0) {\n";
    o << "            int lo = 0, hi = n_items - 1;\n";
    o << "            while (lo < hi) {\n";
    o << "                const int mid = (lo + hi + 1) >> 1;\n";
    o << "                if (items[mid].tile0 <= t) lo = mid; else hi = mid - 1;\n";
    o << "            }\n";
    o << "            s_item = lo;\n";
    o << "        }\n";
    o << "        __syncthreads();\n";
    o << "        const AgItem& it = items[s_item];\n";
    o << "        __syncthreads();\n";
    o << "        const ag_u64 ch = t - it.tile0;\n";
    o << "        switch (it.plan) {\n";
    for (size_t p = 0; p < plans.size(); ++p)
        o << "        case " << p << ": ag_chunk_p" << p << "<" << vecs[p] << ">(it.a, ch); break;\n";
    o << "        default: break;\n        }\n    }\n}\n";
    return o.str();
}

}  // namespace ag
