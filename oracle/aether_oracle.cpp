// aether_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see aether_oracle.h).
//
// CPU restatement of the reference's fused-expression path. Built with
// -ffp-contract=off so every a*b+c rounds twice, as the reference's own
// bit-identity builds do (docs/content/numerics_contract.rst:109-146).
// Each function names the reference file:line whose behaviour it restates.

#include "aether_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Philox4x32-10 -- random/detail/Philox.h:95-133 (Salmon et al., SC'11, with
// cuRAND's block layout).
// ---------------------------------------------------------------------------
constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;

struct Q4 {
    uint32_t x, y, z, w;
};

inline Q4 philox(Q4 c, uint32_t kx, uint32_t ky) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            kx += kW0;
            ky += kW1;
        }
        const uint64_t p0 = uint64_t(kM0) * c.x;
        const uint64_t p1 = uint64_t(kM1) * c.z;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c = Q4{hi1 ^ c.y ^ kx, lo1, hi0 ^ c.w ^ ky, lo0};
    }
    return c;
}

// Backend.h:136-150: the block owned by (seed, global, counter).
inline Q4 block(uint64_t seed, uint32_t global, uint64_t counter) {
    return philox(Q4{uint32_t(counter), uint32_t(counter >> 32), global, 0u}, uint32_t(seed), uint32_t(seed >> 32));
}

// Backend.h:75-82.
inline uint64_t splitmix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

constexpr double k2m32 = 2.3283064365386963e-10;   // 2^-32
constexpr double k2m53 = 1.1102230246251565e-16;   // 2^-53
constexpr double kPi = 3.1415926535897932;
constexpr float k2m32f2pi = 2.3283064e-10f * 6.2831855f;

// Backend.h:123-131 (double: w*2^-32 + 2^-33; float: (2*(w>>9)+1)*2^-24).
inline double u01d(uint32_t w) { return w * k2m32 + (k2m32 / 2.0); }
inline float u01f(uint32_t w) { return float(((w >> 9) << 1) | 1u) * 5.9604645e-8f; }
// Backend.h:152-157.
inline double u01hq(uint32_t x, uint32_t y) {
    const uint64_t z = uint64_t(x) ^ (uint64_t(y) << 21);
    return double(z) * k2m53 + (k2m53 / 2.0);
}

// Backend.h:209-236 (Box-Muller, first normal only). `T` selects the
// precision of the transcendental evaluation; the word -> real conversions
// and the v*pi product are always the double ones of the reference.
template <class T>
T normal_d(uint64_t seed, uint32_t global, uint64_t counter) {
    const Q4 x = block(seed, global, counter);
    const double u = u01hq(x.x, x.y);
    const uint64_t zy = uint64_t(x.z) ^ (uint64_t(x.w) << 21);
    const double v = double(zy) * (k2m53 * 2.0) + k2m53;
    const double arg = v * kPi;
    const T s = std::sqrt(T(-2.0) * std::log(T(u)));
    return s * std::sin(T(arg));
}
inline float normal_f(uint64_t seed, uint32_t global, uint64_t counter) {
    const Q4 x = block(seed, global, counter);
    const float u = u01f(x.x);
    const float v = float(x.y) * k2m32f2pi + (k2m32f2pi / 2.0f);
    const float s = std::sqrt(-2.0f * std::log(u));
    return s * std::sin(v);
}

// Per-distribution salts, random/detail/DistributionLeaf.h:117,184,249,313,373.
constexpr uint64_t kSaltUniform = 0x243F6A8885A308D3ULL;
constexpr uint64_t kSaltNormal = 0x13198A2E03707344ULL;
constexpr uint64_t kSaltLognormal = 0xA4093822299F31D0ULL;
constexpr uint64_t kSaltExponential = 0x082EFA98EC4E6C89ULL;
constexpr uint64_t kSaltBernoulli = 0x452821E638D01377ULL;

// ---------------------------------------------------------------------------
// Compensated sums -- accum/TwoSum.h:86-100 (host arm: Knuth two-sum),
// accum/atomic.h:141-191 (neumaierAdd_, pairCombine_, reduce32Host_).
// ---------------------------------------------------------------------------
template <class T>
inline T two_sum_err(T a, T b, T s) {
    volatile T bb = s - a;
    volatile T t1 = s - bb;
    return (a - t1) + (b - bb);
}
template <class T>
inline void pair_combine(T ah, T ac, T bh, T bc, T& oh, T& oc) {
    const T s = ah + bh;
    const T e = two_sum_err(ah, bh, s);
    oh = s;
    oc = std::isfinite(s) ? (ac + bc) + e : T(0);
}
template <class T>
inline void neumaier_add(T& hi, T& comp, T term) {
    const T s = hi + term;
    const T e = two_sum_err(hi, term, s);
    hi = s;
    comp = std::isfinite(s) ? comp + e : T(0);
}
template <class T>
void reduce32(const T* hi, const T* comp, T& oh, T& oc) {
    T h[32], c[32];
    for (int l = 0; l < 32; ++l) {
        h[l] = hi[l];
        c[l] = comp[l];
    }
    for (int off = 16; off >= 1; off >>= 1) {
        T nh[32], nc[32];
        for (int l = 0; l < 32; ++l) pair_combine(h[l], c[l], h[l ^ off], c[l ^ off], nh[l], nc[l]);
        for (int l = 0; l < 32; ++l) {
            h[l] = nh[l];
            c[l] = nc[l];
        }
    }
    oh = h[0];
    oc = c[0];
}

// ---------------------------------------------------------------------------
// IR parser. The grammar is the engine's own (aether-ir/1); each node's
// evaluation below restates the reference node it lowers.
// ---------------------------------------------------------------------------
struct Node {
    std::string op;
    std::vector<int> kids;
    std::vector<int> shape;   // element extents (empty = rank 0)
    int comps = 1;
    bool is_bool = false;
    int k = 0;                 // slot (in/sc/key) or integer argument
    std::vector<int> ints;     // further integer arguments
    double lit = 0.0;
    std::string dtype;         // `in` operand storage type
};

struct Plan {
    std::string dst_dtype;
    std::vector<int> dst_shape;
    int dst_comps = 1;
    std::string op;
    std::vector<Node> nodes;
    int root = -1;
};

struct Lexer {
    const char* p;
    explicit Lexer(const char* s) : p(s) {}
    void ws() {
        while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') ++p;
    }
    std::string tok() {
        ws();
        if (!*p) throw std::runtime_error("ir: unexpected end");
        if (*p == '(' || *p == ')') return std::string(1, *p++);
        const char* s = p;
        if (*p == '[') {
            while (*p && *p != ']') ++p;
            if (*p != ']') throw std::runtime_error("ir: unterminated shape");
            ++p;
            return std::string(s, p);
        }
        while (*p && *p != ' ' && *p != '(' && *p != ')' && *p != '\n' && *p != '\t') ++p;
        return std::string(s, p);
    }
    std::string peek() {
        const char* save = p;
        std::string t = tok();
        p = save;
        return t;
    }
};

std::vector<int> parse_shape(const std::string& t) {
    if (t.size() < 2 || t.front() != '[' || t.back() != ']') throw std::runtime_error("ir: bad shape " + t);
    std::vector<int> s;
    std::string inner = t.substr(1, t.size() - 2);
    size_t i = 0;
    while (i < inner.size()) {
        size_t j = inner.find(',', i);
        if (j == std::string::npos) j = inner.size();
        s.push_back(std::stoi(inner.substr(i, j - i)));
        i = j + 1;
    }
    return s;
}
int prod(const std::vector<int>& s) {
    int p = 1;
    for (int v : s) p *= v;
    return p;
}

struct Parser {
    Lexer lx;
    Plan plan;
    std::map<std::string, int> memo;   // structural CSE: same text, same node
    int ctx = 0;                       // 1 inside an at0 subtree
    explicit Parser(const char* s) : lx(s) {}

    void expect(const char* t) {
        std::string g = lx.tok();
        if (g != t) throw std::runtime_error(std::string("ir: expected ") + t + " got " + g);
    }
    int integer() { return std::stoi(lx.tok()); }

    int add(Node n) {
        plan.nodes.push_back(std::move(n));
        return int(plan.nodes.size()) - 1;
    }
    const Node& N(int i) const { return plan.nodes[i]; }

    int expr() {
        const char* start = lx.p;
        expect("(");
        Node n;
        n.op = lx.tok();
        const std::string& op = n.op;
        auto kid = [&]() { int c = expr(); n.kids.push_back(c); return c; };
        auto same_shape = [&](int a, int b) {
            if (N(a).shape != N(b).shape) throw std::runtime_error("ir: shape mismatch in " + op);
        };
        auto need_rank0 = [&](int a) {
            if (!N(a).shape.empty()) throw std::runtime_error("ir: rank-0 operand required in " + op);
        };
        static const char* kUnary[] = {"neg", "abs", "sign", "sqrt", "rsqrt", "exp", "expm1", "log", "log1p",
                                       "log2", "log10", "exp2", "sin", "cos", "tan", "asin", "acos", "atan",
                                       "tanh", "sinh", "cosh", "sq", "floor", "ceil", "trunc", "cbrt", "erf"};
        static const char* kBinary[] = {"add", "sub", "mul", "div", "pow", "min", "max", "atan2", "hypot"};
        static const char* kCmp[] = {"gt", "lt", "ge", "le", "eq", "ne"};
        auto in_list = [&](const char* const* l, size_t cnt) {
            for (size_t i = 0; i < cnt; ++i)
                if (op == l[i]) return true;
            return false;
        };
        if (op == "in") {
            n.k = integer();
            n.dtype = lx.tok();
            n.shape = parse_shape(lx.tok());
        } else if (op == "sc") {
            n.k = integer();
            if (lx.peek() == "+") lx.tok();   // sign hint: the value is >= 0
        } else if (op == "lit") {
            n.lit = std::strtod(lx.tok().c_str(), nullptr);
        } else if (op == "bcast") {
            int a = kid();
            need_rank0(a);
            n.shape = parse_shape(lx.tok());
            n.is_bool = N(a).is_bool;
        } else if (op == "at0") {
            // The subtree evaluated at sample 0: Expression's eager folds
            // (norm, rNorm, dot, ...) read their operand at
            // SampleIndex::make(0) (expr/Expression.h:148-173).
            const int save = ctx;
            ctx = 1;
            int a = kid();
            ctx = save;
            n.shape = N(a).shape;
            n.is_bool = N(a).is_bool;
        } else if (in_list(kUnary, sizeof(kUnary) / sizeof(*kUnary))) {
            int a = kid();
            n.shape = N(a).shape;
        } else if (in_list(kBinary, sizeof(kBinary) / sizeof(*kBinary))) {
            int a = kid(), b = kid();
            same_shape(a, b);
            n.shape = N(a).shape;
        } else if (op == "scale" || op == "mins" || op == "maxs" || op == "pows") {
            int a = kid(), s = kid();
            need_rank0(s);
            n.shape = N(a).shape;
        } else if (op == "clamp") {
            int a = kid(), lo = kid(), hi = kid();
            need_rank0(lo);
            need_rank0(hi);
            n.shape = N(a).shape;
        } else if (in_list(kCmp, sizeof(kCmp) / sizeof(*kCmp)) || op == "and" || op == "or") {
            int a = kid(), b = kid();
            same_shape(a, b);
            n.shape = N(a).shape;
            n.is_bool = true;
        } else if (op == "not") {
            int a = kid();
            n.shape = N(a).shape;
            n.is_bool = true;
        } else if (op == "select") {
            int c = kid(), a = kid(), b = kid();
            same_shape(a, b);
            if (!N(c).shape.empty() && N(c).shape != N(a).shape) throw std::runtime_error("ir: select cond shape");
            n.shape = N(a).shape;
            n.is_bool = N(a).is_bool;
        } else if (op == "comp") {
            kid();
            n.k = integer();
        } else if (op == "seg") {
            int a = kid();
            n.k = integer();
            n.ints = {integer()};
            if (N(a).shape.size() != 1) throw std::runtime_error("ir: seg needs rank 1");
            n.shape = {n.ints[0]};
        } else if (op == "row" || op == "col") {
            int a = kid();
            n.k = integer();
            if (N(a).shape.size() != 2) throw std::runtime_error("ir: row/col needs rank 2");
            n.shape = {op == "row" ? N(a).shape[1] : N(a).shape[0]};
        } else if (op == "transpose") {
            int a = kid();
            if (N(a).shape.size() != 2) throw std::runtime_error("ir: transpose needs rank 2");
            n.shape = {N(a).shape[1], N(a).shape[0]};
        } else if (op == "block") {
            kid();
            n.ints = {integer(), integer(), integer(), integer()};
            n.shape = {n.ints[2], n.ints[3]};
        } else if (op == "stack") {
            while (lx.peek() != ")") {
                int a = kid();
                need_rank0(a);
            }
            n.shape = {int(n.kids.size())};
        } else if (op == "reshape") {
            kid();
            n.shape = parse_shape(lx.tok());
        } else if (op == "cross") {
            int a = kid(), b = kid();
            same_shape(a, b);
            n.shape = {3};
        } else if (op == "unit" || op == "qconj") {
            int a = kid();
            n.shape = N(a).shape;
        } else if (op == "qmul") {
            kid();
            kid();
            n.shape = {4};
        } else if (op == "qrot") {
            kid();
            kid();
            n.shape = {3};
        } else if (op == "pureq") {
            kid();
            n.shape = {4};
        } else if (op == "inv") {
            int a = kid();
            n.shape = N(a).shape;
        } else if (op == "det" || op == "trace") {
            kid();
        } else if (op == "matvec") {
            int m = kid();
            kid();
            n.shape = {N(m).shape[0]};
        } else if (op == "matmul") {
            int a = kid(), b = kid();
            n.shape = {N(a).shape[0], N(b).shape[1]};
        } else if (op == "outer") {
            int a = kid(), b = kid();
            n.shape = {N(a).shape[0], N(b).shape[0]};
        } else if (op == "dot") {
            int a = kid(), b = kid();
            same_shape(a, b);
        } else if (op == "sqnorm" || op == "norm" || op == "rnorm" || op == "sum" || op == "maxnorm") {
            kid();
        } else if (op == "uniform" || op == "normal" || op == "lognormal") {
            n.k = integer();
            kid();
            kid();
            n.shape = {integer()};
        } else if (op == "exponential" || op == "bernoulli") {
            n.k = integer();
            kid();
            n.shape = {integer()};
        } else {
            throw std::runtime_error("ir: unknown op " + op);
        }
        expect(")");
        n.comps = prod(n.shape);
        std::string text = std::to_string(ctx) + std::string(start, lx.p);
        auto it = memo.find(text);
        if (it != memo.end()) return it->second;
        int id = add(std::move(n));
        memo.emplace(std::move(text), id);
        return id;
    }

    Plan run() {
        expect("(");
        expect("plan");
        plan.dst_dtype = lx.tok();
        plan.dst_shape = parse_shape(lx.tok());
        plan.dst_comps = prod(plan.dst_shape);
        plan.op = lx.tok();
        plan.root = expr();
        expect(")");
        if (plan.nodes[plan.root].shape != plan.dst_shape) throw std::runtime_error("ir: root shape != dst shape");
        return plan;
    }
};

// ---------------------------------------------------------------------------
// Interpreter: evaluate the tree over a block of samples, node by node, in
// working type T. Each case states the reference node it follows.
// ---------------------------------------------------------------------------
constexpr int kB = 256;

template <class T>
struct Eval {
    const Plan& P;
    const OrcArgs& A;
    bool elem_f32;   // the plan's element type (drives random draws and scalars)
    std::vector<std::vector<T>> val;
    std::vector<char> done;
    uint64_t s0 = 0;
    int nb = 0;

    Eval(const Plan& p, const OrcArgs& a, bool f32) : P(p), A(a), elem_f32(f32), val(p.nodes.size()),
                                                      done(p.nodes.size(), 0) {}

    T scalar(double v) const { return elem_f32 ? T(float(v)) : T(v); }

    T unary(const std::string& op, T x) const {
        using std::abs;
        if (op == "neg") return -x;
        if (op == "abs") return std::fabs(x);
        if (op == "sign") return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));   // math/math.h:162-171
        if (op == "sqrt") return std::sqrt(x);
        if (op == "rsqrt") return T(1) / std::sqrt(x);                            // math/root.h:64-76 (host)
        if (op == "exp") return std::exp(x);
        if (op == "expm1") return std::expm1(x);
        if (op == "log") return std::log(x);
        if (op == "log1p") return std::log1p(x);
        if (op == "log2") return std::log2(x);
        if (op == "log10") return std::log10(x);
        if (op == "exp2") return std::exp2(x);
        if (op == "sin") return std::sin(x);
        if (op == "cos") return std::cos(x);
        if (op == "tan") return std::tan(x);
        if (op == "asin") return std::asin(x);
        if (op == "acos") return std::acos(x);
        if (op == "atan") return std::atan(x);
        if (op == "tanh") return std::tanh(x);
        if (op == "sinh") return std::sinh(x);
        if (op == "cosh") return std::cosh(x);
        if (op == "sq") return x * x;
        if (op == "floor") return std::floor(x);
        if (op == "ceil") return std::ceil(x);
        if (op == "trunc") return std::trunc(x);
        if (op == "cbrt") return std::cbrt(x);
        if (op == "erf") return std::erf(x);
        throw std::runtime_error("oracle: unary " + op);
    }
    T binary(const std::string& op, T a, T b) const {
        if (op == "add") return a + b;                 // expr/nodes/Arithmetic.h:62-70
        if (op == "sub") return a - b;
        if (op == "mul") return a * b;                 // Arithmetic.h:101-104 (Hadamard)
        if (op == "div") return a / b;                 // expr/nodes/Elementwise.h:589-617
        if (op == "pow") return std::pow(a, b);        // Elementwise.h:620-650
        if (op == "min") return std::fmin(a, b);       // Elementwise.h:652-680
        if (op == "max") return std::fmax(a, b);
        if (op == "atan2") return std::atan2(a, b);
        if (op == "hypot") return std::hypot(a, b);
        throw std::runtime_error("oracle: binary " + op);
    }

    // The draw for sample `g`, component `c`, computed in the plan's element
    // type and widened to T (random/detail/DistributionLeaf.h:125-131,192-199).
    T draw01(uint64_t seed, uint32_t g, uint64_t c) const {
        const Q4 x = block(seed, g, c);
        return elem_f32 ? T(u01f(x.x)) : T(u01d(x.x));
    }
    T drawn(uint64_t seed, uint32_t g, uint64_t c) const {
        if (elem_f32) return T(normal_f(seed, g, c));
        if (sizeof(T) > sizeof(double)) return T(normal_d<T>(seed, g, c));
        return T(normal_d<double>(seed, g, c));
    }

    const T* get(int id) {
        if (done[id]) return val[id].data();
        const Node& n = P.nodes[id];
        std::vector<T>& out = val[id];
        out.assign(size_t(n.comps) * nb, T(0));
        auto K = [&](int j) { return get(n.kids[j]); };
        auto at = [&](const T* p, int c, int s) { return p[size_t(c) * nb + s]; };
        auto O = [&](int c, int s) -> T& { return out[size_t(c) * nb + s]; };
        const std::string& op = n.op;

        if (op == "in") {   // view/View.h:234-246,369-377: data[c*pitch + i]
            if (n.k >= int(A.n_operands)) throw std::runtime_error("oracle: operand slot");
            const OrcOperand& o = A.operands[n.k];
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) {
                    const uint64_t idx = uint64_t(c) * o.pitch + s0 + s;
                    if (n.dtype == "f64") O(c, s) = T(static_cast<const double*>(o.ptr)[idx]);
                    else if (n.dtype == "f32") O(c, s) = T(static_cast<const float*>(o.ptr)[idx]);
                    else if (n.dtype == "i32") O(c, s) = T(static_cast<const int32_t*>(o.ptr)[idx]);
                    else if (n.dtype == "u8") O(c, s) = T(static_cast<const uint8_t*>(o.ptr)[idx] != 0);
                    else throw std::runtime_error("oracle: dtype " + n.dtype);
                }
        } else if (op == "sc") {   // a scalar captured by value (Arithmetic.h:118-128)
            if (n.k >= int(A.n_scalars)) throw std::runtime_error("oracle: scalar slot");
            for (int s = 0; s < nb; ++s) O(0, s) = scalar(A.scalars[n.k]);
        } else if (op == "lit") {
            for (int s = 0; s < nb; ++s) O(0, s) = scalar(n.lit);
        } else if (op == "bcast") {   // expr/nodes/Constant.h:68-150
            const T* a = K(0);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = a[s];
        } else if (op == "at0") {
            Eval<T> sub(P, A, elem_f32);
            sub.reset(0, 1);
            const T* a = sub.get(n.kids[0]);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = a[c];
        } else if (n.kids.size() == 1 && (op == "neg" || op == "abs" || op == "sign" || op == "sqrt" ||
                   op == "rsqrt" || op == "exp" || op == "expm1" || op == "log" || op == "log1p" ||
                   op == "log2" || op == "log10" || op == "exp2" || op == "sin" || op == "cos" || op == "tan" ||
                   op == "asin" || op == "acos" || op == "atan" || op == "tanh" || op == "sinh" ||
                   op == "cosh" || op == "sq" || op == "floor" || op == "ceil" || op == "trunc" ||
                   op == "cbrt" || op == "erf")) {   // Elementwise.h:112-496
            const T* a = K(0);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = unary(op, at(a, c, s));
        } else if (op == "add" || op == "sub" || op == "mul" || op == "div" || op == "pow" || op == "min" ||
                   op == "max" || op == "atan2" || op == "hypot") {
            const T* a = K(0);
            const T* b = K(1);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = binary(op, at(a, c, s), at(b, c, s));
        } else if (op == "scale") {   // CWiseScale: factor * e (Arithmetic.h:130-140)
            const T* a = K(0);
            const T* f = K(1);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = f[s] * at(a, c, s);
        } else if (op == "mins" || op == "maxs" || op == "pows") {   // Elementwise.h:62-110,714-739
            const T* a = K(0);
            const T* f = K(1);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) {
                    const T x = at(a, c, s);
                    O(c, s) = op == "mins" ? std::fmin(x, f[s]) : op == "maxs" ? std::fmax(x, f[s]) : std::pow(x, f[s]);
                }
        } else if (op == "clamp") {   // Elementwise.h:138-167: fmin(fmax(e, lo), hi)
            const T* a = K(0);
            const T* lo = K(1);
            const T* hi = K(2);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = std::fmin(std::fmax(at(a, c, s), lo[s]), hi[s]);
        } else if (op == "gt" || op == "lt" || op == "ge" || op == "le" || op == "eq" || op == "ne" || op == "and" ||
                   op == "or") {
            const T* a = K(0);
            const T* b = K(1);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) {
                    const T x = at(a, c, s), y = at(b, c, s);
                    bool r = op == "gt" ? x > y : op == "lt" ? x < y : op == "ge" ? x >= y : op == "le" ? x <= y
                           : op == "eq" ? x == y : op == "ne" ? x != y : op == "and" ? (x != 0 && y != 0)
                                                                                    : (x != 0 || y != 0);
                    O(c, s) = r ? T(1) : T(0);
                }
        } else if (op == "not") {
            const T* a = K(0);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = at(a, c, s) != 0 ? T(0) : T(1);
        } else if (op == "select") {   // Elementwise.h:809-846
            const T* cnd = K(0);
            const T* a = K(1);
            const T* b = K(2);
            const bool per_sample = P.nodes[n.kids[0]].shape.empty();
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) {
                    const T cv = per_sample ? cnd[s] : at(cnd, c, s);
                    O(c, s) = cv != T(0) ? at(a, c, s) : at(b, c, s);
                }
        } else if (op == "comp") {
            const T* a = K(0);
            for (int s = 0; s < nb; ++s) O(0, s) = at(a, n.k, s);
        } else if (op == "seg") {   // expr/nodes/Structural.h (Segment)
            const T* a = K(0);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = at(a, n.k + c, s);
        } else if (op == "row" || op == "col") {
            const T* a = K(0);
            const auto& sh = P.nodes[n.kids[0]].shape;
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s)
                    O(c, s) = op == "row" ? at(a, n.k * sh[1] + c, s) : at(a, c * sh[1] + n.k, s);
        } else if (op == "transpose") {
            const T* a = K(0);
            const auto& sh = P.nodes[n.kids[0]].shape;
            for (int r = 0; r < sh[1]; ++r)
                for (int c = 0; c < sh[0]; ++c)
                    for (int s = 0; s < nb; ++s) O(r * sh[0] + c, s) = at(a, c * sh[1] + r, s);
        } else if (op == "block") {
            const T* a = K(0);
            const auto& sh = P.nodes[n.kids[0]].shape;
            for (int r = 0; r < n.ints[2]; ++r)
                for (int c = 0; c < n.ints[3]; ++c)
                    for (int s = 0; s < nb; ++s)
                        O(r * n.ints[3] + c, s) = at(a, (n.ints[0] + r) * sh[1] + n.ints[1] + c, s);
        } else if (op == "stack") {
            for (int c = 0; c < n.comps; ++c) {
                const T* a = K(c);
                for (int s = 0; s < nb; ++s) O(c, s) = a[s];
            }
        } else if (op == "reshape") {
            const T* a = K(0);
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) O(c, s) = at(a, c, s);
        } else if (op == "cross") {   // expr/nodes/Geometric.h:55-72
            const T* l = K(0);
            const T* r = K(1);
            for (int s = 0; s < nb; ++s) {
                const T l0 = at(l, 0, s), l1 = at(l, 1, s), l2 = at(l, 2, s);
                const T r0 = at(r, 0, s), r1 = at(r, 1, s), r2 = at(r, 2, s);
                O(0, s) = l1 * r2 - l2 * r1;
                O(1, s) = l2 * r0 - l0 * r2;
                O(2, s) = l0 * r1 - l1 * r0;
            }
        } else if (op == "unit") {   // Geometric.h:99-103: e * rNorm(), rNorm = 1/sqrt(squaredNorm)
            const T* a = K(0);
            for (int s = 0; s < nb; ++s) {
                T acc = at(a, 0, s) * at(a, 0, s);
                for (int c = 1; c < n.comps; ++c) acc = at(a, c, s) * at(a, c, s) + acc;
                const T rn = T(1) / std::sqrt(acc);
                for (int c = 0; c < n.comps; ++c) O(c, s) = at(a, c, s) * rn;
            }
        } else if (op == "qmul") {   // expr/nodes/Quaternion.h:60-79 (Hamilton product)
            const T* l = K(0);
            const T* r = K(1);
            for (int s = 0; s < nb; ++s) {
                const T l0 = at(l, 0, s), l1 = at(l, 1, s), l2 = at(l, 2, s), l3 = at(l, 3, s);
                const T r0 = at(r, 0, s), r1 = at(r, 1, s), r2 = at(r, 2, s), r3 = at(r, 3, s);
                O(0, s) = l0 * r0 - l1 * r1 - l2 * r2 - l3 * r3;
                O(1, s) = l0 * r1 + l1 * r0 + l2 * r3 - l3 * r2;
                O(2, s) = l0 * r2 - l1 * r3 + l2 * r0 + l3 * r1;
                O(3, s) = l0 * r3 + l1 * r2 - l2 * r1 + l3 * r0;
            }
        } else if (op == "qconj") {   // Quaternion.h:103-108
            const T* a = K(0);
            for (int s = 0; s < nb; ++s) {
                O(0, s) = at(a, 0, s);
                for (int c = 1; c < 4; ++c) O(c, s) = -at(a, c, s);
            }
        } else if (op == "qrot") {   // Quaternion.h:142-168 (Rodrigues: t = 2(u x v), v + w t + u x t)
            const T* q = K(0);
            const T* v = K(1);
            const T two = scalar(2.0);
            for (int s = 0; s < nb; ++s) {
                const T w = at(q, 0, s), ux = at(q, 1, s), uy = at(q, 2, s), uz = at(q, 3, s);
                const T vx = at(v, 0, s), vy = at(v, 1, s), vz = at(v, 2, s);
                const T tx = two * (uy * vz - uz * vy);
                const T ty = two * (uz * vx - ux * vz);
                const T tz = two * (ux * vy - uy * vx);
                O(0, s) = vx + w * tx + (uy * tz - uz * ty);
                O(1, s) = vy + w * ty + (uz * tx - ux * tz);
                O(2, s) = vz + w * tz + (ux * ty - uy * tx);
            }
        } else if (op == "pureq") {   // Quaternion.h:192-203
            const T* a = K(0);
            for (int s = 0; s < nb; ++s) {
                O(0, s) = T(0);
                for (int c = 1; c < 4; ++c) O(c, s) = at(a, c - 1, s);
            }
        } else if (op == "inv" || op == "det") {   // expr/nodes/Inverse.h:73-118; Expression.h:400-428
            const T* m = K(0);
            const int dim = P.nodes[n.kids[0]].shape[0];
            for (int s = 0; s < nb; ++s) {
                if (dim == 2) {
                    const T a = at(m, 0, s), b = at(m, 1, s), c = at(m, 2, s), d = at(m, 3, s);
                    const T det = a * d - b * c;
                    if (op == "det") {
                        O(0, s) = det;
                    } else {
                        O(0, s) = d / det;
                        O(1, s) = -b / det;
                        O(2, s) = -c / det;
                        O(3, s) = a / det;
                    }
                } else {
                    const T a = at(m, 0, s), b = at(m, 1, s), c = at(m, 2, s);
                    const T d = at(m, 3, s), e = at(m, 4, s), f = at(m, 5, s);
                    const T g = at(m, 6, s), h = at(m, 7, s), k = at(m, 8, s);
                    const T det = a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
                    if (op == "det") {
                        O(0, s) = det;
                    } else {
                        O(0, s) = (e * k - f * h) / det;
                        O(1, s) = (c * h - b * k) / det;
                        O(2, s) = (b * f - c * e) / det;
                        O(3, s) = (f * g - d * k) / det;
                        O(4, s) = (a * k - c * g) / det;
                        O(5, s) = (c * d - a * f) / det;
                        O(6, s) = (d * h - e * g) / det;
                        O(7, s) = (b * g - a * h) / det;
                        O(8, s) = (a * e - b * d) / det;
                    }
                }
            }
        } else if (op == "trace") {   // Expression.h:381-398
            const T* m = K(0);
            const int dim = P.nodes[n.kids[0]].shape[0];
            for (int s = 0; s < nb; ++s) {
                T t = at(m, 0, s) + at(m, dim + 1, s);
                if (dim == 3) t = t + at(m, 8, s);
                O(0, s) = t;
            }
        } else if (op == "matvec" || op == "matmul" || op == "outer") {
            // expr/nodes/Product.h: each output element is a dot fold over the
            // shared index, accumulated in ascending index order.
            const T* a = K(0);
            const T* b = K(1);
            const auto& sa = P.nodes[n.kids[0]].shape;
            const auto& sb = P.nodes[n.kids[1]].shape;
            for (int s = 0; s < nb; ++s) {
                if (op == "outer") {
                    for (int i = 0; i < sa[0]; ++i)
                        for (int j = 0; j < sb[0]; ++j) O(i * sb[0] + j, s) = at(a, i, s) * at(b, j, s);
                } else if (op == "matvec") {
                    for (int i = 0; i < sa[0]; ++i) {
                        T acc = at(a, i * sa[1], s) * at(b, 0, s);
                        for (int k = 1; k < sa[1]; ++k) acc = at(a, i * sa[1] + k, s) * at(b, k, s) + acc;
                        O(i, s) = acc;
                    }
                } else {
                    for (int i = 0; i < sa[0]; ++i)
                        for (int j = 0; j < sb[1]; ++j) {
                            T acc = at(a, i * sa[1], s) * at(b, j, s);
                            for (int k = 1; k < sa[1]; ++k)
                                acc = at(a, i * sa[1] + k, s) * at(b, k * sb[1] + j, s) + acc;
                            O(i * sb[1] + j, s) = acc;
                        }
                }
            }
        } else if (op == "dot" || op == "sqnorm" || op == "norm" || op == "rnorm" || op == "sum" || op == "maxnorm") {
            // expr/Reduce.h:149-188: acc = T(x0); acc = Reduce(T(x_{k+1}), acc)
            const T* a = K(0);
            const T* b = op == "dot" ? K(1) : nullptr;
            const int m = P.nodes[n.kids[0]].comps;
            for (int s = 0; s < nb; ++s) {
                auto term = [&](int c) -> T {
                    const T x = at(a, c, s);
                    if (op == "dot") return x * at(b, c, s);
                    if (op == "sum") return x;
                    if (op == "maxnorm") return x < T(0) ? T(-x) : x;
                    return x * x;
                };
                T acc = term(0);
                for (int c = 1; c < m; ++c) {
                    const T t = term(c);
                    acc = op == "maxnorm" ? (t > acc ? t : acc) : t + acc;
                }
                if (op == "norm") acc = std::sqrt(acc);
                if (op == "rnorm") acc = T(1) / std::sqrt(acc);
                O(0, s) = acc;
            }
        } else if (op == "uniform" || op == "normal" || op == "lognormal" || op == "exponential" ||
                   op == "bernoulli") {
            if (n.k >= int(A.n_keys)) throw std::runtime_error("oracle: key slot");
            const uint64_t key = A.keys[n.k];
            const T* p0 = K(0);
            const T* p1 = n.kids.size() > 1 ? K(1) : nullptr;
            const bool b0 = P.nodes[n.kids[0]].shape.empty();
            const bool b1 = p1 && P.nodes[n.kids[1]].shape.empty();
            for (int c = 0; c < n.comps; ++c)
                for (int s = 0; s < nb; ++s) {
                    const uint32_t g = uint32_t(A.sample_offset + s0 + s);
                    const T x0 = b0 ? p0[s] : at(p0, c, s);
                    const T x1 = p1 ? (b1 ? p1[s] : at(p1, c, s)) : T(0);
                    if (op == "uniform") {   // DistributionLeaf.h:125-131
                        O(c, s) = x0 + (x1 - x0) * draw01(key ^ kSaltUniform, g, uint64_t(c));
                    } else if (op == "normal") {   // DistributionLeaf.h:192-199
                        O(c, s) = x0 + x1 * drawn(key ^ kSaltNormal, g, uint64_t(c));
                    } else if (op == "lognormal") {   // DistributionLeaf.h:257-264
                        O(c, s) = std::exp(x0 + x1 * drawn(key ^ kSaltLognormal, g, uint64_t(c)));
                    } else if (op == "exponential") {   // DistributionLeaf.h:329-333
                        O(c, s) = -std::log(draw01(key ^ kSaltExponential, g, uint64_t(c))) / x0;
                    } else {   // DistributionLeaf.h:380-385
                        O(c, s) = draw01(key ^ kSaltBernoulli, g, uint64_t(c)) < x0 ? T(1) : T(0);
                    }
                }
        } else {
            throw std::runtime_error("oracle: no evaluator for " + op);
        }
        done[id] = 1;
        return out.data();
    }

    void reset(uint64_t start, int count) {
        s0 = start;
        nb = count;
        std::fill(done.begin(), done.end(), 0);
    }
};

template <class T>
int run_plan(const Plan& P, int mode, const OrcArgs& A, int nthreads) {
    const bool f32 = P.dst_dtype != "f64";
    const uint64_t nblocks = (A.n + kB - 1) / kB;
    const bool want_sum = P.op == "sum" || P.op == "setsum";
    const bool want_store = P.op != "sum";
    std::vector<long double> part_hi(want_sum ? nblocks : 0), part_c(want_sum ? nblocks : 0);
    std::string err;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t b = 0; b < int64_t(nblocks); ++b) {
        try {
            Eval<T> local(P, A, f32);
            const uint64_t start = uint64_t(b) * kB;
            const int cnt = int(std::min<uint64_t>(kB, A.n - start));
            local.reset(start, cnt);
            const T* r = local.get(P.root);
            if (want_store) {
                for (int c = 0; c < P.dst_comps; ++c)
                    for (int s = 0; s < cnt; ++s) {
                        const uint64_t idx = uint64_t(c) * A.dst_pitch + start + s;
                        const T v = r[size_t(c) * cnt + s];
                        if (mode == 0 && f32) {
                            float* d = static_cast<float*>(A.dst);
                            float old = d[idx];
                            float nv = float(v);
                            d[idx] = P.op == "add" ? old + nv : P.op == "sub" ? old - nv : nv;
                        } else {
                            double* d = static_cast<double*>(A.dst);
                            double old = d[idx];
                            double nv = double(v);
                            d[idx] = P.op == "add" ? old + nv : P.op == "sub" ? old - nv : nv;
                        }
                    }
            }
            if (want_sum) {
                long double h = 0, c = 0;
                for (int s = 0; s < cnt; ++s) neumaier_add<long double>(h, c, (long double)r[s]);
                part_hi[b] = h;
                part_c[b] = c;
            }
        } catch (const std::exception& e) {
#ifdef _OPENMP
#pragma omp critical
#endif
            err = e.what();
        }
    }
    if (!err.empty()) {
        g_err = err;
        return 1;
    }
    if (want_sum) {
        long double h = 0, c = 0;
        for (uint64_t b = 0; b < nblocks; ++b) {
            neumaier_add<long double>(h, c, part_hi[b]);
            neumaier_add<long double>(h, c, part_c[b]);
        }
        const long double tot = h + c;
        const double hi = double(tot);
        A.reduce_out[0] = hi;
        A.reduce_out[1] = double(tot - (long double)hi);
    }
    return 0;
}

}  // namespace

extern "C" {

uint64_t orc_splitmix64(uint64_t x) { return splitmix(x); }
// random/Generator.h:64-67
uint64_t orc_generator_key(uint64_t seed, uint64_t stream_id) { return splitmix(seed ^ splitmix(stream_id)); }
// random/Generator.h:78-81
uint64_t orc_substream_key(uint64_t key, uint64_t k) {
    return splitmix(key ^ splitmix(k ^ 0x2545F4914F6CDD1DULL));
}
void orc_philox4x32_10(const uint32_t ctr[4], uint32_t kx, uint32_t ky, uint32_t out[4]) {
    Q4 r = philox(Q4{ctr[0], ctr[1], ctr[2], ctr[3]}, kx, ky);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}
// Backend.h:166-172
uint64_t orc_random_bits64(uint64_t seed, uint32_t global, uint64_t counter) {
    const Q4 x = block(seed, global, counter);
    return (uint64_t(x.y) << 32) | x.x;
}
double orc_uniform01_f64(uint64_t seed, uint32_t global, uint64_t counter) {
    return u01d(block(seed, global, counter).x);
}
float orc_uniform01_f32(uint64_t seed, uint32_t global, uint64_t counter) {
    return u01f(block(seed, global, counter).x);
}
double orc_normal_f64(uint64_t seed, uint32_t global, uint64_t counter) {
    return normal_d<double>(seed, global, counter);
}
float orc_normal_f32(uint64_t seed, uint32_t global, uint64_t counter) { return normal_f(seed, global, counter); }
// The keyed block of (seed, global, counter) and the word -> real conversions
// themselves (Backend.h:75-101, :123-131, :152-157).
void orc_philox_block(uint64_t seed, uint32_t global, uint64_t counter, uint32_t out[4]) {
    const Q4 r = block(seed, global, counter);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}
double orc_u01_from_word_f64(uint32_t w) { return u01d(w); }
float orc_u01_from_word_f32(uint32_t w) { return u01f(w); }
double orc_u01_hq(uint32_t x, uint32_t y) { return u01hq(x, y); }
// Mean and standard error of z^2 z'^2 over n seeds splitmix64(salt + k), z at
// counter 5 and z' at counter 5 + lag of global 0: 1 for independent standard
// normals (tests/test_RandomIndependence.cpp:29-48).
void orc_lag_fourth_moment(uint64_t salt, uint64_t lag, int n, int f32, double* mean, double* se) {
    double sum = 0.0, sum2 = 0.0;
    for (int k = 0; k < n; ++k) {
        const uint64_t seed = splitmix(salt + uint64_t(k));
        const double z = f32 ? double(normal_f(seed, 0, 5)) : normal_d<double>(seed, 0, 5);
        const double y = f32 ? double(normal_f(seed, 0, 5 + lag)) : normal_d<double>(seed, 0, 5 + lag);
        const double q = z * z * y * y;
        sum += q;
        sum2 += q * q;
    }
    *mean = sum / n;
    *se = std::sqrt((sum2 / n - *mean * *mean) / n);
}

const char* orc_last_error(void) { return g_err.c_str(); }

int orc_eval(const char* ir, int mode, const OrcArgs* args, int nthreads) {
    try {
        Parser ps(ir);
        Plan P = ps.run();
        if ((P.op == "sum" || P.op == "setsum") && !args->reduce_out) throw std::runtime_error("oracle: reduce_out");
        const bool f32 = P.dst_dtype != "f64";
        if (mode == 0) return f32 ? run_plan<float>(P, 0, *args, nthreads) : run_plan<double>(P, 0, *args, nthreads);
        if (mode == 1) return run_plan<double>(P, 1, *args, nthreads);
        return run_plan<long double>(P, 2, *args, nthreads);
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void orc_pair_combine_f64(double ah, double ac, double bh, double bc, double* oh, double* oc) {
    pair_combine(ah, ac, bh, bc, *oh, *oc);
}
void orc_neumaier_add_f64(double* hi, double* comp, double term) { neumaier_add(*hi, *comp, term); }
void orc_reduce32_f64(const double* h, const double* c, double* oh, double* oc) { reduce32(h, c, *oh, *oc); }
void orc_reduce32_f32(const float* h, const float* c, float* oh, float* oc) { reduce32(h, c, *oh, *oc); }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#ifdef _OPENMP
#define ORC_PARFOR _Pragma("omp parallel for schedule(static) num_threads(nt)")
#else
#define ORC_PARFOR
#endif

static int threads_of(int nthreads) { return nthreads > 0 ? nthreads : orc_max_threads(); }

// The consumer loop of the reference (tests/test_Random_common.h:63-70):
// dst[SampleIndex::make(k)] = generator.uniform<double,N>(lo, hi).
void orc_fill_uniform_f64(uint64_t key, double lo, double hi, int comps, uint64_t n, uint64_t pitch, double* out,
                          int nthreads) {
    const int nt = threads_of(nthreads);
    (void)nt;
    ORC_PARFOR
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (int c = 0; c < comps; ++c)
            out[uint64_t(c) * pitch + i] = lo + (hi - lo) * u01d(block(key ^ kSaltUniform, uint32_t(i), c).x);
}
void orc_fill_uniform_f32(uint64_t key, float lo, float hi, int comps, uint64_t n, uint64_t pitch, float* out,
                          int nthreads) {
    const int nt = threads_of(nthreads);
    (void)nt;
    ORC_PARFOR
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (int c = 0; c < comps; ++c)
            out[uint64_t(c) * pitch + i] = lo + (hi - lo) * u01f(block(key ^ kSaltUniform, uint32_t(i), c).x);
}
void orc_fill_normal_f64(uint64_t key, double mean, double sd, int comps, uint64_t n, uint64_t pitch, double* out,
                         uint32_t sample_offset, int nthreads) {
    const int nt = threads_of(nthreads);
    (void)nt;
    ORC_PARFOR
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (int c = 0; c < comps; ++c)
            out[uint64_t(c) * pitch + i] =
                mean + sd * normal_d<double>(key ^ kSaltNormal, uint32_t(sample_offset + i), c);
}
void orc_cfg1_f64(const double* a, const double* b, const double* c, double* d, uint64_t n, uint64_t pitch,
                  int nthreads) {
    const int nt = threads_of(nthreads);
    (void)nt;
    ORC_PARFOR
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (int q = 0; q < 3; ++q) {
            const uint64_t j = uint64_t(q) * pitch + i;
            const double cc = (c[j] * c[j]) * -1.0;
            d[j] = (a[j] + b[j] * c[j]) + std::sin(a[j]) * std::exp(cc);
        }
}
void orc_cfg2a_f64(const double* a, const double* b, const double* c, const double* d0, double* d, uint64_t n,
                   uint64_t pitch, int nthreads) {
    const int nt = threads_of(nthreads);
    (void)nt;
    ORC_PARFOR
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (int q = 0; q < 3; ++q) {
            const uint64_t j = uint64_t(q) * pitch + i;
            const double L = std::log1p(std::fabs(c[j]));
            d[j] = std::sqrt(a[j] * a[j] + b[j] * b[j]) * L + 1.0 / std::sqrt(1.0 + d0[j] * d0[j]);
        }
}

}  // extern "C"
