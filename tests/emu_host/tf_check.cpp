// tf_check.cpp -- host check of the triple-float kernels of ag_tf64.cuh
// against __float128 (113-bit) arithmetic. Prints one JSON object: per
// operation the maximum and mean error over a seeded corpus, in units of
// 2^-53 of the exact result (of the larger operand for sums, whose
// cancellations the term scale absorbs), and for the large streaming
// expression d = sqrt(a*a+b*b)*log1p(|c|) + rsqrt(1+d0*d0) the error of the
// reassembled double in ulps of the term scale. Test infrastructure.
#include "host_shim.h"

#include <quadmath.h>

namespace ag {
// Native functions the bridge calls (not exercised by this check).
inline double f_exp(double x) { return std::exp(x); }
inline double f_sin(double x) { return std::sin(x); }
inline double f_cos(double x) { return std::cos(x); }
inline double normal_f64(ag_u64, ag_u32, ag_u32) { return std::nan(""); }
}  // namespace ag

#include "../../include/aether/gb300/ag_tf64.cuh"
#include "../../include/aether/gb300/ag_tf64_trig.cuh"

#include <cstdio>
#include <random>
#include <string>
#include <vector>

using namespace ag::t64;
typedef __float128 Q;

static Q val(tf v) { return (Q)v.x + (Q)v.y + (Q)v.z; }
static const Q U = ldexpq((Q)1, -53);   // 2^-53

struct Stat {
    double max_e = 0, sum = 0;
    long n = 0, bad = 0;
    void add(Q got, Q ref, Q scale) {
        const Q e = fabsq(got - ref) / (scale > 0 ? scale : (Q)1) / U;
        if (!(e == e)) {
            ++bad;
            return;
        }
        if ((double)e > max_e) max_e = (double)e;
        sum += (double)e;
        ++n;
    }
};

int main() {
    std::mt19937_64 rng(20261204);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    auto logu = [&](double lo2, double hi2) { return std::exp2(lo2 + (hi2 - lo2) * u01(rng)); };
    auto sgn = [&] { return u01(rng) < 0.5 ? -1.0 : 1.0; };
    const int N = 200000;
    std::vector<std::pair<std::string, Stat>> out;

    auto split = [](double x, bool& ok) { return from_double_ck(x, ok); };
    {   // the split is exact, and the reassembly returns the double
        Stat s;
        long mismatches = 0;
        for (int i = 0; i < N; ++i) {
            const double x = sgn() * logu(-40, 60);
            bool ok = true;
            const tf t = split(x, ok);
            if (!ok) continue;
            s.add(val(t), (Q)x, fabsq((Q)x));
            if (to_double(t) != x) ++mismatches;
        }
        s.bad += mismatches;
        out.push_back({"split", s});
    }
    auto binop = [&](const char* name, auto f, auto ref, bool rel_to_operands) {
        Stat s;
        for (int i = 0; i < N; ++i) {
            const double a = sgn() * logu(-20, 20), b = sgn() * logu(-20, 20);
            bool ok = true;
            const tf ta = split(a, ok), tb = split(b, ok);
            const tf r = f(ta, tb);
            const Q exact = ref((Q)a, (Q)b);
            s.add(val(r), exact, rel_to_operands ? fmaxq(fabsq((Q)a), fabsq((Q)b)) : fabsq(exact));
        }
        out.push_back({name, s});
    };
    binop("add", [](tf a, tf b) { return add(a, b); }, [](Q a, Q b) { return a + b; }, true);
    binop("sub", [](tf a, tf b) { return sub(a, b); }, [](Q a, Q b) { return a - b; }, true);
    binop("mul", [](tf a, tf b) { return mul(a, b); }, [](Q a, Q b) { return a * b; }, false);
    binop("div", [](tf a, tf b) { return div(a, b); }, [](Q a, Q b) { return a / b; }, false);
    binop("sqr_then_mul", [](tf a, tf b) { return mul(sqr(a), b); }, [](Q a, Q b) { return a * a * b; }, false);
    {   // sums of products under cancellation: (a b) - (a b (1 + small))
        Stat s;
        for (int i = 0; i < N; ++i) {
            const double a = sgn() * logu(-20, 20), b = a * (1.0 + (u01(rng) - 0.5) * 1e-9);
            bool ok = true;
            const tf ta = split(a, ok), tb = split(b, ok);
            const tf r = sub(mul(ta, ta), mul(ta, tb));
            s.add(val(r), (Q)a * (Q)a - (Q)a * (Q)b, (Q)a * (Q)a);
        }
        out.push_back({"cancel", s});
    }
    auto unop = [&](const char* name, auto gen, auto f, auto ref) {
        Stat s;
        for (int i = 0; i < N; ++i) {
            const double x = gen();
            bool ok = true;
            const tf t = split(x, ok);
            if (!ok) continue;
            const tf r = f(t);
            if (!out_ok(r)) continue;   // the generated kernel recomputes these natively
            const Q exact = ref((Q)x);
            s.add(val(r), exact, fabsq(exact));
        }
        out.push_back({name, s});
    };
    unop("sqrt", [&] { return logu(-40, 60); }, [](tf x) { return sqrt_(x); }, [](Q x) { return sqrtq(x); });
    unop("rsqrt", [&] { return logu(-40, 60); }, [](tf x) { return rsqrt_(x); }, [](Q x) { return 1 / sqrtq(x); });
    unop("recip", [&] { return sgn() * logu(-40, 60); }, [](tf x) { return recip(x); }, [](Q x) { return 1 / x; });
    unop("log", [&] { return logu(-40, 60); }, [](tf x) { return log_(x); }, [](Q x) { return logq(x); });
    unop("log_near_1", [&] { return 1.0 + (u01(rng) - 0.5) * 1e-3; }, [](tf x) { return log_(x); },
         [](Q x) { return logq(x); });
    unop("log1p", [&] { return 4.0 * u01(rng); }, [](tf x) { return log1p_(x); }, [](Q x) { return log1pq(x); });
    unop("log1p_nn", [&] { return logu(-40, 60); }, [](tf x) { return log1p_nn_(x); },
         [](Q x) { return log1pq(x); });
    unop("log1p_neg", [&] { return -0.99 * u01(rng); }, [](tf x) { return log1p_(x); },
         [](Q x) { return log1pq(x); });

    auto flagged = [&](const char* name, auto gen, auto f, auto ref) {
        Stat s;
        long native = 0;
        for (int i = 0; i < N; ++i) {
            const double x = gen();
            bool ok = true;
            const tf t = split(x, ok);
            if (!ok) continue;
            const tf r = f(t, ok);
            if (!ok || !out_ok(r)) {   // lanes the generated kernel computes natively
                ++native;
                continue;
            }
            const Q exact = ref((Q)x);
            s.add(val(r), exact, fabsq(exact));
        }
        s.bad += native > N / 1000 ? native : 0;   // more than 0.1 % native lanes is a failure
        out.push_back({name, s});
    };
    flagged("exp", [&] { return -54.0 + 140.0 * u01(rng); }, [](tf x, bool& ok) { return exp_(x, ok); },
            [](Q x) { return expq(x); });
    flagged("exp_small", [&] { return sgn() * logu(-40, -1); }, [](tf x, bool& ok) { return exp_(x, ok); },
            [](Q x) { return expq(x); });
    flagged("sin", [&] { return sgn() * logu(-30, 9.99); }, [](tf x, bool& ok) { return sin_(x, ok); },
            [](Q x) { return sinq(x); });
    flagged("cos", [&] { return sgn() * logu(-30, 9.99); }, [](tf x, bool& ok) { return cos_(x, ok); },
            [](Q x) { return cosq(x); });
    flagged("sin_unit", [&] { return 2.0 * u01(rng) - 1.0; }, [](tf x, bool& ok) { return sin_(x, ok); },
            [](Q x) { return sinq(x); });
    {   // near nonzero multiples of pi/2: beyond 2^-22 of them every lane is kept
        Stat s;
        long native = 0;
        const Q pio2 = acosq((Q)0);   // pi/2
        for (int i = 0; i < N; ++i) {
            const int q = 1 + (int)(u01(rng) * 600);
            const double x = (double)(q * pio2) + sgn() * logu(-21, -3);
            bool ok = true;
            const tf t = split(x, ok);
            const tf r = (i % 2) ? sin_(t, ok) : cos_(t, ok);
            if (!ok) {
                ++native;
                continue;
            }
            const Q exact = (i % 2) ? sinq((Q)x) : cosq((Q)x);
            s.add(val(r), exact, fabsq(exact));
        }
        s.bad += native;
        out.push_back({"trig_near_multiples", s});
    }

    {   // the large streaming expression, reassembled, in ulps of its term scale
        Stat s;
        long fallback = 0;
        for (int i = 0; i < N; ++i) {
            const double a = (u01(rng) - 0.5) * 8.0, b = (u01(rng) - 0.5) * 8.0, c = (u01(rng) - 0.5) * 8.0,
                         d0 = (u01(rng) - 0.5) * 8.0;
            bool ok = true;
            const tf ta = split(a, ok), tb = split(b, ok), tc = split(c, ok), td = split(d0, ok);
            if (!ok) {
                ++fallback;
                continue;
            }
            const tf r = add_fast(mul(sqrt_(add_fast(sqr(ta), sqr(tb))), log1p_nn_(abs_(tc))),
                                  rsqrt_(add_fast(mk3(1.0f, 0.0f, 0.0f), sqr(td))));
            if (!out_ok(r)) {
                ++fallback;
                continue;
            }
            const double got = to_double(r);
            const Q t1 = sqrtq((Q)a * a + (Q)b * b) * log1pq(fabsq((Q)c)), t2 = 1 / sqrtq(1 + (Q)d0 * d0);
            const Q scale = fmaxq(fabsq(t1), fabsq(t2));
            // one ulp of the term scale: 2^(floor(log2 scale) - 52)
            const Q ulp = ldexpq((Q)1, ilogbq(scale) - 52);
            const Q e = fabsq((Q)got - (t1 + t2)) / ulp;
            if ((double)e > s.max_e) s.max_e = (double)e;
            s.sum += (double)e;
            ++s.n;
        }
        s.bad = fallback;
        out.push_back({"expr_term_ulps", s});
    }

    std::printf("{");
    for (size_t k = 0; k < out.size(); ++k) {
        const Stat& s = out[k].second;
        std::printf("%s\"%s\": {\"max\": %.4f, \"mean\": %.6f, \"n\": %ld, \"bad\": %ld}", k ? ", " : "",
                    out[k].first.c_str(), s.max_e, s.n ? s.sum / s.n : 0.0, s.n, s.bad);
    }
    std::printf("}\n");
    return 0;
}
