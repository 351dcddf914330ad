// emu_check.cpp -- host check of the double-float kernels of ag_emu64.cuh
// against long double. Prints one JSON object: per function the maximum
// relative error in units of 2^-53 over a seeded corpus. Test infrastructure.
#include "host_shim.h"

#include "../../include/aether/gb300/ag_emu64.cuh"
#include "../../include/aether/gb300/ag_emu64_bm.cuh"

#include <cstdio>
#include <random>
#include <string>
#include <vector>

using namespace ag::e64;
typedef long double LD;

static LD val(df x) { return (LD)x.hi + (LD)x.lo; }
static const LD U = 1.1102230246251565404e-16L;   // 2^-53

struct Stat {
    double max_rel = 0, sum = 0;
    long n = 0, bad = 0;
    void add(LD got, LD ref) {
        if (std::isnan((double)ref) && std::isnan((double)got)) return;
        LD e = fabsl(got - ref) / (fabsl(ref) > 0 ? fabsl(ref) : 1.0L) / U;
        if (!(e == e)) {
            ++bad;
            return;
        }
        if (e > max_rel) max_rel = (double)e;
        sum += (double)e;
        ++n;
    }
};

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    auto logu = [&](double lo2, double hi2) { return std::exp2(lo2 + (hi2 - lo2) * u01(rng)); };
    const int N = 200000;
    std::vector<std::pair<std::string, Stat>> out;
    auto run = [&](const char* name, auto gen, auto f, auto ref) {
        Stat s;
        for (int i = 0; i < N; ++i) {
            double x = gen();
            bool ok = true;
            df r = f(from_double(x), ok);
            if (!ok || !out_ok(r)) continue;   // the generated kernel recomputes these natively
            s.add(val(r), ref((LD)x));
        }
        out.push_back({name, s});
    };
    auto nf = [](auto fn) { return [fn](df x, bool&) { return fn(x); }; };
    run("roundtrip", [&] { return (u01(rng) - 0.5) * 8.0; }, nf([](df x) { return x; }), [](LD x) { return x; });
    run("sqrt", [&] { return logu(-50, 50); }, nf(sqrt_), [](LD x) { return sqrtl(x); });
    run("rsqrt", [&] { return logu(-50, 50); }, nf(rsqrt_), [](LD x) { return 1.0L / sqrtl(x); });
    auto expf_ = [](df x, bool& ok) { return exp_(x, ok); };
    run("exp", [&] { return (u01(rng) - 0.5) * 160.0; }, expf_, [](LD x) { return expl(x); });
    run("exp_small", [&] { return -u01(rng); }, expf_, [](LD x) { return expl(x); });
    run("log", [&] { return logu(-60, 60); }, nf(log_), [](LD x) { return logl(x); });
    run("log_0.5_2", [&] { return 0.5 + 1.5 * u01(rng); }, nf(log_), [](LD x) { return logl(x); });
    run("log1p", [&] { return 4.0 * u01(rng); }, nf(log1p_), [](LD x) { return log1pl(x); });
    run("log1p_tiny", [&] { return logu(-40, -6) * (u01(rng) < 0.5 ? -1 : 1); }, nf(log1p_),
        [](LD x) { return log1pl(x); });
    run("log1p_neg", [&] { return -0.99 * u01(rng); }, nf(log1p_), [](LD x) { return log1pl(x); });
    run("sin", [&] { return 2.0 * u01(rng) - 1.0; }, [](df x, bool& ok) { return sin_(x, ok); },
        [](LD x) { return sinl(x); });
    run("cos", [&] { return 2.0 * u01(rng) - 1.0; }, [](df x, bool& ok) { return cos_(x, ok); },
        [](LD x) { return cosl(x); });
    // large float arguments (the precision form's inputs: exact in a float),
    // 6000 <= |x| < 2^24 (the integer Payne-Hanek range), against sinl/cosl
    {
        Stat s;
        for (int i = 0; i < N; ++i) {
            const float x = (float)((u01(rng) < 0.5 ? -1 : 1) * logu(12.6, 23.99));
            bool ok = true;
            const df r = (i % 2) ? sin_(mk(x, 0.0f), ok) : cos_(mk(x, 0.0f), ok);
            if (!ok || !out_ok(r)) continue;
            s.add(val(r), (i % 2) ? sinl((LD)x) : cosl((LD)x));
        }
        out.push_back({"trig_large_f32", s});
    }
    run("sin_100", [&] { return 200.0 * u01(rng) - 100.0; }, [](df x, bool& ok) { return sin_(x, ok); },
        [](LD x) { return sinl(x); });
    run("sinpi", [&] { return 2.0 * u01(rng); }, nf(sinpi_),
        [](LD x) { return sinl(x * 3.14159265358979323846264338327950288L); });
    run("recip", [&] { return logu(-30, 30); }, nf(recip), [](LD x) { return 1.0L / x; });
    // binary arithmetic
    {
        Stat sa, sm, sd;
        for (int i = 0; i < N; ++i) {
            double a = (u01(rng) - 0.5) * 8, b = (u01(rng) - 0.5) * 8;
            df A = from_double(a), B = from_double(b);
            sa.add(val(add(A, B)), (LD)a + (LD)b);
            sm.add(val(mul(A, B)), (LD)a * (LD)b);
            sd.add(val(div(A, B)), (LD)a / (LD)b);
        }
        out.push_back({"add", sa});
        out.push_back({"mul", sm});
        out.push_back({"div", sd});
    }
    // config 2a composite: sqrt(a*a+b*b)*log1p(|c|) + rsqrt(1+d0*d0), through to_double
    {
        Stat s;
        for (int i = 0; i < N; ++i) {
            double a = (u01(rng) - 0.5) * 8, b = (u01(rng) - 0.5) * 8, c = (u01(rng) - 0.5) * 8,
                   d0 = (u01(rng) - 0.5) * 8;
            df A = from_double(a), B = from_double(b), C = from_double(c), D = from_double(d0);
            df r = add(mul(sqrt_(add(mul(A, A), mul(B, B))), log1p_(abs_(C))),
                       rsqrt_(add(dfc(1.0), mul(D, D))));
            LD ref = sqrtl((LD)a * a + (LD)b * b) * log1pl(fabsl((LD)c)) + 1.0L / sqrtl(1.0L + (LD)d0 * d0);
            s.add((LD)to_double(r), ref);
        }
        out.push_back({"cfg2a", s});
    }
    // the same expression in the generated form: sums of unnormalised
    // squares, add_fast for sums of non-negative terms, log1p of |input|
    {
        Stat s;
        for (int i = 0; i < N; ++i) {
            double a = (u01(rng) - 0.5) * 8, b = (u01(rng) - 0.5) * 8, c = (u01(rng) - 0.5) * 8,
                   d0 = (u01(rng) - 0.5) * 8;
            bool ok = true;
            df A = from_double_ck(a, ok), B = from_double_ck(b, ok), C = from_double_ck(c, ok), D = from_double_ck(d0, ok);
            df r = add_fast_u(mul(sqrt_nn_(add_fast(sqr_u(A), sqr_u(B))), log1p_nn_(abs_(C))),
                            rsqrt_(add_fast(dfc(1.0), sqr_u(D))));
            LD ref = sqrtl((LD)a * a + (LD)b * b) * log1pl(fabsl((LD)c)) + 1.0L / sqrtl(1.0L + (LD)d0 * d0);
            if (ok) s.add((LD)to_double(r), ref);
        }
        out.push_back({"cfg2a_gen", s});
    }
    // config 1 composite: a + b*c + sin(a)*exp(-c*c)
    {
        Stat s;
        for (int i = 0; i < N; ++i) {
            double a = 2 * u01(rng) - 1, b = 2 * u01(rng) - 1, c = 2 * u01(rng) - 1;
            df A = from_double(a), B = from_double(b), C = from_double(c);
            bool ok = true;
            df r = add(add(A, mul(B, C)), mul(sin_(A, ok), exp_(mul(dfc(-1.0), mul(C, C)), ok)));
            LD ref = (LD)a + (LD)b * c + sinl((LD)a) * expl(-(LD)c * c);
            LD scale = fabsl((LD)a) + fabsl((LD)b * c) + fabsl(sinl((LD)a) * expl(-(LD)c * c));
            // error relative to the magnitude of the terms (the sum can cancel)
            LD e = fabsl((LD)to_double(r) - ref) / scale / U;
            if (e > s.max_rel) s.max_rel = (double)e;
            s.sum += (double)e;
            ++s.n;
        }
        out.push_back({"cfg1_termscale", s});
    }
    // Box-Muller normals against the double-precision formula in long double
    {
        Stat s;
        for (int i = 0; i < N; ++i) {
            const ag_u64 seed = 0x1234567ull;
            const ag::q4 x = ag::philox_block(seed, (ag_u32)i, 0u);
            const ag_u64 z = (ag_u64)x.x ^ ((ag_u64)x.y << 21);
            const ag_u64 zy = (ag_u64)x.z ^ ((ag_u64)x.w << 21);
            // the reference's uniforms are doubles (random/detail/Backend.h):
            // z 2^-53 + 2^-54 and zy 2^-52 + 2^-53, each rounded once
            volatile double u0 = (double)z * 1.1102230246251565e-16, v0 = (double)zy * 2.2204460492503131e-16;
            const LD u = (LD)(double)(u0 + 5.5511151231257827e-17);
            const LD v = (LD)(double)(v0 + 1.1102230246251565e-16);
            const LD ref = sqrtl(-2.0L * logl(u)) * sinl(v * 3.14159265358979323846264338327950288L);
            const double got = to_double(normal_df(seed, (ag_u32)i, 0u));
            // the unnormalised form reassembles to the same double
            if (to_double(normal_df<true>(seed, (ag_u32)i, 0u)) != got) ++s.bad;
            // TIER-TOL form: |got - ref| / (1 + |ref|)
            LD e = fabsl((LD)got - ref) / (1.0L + fabsl(ref)) / U;
            if (e > s.max_rel) s.max_rel = (double)e;
            s.sum += (double)e;
            ++s.n;
        }
        out.push_back({"normal_abs_rel", s});
    }
    // At scale: 2^22 samples of each, Philox-seeded, in parallel (the maxima
    // of the long tails that 2*10^5 draws do not reach)
    {
        const long M = 1L << 22;
        double mx_e = 0, mx_n = 0, sum_e = 0, sum_n = 0;
        long cnt_e = 0;
#pragma omp parallel for reduction(max : mx_e, mx_n) reduction(+ : sum_e, sum_n, cnt_e)
        for (long i = 0; i < M; ++i) {
            double v[4];
            for (int k = 0; k < 4; ++k) {
                const ag::q4 x = ag::philox_block(0x9E3779B97F4A7C15ull + 977ull * (ag_u64)k, (ag_u32)i, 0u);
                const ag_u64 z = (ag_u64)x.x ^ ((ag_u64)x.y << 21);
                v[k] = ((double)z * 1.1102230246251565e-16 + 5.5511151231257827e-17) * 8.0 - 4.0;
            }
            bool ok = true;
            df A = from_double_ck(v[0], ok), B = from_double_ck(v[1], ok), C = from_double_ck(v[2], ok),
               D = from_double_ck(v[3], ok);
            df r = add_fast_u(mul(sqrt_nn_(add_fast(sqr_u(A), sqr_u(B))), log1p_nn_(abs_(C))),
                              rsqrt_(add_fast(dfc(1.0), sqr_u(D))));
            if (ok && out_ok(r)) {
                const LD t1 = sqrtl((LD)v[0] * v[0] + (LD)v[1] * v[1]) * log1pl(fabsl((LD)v[2]));
                const LD t2 = 1.0L / sqrtl(1.0L + (LD)v[3] * v[3]);
                const double e = (double)(fabsl((LD)to_double(r) - (t1 + t2)) / fmaxl(fabsl(t1), fabsl(t2)) / U);
                mx_e = e > mx_e ? e : mx_e;
                sum_e += e;
                ++cnt_e;
            }
            const ag_u64 seed = 0x48f0bd76c5a9c07dull;
            const ag::q4 x = ag::philox_block(seed, (ag_u32)i, 0u);
            const ag_u64 z = (ag_u64)x.x ^ ((ag_u64)x.y << 21), zy = (ag_u64)x.z ^ ((ag_u64)x.w << 21);
            volatile double u0 = (double)z * 1.1102230246251565e-16, v0 = (double)zy * 2.2204460492503131e-16;
            const LD u = (LD)(double)(u0 + 5.5511151231257827e-17), vv = (LD)(double)(v0 + 1.1102230246251565e-16);
            const LD ref = sqrtl(-2.0L * logl(u)) * sinl(vv * 3.14159265358979323846264338327950288L);
            const double e = (double)(fabsl((LD)to_double(normal_df(seed, (ag_u32)i, 0u)) - ref) / (1.0L + fabsl(ref)) / U);
            mx_n = e > mx_n ? e : mx_n;
            sum_n += e;
        }
        Stat a, b;
        a.max_rel = mx_e, a.sum = sum_e, a.n = cnt_e;
        b.max_rel = mx_n, b.sum = sum_n, b.n = M;
        out.push_back({"cfg2a_gen_2p22", a});
        out.push_back({"normal_2p22", b});
    }
    std::printf("{");
    for (size_t i = 0; i < out.size(); ++i)
        std::printf("%s\"%s\": {\"max\": %.3f, \"mean\": %.3f, \"n\": %ld, \"bad\": %ld}", i ? ", " : "",
                    out[i].first.c_str(), out[i].second.max_rel,
                    out[i].second.n ? out[i].second.sum / out[i].second.n : 0.0, out[i].second.n, out[i].second.bad);
    std::printf("}\n");
    return 0;
}
