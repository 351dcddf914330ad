// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own headers (compiled in AETHER_CPP_MODE by
// `make -C oracle ref`) on seeded inputs drawn by the reference's own
// Generator, and dumps inputs and outputs for tests/golden/make_golden.py.
// This file is a consumer of the reference API: every loop is the user loop
// the reference documents (tests/test_Random_common.h:63-70), one sample per
// iteration with `dst[i] = expr`.
//
// usage: aether_ref <out_dir>     (prints a JSON manifest on stdout)
//        aether_ref --bench [steps] (times the CPU arm's sample through the
//                                    reference's headers, one JSON line)

#include <aether/aether.h>

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using aether::SampleIndex;
using aether::random::Generator;

static std::string g_dir;
static bool g_first = true;

template <class T>
static void dump(const std::string& name, const T* data, std::size_t comps, std::size_t n, std::size_t pitch,
                 const char* dtype) {
    const std::string path = g_dir + "/" + name + ".bin";
    std::FILE* f = std::fopen(path.c_str(), "wb");
    for (std::size_t c = 0; c < comps; ++c) std::fwrite(data + c * pitch, sizeof(T), n, f);
    std::fclose(f);
    std::printf("%s{\"name\":\"%s\",\"dtype\":\"%s\",\"comps\":%zu,\"n\":%zu}", g_first ? "" : ",\n", name.c_str(),
                dtype, comps, n);
    g_first = false;
}

template <class T, std::size_t... Es>
static void dumpArray(const std::string& name, aether::Array<T, Es...>& a) {
    constexpr std::size_t comps = (Es * ... * std::size_t{1});
    const T* base = a.hostView().data();
    dump<T>(name, base, comps, a.samples(), a.capacity(), sizeof(T) == 8 ? "f64" : "f32");
}

template <class T, std::size_t N, class Leaf>
static void fill(aether::Array<T, N>& a, const Leaf& leaf) {
    auto v = a.hostView();
    for (std::size_t k = 0; k < a.samples(); ++k) v[SampleIndex::make(k)] = leaf;
}

// The CPU arm's sample timed through the reference's own headers: config 2a
// on 2^23 samples and the N(0, 1) fill of 2^25 doubles, inputs from
// Generator(7), each an OpenMP loop over SampleIndex::make(k) assigning
// `view[i] = expr` (the user loop, tests/test_Random_common.h:63-70), as the
// oracle's restatement runs them; prints the median of `steps` steps as JSON.
static int bench(int steps) {
    const std::size_t n = std::size_t(1) << 23, nf = std::size_t(1) << 25;
    Generator g(7);
    aether::Array<double, 3> a(n), b(n), c(n), d0(n), d(n);
    aether::Array<double, 1> z(nf);
    aether::Array<double, 3>* in[4] = {&a, &b, &c, &d0};
    for (int s = 0; s < 4; ++s) {
        auto v = in[s]->hostView();
        const auto leaf = g.substream(std::uint64_t(s)).uniform<double, 3>(-4.0, 4.0);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < long(n); ++k) v[SampleIndex::make(std::size_t(k))] = leaf;
    }
    auto av = a.hostView(), bv = b.hostView(), cv = c.hostView(), d0v = d0.hostView(), dv = d.hostView();
    auto zv = z.hostView();
    const auto normal = g.substream(4).normal<double, 1>(0.0, 1.0);
    std::vector<double> ts;
    for (int it = 0; it < steps + 1; ++it) {
        const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(static)
        for (long k = 0; k < long(n); ++k) {
            aether::Item<double, 3> L;
            for (std::size_t q = 0; q < 3; ++q) L(q) = aether::math::log1p(aether::math::abs(cv(q, std::size_t(k))));
            dv[SampleIndex::make(std::size_t(k))] = aether::cwiseSqrt(av * av + bv * bv) * L +
                                                     aether::cwiseRsqrt(aether::constant<aether::extents<3>>(1.0) + d0v * d0v);
        }
#pragma omp parallel for schedule(static)
        for (long k = 0; k < long(nf); ++k) zv[SampleIndex::make(std::size_t(k))] = normal;
        if (it) ts.push_back(omp_get_wtime() - t0);
    }
    std::sort(ts.begin(), ts.end());
    const double t = ts[ts.size() / 2];
    std::printf("{\"threads\": %d, \"s_per_step\": %.6f, \"gbs\": %.4f}\n", omp_get_max_threads(), t,
                (double(n) * 120 + double(nf) * 8) / t / 1e9);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    if (std::string(argv[1]) == "--bench") return bench(argc > 2 ? std::atoi(argv[2]) : 5);
    g_dir = argv[1];
    std::printf("[\n");

    // Config 1: Array<double,3>, inputs Generator(42).substream(0..2).uniform(-1,1).
    {
        const std::size_t n = 1000;
        Generator g(42);
        aether::Array<double, 3> a(n), b(n), c(n), d(n);
        fill(a, g.substream(0).uniform<double, 3>(-1.0, 1.0));
        fill(b, g.substream(1).uniform<double, 3>(-1.0, 1.0));
        fill(c, g.substream(2).uniform<double, 3>(-1.0, 1.0));
        auto av = a.hostView();
        auto bv = b.hostView();
        auto cv = c.hostView();
        auto dv = d.hostView();
        for (std::size_t k = 0; k < n; ++k)
            dv[SampleIndex::make(k)] = av + bv * cv + aether::cwiseSin(av) * aether::cwiseExp((cv * cv) * (-1.0));
        dumpArray("cfg1_a", a);
        dumpArray("cfg1_b", b);
        dumpArray("cfg1_c", c);
        dumpArray("cfg1_d", d);
    }
    // Config 2a: four Array<double,3> from Generator(7).substream(0..3).uniform(-4,4).
    {
        const std::size_t n = 1000;
        Generator g(7);
        aether::Array<double, 3> a(n), b(n), c(n), d0(n), d(n);
        fill(a, g.substream(0).uniform<double, 3>(-4.0, 4.0));
        fill(b, g.substream(1).uniform<double, 3>(-4.0, 4.0));
        fill(c, g.substream(2).uniform<double, 3>(-4.0, 4.0));
        fill(d0, g.substream(3).uniform<double, 3>(-4.0, 4.0));
        auto av = a.hostView();
        auto bv = b.hostView();
        auto cv = c.hostView();
        auto d0v = d0.hostView();
        auto dv = d.hostView();
        for (std::size_t k = 0; k < n; ++k) {
            aether::Item<double, 3> L;
            for (std::size_t q = 0; q < 3; ++q) L(q) = aether::math::log1p(aether::math::abs(cv(q, k)));
            dv[SampleIndex::make(k)] = aether::cwiseSqrt(av * av + bv * bv) * L
                + aether::cwiseRsqrt(aether::constant<aether::extents<3>>(1.0) + d0v * d0v);
        }
        dumpArray("cfg2a_a", a);
        dumpArray("cfg2a_b", b);
        dumpArray("cfg2a_c", c);
        dumpArray("cfg2a_d0", d0);
        dumpArray("cfg2a_d", d);
    }
    // Config 2b: normal fill Generator(7).substream(4).normal<double,1>(0,1).
    {
        const std::size_t n = 4096;
        aether::Array<double, 1> x(n);
        fill(x, Generator(7).substream(4).normal<double, 1>(0.0, 1.0));
        dumpArray("cfg2b_x", x);
    }
    // FP32 leaves.
    {
        const std::size_t n = 1000;
        aether::Array<float, 3> u(n);
        aether::Array<float, 1> z(n);
        fill(u, Generator(3).substream(0).uniform<float, 3>(-1.0f, 1.0f));
        fill(z, Generator(3).substream(1).normal<float, 1>(0.0f, 1.0f));
        dumpArray("f32_uniform", u);
        dumpArray("f32_normal", z);
    }
    // Remaining distribution leaves, double.
    {
        const std::size_t n = 1000;
        Generator g(11);
        aether::Array<double, 2> ln(n), ex(n), be(n), ui(n);
        fill(ln, g.lognormal<double, 2>(0.1, 0.5));
        fill(ex, g.exponential<double, 2>(1.5));
        fill(be, g.bernoulli<double, 2>(0.3));
        aether::Item<double, 2> lo, hi;
        lo(0) = -2.0;
        lo(1) = 10.0;
        hi(0) = 2.0;
        hi(1) = 11.0;
        fill(ui, g.uniform<double, 2>(lo, hi));
        dumpArray("leaf_lognormal", ln);
        dumpArray("leaf_exponential", ex);
        dumpArray("leaf_bernoulli", be);
        dumpArray("leaf_uniform_item", ui);
    }
    // The rest of the leaf API, read per sample with get<I>(i) as the
    // reference's random tests do: per-component (Item) parameters of every
    // distribution, uniformInt, multivariateNormal from cholesky, the
    // index-free get<I>() draws and the free-function spelling.
    {
        const std::size_t n = 1000;
        Generator g(21);
        aether::Item<double, 3> m3, s3, l3, p3;
        m3(0) = -1.0; m3(1) = 0.0; m3(2) = 2.5;
        s3(0) = 0.5; s3(1) = 1.0; s3(2) = 3.0;
        l3(0) = 0.5; l3(1) = 2.0; l3(2) = 8.0;
        p3(0) = 0.1; p3(1) = 0.5; p3(2) = 0.9;
        const auto nrm = g.substream(0).normal<double, 3>(m3, s3);
        const auto lgn = g.substream(1).lognormal<double, 3>(m3, s3);
        const auto ex = g.substream(2).exponential<double, 3>(l3);
        const auto be = g.substream(3).bernoulli<double, 3>(p3);
        const auto ri = g.substream(4).uniformInt<int, 3>(-5, 17);
        const auto rl = g.substream(5).uniformInt<long long, 2>(-(1LL << 40), 1LL << 41);
        const double cov[3][3] = {{2.0, 0.5, 0.1}, {0.5, 1.0, 0.3}, {0.1, 0.3, 0.5}};
        const auto L = aether::random::cholesky<double, 3>(cov);
        aether::Item<double, 3> mu;
        mu(0) = 1.0; mu(1) = -2.0; mu(2) = 0.5;
        const auto mvn = g.substream(6).multivariateNormal<double, 3>(mu, L);
        const float covf[2][2] = {{1.5f, -0.4f}, {-0.4f, 0.8f}};
        const auto Lf = aether::random::cholesky<float, 2>(covf);
        aether::Item<float, 2> muf;
        muf(0) = 0.25f; muf(1) = -0.75f;
        const auto mvnf = g.substream(7).multivariateNormal<float, 2>(muf, Lf);
        const auto fu = aether::random::uniform<double, 2>(-3.0, 3.0);
        const auto fs = aether::random::seed(99).normal<double, 2>(0.0, 1.0);
        std::vector<double> vn(3 * n), vl(3 * n), ve(3 * n), vb(3 * n), vm(3 * n), vfu(2 * n), vfs(2 * n);
        std::vector<int> vi(3 * n);
        std::vector<long long> vll(2 * n);
        std::vector<float> vmf(2 * n);
        for (std::size_t k = 0; k < n; ++k) {
            const SampleIndex i = SampleIndex::make(k);
            vn[k] = nrm.get<0>(i); vn[n + k] = nrm.get<1>(i); vn[2 * n + k] = nrm.get<2>(i);
            vl[k] = lgn.get<0>(i); vl[n + k] = lgn.get<1>(i); vl[2 * n + k] = lgn.get<2>(i);
            ve[k] = ex.get<0>(i); ve[n + k] = ex.get<1>(i); ve[2 * n + k] = ex.get<2>(i);
            vb[k] = be.get<0>(i); vb[n + k] = be.get<1>(i); vb[2 * n + k] = be.get<2>(i);
            vi[k] = ri.get<0>(i); vi[n + k] = ri.get<1>(i); vi[2 * n + k] = ri.get<2>(i);
            vll[k] = rl.get<0>(i); vll[n + k] = rl.get<1>(i);
            vm[k] = mvn.get<0>(i); vm[n + k] = mvn.get<1>(i); vm[2 * n + k] = mvn.get<2>(i);
            vmf[k] = mvnf.get<0>(i); vmf[n + k] = mvnf.get<1>(i);
            vfu[k] = fu.get<0>(i); vfu[n + k] = fu.get<1>(i);
            vfs[k] = fs.get<0>(i); vfs[n + k] = fs.get<1>(i);
        }
        dump<double>("leafi_normal", vn.data(), 3, n, n, "f64");
        dump<double>("leafi_lognormal", vl.data(), 3, n, n, "f64");
        dump<double>("leafi_exponential", ve.data(), 3, n, n, "f64");
        dump<double>("leafi_bernoulli", vb.data(), 3, n, n, "f64");
        dump<int>("leaf_uniform_int", vi.data(), 3, n, n, "i32");
        dump<long long>("leaf_uniform_int64", vll.data(), 2, n, n, "i64");
        dump<double>("leaf_mvn", vm.data(), 3, n, n, "f64");
        dump<float>("leaf_mvn_f32", vmf.data(), 2, n, n, "f32");
        dump<double>("free_uniform", vfu.data(), 2, n, n, "f64");
        dump<double>("free_seed_normal", vfs.data(), 2, n, n, "f64");
        dump<double>("mvn_cholesky", L.data, 1, 6, 6, "f64");
        // index-free draws: one value per component, the same at every sample
        const auto u = g.substream(8).uniform<double, 3>(-1.0, 1.0);
        const auto z = g.substream(9).normal<float, 2>(0.0f, 1.0f);
        const double fr[] = {u.get<0>(), u.get<1>(), u.get<2>(), double(z.get<0>()), double(z.get<1>()),
                             nrm.get<2>(), lgn.get<0>(), ex.get<1>(), be.get<2>(), double(ri.get<0>()),
                             double(ri.get<2>()), double(rl.get<1>()), mvn.get<0>(), mvn.get<2>(),
                             double(mvnf.get<1>()), fu.get<1>()};
        dump<double>("index_free", fr, 1, sizeof(fr) / sizeof(*fr), sizeof(fr) / sizeof(*fr), "f64");
    }
    // Geometry (config 4 node kinds) on uniform(-1,1) inputs, Generator(5).
    {
        const std::size_t n = 777;
        Generator g(5);
        aether::Array<double, 3> a(n), b(n), cr(n), rot(n), un(n), uni(n);
        aether::Array<double, 4> q(n), p(n), qm(n);
        aether::Array<double, 9> m9(n);
        aether::Array<double, 3, 3> M(n), Minv(n);
        aether::Array<double, 1> det(n), tr(n);
        fill(a, g.substream(0).uniform<double, 3>(-1.0, 1.0));
        fill(b, g.substream(1).uniform<double, 3>(-1.0, 1.0));
        fill(q, g.substream(2).uniform<double, 4>(-1.0, 1.0));
        fill(p, g.substream(3).uniform<double, 4>(-1.0, 1.0));
        fill(m9, g.substream(4).uniform<double, 9>(-1.0, 1.0));
        auto av = a.hostView();
        auto bv = b.hostView();
        auto qv = q.hostView();
        auto pv = p.hostView();
        auto m9v = m9.hostView();
        auto Mv = M.hostView();
        for (std::size_t k = 0; k < n; ++k)
            for (std::size_t r = 0; r < 3; ++r)
                for (std::size_t c = 0; c < 3; ++c) Mv(r, c, k) = m9v(r * 3 + c, k);
        auto crv = cr.hostView();
        auto rotv = rot.hostView();
        auto unv = un.hostView();
        auto univ = uni.hostView();
        auto qmv = qm.hostView();
        auto Miv = Minv.hostView();
        auto detv = det.hostView();
        auto trv = tr.hostView();
        for (std::size_t k = 0; k < n; ++k) {
            const SampleIndex i = SampleIndex::make(k);
            crv[i] = av.cross(bv);
            rotv[i] = qv.quatRotate(av);
            qmv[i] = qv.quatMul(pv);
            unv[i] = av.unitVector();
            aether::Item<double, 3> ai = av[i].get();
            aether::Item<double, 3> ui = ai.unitVector();
            for (std::size_t q = 0; q < 3; ++q) univ(q, k) = ui(q);
            Miv[i] = Mv.inverse();
            aether::Item<double, 3, 3> mi = Mv[i].get();
            detv(0, k) = mi.det();
            trv(0, k) = mi.trace();
        }
        dumpArray("geo_a", a);
        dumpArray("geo_b", b);
        dumpArray("geo_q", q);
        dumpArray("geo_p", p);
        dumpArray("geo_m", m9);
        dumpArray("geo_cross", cr);
        dumpArray("geo_qrot", rot);
        dumpArray("geo_qmul", qm);
        dumpArray("geo_unit", un);
        dumpArray("geo_unit_item", uni);
        dumpArray("geo_inv", Minv);
        dumpArray("geo_det", det);
        dumpArray("geo_trace", tr);
    }
    // Per-sample dot over 8 components (config 3's fold), double and float.
    {
        const std::size_t n = 600;
        Generator g(9);
        aether::Array<double, 8> x(n), y(n);
        aether::Array<float, 8> xf(n), yf(n);
        aether::Array<double, 1> dd(n);
        aether::Array<float, 1> df(n);
        fill(x, g.substream(0).uniform<double, 8>(-1.0, 1.0));
        fill(y, g.substream(1).uniform<double, 8>(-1.0, 1.0));
        fill(xf, g.substream(2).uniform<float, 8>(-1.0f, 1.0f));
        fill(yf, g.substream(3).uniform<float, 8>(-1.0f, 1.0f));
        auto xv = x.hostView();
        auto yv = y.hostView();
        auto xfv = xf.hostView();
        auto yfv = yf.hostView();
        auto ddv = dd.hostView();
        auto dfv = df.hostView();
        for (std::size_t k = 0; k < n; ++k) {
            const SampleIndex i = SampleIndex::make(k);
            aether::Item<double, 8> xi = xv[i].get(), yi = yv[i].get();
            aether::Item<float, 8> xfi = xfv[i].get(), yfi = yfv[i].get();
            ddv(0, k) = xi.dot(yi);
            dfv(0, k) = xfi.dot(yfi);
        }
        dumpArray("dot_x", x);
        dumpArray("dot_y", y);
        dumpArray("dot_xf", xf);
        dumpArray("dot_yf", yf);
        dumpArray("dot_d", dd);
        dumpArray("dot_f", df);
    }
    // Elementwise nodes on a corpus: uniform(-4,4) values then specials.
    {
        const std::size_t nr = 480;
        const double specials[] = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1e-300, -1e-300, 1e-10, 3.0, 7.5, -7.5,
                                   0.999999, 1.000001, 2.0, 4.0};
        const std::size_t ns = sizeof(specials) / sizeof(*specials);
        const std::size_t n = nr + ns;
        aether::Array<double, 1> x(n), y(n);
        auto xv = x.hostView();
        auto yv = y.hostView();
        Generator g(13);
        {
            auto lx = g.substream(0).uniform<double, 1>(-4.0, 4.0);
            auto ly = g.substream(1).uniform<double, 1>(0.25, 3.0);
            for (std::size_t k = 0; k < nr; ++k) {
                xv[SampleIndex::make(k)] = lx;
                yv[SampleIndex::make(k)] = ly;
            }
        }
        for (std::size_t k = 0; k < ns; ++k) {
            xv(0, nr + k) = specials[k];
            yv(0, nr + k) = 1.5;
        }
        dumpArray("cw_x", x);
        dumpArray("cw_y", y);
        aether::Array<double, 1> o(n);
        auto ov = o.hostView();
#define AETHER_REF_CASE(NAME, EXPR)                                                   \
    for (std::size_t k = 0; k < n; ++k) ov[SampleIndex::make(k)] = (EXPR);           \
    dumpArray(NAME, o);
        AETHER_REF_CASE("cw_sqrt", aether::cwiseSqrt(xv))
        AETHER_REF_CASE("cw_rsqrt", aether::cwiseRsqrt(xv))
        AETHER_REF_CASE("cw_exp", aether::cwiseExp(xv))
        AETHER_REF_CASE("cw_log", aether::cwiseLog(xv))
        AETHER_REF_CASE("cw_sin", aether::cwiseSin(xv))
        AETHER_REF_CASE("cw_cos", aether::cwiseCos(xv))
        AETHER_REF_CASE("cw_tan", aether::cwiseTan(xv))
        AETHER_REF_CASE("cw_asin", aether::cwiseAsin(xv))
        AETHER_REF_CASE("cw_acos", aether::cwiseAcos(xv))
        AETHER_REF_CASE("cw_atan", aether::cwiseAtan(xv))
        AETHER_REF_CASE("cw_tanh", aether::cwiseTanh(xv))
        AETHER_REF_CASE("cw_abs", aether::cwiseAbs(xv))
        AETHER_REF_CASE("cw_sign", aether::cwiseSign(xv))
        AETHER_REF_CASE("cw_mins", aether::cwiseMin(xv, 0.25))
        AETHER_REF_CASE("cw_maxs", aether::cwiseMax(xv, -0.25))
        AETHER_REF_CASE("cw_min", aether::cwiseMin(xv, yv))
        AETHER_REF_CASE("cw_max", aether::cwiseMax(xv, yv))
        AETHER_REF_CASE("cw_clamp", aether::clamp(xv, -0.5, 0.5))
        AETHER_REF_CASE("cw_div", aether::cwiseDiv(xv, yv))
        AETHER_REF_CASE("cw_pow", aether::cwisePow(aether::cwiseAbs(xv), yv))
        AETHER_REF_CASE("cw_pows", aether::cwisePow(aether::cwiseAbs(xv), 1.75))
        AETHER_REF_CASE("cw_scale", 2.5 * xv)
        AETHER_REF_CASE("cw_divs", xv / 3.0)
        AETHER_REF_CASE("cw_sub", xv - yv)
#undef AETHER_REF_CASE
    }
    std::printf("\n]\n");
    return 0;
}
