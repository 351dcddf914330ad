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

#include <aether/aether.h>

#include <cmath>
#include <cstdio>
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

int main(int argc, char** argv) {
    if (argc < 2) return 2;
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
