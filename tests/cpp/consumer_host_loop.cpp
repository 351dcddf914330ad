// The per-sample consumer API on the host: the reference's CPU usage pattern
// (a loop over SampleIndex::make(k) assigning `view[i] = expression` into
// make_view'd host memory, tests/test_Random_common.h:63-70), compiled by a
// host compiler with contraction off. Random leaves are drawn per sample by
// the header's own Philox, the math facade routes to std::. Writes every
// array's planes (n samples each) to argv[1].
//
// usage: consumer_host_loop <out.bin> <n>
#include <aether/aether.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::size_t n = std::strtoull(argv[2], nullptr, 10);
    using aether::dyn;
    using aether::SampleIndex;
    const aether::Device cpu(aether::kDLCPU);

    std::vector<double> A(3 * n), B(3 * n), C(3 * n), D0(3 * n), Q(4 * n), M(9 * n), Z(n);
    std::vector<double> D1(3 * n), D2(3 * n), CR(3 * n), QR(3 * n), MI(9 * n), DT(n), N2(2 * n);
    auto a = aether::make_view<double, 3, dyn>(A.data(), cpu, n);
    auto b = aether::make_view<double, 3, dyn>(B.data(), cpu, n);
    auto c = aether::make_view<double, 3, dyn>(C.data(), cpu, n);
    auto d0 = aether::make_view<double, 3, dyn>(D0.data(), cpu, n);
    auto q = aether::make_view<double, 4, dyn>(Q.data(), cpu, n);
    auto m9 = aether::make_view<double, 9, dyn>(M.data(), cpu, n);
    auto m = aether::make_view<double, 3, 3, dyn>(M.data(), cpu, n);
    auto z = aether::make_view<double, 1, dyn>(Z.data(), cpu, n);
    auto d1 = aether::make_view<double, 3, dyn>(D1.data(), cpu, n);
    auto d2 = aether::make_view<double, 3, dyn>(D2.data(), cpu, n);
    auto cr = aether::make_view<double, 3, dyn>(CR.data(), cpu, n);
    auto qr = aether::make_view<double, 3, dyn>(QR.data(), cpu, n);
    auto mi = aether::make_view<double, 3, 3, dyn>(MI.data(), cpu, n);
    auto dt = aether::make_view<double, dyn>(DT.data(), cpu, n);
    auto n2 = aether::make_view<double, 2, dyn>(N2.data(), cpu, n);

    const aether::random::Generator g(42);
    for (std::size_t k = 0; k < n; ++k) {
        const SampleIndex i = SampleIndex::make(k);
        a[i] = g.substream(0).uniform<double, 3>(-1.0, 1.0);
        b[i] = g.substream(1).uniform<double, 3>(-1.0, 1.0);
        c[i] = g.substream(2).uniform<double, 3>(-1.0, 1.0);
        d0[i] = g.substream(3).uniform<double, 3>(-4.0, 4.0);
        q[i] = g.substream(4).uniform<double, 4>(-1.0, 1.0);
        m9[i] = g.substream(5).uniform<double, 9>(-1.0, 1.0);
        z[i] = g.substream(6).normal<double, 1>(0.0, 1.0);
        n2[i] = g.substream(7).normal<double, 2>(0.5, 2.0);
    }
    for (std::size_t k = 0; k < n; ++k) {
        const SampleIndex i = SampleIndex::make(k);
        d1[i] = a + b * c + aether::cwiseSin(a) * aether::cwiseExp((c * c) * (-1.0));
        const aether::Vec3d cc = c[i].get();
        const aether::Vec3d L{aether::math::log1p(aether::math::abs(cc(0))), aether::math::log1p(aether::math::abs(cc(1))),
                              aether::math::log1p(aether::math::abs(cc(2)))};
        d2[i] = aether::cwiseSqrt(a * a + b * b) * L +
                aether::cwiseRsqrt(aether::constant<aether::extents<3>>(1.0) + d0 * d0);
        cr[i] = a.cross(b);
        qr[i] = q.quatRotate(b);
        const aether::Mat33d Mi = m[i].get();
        if (aether::math::abs(Mi.det()) > 1e-300)
            mi[i] = Mi.inverse();
        else
            mi[i] = 0.0;
        const aether::Vec3d x = a[i].get(), y = b[i].get();
        dt(i.global()) = x.dot(y);
    }

    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    for (const std::vector<double>* v : {&A, &B, &C, &D0, &Q, &M, &Z, &N2, &D1, &D2, &CR, &QR, &MI, &DT})
        std::fwrite(v->data(), sizeof(double), v->size(), f);
    std::fclose(f);
    std::printf("host loop ok\n");
    return 0;
}
