// A consumer of the C++ front end on the device: the plain fused assignment
// of the reference's first configuration, written the way an aether user
// writes it, plus a host-view round trip, a compensated global sum and a
// refused assignment. Writes a, b, c, d (capacity layout) and the sum to the
// file named by argv[1]; prints "consumer ok" when its own checks pass.
#include <aether/aether.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::size_t n = std::strtoull(argv[2], nullptr, 10);
    aether::Array<double, 3> a(n), b(n), c(n), d(n);
    aether::random::Generator g(42);
    a.deviceView() = g.substream(0).uniform<double, 3>(-1.0, 1.0);
    b.deviceView() = g.substream(1).uniform<double, 3>(-1.0, 1.0);
    c.deviceView() = g.substream(2).uniform<double, 3>(-1.0, 1.0);
    auto A = a.deviceView(), B = b.deviceView(), C = c.deviceView();
    d.deviceView() = A + B * C + aether::cwiseSin(A) * aether::cwiseExp((C * C) * -1.0);
    const auto sum = aether::globalSum(aether::per_sample::dot(A, B), n);
    a.download();
    b.download();
    c.download();
    d.download();

    // host view -> device -> host
    aether::Array<double> x(n), y(n);
    auto xh = x.hostView();
    for (std::size_t i = 0; i < n; ++i) xh(i) = double(i) * 0.5;
    x.upload();
    y.deviceView() = x.deviceView() * 2.0 + 1.0;
    y.download();
    auto yh = y.hostView();
    for (std::size_t i = 0; i < n; ++i)
        if (yh(i) != double(i) + 1.0) {
            std::printf("round trip mismatch at %zu\n", i);
            return 1;
        }
    // runtime-typed evaluation: cast d to float through its descriptor
    aether::Array<float, 3> fl(n);
    aether::eval::runtimeEval(aether::eval::RuntimeOp::Assign, aether::fromView(d.deviceView()), aether::RuntimeView{},
                              aether::fromView(fl.deviceView()));
    fl.download();
    {
        auto fh = fl.hostView();
        auto dh = d.hostView();
        for (std::size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                if (fh(k, i) != float(dh(k, i))) {
                    std::printf("runtimeEval cast mismatch at %zu\n", i);
                    return 1;
                }
    }
    // compensated accumulation plane: a + b - a delivers b (to within one ulp)
    {
        aether::accum::Plane<3> plane(n);
        plane += A * 1e6;
        plane += B;
        plane += A * -1e6;
        aether::Array<double, 3> got(n);
        plane.deliver(got.deviceView());
        got.download();
        auto gh = got.hostView();
        auto bh = b.hostView();
        for (std::size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                if (std::fabs(gh(k, i) - bh(k, i)) > std::fabs(std::nextafter(bh(k, i), 1e300) - bh(k, i))) {
                    std::printf("accumulation plane mismatch at %zu\n", i);
                    return 1;
                }
    }
    try {
        d.deviceView() = aether::Expr(aether::per_sample::dot(A, B)) + aether::Expr(aether::constant<aether::extents<2>>(1.0));
        std::printf("shape mismatch was not refused\n");
        return 1;
    } catch (const aether::Error&) {
    }

    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    for (auto* arr : {&a, &b, &c, &d}) {
        auto h = arr->hostView();
        std::fwrite(h.data(), sizeof(double), 3 * arr->capacity(), f);
    }
    std::fwrite(&sum.first, sizeof(double), 1, f);
    std::fwrite(&sum.second, sizeof(double), 1, f);
    std::fclose(f);
    std::printf("consumer ok\n");
    return 0;
}
