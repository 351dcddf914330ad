// The per-sample expression surface on Items and views, the cases of the
// reference's tests/test_ExprDepth.cpp, test_ExprStructural, test_ExprReduce,
// test_ItemRank0, test_Tile and the Item factories of view/Item.h:195-225
// (a default-constructed Item is zero): a 48-operand
// chained sum and a 24-operand sum of scaled terms, exact; head, tail and
// segment reads alone and inside arithmetic; dot, sum, the norm family and
// maxNorm by hand; isFinite; rank-0 items; the public reduction functors.
//
// The same checks run on the host (a host compiler) and in one kernel thread
// (nvcc -x cu), each writing a failure count; the program prints
// "expr surface ok" when both report none.
//
// usage: expr_surface
#include <aether/aether.h>

#include <cstdio>

namespace {

using aether::Vec3d;

#define EXPECT(c) fails += (c) ? 0 : 1

AETHER_DEVICEANDHOST() int depth() {
    int fails = 0;
    const Vec3d a = Vec3d::filled(1.0);
    const Vec3d sum48 = a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a +
                        a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a;
    for (int i = 0; i < 3; ++i) EXPECT(sum48(i) == 48.0);
    const Vec3d b = Vec3d::filled(2.0);
    const Vec3d chain = a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a +
                        1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b + a + 1.0 * b;
    for (int i = 0; i < 3; ++i) EXPECT(chain(i) == 36.0);
    return fails;
}

AETHER_DEVICEANDHOST() int structural() {
    int fails = 0;
    const aether::Vec<double, 6> v{1.0, 2.0, 3.0, 4.0, 5.0, 6.0};
    const aether::Vec<double, 3> s = v.segment<2, 3>();
    EXPECT(s(0) == 3.0 && s(1) == 4.0 && s(2) == 5.0);
    const aether::Vec<double, 2> h = v.head<2>();
    EXPECT(h(0) == 1.0 && h(1) == 2.0);
    const aether::Vec<double, 2> t = v.tail<2>();
    EXPECT(t(0) == 5.0 && t(1) == 6.0);
    const aether::Vec<double, 3> m = v.segment<1, 3>() * 2.0 + v.head<3>();
    EXPECT(m(0) == 5.0 && m(1) == 8.0 && m(2) == 11.0);
    const aether::Vec<double, 4> q{0.5, 1.0, 2.0, 3.0};
    const Vec3d back = q.asBack3DVector();
    EXPECT(back(0) == 1.0 && back(1) == 2.0 && back(2) == 3.0);
    return fails;
}

AETHER_DEVICEANDHOST() int reduce() {
    int fails = 0;
    const Vec3d a{1.0, 2.0, 2.0}, b{3.0, -1.0, 0.5};
    EXPECT(a.dot(b) == 0.5 * 2.0 + (-2.0 + 3.0));   // right-nested: e2 + (e1 + e0)
    EXPECT(a.sum() == 5.0);
    EXPECT(a.squaredNorm() == 9.0 && a.norm() == 3.0);
    EXPECT(aether::math::abs(a.rNorm() - 1.0 / 3.0) <= 1e-16 && a.rSquaredNorm() == 1.0 / 9.0);
    EXPECT(a.cubedNorm() == 27.0 && a.rCubedNorm() == 1.0 / 27.0);
    EXPECT(b.maxNorm() == 3.0);
    const aether::Vec<double, 4> q{1.0, 1.0, 1.0, 1.0};
    EXPECT(q.dot(q) == 4.0 && q.norm() == 2.0);   // on a quaternion too
    volatile double zero = 0.0;
    Vec3d f = Vec3d::filled(1.0);
    EXPECT(aether::isFinite(f));
    f(1) = zero / zero;
    EXPECT(!aether::isFinite(f));
    f = Vec3d::filled(1.0);
    f(2) = 1.0 / zero;
    EXPECT(!aether::isFinite(f));
    EXPECT(aether::isFinite(a + b * 2.0));
    EXPECT(aether::SumOp<double>{}(1.5, 2.0) == 3.5 && aether::TimesOp<double>{}(1.5, 2.0) == 3.0);
    EXPECT(aether::MaxOp<double>{}(-1.0, 2.0) == 2.0 && aether::LogicalAndOp{}(true, false) == false);
    return fails;
}

AETHER_DEVICEANDHOST() int items() {
    int fails = 0;
    aether::Item<double> r0(2.5);
    EXPECT(r0() == 2.5);
    r0() = -1.0;
    EXPECT(r0.get<>() == -1.0 && r0.size() == 1);
    const aether::Mat33d I = aether::Mat33d::Identity(), Z = aether::Mat33d::Zeros(), O = aether::Mat33d::Ones();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            EXPECT(I(r, c) == (r == c ? 1.0 : 0.0));
            EXPECT(Z(r, c) == 0.0 && O(r, c) == 1.0);
        }
    EXPECT(aether::Mat33d::size() == 9);
    EXPECT(sizeof(aether::idx_t) == 4 && sizeof(aether::dims_t) == 4 && aether::abi()[0] == 'a');
    // a rank-0 item read from a scalar view at a sample
    double plane[4] = {0.25, 0.5, 0.75, 1.0};
    const auto sv = aether::make_view<double, aether::dyn>(plane, aether::Device(aether::kDLCPU), 4);
    const aether::Item<double> at2 = sv[aether::SampleIndex::make(std::size_t(2))].get();
    EXPECT(at2() == 0.75);
    return fails;
}

AETHER_DEVICEANDHOST() int tiles() {
    int fails = 0;
    const aether::Tile<double, 3, 4> zero;   // a default-constructed item is zero
    for (std::size_t k = 0; k < zero.size(); ++k) EXPECT(zero.data()[k] == 0.0);
    const aether::Tile<double, 3, 4> t{1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0};
    const aether::Vec3d s2 = aether::slot<2, 3>(t);
    EXPECT(s2(0) == 7.0 && s2(1) == 8.0 && s2(2) == 9.0);
    const aether::Vec3d sum = aether::slot<0, 3>(t) + aether::slot<3, 3>(t);
    EXPECT(sum(0) == 11.0 && sum(2) == 15.0);
    const aether::Mat33d m;
    EXPECT(m(1, 2) == 0.0 && m.sum() == 0.0);
    return fails;
}

AETHER_DEVICEANDHOST() int all() { return depth() + structural() + reduce() + items() + tiles(); }

#if defined(__CUDACC__)
AETHER_KERNEL() void surface_kernel(int* fails) { *fails = all(); }
#endif

}  // namespace

int main() {
    const int host = all();
#if defined(__CUDACC__)
    int* d = nullptr;
    AETHER_CHECK_CUDA(cudaMalloc(&d, sizeof(int)));
    surface_kernel<<<1, 1>>>(d);
    aether::cuda::checkLastLaunch("surface_kernel");
    int dev = -1;
    AETHER_CHECK_CUDA(cudaMemcpy(&dev, d, sizeof(int), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaFree(d));
#else
    const int dev = 0;
#endif
    std::printf("host failures %d, device failures %d\n", host, dev);
    if (host || dev) return 1;
    std::printf("expr surface ok\n");
    return 0;
}
