// aether::rt (aether/rt.h), the rolled-loop twins, against the static forms
// they stand in for (the reference's tests/test_ExprRt): dot, sum, the norm
// family, maxNorm, isFinite and matDot over 144- and 3-element operands;
// matVec (=, +=, -=, and through transposed) over an 8x40 matrix; matMat over
// 3x4 by 4x5; store. Items on the host, per-sample proxies view[i] over
// arrays of samples on the host and in a kernel. Every result must equal the
// static form's bits (built with contraction off: -ffp-contract=off on the
// host, --fmad=false and -Xcompiler -ffp-contract=off in the nvcc build).
// Prints "rt twins ok".
#include <aether/aether.h>
#include <aether/rt.h>

#include <cstdio>
#include <vector>

namespace {

constexpr int kS = 67;   // samples
constexpr int kL = 144, kR = 8, kC = 40;

template <class T>
AETHER_DEVICEANDHOST() T val(int s, int k, int salt) {
    const unsigned h = unsigned(s) * 2654435761u + unsigned(k) * 40503u + unsigned(salt) * 97u;
    return T(int((h >> 7) % 2001) - 1000) / T(257) + T(salt) * T(0.125);
}

#define EXPECT_SAME(a, b) fails += ((a) == (b)) ? 0 : 1

// One sample of every check, on views whose sample mode is the last.
template <class VL, class VM, class VV, class VO, class VA, class VB, class VP>
AETHER_DEVICEANDHOST() int checkSample(int s, VL& x, VL& y, VM& m, VV& v, VO& o1, VO& o2, VA& a, VB& b, VP& p1, VP& p2) {
    int fails = 0;
    const aether::SampleIndex i = aether::SampleIndex::make(std::size_t(s));
    auto xs = x[i];
    auto ys = y[i];
    // the static forms, each evaluated at this sample
    const auto X = xs.get(), Y = ys.get();
    EXPECT_SAME(aether::rt::dot(xs, ys), X.dot(Y));
    EXPECT_SAME(aether::rt::sum(xs), X.sum());
    EXPECT_SAME(aether::rt::squaredNorm(xs), X.squaredNorm());
    EXPECT_SAME(aether::rt::norm(xs), X.norm());
    EXPECT_SAME(aether::rt::rNorm(xs), X.rNorm());
    EXPECT_SAME(aether::rt::rSquaredNorm(xs), X.rSquaredNorm());
    EXPECT_SAME(aether::rt::cubedNorm(xs), X.cubedNorm());
    EXPECT_SAME(aether::rt::rCubedNorm(xs), X.rCubedNorm());
    EXPECT_SAME(aether::rt::maxNorm(xs), X.maxNorm());
    EXPECT_SAME(aether::rt::isFinite(xs), aether::isFinite(X));
    // matVec: rolled into o1, static into o2
    auto ms = m[i];
    auto vs = v[i];
    auto o1s = o1[i];
    auto o2s = o2[i];
    aether::rt::matVec(o1s, ms, vs);
    o2s = m * v;
    for (int r = 0; r < kR; ++r) EXPECT_SAME(o1s.at(r), o2s.at(r));
    aether::rt::matVecAdd(o1s, ms, vs);
    o2s += m * v;
    aether::rt::matVecSub(o1s, ms, vs);
    o2s -= m * v;
    for (int r = 0; r < kR; ++r) EXPECT_SAME(o1s.at(r), o2s.at(r));
    // matMat and matDot over 3x4 by 4x5; transposed
    auto as = a[i];
    auto bs = b[i];
    auto p1s = p1[i];
    auto p2s = p2[i];
    aether::rt::matMat(p1s, as, bs);
    p2s = a * b;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 5; ++c) EXPECT_SAME(p1s.at(r, c), p2s.at(r, c));
    const auto A = as.get();
    EXPECT_SAME(aether::rt::matDot(as, as), A.matDot(A));
    // (A^T) (A) is 4x4: rolled through transposed vs the static transpose
    aether::Mat<double, 4, 4> t1, t2;
    aether::rt::matMat(t1, aether::rt::transposed(A), A);
    t2 = A.transpose() * A;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) EXPECT_SAME(t1(r, c), t2(r, c));
    // store: rolled element copy of an Item
    aether::rt::store(p1s, p2s.get());
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 5; ++c) EXPECT_SAME(p1s.at(r, c), p2s.at(r, c));
    return fails;
}

struct Storage {
    std::vector<double> x, y, m, v, o1, o2, a, b, p1, p2;
    Storage()
        : x(kL * kS), y(kL * kS), m(kR * kC * kS), v(kC * kS), o1(kR * kS), o2(kR * kS), a(12 * kS), b(20 * kS),
          p1(15 * kS), p2(15 * kS) {
        for (int s = 0; s < kS; ++s) {
            for (int k = 0; k < kL; ++k) x[k * kS + s] = val<double>(s, k, 1), y[k * kS + s] = val<double>(s, k, 2);
            for (int k = 0; k < kR * kC; ++k) m[k * kS + s] = val<double>(s, k, 3);
            for (int k = 0; k < kC; ++k) v[k * kS + s] = val<double>(s, k, 4);
            for (int k = 0; k < 12; ++k) a[k * kS + s] = val<double>(s, k, 5);
            for (int k = 0; k < 20; ++k) b[k * kS + s] = val<double>(s, k, 6);
        }
    }
};

template <class P>
AETHER_DEVICEANDHOST() int checkAll(P* x, P* y, P* m, P* v, P* o1, P* o2, P* a, P* b, P* p1, P* p2, aether::Device d,
                                     int s0, int s1) {
    auto X = aether::make_view<double, kL, aether::dyn>(x, d, kS);
    auto Y = aether::make_view<double, kL, aether::dyn>(y, d, kS);
    auto M = aether::make_view<double, kR, kC, aether::dyn>(m, d, kS);
    auto V = aether::make_view<double, kC, aether::dyn>(v, d, kS);
    auto O1 = aether::make_view<double, kR, aether::dyn>(o1, d, kS);
    auto O2 = aether::make_view<double, kR, aether::dyn>(o2, d, kS);
    auto A = aether::make_view<double, 3, 4, aether::dyn>(a, d, kS);
    auto B = aether::make_view<double, 4, 5, aether::dyn>(b, d, kS);
    auto P1 = aether::make_view<double, 3, 5, aether::dyn>(p1, d, kS);
    auto P2 = aether::make_view<double, 3, 5, aether::dyn>(p2, d, kS);
    int fails = 0;
    for (int s = s0; s < s1; ++s) fails += checkSample(s, X, Y, M, V, O1, O2, A, B, P1, P2);
    return fails;
}

#if defined(__CUDACC__)
AETHER_KERNEL() void twinsKernel(double* x, double* y, double* m, double* v, double* o1, double* o2, double* a,
                                 double* b, double* p1, double* p2, int* fails) {
    const int s = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (s >= kS) return;
    const int f = checkAll(x, y, m, v, o1, o2, a, b, p1, p2, aether::Device(aether::kDLCUDA), s, s + 1);
    if (f) atomicAdd(fails, f);
}
#endif

}  // namespace

int main() {
    Storage h;
    int fails = checkAll(h.x.data(), h.y.data(), h.m.data(), h.v.data(), h.o1.data(), h.o2.data(), h.a.data(),
                         h.b.data(), h.p1.data(), h.p2.data(), aether::Device(aether::kDLCPU), 0, kS);
    // Items on the host: a non-finite component and the 3-vectors
    const aether::Vec3d q{1.0, -2.5, 0.75};
    fails += aether::rt::dot(q, q) == q.dot(q) ? 0 : 1;
    fails += aether::rt::maxNorm(q) == 2.5 ? 0 : 1;
    aether::Vec3d bad = q;
    volatile double zero = 0.0;
    bad(1) = 1.0 / zero;
    fails += (!aether::rt::isFinite(bad) && aether::rt::isFinite(q)) ? 0 : 1;
    std::printf("host failures %d\n", fails);
#if defined(__CUDACC__)
    std::vector<double*> d(10);
    std::vector<std::vector<double>*> src = {&h.x, &h.y, &h.m, &h.v, &h.o1, &h.o2, &h.a, &h.b, &h.p1, &h.p2};
    for (int k = 0; k < 10; ++k) {
        AETHER_CHECK_CUDA(cudaMalloc(&d[k], src[k]->size() * sizeof(double)));
        AETHER_CHECK_CUDA(cudaMemcpy(d[k], src[k]->data(), src[k]->size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    int* df = nullptr;
    AETHER_CHECK_CUDA(cudaMalloc(&df, sizeof(int)));
    AETHER_CHECK_CUDA(cudaMemset(df, 0, sizeof(int)));
    twinsKernel<<<(kS + 31) / 32, 32>>>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9], df);
    aether::cuda::checkLastLaunch("twinsKernel");
    int devFails = -1;
    AETHER_CHECK_CUDA(cudaMemcpy(&devFails, df, sizeof(int), cudaMemcpyDeviceToHost));
    for (double* p : d) AETHER_CHECK_CUDA(cudaFree(p));
    AETHER_CHECK_CUDA(cudaFree(df));
    std::printf("device failures %d\n", devFails);
    fails += devFails;
#endif
    if (fails) return 1;
    std::printf("rt twins ok\n");
    return 0;
}
