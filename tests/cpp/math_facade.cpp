// Every function of aether::math over one corpus, on the host (a host
// compiler) or in a kernel (nvcc -x cu), written as raw doubles for the test
// to compare: exact operations bit for bit, transcendentals within the
// reference's device-versus-host table (tests/test_MathParity_common.h:229-250).
//
// usage: math_facade <out.bin>
// out.bin: kFns rows of kN doubles (f(x), or f(x, y) for the binary ones).
#include <aether/aether.h>

#include <cmath>
#include <cstdio>
#include <vector>

namespace {

constexpr int kN = 512;
constexpr int kFns = 43;

// x over [-12, 12] with specials; y over [0.25, 3] with signs mixed
AETHER_DEVICEANDHOST() double corpus_x(int i) {
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.5, -2.5, 1e-300, 3.0, 1e300, -7.75};
    return i < 12 ? sp[i] : -12.0 + 24.0 * double(i) / double(kN);
}
AETHER_DEVICEANDHOST() double corpus_y(int i) {
    const double v = 0.25 + 2.75 * double((i * 37) % kN) / double(kN);
    return (i % 3 == 0) ? -v : v;
}

AETHER_DEVICEANDHOST() double eval(int f, double x, double y) {
    namespace m = aether::math;
    const double ax = m::abs(x);
    switch (f) {
    case 0: return m::sqrt(ax);
    case 1: return m::rsqrt(ax + 0.5);
    case 2: return m::exp(m::min(x, 700.0));
    case 3: return m::log(ax + 1e-3);
    case 4: return m::log1p(ax);
    case 5: return m::sin(x);
    case 6: return m::cos(x);
    case 7: return m::cbrt(x);
    case 8: return m::exp2(x);
    case 9: return m::expm1(x);
    case 10: return m::log2(ax + 1e-3);
    case 11: return m::log10(ax + 1e-3);
    case 12: return m::tan(x);
    case 13: return m::asin(m::clip(x / 12.0, -1.0, 1.0));
    case 14: return m::acos(m::clip(x / 12.0, -1.0, 1.0));
    case 15: return m::atan(x);
    case 16: return m::sinh(m::clip(x, -10.0, 10.0));
    case 17: return m::cosh(m::clip(x, -10.0, 10.0));
    case 18: return m::tanh(x);
    case 19: return m::erf(x);
    case 20: return m::abs(x);
    case 21: return m::floor(x);
    case 22: return m::ceil(x);
    case 23: return m::trunc(x);
    case 24: return m::round(x);
    case 25: return m::rint(x);
    case 26: return m::asinh(x);
    case 27: return m::acosh(ax + 1.0);
    case 28: return m::atanh(m::clip(x / 13.0, -0.99, 0.99));
    case 29: return m::erfc(x);
    case 30: return m::exp10(m::clip(x, -12.0, 12.0));
    case 31: return m::pow(ax + 0.5, y);
    case 32: return m::atan2(x, y);
    case 33: return m::hypot(x, y);
    case 34: return m::min(x, y);
    case 35: return m::max(x, y);
    case 36: return m::fmod(x, y);
    case 37: return m::fdim(x, y);
    case 38: return m::copysign(x, y);
    case 39: return m::remainder(x, y);
    case 40: return m::sign(x);
    case 41: return m::clip(x, -1.0, y);
    default: return double(m::isnan(x / y) * 4 + m::isinf(x * 1e300) * 2 + m::isfinite(x * 1e300));
    }
}

#if defined(__CUDACC__)
AETHER_KERNEL() void facade_kernel(double* out) {
    const int i = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= kN * kFns) return;
    const int f = i / kN, k = i % kN;
    out[i] = eval(f, corpus_x(k), corpus_y(k));
}
#endif

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::vector<double> out(size_t(kN) * kFns);
#if defined(__CUDACC__)
    double* d = nullptr;
    AETHER_CHECK_CUDA(cudaMalloc(&d, out.size() * sizeof(double)));
    facade_kernel<<<(unsigned(out.size()) + 255) / 256, 256>>>(d);
    aether::cuda::checkLastLaunch("facade_kernel");
    AETHER_CHECK_CUDA(cudaMemcpy(out.data(), d, out.size() * sizeof(double), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaFree(d));
#else
    for (int f = 0; f < kFns; ++f)
        for (int k = 0; k < kN; ++k) out[size_t(f) * kN + k] = eval(f, corpus_x(k), corpus_y(k));
#endif
    std::FILE* fp = std::fopen(argv[1], "wb");
    if (!fp) return 1;
    std::fwrite(out.data(), sizeof(double), out.size(), fp);
    std::fclose(fp);
    std::printf("math facade ok\n");
    return 0;
}
