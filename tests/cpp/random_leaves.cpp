// The rest of aether::random's leaf API, drawn per sample with get<I>(i)
// the way the reference's random tests read leaves: Item (per-component)
// parameters of normal, lognormal, exponential and bernoulli, uniformInt in
// 32 and 64 bits, multivariateNormal from cholesky in double and float, the
// free-function spelling (the default seed and seed(s)) and the index-free
// get<I>() draws. The same cases as the reference driver's, at the same seeds.
//
// Compiled by a host compiler the samples run in a host loop; compiled by
// nvcc (-x cu) one thread draws one sample in a kernel.
//
// usage: random_leaves <out.bin> <n>
// out.bin: 19 f64 planes (normal 3, lognormal 3, exponential 3, bernoulli 3,
// mvn 3, free uniform 2, seed(99) normal 2), the 16 index-free f64 values,
// 3 i32 planes (uniformInt), 2 i64 planes (uniformInt 64-bit), 2 f32 planes
// (float mvn), then the 6 packed f64 entries of the cholesky factor.
#include <aether/aether.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

using aether::SampleIndex;

namespace {

struct Out {
    double* f64;
    double* index_free;
    int* i32;
    long long* i64;
    float* f32;
    std::size_t n;
};

template <class N, class LG, class EX, class BE, class RI, class RL, class MV, class MF, class FU, class FS>
AETHER_DEVICEANDHOST() void drawSample(std::size_t k, const Out& o, const N& nrm, const LG& lgn, const EX& ex,
                                       const BE& be, const RI& ri, const RL& rl, const MV& mvn, const MF& mvnf,
                                       const FU& fu, const FS& fs) {
    const std::size_t n = o.n;
    const SampleIndex i = SampleIndex::make(k);
    double* f = o.f64;
    f[0 * n + k] = nrm.template get<0>(i);
    f[1 * n + k] = nrm.template get<1>(i);
    f[2 * n + k] = nrm.template get<2>(i);
    f[3 * n + k] = lgn.template get<0>(i);
    f[4 * n + k] = lgn.template get<1>(i);
    f[5 * n + k] = lgn.template get<2>(i);
    f[6 * n + k] = ex.template get<0>(i);
    f[7 * n + k] = ex.template get<1>(i);
    f[8 * n + k] = ex.template get<2>(i);
    f[9 * n + k] = be.template get<0>(i);
    f[10 * n + k] = be.template get<1>(i);
    f[11 * n + k] = be.template get<2>(i);
    f[12 * n + k] = mvn.template get<0>(i);
    f[13 * n + k] = mvn.template get<1>(i);
    f[14 * n + k] = mvn.template get<2>(i);
    f[15 * n + k] = fu.template get<0>(i);
    f[16 * n + k] = fu.template get<1>(i);
    f[17 * n + k] = fs.template get<0>(i);
    f[18 * n + k] = fs.template get<1>(i);
    o.i32[0 * n + k] = ri.template get<0>(i);
    o.i32[1 * n + k] = ri.template get<1>(i);
    o.i32[2 * n + k] = ri.template get<2>(i);
    o.i64[0 * n + k] = rl.template get<0>(i);
    o.i64[1 * n + k] = rl.template get<1>(i);
    o.f32[0 * n + k] = mvnf.template get<0>(i);
    o.f32[1 * n + k] = mvnf.template get<1>(i);
}

template <class U, class Z, class N, class LG, class EX, class BE, class RI, class RL, class MV, class MF, class FU>
AETHER_DEVICEANDHOST() void drawIndexFree(double* fr, const U& u, const Z& z, const N& nrm, const LG& lgn, const EX& ex,
                                          const BE& be, const RI& ri, const RL& rl, const MV& mvn, const MF& mvnf,
                                          const FU& fu) {
    fr[0] = u.template get<0>();
    fr[1] = u.template get<1>();
    fr[2] = u.template get<2>();
    fr[3] = double(z.template get<0>());
    fr[4] = double(z.template get<1>());
    fr[5] = nrm.template get<2>();
    fr[6] = lgn.template get<0>();
    fr[7] = ex.template get<1>();
    fr[8] = be.template get<2>();
    fr[9] = double(ri.template get<0>());
    fr[10] = double(ri.template get<2>());
    fr[11] = double(rl.template get<1>());
    fr[12] = mvn.template get<0>();
    fr[13] = mvn.template get<2>();
    fr[14] = double(mvnf.template get<1>());
    fr[15] = fu.template get<1>();
}

#if defined(__CUDACC__)
template <class U, class Z, class N, class LG, class EX, class BE, class RI, class RL, class MV, class MF, class FU,
          class FS>
AETHER_KERNEL() void leavesKernel(Out o, U u, Z z, N nrm, LG lgn, EX ex, BE be, RI ri, RL rl, MV mvn, MF mvnf, FU fu,
                                  FS fs) {
    const std::size_t k = std::size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k == 0) drawIndexFree(o.index_free, u, z, nrm, lgn, ex, be, ri, rl, mvn, mvnf, fu);
    if (k < o.n) drawSample(k, o, nrm, lgn, ex, be, ri, rl, mvn, mvnf, fu, fs);
}
#endif

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::size_t n = std::strtoull(argv[2], nullptr, 10);

    const aether::random::Generator g(21);
    aether::Item<double, 3> m3, s3, l3, p3, mu;
    m3(0) = -1.0; m3(1) = 0.0; m3(2) = 2.5;
    s3(0) = 0.5; s3(1) = 1.0; s3(2) = 3.0;
    l3(0) = 0.5; l3(1) = 2.0; l3(2) = 8.0;
    p3(0) = 0.1; p3(1) = 0.5; p3(2) = 0.9;
    mu(0) = 1.0; mu(1) = -2.0; mu(2) = 0.5;
    const double cov[3][3] = {{2.0, 0.5, 0.1}, {0.5, 1.0, 0.3}, {0.1, 0.3, 0.5}};
    const auto L = aether::random::cholesky<double, 3>(cov);
    const float covf[2][2] = {{1.5f, -0.4f}, {-0.4f, 0.8f}};
    const auto Lf = aether::random::cholesky<float, 2>(covf);
    aether::Item<float, 2> muf;
    muf(0) = 0.25f; muf(1) = -0.75f;

    const auto nrm = g.substream(0).normal<double, 3>(m3, s3);
    const auto lgn = g.substream(1).lognormal<double, 3>(m3, s3);
    const auto ex = g.substream(2).exponential<double, 3>(l3);
    const auto be = g.substream(3).bernoulli<double, 3>(p3);
    const auto ri = g.substream(4).uniformInt<int, 3>(-5, 17);
    const auto rl = g.substream(5).uniformInt<long long, 2>(-(1LL << 40), 1LL << 41);
    const auto mvn = g.substream(6).multivariateNormal<double, 3>(mu, L);
    const auto mvnf = g.substream(7).multivariateNormal<float, 2>(muf, Lf);
    const auto fu = aether::random::uniform<double, 2>(-3.0, 3.0);
    const auto fs = aether::random::seed(99).normal<double, 2>(0.0, 1.0);
    const auto u = g.substream(8).uniform<double, 3>(-1.0, 1.0);
    const auto z = g.substream(9).normal<float, 2>(0.0f, 1.0f);

    std::vector<double> F(19 * n), FR(16);
    std::vector<int> I32(3 * n);
    std::vector<long long> I64(2 * n);
    std::vector<float> F32(2 * n);
#if defined(__CUDACC__)
    Out d{nullptr, nullptr, nullptr, nullptr, nullptr, n};
    AETHER_CHECK_CUDA(cudaMalloc(&d.f64, F.size() * sizeof(double)));
    AETHER_CHECK_CUDA(cudaMalloc(&d.index_free, FR.size() * sizeof(double)));
    AETHER_CHECK_CUDA(cudaMalloc(&d.i32, I32.size() * sizeof(int)));
    AETHER_CHECK_CUDA(cudaMalloc(&d.i64, I64.size() * sizeof(long long)));
    AETHER_CHECK_CUDA(cudaMalloc(&d.f32, F32.size() * sizeof(float)));
    const auto cfg = aether::cuda::launchConfig(n, 128);
    leavesKernel<<<cfg.blocks, cfg.threads>>>(d, u, z, nrm, lgn, ex, be, ri, rl, mvn, mvnf, fu, fs);
    aether::cuda::checkLastLaunch("leavesKernel");
    AETHER_CHECK_CUDA(cudaMemcpy(F.data(), d.f64, F.size() * sizeof(double), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(FR.data(), d.index_free, FR.size() * sizeof(double), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(I32.data(), d.i32, I32.size() * sizeof(int), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(I64.data(), d.i64, I64.size() * sizeof(long long), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(F32.data(), d.f32, F32.size() * sizeof(float), cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaFree(d.f64));
    AETHER_CHECK_CUDA(cudaFree(d.index_free));
    AETHER_CHECK_CUDA(cudaFree(d.i32));
    AETHER_CHECK_CUDA(cudaFree(d.i64));
    AETHER_CHECK_CUDA(cudaFree(d.f32));
#else
    const Out h{F.data(), FR.data(), I32.data(), I64.data(), F32.data(), n};
    drawIndexFree(h.index_free, u, z, nrm, lgn, ex, be, ri, rl, mvn, mvnf, fu);
    for (std::size_t k = 0; k < n; ++k) drawSample(k, h, nrm, lgn, ex, be, ri, rl, mvn, mvnf, fu, fs);
#endif

    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    std::fwrite(F.data(), sizeof(double), F.size(), f);
    std::fwrite(FR.data(), sizeof(double), FR.size(), f);
    std::fwrite(I32.data(), sizeof(int), I32.size(), f);
    std::fwrite(I64.data(), sizeof(long long), I64.size(), f);
    std::fwrite(F32.data(), sizeof(float), F32.size(), f);
    std::fwrite(L.data, sizeof(double), 6, f);
    std::fclose(f);
    std::printf("random leaves ok\n");
    return 0;
}
