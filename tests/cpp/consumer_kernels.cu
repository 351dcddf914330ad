// A consumer that writes its own kernels against include/aether, spelled the
// way a user of the reference writes them (tests/test_GraphCapture.cu:45-58
// is the idiom): typed strided views as kernel parameters, one sample per
// thread from SampleIndex::make, `view[i] = expression`, Items read with
// `view[i].get()`, aether::math on register values, random leaves drawn per
// sample, launchConfig / checkLastLaunch / AETHER_CHECK_CUDA around the
// launches, and a captured launch replayed from a CUDA graph.
//
// usage: consumer_kernels <out.bin> <n>
// Writes every array's planes (capacity layout) to out.bin and prints
// "consumer kernels ok" when its own checks (graph replay identical to the
// uncaptured launch; Item and view forms of cross identical) pass.
#include <aether/aether.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

using aether::Array;
using aether::SampleIndex;
using aether::Vec3d;
using aether::Mat33d;

using StridedScalar = aether::View<double, aether::extents<aether::dyn>, aether::layout_stride>;
using Strided3 = aether::View<double, aether::extents<3, aether::dyn>, aether::layout_stride>;
using Strided4 = aether::View<double, aether::extents<4, aether::dyn>, aether::layout_stride>;
using Strided9 = aether::View<double, aether::extents<9, aether::dyn>, aether::layout_stride>;
using Strided33 = aether::View<double, aether::extents<3, 3, aether::dyn>, aether::layout_stride>;

/** out = a + s*b, rank 1. */
AETHER_KERNEL()
void graphAxpyKernel(StridedScalar a, StridedScalar b, double s, StridedScalar out) {
    const SampleIndex i = SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= a.samples()) return;
    out(i.global()) = a(i.global()) + s * b(i.global());
}

/** Per-sample Philox draws: a uniform fill of 3, 4 and 9 components. */
AETHER_KERNEL()
void fillKernel(Strided3 a, Strided3 b, Strided3 c, Strided3 d0, Strided4 q, Strided9 m, aether::random::Generator g) {
    const SampleIndex i = SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= a.samples()) return;
    a[i] = g.substream(0).uniform<double, 3>(-1.0, 1.0);
    b[i] = g.substream(1).uniform<double, 3>(-1.0, 1.0);
    c[i] = g.substream(2).uniform<double, 3>(-1.0, 1.0);
    d0[i] = g.substream(3).uniform<double, 3>(-4.0, 4.0);
    q[i] = g.substream(4).uniform<double, 4>(-1.0, 1.0);
    m[i] = g.substream(5).uniform<double, 9>(-1.0, 1.0);
}

/** The plain fused assignment: d = a + b*c + sin(a) exp(-c*c). */
AETHER_KERNEL()
void cfg1Kernel(Strided3 a, Strided3 b, Strided3 c, Strided3 d) {
    const SampleIndex i = SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= d.samples()) return;
    d[i] = a + b * c + aether::cwiseSin(a) * aether::cwiseExp((c * c) * (-1.0));
}

/** d = sqrt(a*a+b*b) * log1p(|c|) + rsqrt(1 + d0*d0), log1p per component of
 *  the sample's Item. */
AETHER_KERNEL()
void cfg2aKernel(Strided3 a, Strided3 b, Strided3 c, Strided3 d0, Strided3 d) {
    const SampleIndex i = SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= d.samples()) return;
    const Vec3d cc = c[i].get();
    const Vec3d L{aether::math::log1p(aether::math::abs(cc(0))), aether::math::log1p(aether::math::abs(cc(1))),
                  aether::math::log1p(aether::math::abs(cc(2)))};
    d[i] = aether::cwiseSqrt(a * a + b * b) * L + aether::cwiseRsqrt(aether::constant<aether::extents<3>>(1.0) + d0 * d0);
}

/** Geometry per sample: cross product (view and Item forms), quaternion
 *  rotation, the 3x3 inverse guarded by its determinant, a dot product. */
AETHER_KERNEL()
void geometryKernel(Strided3 a, Strided3 b, Strided4 q, Strided33 m, Strided3 cr, Strided3 cr2, Strided3 qr,
                    Strided33 mi, StridedScalar dt) {
    const SampleIndex i = SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (i.global() >= a.samples()) return;
    cr[i] = a.cross(b);
    const Vec3d x = a[i].get(), y = b[i].get();
    cr2[i] = x.cross(y);
    qr[i] = q.quatRotate(b);
    const Mat33d M = m[i].get();
    const double det = M.det();
    if (aether::math::abs(det) > 1e-300)
        mi[i] = M.inverse();
    else
        mi[i] = 0.0;
    dt(i.global()) = x.dot(y);
}

/** The plain fused assignment again, two samples per thread (BundleIndex). */
AETHER_KERNEL()
void cfg1BundleKernel(Strided3 a, Strided3 b, Strided3 c, Strided3 d) {
    const aether::BundleIndex<2> bi = aether::BundleIndex<2>::make(threadIdx.x, blockIdx.x, blockDim.x);
    if (!bi.mask(d.samples()).lane(0)) return;
    d[bi] = a + b * c + aether::cwiseSin(a) * aether::cwiseExp((c * c) * (-1.0));
}

template <class A>
void write(std::FILE* f, A& arr) {
    arr.download();
    auto h = arr.hostView();
    std::fwrite(h.data(), sizeof(double), A::components * arr.capacity(), f);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const std::size_t n = std::strtoull(argv[2], nullptr, 10);

    Array<double, 3> a(n), b(n), c(n), d0(n), d1(n), d2(n), cr(n), cr2(n), qr(n);
    Array<double, 4> q(n);
    Array<double, 3, 3> m(n), mi(n);
    Array<double> dt(n);

    // the 3x3 array's planes seen as 9 components (the same capacity layout)
    using Ext9 = aether::extents<9, aether::dyn>;
    const aether::offset_t st9[2] = {aether::offset_t(m.capacity()), 1};
    Strided9 m9(m.deviceView().data(), Strided9::mapping_type(Ext9(n), st9), aether::Device(aether::kDLCUDA, 0));

    const auto cfg = aether::cuda::launchConfig(n, 128);
    fillKernel<<<cfg.blocks, cfg.threads>>>(a.deviceView(), b.deviceView(), c.deviceView(), d0.deviceView(),
                                            q.deviceView(), m9, aether::random::Generator(42));
    aether::cuda::checkLastLaunch("fillKernel");
    cfg1Kernel<<<cfg.blocks, cfg.threads>>>(a.deviceView(), b.deviceView(), c.deviceView(), d1.deviceView());
    aether::cuda::checkLastLaunch("cfg1Kernel");
    Array<double, 3> d1b(n);
    const auto cfgb = aether::cuda::bundleLaunchConfig(n, 2, 128);
    cfg1BundleKernel<<<cfgb.blocks, cfgb.threads>>>(a.deviceView(), b.deviceView(), c.deviceView(), d1b.deviceView());
    aether::cuda::checkLastLaunch("cfg1BundleKernel");
    cfg2aKernel<<<cfg.blocks, cfg.threads>>>(a.deviceView(), b.deviceView(), c.deviceView(), d0.deviceView(),
                                             d2.deviceView());
    aether::cuda::checkLastLaunch("cfg2aKernel");
    geometryKernel<<<cfg.blocks, cfg.threads>>>(a.deviceView(), b.deviceView(), q.deviceView(), m.deviceView(),
                                                cr.deviceView(), cr2.deviceView(), qr.deviceView(), mi.deviceView(),
                                                dt.deviceView());
    aether::cuda::checkLastLaunch("geometryKernel");

    // capture: a launch and a stream-ordered download in one graph, replayed
    const std::size_t kN = 500;
    Array<double> x(kN), y(kN), outU(kN), outC(kN);
    {
        auto xh = x.hostView();
        auto yh = y.hostView();
        for (std::size_t k = 0; k < kN; ++k) {
            xh(k) = double(k) * 0.21 - 4.0;
            yh(k) = double(k) * 0.05 + 1.0;
        }
    }
    x.upload();
    y.upload();
    const auto c2 = aether::cuda::launchConfig(kN, 128);
    graphAxpyKernel<<<c2.blocks, c2.threads>>>(x.deviceView(), y.deviceView(), 2.25, outU.deviceView());
    aether::cuda::checkLastLaunch("graphAxpyKernel(uncaptured)");
    outU.download();
    cudaStream_t stream = nullptr;
    AETHER_CHECK_CUDA(cudaStreamCreate(&stream));
    AETHER_CHECK_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    graphAxpyKernel<<<c2.blocks, c2.threads, 0, stream>>>(x.deviceView(), y.deviceView(), 2.25, outC.deviceView());
    AETHER_CHECK_CUDA(cudaPeekAtLastError());
    outC.download(stream);
    cudaGraph_t graph = nullptr;
    AETHER_CHECK_CUDA(cudaStreamEndCapture(stream, &graph));
    cudaGraphExec_t exec = nullptr;
    AETHER_CHECK_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    for (int rep = 0; rep < 3; ++rep) {
        AETHER_CHECK_CUDA(cudaGraphLaunch(exec, stream));
        AETHER_CHECK_CUDA(cudaStreamSynchronize(stream));
        if (std::memcmp(outC.hostView().data(), outU.hostView().data(), kN * sizeof(double)) != 0) {
            std::printf("graph replay %d differs from the uncaptured launch\n", rep);
            return 1;
        }
    }
    AETHER_CHECK_CUDA(cudaGraphExecDestroy(exec));
    AETHER_CHECK_CUDA(cudaGraphDestroy(graph));
    AETHER_CHECK_CUDA(cudaStreamDestroy(stream));
    {
        auto uh = outU.hostView();
        auto xh = x.hostView();
        auto yh = y.hostView();
        for (std::size_t k = 0; k < kN; ++k) {
            // a + s*b with or without FMA contraction, as the kernel was compiled
            volatile double prod = 2.25 * yh(k);
            const double separate = xh(k) + prod, fused = std::fma(2.25, yh(k), xh(k));
            if (uh(k) != separate && uh(k) != fused) {
                std::printf("axpy value at %zu\n", k);
                return 1;
            }
        }
    }

    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    write(f, a);
    write(f, b);
    write(f, c);
    write(f, d0);
    write(f, q);
    write(f, m);
    write(f, d1);
    write(f, d2);
    write(f, cr);
    write(f, cr2);
    write(f, qr);
    write(f, mi);
    write(f, dt);
    std::fclose(f);
    d1b.download();
    {
        auto x1 = d1.hostView();
        auto x2 = d1b.hostView();
        for (std::size_t k = 0; k < n; ++k)
            for (int j = 0; j < 3; ++j)
                if (x1(j, k) != x2(j, k)) {
                    std::printf("bundle assignment differs at sample %zu\n", k);
                    return 1;
                }
    }
    if (std::memcmp(cr.hostView().data(), cr2.hostView().data(), 3 * cr.capacity() * sizeof(double)) != 0) {
        std::printf("cross: view and Item forms differ\n");
        return 1;
    }
    std::printf("consumer kernels ok\n");
    return 0;
}
