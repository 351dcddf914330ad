// reshaped<Ms...> (aether/reshape.h), copyAsync(View, View, Stream)
// (aether/view_copy.h) and accum::AppendCounter (aether/append_counter.h):
// the cases of the reference's tests/test_Reshape, test_ViewCopyAsync and
// test_AppendCounter.
//
// A host compiler runs the host cases: reshaping host views, and the append
// counter's view over host words (sequential slots, 8 threads racing, the
// overflow). nvcc -x cu, linked to the engine, adds the device cases: views
// copied between device and page-locked host memory and the refusals, work
// views staging samples in shared memory (view/WorkView.h), and kernels
// appending into an Array's spare capacity up to and past it.
// Prints "view tools ok".
#include <aether/aether.h>

#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <thread>
#include <vector>

namespace {

int failures = 0;
#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                              \
        }                                                            \
    } while (0)

template <class F>
std::string thrown(F f) {
    try {
        f();
    } catch (const aether::Error& e) {
        return e.what();
    }
    return "";
}

const aether::Device kCpu(aether::kDLCPU);

void reshapes() {
    // components first, then the samples folded row-major into (4, dyn)
    const std::size_t n = 24;
    std::vector<double> d(3 * n);
    for (std::size_t k = 0; k < d.size(); ++k) d[k] = double(k);
    auto flat = aether::make_view<double, 3, aether::dyn>(d.data(), kCpu, n);
    auto f = aether::reshaped<4, aether::dyn>(flat);
    static_assert(decltype(f)::extents_type::Rank == 3, "(3, 4, dyn)");
    CHECK(f.extent(0) == 3 && f.extent(1) == 4 && f.extent(2) == 6);
    bool same = true;
    for (std::size_t c = 0; c < 3; ++c)
        for (std::size_t a = 0; a < 4; ++a)
            for (std::size_t b = 0; b < 6; ++b) same &= f(c, a, b) == flat(c, a * 6 + b);
    CHECK(same);
    // writes through the folded view land where the flat view reads
    f(2, 3, 5) = -1.0;
    CHECK(flat(2, 23) == -1.0 && f.data() == flat.data() && f.device() == kCpu);
    // the dynamic mode may come first
    auto g = aether::reshaped<aether::dyn, 4>(flat);
    CHECK(g.extent(1) == 6 && g.extent(2) == 4 && g(1, 2, 3) == flat(1, 2 * 4 + 3));
    // a scalar view reshapes straight into modes
    std::vector<float> s(32);
    for (std::size_t k = 0; k < s.size(); ++k) s[k] = float(k);
    auto sv = aether::make_view<float, aether::dyn>(s.data(), kCpu, s.size());
    auto sm = aether::reshaped<aether::dyn, 8>(sv);
    CHECK(sm.extent(0) == 4 && sm.extent(1) == 8 && sm(3, 7) == 31.0f);
    auto three = aether::reshaped<2, aether::dyn, 4>(sv);
    CHECK(three.extent(1) == 4 && three(1, 2, 3) == float(1 * 16 + 2 * 4 + 3));
    // a product that does not divide the samples is refused
    std::vector<double> ten(10);
    auto tv = aether::make_view<double, aether::dyn>(ten.data(), kCpu, ten.size());
    const std::string w = thrown([&] { (void)aether::reshaped<4, aether::dyn>(tv); });
    CHECK(w.find("reshaped failed on view") != std::string::npos &&
          w.find("static mode product 4 does not divide samples()=10") != std::string::npos);
}

// The counter's view over host words: the logic without a device.
void appendViewOnHost() {
    std::uint32_t counter = 0, flag = 0;
    const aether::accum::AppendCounterView v(&counter, 8, aether::DeviceFlagView(&flag));
    for (aether::offset_t k = 0; k < 8; ++k) CHECK(v.tryAppend() == k);
    CHECK(flag == 0);
    CHECK(v.tryAppend() == aether::accum::npos && flag == 1 && counter == 9);
    // 8 threads x 1000 appends into 5000 slots: every slot once, the rest npos
    std::uint32_t c2 = 0, f2 = 0;
    const aether::accum::AppendCounterView w(&c2, 5000, aether::DeviceFlagView(&f2));
    std::vector<std::vector<aether::offset_t>> got(8);
    std::vector<std::thread> th;
    for (int t = 0; t < 8; ++t)
        th.emplace_back([&, t] {
            for (int k = 0; k < 1000; ++k) got[t].push_back(w.tryAppend());
        });
    for (auto& x : th) x.join();
    std::set<aether::offset_t> slots;
    std::size_t misses = 0;
    for (const auto& g : got)
        for (const aether::offset_t s : g) {
            if (s == aether::accum::npos)
                ++misses;
            else
                slots.insert(s);
        }
    CHECK(slots.size() == 5000 && *slots.rbegin() == 4999 && misses == 3000 && f2 == 1 && c2 == 8000);
}

}  // namespace

#if defined(__CUDACC__)
namespace {

// Work views in shared memory (view/WorkView.h): a block stages its samples
// of `a` in a static shared array and of `b` in a carve of the dynamic one,
// then writes out[i] = a[i] + b[the mirrored sample of the same block].
using Planes3 = aether::Array<double, 3>::ViewT;
AETHER_KERNEL() void stageKernel(Planes3 a, Planes3 b, Planes3 out) {
    AETHER_SHARED() double bufA[3 * 128];
    extern __shared__ unsigned char raw[];
    const aether::offset_t bs = blockDim.x;
    auto wa = aether::make_work_view<double, 3>(bufA, bs);
    auto wb = aether::make_work_view<double, 3>(reinterpret_cast<double*>(raw), bs);
    const aether::SampleIndex i = aether::SampleIndex::make(threadIdx.x, blockIdx.x, blockDim.x);
    const bool live = i.global() < a.samples();
    if (live) {
        wa[aether::SampleIndex::make(std::size_t(i.work()))] = a[i].get();
        for (int c = 0; c < 3; ++c) wb(c, i.work()) = b(c, i.global());
    }
    __syncthreads();
    const aether::offset_t mirror = bs - 1 - i.work();
    if (live && blockIdx.x * bs + mirror < a.samples())
        for (int c = 0; c < 3; ++c) out(c, i.global()) = wa(c, i.work()) + wb(c, mirror);
}

AETHER_KERNEL() void appendKernel(aether::accum::AppendCounterView counter,
                                  aether::View<double, aether::extents<2, aether::dyn>, aether::layout_stride> spare,
                                  unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const aether::offset_t slot = counter.tryAppend();
    if (slot == aether::accum::npos) return;
    spare(0, slot) = double(i);
    spare(1, slot) = -double(i);
}

void copies() {
    const std::size_t n = 1000;
    aether::Array<double, 3> a(n), b(n), c(n), wide(2 * n);
    {
        auto h = a.hostView();
        for (std::size_t s = 0; s < n; ++s)
            for (std::size_t k = 0; k < 3; ++k) h(k, s) = double(k * 10000 + s) + 0.25;
    }
    cudaStream_t st = nullptr;
    AETHER_CHECK_CUDA(cudaStreamCreate(&st));
    aether::copyAsync(a.deviceView(), a.hostView(), st);     // page-locked host -> device
    aether::copyAsync(b.deviceView(), a.deviceView(), st);   // device -> device
    aether::copyAsync(c.hostView(), b.deviceView(), st);     // device -> page-locked host
    AETHER_CHECK_CUDA(cudaStreamSynchronize(st));
    bool same = true;
    for (std::size_t s = 0; s < n; ++s)
        for (std::size_t k = 0; k < 3; ++k) same &= c.hostView()(k, s) == a.hostView()(k, s);
    CHECK(same);
    // a source read-only view is fine
    aether::copyAsync(b.deviceView(), a.deviceView().as_const(), st);
    AETHER_CHECK_CUDA(cudaStreamSynchronize(st));
    // equal shapes with other plane pitches are refused, as are pageable views
    wide.resize(n);
    CHECK(thrown([&] { aether::copyAsync(wide.deviceView(), a.deviceView(), st); }).find("strides mismatch at mode 0") !=
          std::string::npos);
    std::vector<double> pageable(3 * a.capacity());
    auto pv = aether::View<double, aether::extents<3, aether::dyn>, aether::layout_stride>(
        pageable.data(), a.deviceView().mapping(), kCpu);
    CHECK(thrown([&] { aether::copyAsync(a.deviceView(), pv, st); }).find("no asynchronous copy for this pair") !=
          std::string::npos);
    aether::Array<double, 3> shorter(n - 1);
    CHECK(thrown([&] { aether::copyAsync(shorter.deviceView(), a.deviceView(), st); }).find("extents mismatch") !=
          std::string::npos);
    AETHER_CHECK_CUDA(cudaStreamDestroy(st));
}

void workViews() {
    const std::size_t n = 1000;   // 8 blocks of 128, the last one partial
    aether::Array<double, 3> a(n), b(n), out(n);
    auto ha = a.hostView();
    auto hb = b.hostView();
    auto ho = out.hostView();
    for (std::size_t s = 0; s < n; ++s)
        for (std::size_t c = 0; c < 3; ++c) {
            ha(c, s) = double(c * 1000 + s);
            hb(c, s) = 0.5 * double(s) - double(c);
            ho(c, s) = -1.0;
        }
    a.upload();
    b.upload();
    out.upload();
    stageKernel<<<(unsigned(n) + 127) / 128, 128, 3 * 128 * sizeof(double)>>>(a.deviceView(), b.deviceView(),
                                                                               out.deviceView());
    aether::cuda::checkLastLaunch("stageKernel");
    out.download();
    bool ok = true;
    for (std::size_t s = 0; s < n; ++s) {
        const std::size_t blk = s / 128, m = blk * 128 + (127 - s % 128);
        for (std::size_t c = 0; c < 3; ++c)
            ok &= out.hostView()(c, s) == (m < n ? ha(c, s) + hb(c, m) : -1.0);
    }
    CHECK(ok);
}

void appends() {
    // 2000 threads into 1500 spare samples: exactly 1500 land, each once,
    // the flag rises, and the 36 samples already there are untouched
    aether::Array<double, 2> arr(36);   // 36 samples already there
    arr.reserve(1536);                  // spare = 1536 - 36 = 1500
    {
        auto h = arr.hostView();
        for (std::size_t s = 0; s < 36; ++s) h(0, s) = h(1, s) = 7.0;
    }
    arr.upload();
    const std::size_t spare = arr.capacity() - arr.samples();
    CHECK(spare == 1500);
    aether::accum::AppendCounter counter(spare);
    appendKernel<<<8, 250>>>(counter.deviceView(), arr.deviceSpare(), 2000u);
    aether::cuda::checkLastLaunch("appendKernel");
    AETHER_CHECK_CUDA(cudaDeviceSynchronize());
    CHECK(counter.rawCount() == 2000 && counter.overflowed());
    CHECK(counter.commit(arr) == 1500 && arr.samples() == 1536 && counter.rawCount() == 0);
    const std::string w = thrown([&] { counter.checkOverflow("appends"); });
    CHECK(w.find("appends: device flag set") != std::string::npos && !counter.overflowed());
    arr.download();
    std::set<long> ids;
    bool paired = true, kept = true;
    auto h = arr.hostView();
    for (std::size_t s = 0; s < 36; ++s) kept &= h(0, s) == 7.0 && h(1, s) == 7.0;
    for (std::size_t s = 36; s < 1536; ++s) {
        ids.insert(long(h(0, s)));
        paired &= h(1, s) == -h(0, s);
    }
    CHECK(kept && paired && ids.size() == 1500 && *ids.rbegin() < 2000);
    // a second step within the capacity: no overflow, every append lands
    aether::Array<double, 2> more(0);
    more.reserve(640);
    aether::accum::AppendCounter c2(more.capacity());
    appendKernel<<<2, 256>>>(c2.deviceView(), more.deviceSpare(), 500u);
    aether::cuda::checkLastLaunch("appendKernel");
    AETHER_CHECK_CUDA(cudaDeviceSynchronize());
    CHECK(c2.commit(more) == 500 && !c2.overflowed() && more.samples() == 500);
}

}  // namespace
#endif

int main() {
    reshapes();
    appendViewOnHost();
#if defined(__CUDACC__)
    copies();
    workViews();
    appends();
#endif
    if (failures) return 1;
    std::printf("view tools ok\n");
    return 0;
}
