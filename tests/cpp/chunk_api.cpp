// aether::Chunk, copy, copyAsync, fill and make_view(chunk) (aether/chunk.h),
// the cases of the reference's tests/test_Chunk, test_Copy and test_Borrow.
// Host cases need only the engine library (host chunks); with nvcc the
// device and page-locked cases run as well. Prints "chunk ok".
#include <aether/aether.h>
#include <aether/chunk.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
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
bool has(const std::string& s, const char* n) { return s.find(n) != std::string::npos; }

const aether::Device kCpu(aether::kDLCPU), kDev(aether::kDLCUDA), kPinned(aether::kDLCUDAHost);

void hostCases() {
    aether::Chunk a = aether::Chunk::allocate(kCpu, 4096);
    CHECK(a.owns() && a.size() == 4096 && a.device() == kCpu && !a.streamOrdered());
    CHECK(reinterpret_cast<std::uintptr_t>(a.data()) % 256 == 0);
    // move-only: the source is emptied, the bytes stay
    std::memset(a.data(), 7, a.size());
    aether::Chunk b = std::move(a);
    CHECK(!a.owns() && a.data() == nullptr && b.owns() && static_cast<unsigned char>(b.data()[4095]) == 7);
    // borrow: no ownership, same bytes
    std::vector<double> host(64, 1.5);
    aether::Chunk br = aether::Chunk::borrow(host.data(), host.size() * sizeof(double), kCpu, 8);
    CHECK(!br.owns() && br.size() == 512);
    // host <-> host copy and fill
    aether::Chunk c = aether::Chunk::allocate(kCpu, 512);
    aether::copy(c, br);
    CHECK(reinterpret_cast<double*>(c.data())[63] == 1.5);
    const double v = -2.25;
    aether::fill(c, &v, sizeof v);
    CHECK(reinterpret_cast<double*>(c.data())[10] == -2.25);
    // a view over a chunk, its size checked
    auto view = aether::make_view<double, 4, aether::dyn>(c, 16);
    CHECK(view(3, 15) == -2.25 && view.device() == kCpu);
    CHECK(has(thrown([&] { (void)aether::make_view<double, 4, aether::dyn>(c, 17); }),
              "the view needs 544 bytes, the chunk holds 512"));
    // refusals: size mismatch, a direct host <-> device pair, bad fill widths,
    // misaligned borrow, alignment above 256 -- all before any device call
    aether::Chunk small = aether::Chunk::allocate(kCpu, 256);
    CHECK(has(thrown([&] { aether::copy(small, c); }), "copy failed on cpu -> cpu, size=512 bytes (size mismatch"));
    aether::Chunk fakeDev = aether::Chunk::borrow(reinterpret_cast<void*>(std::uintptr_t(1) << 20), 512, kDev);
    CHECK(has(thrown([&] { aether::copy(fakeDev, c); }), "illegal device pair"));
    CHECK(has(thrown([&] { aether::copy(c, fakeDev); }), "illegal device pair"));
    aether::Chunk zero = aether::Chunk::allocate(kCpu, 0);
    aether::Chunk zeroDev = aether::Chunk::borrow(nullptr, 0, kDev);
    CHECK(has(thrown([&] { aether::copy(zeroDev, zero); }), "illegal device pair"));   // checked before the empty case
    CHECK(has(thrown([&] { aether::copyAsync(c, br, nullptr); }), "not an asynchronous pair"));
    const char three[3] = {1, 2, 3};
    CHECK(has(thrown([&] { aether::fill(c, three, 3); }), "must be 1..16 bytes and divide the size"));
    CHECK(has(thrown([&] { (void)aether::Chunk::borrow(host.data() + 1, 8, kCpu, 16); }), "not aligned to 16"));
    CHECK(has(thrown([&] { (void)aether::Chunk::allocate(kCpu, 64, 512); }), "alignment must be a power of two"));
}

}  // namespace

#if defined(__CUDACC__)
namespace {

void deviceChunks(cudaStream_t st) {
    const std::size_t n = 1 << 20;
    aether::Chunk pin = aether::Chunk::allocate(kPinned, n * sizeof(double));
    aether::Chunk back = aether::Chunk::allocate(kPinned, n * sizeof(double));
    auto* p = reinterpret_cast<double*>(pin.data());
    for (std::size_t k = 0; k < n; ++k) p[k] = double(k) * 0.5;
    aether::Chunk dev = aether::Chunk::allocate(kDev, n * sizeof(double), st);
    CHECK(dev.streamOrdered() && dev.stream() == st && dev.owns());
    aether::copyAsync(dev, pin, st);   // page-locked -> device
    aether::Chunk dev2 = aether::Chunk::allocate(kDev, n * sizeof(double));
    aether::copyAsync(dev2, dev, st);  // device -> device
    aether::copyAsync(back, dev2, st); // device -> page-locked
    AETHER_CHECK_CUDA(cudaStreamSynchronize(st));
    CHECK(std::memcmp(back.data(), pin.data(), pin.size()) == 0);
    // blocking copies through the copy engines, and a device fill
    const float pattern[2] = {1.0f, -3.0f};   // 8 bytes, not uniform
    aether::fill(dev2, pattern, sizeof pattern, st);
    AETHER_CHECK_CUDA(cudaStreamSynchronize(st));
    aether::copy(back, dev2);
    const float* f = reinterpret_cast<const float*>(back.data());
    CHECK(f[0] == 1.0f && f[1] == -3.0f && f[2 * n - 1] == -3.0f);
    aether::Chunk host = aether::Chunk::allocate(kCpu, n * sizeof(double));
    aether::copy(host, back);          // page-locked -> pageable: a host copy
    CHECK(std::memcmp(host.data(), back.data(), back.size()) == 0);
    CHECK(has(thrown([&] { aether::copyAsync(dev, host, st); }), "not an asynchronous pair"));
    // a device view over a chunk, used by the engine's runtime evaluation
    auto dv = aether::make_view<double, 2, aether::dyn>(dev, n / 2);
    CHECK(dv.device() == kDev && dv.data() == reinterpret_cast<double*>(dev.data()));
    AETHER_CHECK_CUDA(cudaStreamSynchronize(st));
}

void deviceCases() {
    cudaStream_t st = nullptr;
    AETHER_CHECK_CUDA(cudaStreamCreate(&st));
    deviceChunks(st);   // every chunk is gone before its stream is destroyed
    AETHER_CHECK_CUDA(cudaStreamDestroy(st));
}

}  // namespace
#endif

int main() {
    hostCases();
#if defined(__CUDACC__)
    deviceCases();
#endif
    if (failures) return 1;
    std::printf("chunk ok\n");
    return 0;
}
