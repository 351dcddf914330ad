// aether::accum::atomic (aether/accum_atomic.h), the cases of the reference's
// tests/test_Atomic: a concurrent magnitude minimum that keeps the stored
// sign and leaves a slot alone for a larger magnitude, a concurrent integer
// maximum, one-byte bool slots set by many writers (all false stays false,
// neighbours untouched, a one-byte allocation stays in bounds), and a
// compensated sum whose value + residual is the exact total. Host threads
// with a host compiler; with nvcc a kernel of 64 blocks of 256 threads as
// well. Prints "atomic ok".
#include <aether/aether.h>
#include <aether/accum_atomic.h>

#include <cmath>
#include <cstdio>
#include <thread>
#include <vector>

namespace {

namespace at = aether::accum::atomic;

int failures = 0;
#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                              \
        }                                                            \
    } while (0)

constexpr int kWriters = 16384;

// writer w: a magnitude, an int, which bool slot it sets, and a term
AETHER_DEVICEANDHOST() double magnitudeOf(int w) { return 1.0 + double((w * 7919) % kWriters); }
AETHER_DEVICEANDHOST() int intOf(int w) { return (w * 104729) % 100003 - 50000; }
AETHER_DEVICEANDHOST() double termOf(int w) { return (w & 1) ? 1099511627776.0 : double(1 + w % 5) * 0.0009765625; }

struct Slots {
    double* mins;   // [0] starts at -1e300 (a negative sign to keep), [1] at +0.5 (smaller than every writer)
    int* maxi;
    bool* flags;    // 8 byte slots: writers set the even ones only, and only when asked
    bool* lone;     // a one-byte allocation every writer sets
    double* sum;    // value, residual
};

AETHER_DEVICEANDHOST() void write(const Slots& s, int w) {
    at::minAbsReal(&s.mins[0], (w & 1) ? magnitudeOf(w) : -magnitudeOf(w));
    at::minAbsReal(&s.mins[1], magnitudeOf(w));
    at::maxInt(&s.maxi[0], intOf(w));
    at::orBool(&s.flags[2 * (w % 4)], true);
    at::orBool(&s.flags[1], false);   // false writers never set a slot
    at::orBool(s.lone, true);
    auto value = aether::make_view<double, aether::dyn>(s.sum, aether::Device(aether::kDLCPU), 1);
    auto comp = aether::make_view<double, aether::dyn>(s.sum + 1, aether::Device(aether::kDLCPU), 1);
    at::compensatedSum(value, comp, aether::SampleIndex::make(std::size_t(0)), termOf(w));
}

void check(const char* where, const double* mins, int maxi, const bool* flags, bool lone, const double* sum) {
    CHECK(mins[0] == -1.0);   // the smallest magnitude, the stored sign kept
    CHECK(mins[1] == 0.5);    // never replaced by a larger magnitude
    int want = -1000000;
    for (int w = 0; w < kWriters; ++w) want = intOf(w) > want ? intOf(w) : want;
    CHECK(maxi == want);
    for (int k = 0; k < 8; ++k) CHECK(flags[k] == (k % 2 == 0));
    CHECK(lone);
    long double exact = 0.0L;
    for (int w = 0; w < kWriters; ++w) exact += termOf(w);
    CHECK((long double)sum[0] + (long double)sum[1] == exact);
    if (failures) std::printf("%s failed\n", where);
}

void hostThreads() {
    double mins[2] = {-1e300, 0.5};
    int maxi = -1000000;
    bool flags[8] = {};
    bool* lone = new bool(false);
    double sum[2] = {0.0, 0.0};
    const Slots s{mins, &maxi, flags, lone, sum};
    std::vector<std::thread> th;
    for (int t = 0; t < 8; ++t)
        th.emplace_back([&, t] {
            for (int w = t; w < kWriters; w += 8) write(s, w);
        });
    for (auto& x : th) x.join();
    check("host", mins, maxi, flags, *lone, sum);
    delete lone;
}

}  // namespace

#if defined(__CUDACC__)
namespace {

AETHER_KERNEL() void writers(Slots s) {
    const int w = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (w < kWriters) write(s, w);
}

void deviceKernel() {
    double* mins = nullptr;
    int* maxi = nullptr;
    bool *flags = nullptr, *lone = nullptr;
    double* sum = nullptr;
    AETHER_CHECK_CUDA(cudaMalloc(&mins, 2 * sizeof(double)));
    AETHER_CHECK_CUDA(cudaMalloc(&maxi, sizeof(int)));
    AETHER_CHECK_CUDA(cudaMalloc(&flags, 8));
    AETHER_CHECK_CUDA(cudaMalloc(&lone, 1));   // a one-byte allocation
    AETHER_CHECK_CUDA(cudaMalloc(&sum, 2 * sizeof(double)));
    const double m0[2] = {-1e300, 0.5};
    const int i0 = -1000000;
    const bool f0[8] = {};
    const bool l0 = false;
    const double s0[2] = {0.0, 0.0};
    AETHER_CHECK_CUDA(cudaMemcpy(mins, m0, sizeof m0, cudaMemcpyHostToDevice));
    AETHER_CHECK_CUDA(cudaMemcpy(maxi, &i0, sizeof i0, cudaMemcpyHostToDevice));
    AETHER_CHECK_CUDA(cudaMemcpy(flags, f0, sizeof f0, cudaMemcpyHostToDevice));
    AETHER_CHECK_CUDA(cudaMemcpy(lone, &l0, 1, cudaMemcpyHostToDevice));
    AETHER_CHECK_CUDA(cudaMemcpy(sum, s0, sizeof s0, cudaMemcpyHostToDevice));
    writers<<<kWriters / 256, 256>>>(Slots{mins, maxi, flags, lone, sum});
    aether::cuda::checkLastLaunch("writers");
    double hm[2], hs[2];
    int hi = 0;
    bool hf[8], hl = false;
    AETHER_CHECK_CUDA(cudaMemcpy(hm, mins, sizeof hm, cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(&hi, maxi, sizeof hi, cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(hf, flags, sizeof hf, cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(&hl, lone, 1, cudaMemcpyDeviceToHost));
    AETHER_CHECK_CUDA(cudaMemcpy(hs, sum, sizeof hs, cudaMemcpyDeviceToHost));
    check("device", hm, hi, hf, hl, hs);
    for (void* p : {(void*)mins, (void*)maxi, (void*)flags, (void*)lone, (void*)sum}) AETHER_CHECK_CUDA(cudaFree(p));
}

}  // namespace
#endif

int main() {
    hostThreads();
#if defined(__CUDACC__)
    deviceKernel();
#endif
    if (failures) return 1;
    std::printf("atomic ok\n");
    return 0;
}
