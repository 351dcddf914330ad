// aether::accum::run (aether/accum_run.h), the cases of the reference's
// tests/test_Run.cpp: every form adds N = 4133 lane terms into keyed slots
// and must deliver the exact sums (dyadic terms: any order sums them
// exactly), with the number of atomic commits each form promises -- one per
// aligned run, per uniform warp, per sorted run, per full block -- and lane
// by lane for a warp that fails its vote or is not full (the ragged tail).
// The compensated forms must keep, in target + comp, what a plain commit
// rounds away.
//
// A host compiler runs the host path (one Open run per form over the lanes
// in order); nvcc -x cu runs it and then the device kernels.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#if defined(__CUDACC__)
__device__ unsigned long long d_commits[2];
#endif
unsigned long long h_commits[2];
#if defined(__CUDA_ARCH__)
#define AETHER_RUN_COMMIT_HOOK(isRun) atomicAdd(&d_commits[(isRun) ? 0 : 1], 1ull)
#else
#define AETHER_RUN_COMMIT_HOOK(isRun) (++h_commits[(isRun) ? 0 : 1])
#endif

#include <aether/aether.h>
#include <aether/accum_run.h>

namespace {

constexpr int kN = 4133;   // 129 full warps and a tail of 5 lanes
namespace ar = aether::accum::run;

enum Form { kAligned8, kTested32, kTested16, kSorted5, kComp32, kTestedComp, kSortedComp, kBlock, kPlain32, kForms };

AETHER_DEVICEANDHOST() long long keyOf(int form, long long i) {
    switch (form) {
    case kAligned8: return i / 8;
    case kTested32: return i / 32;
    case kTested16: return i / 16;   // two keys per warp: the vote fails
    case kSorted5:
    case kSortedComp: return i / 5;
    case kBlock: return i / 1024;
    default: return i / 64;          // two warps per slot
    }
}
// Dyadic terms; for the compensated forms even warps add 2^47 per lane (a
// warp sums to 2^52) and odd warps small eighths of eighths, so a plain
// commit into a slot that holds 2^52 rounds the small part away.
AETHER_DEVICEANDHOST() double termOf(int form, long long i) {
    if (form == kComp32 || form == kPlain32 || form == kTestedComp)
        return ((i >> 5) & 1) ? double(1 + i % 7) * 0.00390625 : 140737488355328.0;
    return double(1 + (i * 7919) % 97) * 0.015625;
}

template <class V>
AETHER_DEVICEANDHOST() void addOne(int form, V& target, V& comp, long long i, ar::Open<double>& r, bool full) {
    const aether::SampleIndex own = aether::SampleIndex::make(std::size_t(i));
    const aether::SampleIndex at = aether::SampleIndex::make(std::size_t(keyOf(form, i)));
    const double t = termOf(form, i);
    switch (form) {
    case kAligned8: ar::add<8>(target, at, t, own, r); break;
    case kTested32:
    case kTested16: ar::addTested(target, at, t, r); break;
    case kSorted5: ar::addSorted(target, at, t, r); break;
    case kComp32: ar::addCompensated<32>(target, comp, at, t, own, r); break;
    case kTestedComp: ar::addTestedCompensated(target, comp, at, t, r); break;
    case kSortedComp: ar::addSortedCompensated(target, comp, at, t, r); break;
    case kBlock: ar::addCompensatedBlock(target, comp, at, t, own, full, r); break;
    default: ar::add<32>(target, at, t, own, r); break;
    }
}

constexpr int kSlots = kN / 5 + 1;

#if defined(__CUDACC__)
AETHER_KERNEL() void runKernel(int form, double* tgt, double* cmp) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kN) return;
    auto target = aether::make_view<double, aether::dyn>(tgt, aether::Device(aether::kDLCUDA), kSlots);
    auto comp = aether::make_view<double, aether::dyn>(cmp, aether::Device(aether::kDLCUDA), kSlots);
    ar::Open<double> r = ar::open(target);
    addOne(form, target, comp, i, r, ar::blockFull(0, kN));
}
#endif

int failures = 0;
#define CHECK(c)                                                                    \
    do {                                                                            \
        if (!(c)) {                                                                 \
            std::printf("FAIL form %d line %d: %s\n", form, __LINE__, #c);           \
            ++failures;                                                             \
        }                                                                           \
    } while (0)

// The exact slot sums, in long double (every partial sum here fits its 64 bits).
std::vector<long double> exactSums(int form) {
    std::vector<long double> s(kSlots, 0.0L);
    for (long long i = 0; i < kN; ++i) s[keyOf(form, i)] += termOf(form, i);
    return s;
}

void checkSums(int form, const std::vector<double>& tgt, const std::vector<double>& cmp, const char* where) {
    const std::vector<long double> ex = exactSums(form);
    const bool compensated = form == kComp32 || form == kTestedComp || form == kSortedComp || form == kBlock;
    for (int k = 0; k < kSlots; ++k) {
        if (compensated) {
            if ((long double)tgt[k] + (long double)cmp[k] != ex[k]) {
                std::printf("%s form %d slot %d: %.21Lg + %.21Lg vs %.21Lg\n", where, form, k, (long double)tgt[k],
                            (long double)cmp[k], ex[k]);
                ++failures;
                return;
            }
        } else if (form == kPlain32) {
            // two plain commits per slot: the second rounds once, within an ulp
            const double d = std::fabs(double(ex[k]));
            const long double ulp = (long double)(std::nextafter(d, 2.0 * d + 1.0) - d);
            if (std::fabs(double((long double)tgt[k] - ex[k])) > double(ulp)) {
                std::printf("%s form %d slot %d off by more than an ulp\n", where, form, k);
                ++failures;
                return;
            }
        } else if ((long double)tgt[k] != ex[k]) {
            std::printf("%s form %d slot %d: %.17g vs %.17Lg\n", where, form, k, tgt[k], ex[k]);
            ++failures;
            return;
        }
    }
}

#if defined(__CUDACC__)
// Commits each form promises on the device for kN lanes in blocks of `block`.
void expectedDeviceCommits(int form, int block, unsigned long long& runs, unsigned long long& lanes) {
    const long long fullWarps = kN / 32, tail = kN % 32;
    runs = 0;
    lanes = 0;
    switch (form) {
    case kAligned8: runs = fullWarps * 4; lanes = tail; break;
    case kTested32:
    case kTestedComp: runs = fullWarps; lanes = tail; break;
    case kTested16: lanes = kN; break;
    case kSorted5:
    case kSortedComp:
        for (long long w = 0; w < fullWarps; ++w)
            for (long long l = 0; l < 32; ++l) runs += (l == 0 || keyOf(form, 32 * w + l) != keyOf(form, 32 * w + l - 1));
        lanes = tail;
        break;
    case kBlock: {
        const long long fullBlocks = kN / block;
        runs = fullBlocks + (kN - fullBlocks * block) / 32;
        lanes = tail;
        break;
    }
    default: runs = fullWarps; lanes = tail; break;
    }
}
#endif

void hostPath() {
    for (int form = 0; form < kForms; ++form) {
        std::vector<double> tgt(kSlots, 0.0), cmp(kSlots, 0.0);
        auto target = aether::make_view<double, aether::dyn>(tgt.data(), aether::Device(aether::kDLCPU), kSlots);
        auto comp = aether::make_view<double, aether::dyn>(cmp.data(), aether::Device(aether::kDLCPU), kSlots);
        h_commits[0] = h_commits[1] = 0;
        ar::Open<double> r = ar::open(target);
        for (long long i = 0; i < kN; ++i) addOne(form, target, comp, i, r, ar::blockFull(0, kN));
        ar::close(r);
        checkSums(form, tgt, cmp, "host");
        // one commit per change of slot along the lanes, all of them runs
        long long changes = 1;
        for (long long i = 1; i < kN; ++i) changes += keyOf(form, i) != keyOf(form, i - 1);
        CHECK(h_commits[0] == (unsigned long long)changes && h_commits[1] == 0);
    }
}

}  // namespace

int main() {
    hostPath();
#if defined(__CUDACC__)
    double *tgt = nullptr, *cmp = nullptr;
    AETHER_CHECK_CUDA(cudaMalloc(&tgt, kSlots * sizeof(double)));
    AETHER_CHECK_CUDA(cudaMalloc(&cmp, kSlots * sizeof(double)));
    for (int form = 0; form < kForms; ++form) {
        const int block = form == kBlock ? 256 : 128;
        AETHER_CHECK_CUDA(cudaMemset(tgt, 0, kSlots * sizeof(double)));
        AETHER_CHECK_CUDA(cudaMemset(cmp, 0, kSlots * sizeof(double)));
        const unsigned long long zero[2] = {0, 0};
        AETHER_CHECK_CUDA(cudaMemcpyToSymbol(d_commits, zero, sizeof zero));
        runKernel<<<(kN + block - 1) / block, block>>>(form, tgt, cmp);
        aether::cuda::checkLastLaunch("runKernel");
        std::vector<double> ht(kSlots), hc(kSlots);
        unsigned long long got[2];
        AETHER_CHECK_CUDA(cudaMemcpy(ht.data(), tgt, kSlots * sizeof(double), cudaMemcpyDeviceToHost));
        AETHER_CHECK_CUDA(cudaMemcpy(hc.data(), cmp, kSlots * sizeof(double), cudaMemcpyDeviceToHost));
        AETHER_CHECK_CUDA(cudaMemcpyFromSymbol(got, d_commits, sizeof got));
        checkSums(form, ht, hc, "device");
        unsigned long long runs, lanes;
        expectedDeviceCommits(form, block, runs, lanes);
        if (got[0] != runs || got[1] != lanes)
            std::printf("form %d: %llu run and %llu lane commits, expected %llu and %llu\n", form, got[0], got[1], runs,
                        lanes);
        CHECK(got[0] == runs && got[1] == lanes);
        if (form == kPlain32) {
            // the plain commit loses the small part that the compensated one keeps
            const std::vector<long double> ex = exactSums(form);
            bool lost = false;
            for (int k = 0; k < kSlots; ++k) lost |= (long double)ht[k] != ex[k];
            CHECK(lost);
        }
    }
    AETHER_CHECK_CUDA(cudaFree(tgt));
    AETHER_CHECK_CUDA(cudaFree(cmp));
#endif
    if (failures) return 1;
    std::printf("accum run ok\n");
    return 0;
}
