// aether/accum_run.h -- keyed accumulation with one atomic per run of lanes
// that share a slot (accum/run.h), for consumer kernels and host loops.
//
// aether::accum::run::add*(target, at, term, ..., open) adds `term` into
// target(at.global()). On the device, lanes of a warp that add into the same
// slot are summed with shuffles first and one lane commits the run's sum in a
// single atomic; which lanes form a run comes from what the caller knows:
//
//   add<W>     the caller proves the slot is equal over every aligned group of
//              W lanes (W a power of two, 2..32); one vote checks that the
//              warp is full and holds 32 consecutive samples starting on a
//              multiple of 32 (`own` is the lane's own sample index);
//   addTested  no proof: one vote checks that all 32 lanes share one slot;
//   addSorted  slots are non-decreasing in lane order; each maximal run of
//              equal slots is found from head flags (keys out of order only
//              shorten the runs).
//
// A warp that fails its vote, or is not full, commits lane by lane, so every
// form is correct for any key and the facts only make it fast. The
// *Compensated forms keep the plain run sum and make its one commit
// compensated: the sum goes into `target` and the exact two-sum residual of
// that atomic addition into `comp` (delivered value = target + comp).
// addCompensatedBlock folds a whole block's warps through shared memory into
// one commit when the caller proves the block shares a key (blockFull).
//
// On the host every form adds into an Open run the caller holds (open()),
// with a Neumaier step in lane order, and commits it when the slot changes
// and at close(); the device ignores it.
//
// Summation order is the ULP contract's, not a bit-identity across shapes:
// aligned and tested runs use an xor butterfly (offsets W/2 .. 1), sorted
// runs a segmented shuffle-down tree (offsets 1, 2, .., 16, the lower lane
// on the left). AETHER_RUN_COMMIT_HOOK(isRun) is invoked once per atomic
// commit (isRun: a run's commit rather than a lane's own); it does nothing
// unless defined before this header, which a test does to count commits.
#pragma once

#include <cstdint>
#include <cstring>
#include <type_traits>
#include <utility>

#include "aether/layout.h"

#ifndef AETHER_RUN_COMMIT_HOOK
#define AETHER_RUN_COMMIT_HOOK(isRun) ((void)(isRun))
#endif

namespace aether {
namespace accum {
namespace run {

/** The host's open run: the slot being summed, its compensation slot (null
 *  for a plain run) and the partial (s, c). Unused on the device. */
template <class E>
struct Open {
    E* slot = nullptr;
    E* comp = nullptr;
    E s = E(0);
    E c = E(0);
};

namespace detail {

template <class ViewT>
using slot_t = std::remove_cv_t<std::remove_reference_t<decltype(std::declval<ViewT&>()(std::size_t(0)))>>;

/** One atomic addition; the value it replaced. */
template <class E>
AETHER_DEVICEANDHOST() inline E atomic_add(E* slot, E t) {
#if defined(__CUDA_ARCH__)
    return atomicAdd(slot, t);
#else
    // a compare-exchange on the value's bits (C++17 has no atomic_ref)
    using Bits = std::conditional_t<sizeof(E) == 4, uint32_t, uint64_t>;
    static_assert(sizeof(E) == sizeof(Bits), "a 4- or 8-byte element");
    Bits* bits = reinterpret_cast<Bits*>(slot);
    Bits seen = __atomic_load_n(bits, __ATOMIC_RELAXED);
    for (;;) {
        E cur, next;
        std::memcpy(&cur, &seen, sizeof cur);
        next = cur + t;
        Bits want;
        std::memcpy(&want, &next, sizeof want);
        if (__atomic_compare_exchange_n(bits, &seen, want, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return cur;
    }
#endif
}

/** Knuth's two-sum residual: a + b - s exactly, for s = fl(a + b). Additions
 *  only, so contraction cannot change it. */
template <class E>
AETHER_DEVICEANDHOST() inline E two_sum_residual(E a, E b, E s) {
    const E bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

template <class E>
AETHER_DEVICEANDHOST() inline void commit(E* slot, E s, bool isRun) {
    atomic_add(slot, s);
    AETHER_RUN_COMMIT_HOOK(isRun);
}
/** One atomic addition of s into slot; its exact residual plus c into comp. */
template <class E>
AETHER_DEVICEANDHOST() inline void commit_compensated(E* slot, E* comp, E s, E c, bool isRun) {
    const E old = atomic_add(slot, s);
    atomic_add(comp, two_sum_residual(old, s, old + s) + c);
    AETHER_RUN_COMMIT_HOOK(isRun);
}

#if !defined(__CUDA_ARCH__)
template <class E>
inline void flush(Open<E>& r) {
    if (!r.slot) return;
    if (r.comp)
        commit_compensated(r.slot, r.comp, r.s, r.c, true);
    else
        commit(r.slot, r.s + r.c, true);
}
/** Add t into the open run on `slot` (Neumaier), committing the run it
 *  replaces first. */
template <class E>
inline void open_add(Open<E>& r, E* slot, E* comp, E t) {
    if (slot != r.slot) {
        flush(r);
        r = Open<E>{slot, comp, t, E(0)};
        return;
    }
    const E s = r.s + t;
    const E e = two_sum_residual(r.s, t, s);
    r.s = s;
    r.c = (s - s == E(0)) ? r.c + e : E(0);   // a non-finite sum drops the correction
}
#endif

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned lane_id() {
    unsigned l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}
// A full warp of 32 consecutive samples starting on a multiple of 32.
template <class I>
__device__ __forceinline__ bool warp_aligned(unsigned mask, const I& own) {
    return mask == 0xffffffffu && __all_sync(mask, (unsigned(own.global()) & 31u) == lane_id());
}
// A full warp whose 32 keys are all lane 0's.
__device__ __forceinline__ bool warp_uniform(unsigned mask, unsigned long long key) {
    return mask == 0xffffffffu && __all_sync(mask, key == __shfl_sync(mask, key, 0));
}
template <int W, class E>
__device__ __forceinline__ E butterfly(E t) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}
// Bit l set where lane l starts a run: lane 0, or a key unlike the lane below.
__device__ __forceinline__ unsigned run_heads(unsigned long long key, unsigned lane) {
    const unsigned long long below = __shfl_up_sync(0xffffffffu, key, 1);
    return __ballot_sync(0xffffffffu, lane == 0u || key != below);
}
// Each run's head receives the sum of its run: a shuffle-down tree that adds
// a partner only from inside the same run.
template <class E>
__device__ __forceinline__ E segmented_sum(E t, unsigned heads, unsigned lane) {
    if (heads == 0xffffffffu) return t;
    const unsigned after = lane == 31u ? 0u : heads >> (lane + 1u);
    const unsigned end = after ? lane + unsigned(__ffs(int(after))) : 32u;   // first lane of the next run
#pragma unroll
    for (unsigned o = 1; o < 32u; o <<= 1) {
        const E v = __shfl_down_sync(0xffffffffu, t, o);
        if (lane + o < end) t += v;
    }
    return t;
}
#endif

}  // namespace detail

/** A closed host run for `target`'s element type. */
template <class ViewT>
AETHER_DEVICEANDHOST() inline Open<detail::slot_t<ViewT>> open(const ViewT&) {
    return {};
}

/** Commit the host's open run at the end of the caller's range; nothing on
 *  the device. */
template <class E>
AETHER_DEVICEANDHOST() inline void close(Open<E>& r) {
#if !defined(__CUDA_ARCH__)
    detail::flush(r);
    r = Open<E>{};
#else
    (void)r;
#endif
}

/** Add `term` into target(at.global()), one atomic per aligned run of W
 *  lanes (the caller's fact: the slot is equal over each such group). */
template <int W, class ViewT, class T, class I, class E>
AETHER_DEVICEANDHOST() inline void add(ViewT& target, const SampleIndex& at, T term, const I& own, Open<E>& r) {
    static_assert(W >= 2 && W <= 32 && (W & (W - 1)) == 0, "a run is 2..32 lanes, a power of two");
    E* slot = &target(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (detail::warp_aligned(__activemask(), own)) {
        const E s = detail::butterfly<W>(E(term));
        if ((detail::lane_id() & unsigned(W - 1)) == 0u) detail::commit(slot, s, true);
        return;
    }
    detail::commit(slot, E(term), false);
#else
    (void)own;
    detail::open_add(r, slot, static_cast<E*>(nullptr), E(term));
#endif
}

/** As add<32> without a proof: one vote decides. */
template <class ViewT, class T, class E>
AETHER_DEVICEANDHOST() inline void addTested(ViewT& target, const SampleIndex& at, T term, Open<E>& r) {
    E* slot = &target(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (detail::warp_uniform(__activemask(), static_cast<unsigned long long>(at.global()))) {
        const E s = detail::butterfly<32>(E(term));
        if (detail::lane_id() == 0u) detail::commit(slot, s, true);
        return;
    }
    detail::commit(slot, E(term), false);
#else
    detail::open_add(r, slot, static_cast<E*>(nullptr), E(term));
#endif
}

/** Keys non-decreasing in lane order: one atomic per maximal run. */
template <class ViewT, class T, class E>
AETHER_DEVICEANDHOST() inline void addSorted(ViewT& target, const SampleIndex& at, T term, Open<E>& r) {
    E* slot = &target(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (__activemask() == 0xffffffffu) {
        const unsigned lane = detail::lane_id();
        const unsigned heads = detail::run_heads(static_cast<unsigned long long>(at.global()), lane);
        const E s = detail::segmented_sum(E(term), heads, lane);
        if ((heads >> lane) & 1u) detail::commit(slot, s, true);
        return;
    }
    detail::commit(slot, E(term), false);
#else
    detail::open_add(r, slot, static_cast<E*>(nullptr), E(term));
#endif
}

/** Compensated add<W>: the plain run sum, one compensated commit. */
template <int W, class ViewT, class T, class I, class E>
AETHER_DEVICEANDHOST() inline void addCompensated(ViewT& target, ViewT& comp, const SampleIndex& at, T term,
                                                  const I& own, Open<E>& r) {
    static_assert(W >= 2 && W <= 32 && (W & (W - 1)) == 0, "a run is 2..32 lanes, a power of two");
    E* slot = &target(at.global());
    E* cslot = &comp(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (detail::warp_aligned(__activemask(), own)) {
        const E s = detail::butterfly<W>(E(term));
        if ((detail::lane_id() & unsigned(W - 1)) == 0u) detail::commit_compensated(slot, cslot, s, E(0), true);
        return;
    }
    detail::commit_compensated(slot, cslot, E(term), E(0), false);
#else
    (void)own;
    detail::open_add(r, slot, cslot, E(term));
#endif
}

/** Compensated addTested. */
template <class ViewT, class T, class E>
AETHER_DEVICEANDHOST() inline void addTestedCompensated(ViewT& target, ViewT& comp, const SampleIndex& at, T term,
                                                        Open<E>& r) {
    E* slot = &target(at.global());
    E* cslot = &comp(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (detail::warp_uniform(__activemask(), static_cast<unsigned long long>(at.global()))) {
        const E s = detail::butterfly<32>(E(term));
        if (detail::lane_id() == 0u) detail::commit_compensated(slot, cslot, s, E(0), true);
        return;
    }
    detail::commit_compensated(slot, cslot, E(term), E(0), false);
#else
    detail::open_add(r, slot, cslot, E(term));
#endif
}

/** Compensated addSorted. */
template <class ViewT, class T, class E>
AETHER_DEVICEANDHOST() inline void addSortedCompensated(ViewT& target, ViewT& comp, const SampleIndex& at, T term,
                                                        Open<E>& r) {
    E* slot = &target(at.global());
    E* cslot = &comp(at.global());
#if defined(__CUDA_ARCH__)
    (void)r;
    if (__activemask() == 0xffffffffu) {
        const unsigned lane = detail::lane_id();
        const unsigned heads = detail::run_heads(static_cast<unsigned long long>(at.global()), lane);
        const E s = detail::segmented_sum(E(term), heads, lane);
        if ((heads >> lane) & 1u) detail::commit_compensated(slot, cslot, s, E(0), true);
        return;
    }
    detail::commit_compensated(slot, cslot, E(term), E(0), false);
#else
    detail::open_add(r, slot, cslot, E(term));
#endif
}

/** True for a block whose every thread is live and whose samples
 *  [base + blockIdx.x * blockDim.x, + blockDim.x) the caller has proven to
 *  share one key (the key moves in runs of 1024 aligned samples and
 *  blockDim.x divides 1024). Block-uniform; false on the host. */
AETHER_DEVICEANDHOST() inline bool blockFull(long long base, long long count) {
#if defined(__CUDA_ARCH__)
    const long long b = blockDim.x;
    return (1024 % b == 0) && (base % b == 0) && ((static_cast<long long>(blockIdx.x) + 1) * b <= count);
#else
    (void)base;
    (void)count;
    return false;
#endif
}

/** addCompensated<32> for a key uniform over the block: when `full`
 *  (blockFull), the warps' sums fold through shared memory in a fixed tree
 *  and ONE compensated commit is made per block. Every thread of the block
 *  must reach the call (two barriers); a block that is not full takes
 *  addCompensated<32>. */
template <class ViewT, class T, class I, class E>
AETHER_DEVICEANDHOST() inline void addCompensatedBlock(ViewT& target, ViewT& comp, const SampleIndex& at, T term,
                                                       const I& own, bool full, Open<E>& r) {
#if defined(__CUDA_ARCH__)
    if (full) {
        __shared__ E part[32];
        const unsigned lane = detail::lane_id(), warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
        const E s = detail::butterfly<32>(E(term));
        if (lane == 0u) part[warp] = s;
        __syncthreads();
        if (warp == 0u) {
            const E v = detail::butterfly<32>(lane < warps ? part[lane] : E(0));
            if (lane == 0u) detail::commit_compensated(&target(at.global()), &comp(at.global()), v, E(0), true);
        }
        __syncthreads();
        return;
    }
#else
    (void)full;
#endif
    addCompensated<32>(target, comp, at, term, own, r);
}

}  // namespace run
}  // namespace accum
}  // namespace aether
