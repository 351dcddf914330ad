// aether/accum_atomic.h -- the atomic slot updates of accum/atomic.h, for
// consumer kernels and host threads.
//
// aether::accum::atomic:
//   minAbsReal(h, i, v)   |h[i]| <- min(|h[i]|, |v|), keeping the sign already
//                         stored at the slot; returns the value it found;
//   orBool(h, i, v)       a monotone set-to-true of a one-byte bool slot: a
//                         byte store, so it never touches a neighbouring byte
//                         and stays inside a one-byte allocation (read the
//                         result after the kernel); false does nothing;
//   maxInt(h, i, v)       h[i] <- max(h[i], v) for a 32-bit int; returns the
//                         value it found;
//   compensatedSum(v, c, i, t)  v[i] += t in one atomic addition, its exact
//                         two-sum residual atomically into c[i]: v[i] + c[i]
//                         is the sum of the terms whatever their order.
// Each has a view form (slot i of a scalar view) and a raw-pointer form. On
// the device they are CUDA atomics (a compare-and-swap loop for the
// magnitude minimum); on the host, compare-and-swap loops on the slot's bits.
#pragma once

#include <cstdint>
#include <cstring>

#include "aether/layout.h"
#include "aether/math.h"

namespace aether {
namespace accum {
namespace atomic {
namespace detail {

#if !defined(__CUDA_ARCH__)
// Host: replace the 8-byte word at p by f(current) while f says so.
template <class F>
inline double cas_double(double* p, F f) {
    auto* bits = reinterpret_cast<uint64_t*>(p);
    uint64_t seen = __atomic_load_n(bits, __ATOMIC_RELAXED);
    for (;;) {
        double cur;
        std::memcpy(&cur, &seen, sizeof cur);
        double next;
        if (!f(cur, next)) return cur;
        uint64_t want;
        std::memcpy(&want, &next, sizeof want);
        if (__atomic_compare_exchange_n(bits, &seen, want, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return cur;
    }
}
#endif

AETHER_DEVICEANDHOST() inline double min_abs_real(double* p, double v) {
    const double a = math::abs(v);
#if defined(__CUDA_ARCH__)
    auto* w = reinterpret_cast<unsigned long long*>(p);
    unsigned long long seen = *reinterpret_cast<volatile unsigned long long*>(w);
    for (;;) {
        const double cur = __longlong_as_double((long long)seen);
        if (!(a < math::abs(cur))) return cur;
        const unsigned long long want = (unsigned long long)__double_as_longlong(math::copysign(a, cur));
        const unsigned long long got = atomicCAS(w, seen, want);
        if (got == seen) return cur;
        seen = got;
    }
#else
    return cas_double(p, [a](double cur, double& next) {
        if (!(a < math::abs(cur))) return false;
        next = math::copysign(a, cur);
        return true;
    });
#endif
}

AETHER_DEVICEANDHOST() inline void or_bool(bool* p, bool v) {
    if (!v) return;
#if defined(__CUDA_ARCH__)
    *reinterpret_cast<volatile unsigned char*>(p) = 1;
#else
    __atomic_store_n(reinterpret_cast<unsigned char*>(p), static_cast<unsigned char>(1), __ATOMIC_RELAXED);
#endif
}

AETHER_DEVICEANDHOST() inline int max_int(int* p, int v) {
#if defined(__CUDA_ARCH__)
    return atomicMax(p, v);
#else
    int seen = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v > seen && !__atomic_compare_exchange_n(p, &seen, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
    return seen;
#endif
}

AETHER_DEVICEANDHOST() inline double add_double(double* p, double t) {
#if defined(__CUDA_ARCH__)
    return atomicAdd(p, t);
#else
    return cas_double(p, [t](double cur, double& next) {
        next = cur + t;
        return true;
    });
#endif
}

AETHER_DEVICEANDHOST() inline void compensated_sum(double* value, double* comp, double t) {
    const double old = add_double(value, t);
    const double s = old + t;   // the value the atomic stored
    const double bb = s - old;
    add_double(comp, (old - (s - bb)) + (t - bb));
}

}  // namespace detail

template <class ViewT>
AETHER_DEVICEANDHOST() inline double minAbsReal(ViewT& h, const SampleIndex& i, double v) {
    return detail::min_abs_real(&h(i.global()), v);
}
AETHER_DEVICEANDHOST() inline double minAbsReal(double* h, double v) { return detail::min_abs_real(h, v); }

template <class ViewT>
AETHER_DEVICEANDHOST() inline void orBool(ViewT& h, const SampleIndex& i, bool v) {
    detail::or_bool(&h(i.global()), v);
}
AETHER_DEVICEANDHOST() inline void orBool(bool* h, bool v) { detail::or_bool(h, v); }

template <class ViewT>
AETHER_DEVICEANDHOST() inline int maxInt(ViewT& h, const SampleIndex& i, int v) {
    return detail::max_int(&h(i.global()), v);
}
AETHER_DEVICEANDHOST() inline int maxInt(int* h, int v) { return detail::max_int(h, v); }

template <class ViewT>
AETHER_DEVICEANDHOST() inline void compensatedSum(ViewT& value, ViewT& comp, const SampleIndex& i, double t) {
    detail::compensated_sum(&value(i.global()), &comp(i.global()), t);
}

}  // namespace atomic
}  // namespace accum
}  // namespace aether
