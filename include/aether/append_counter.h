// aether/append_counter.h -- device-side appends into an Array's spare
// capacity (accum/AppendCounter.h).
//
// aether::accum::AppendCounter hands out slots in the reserved tail of an
// Array (its deviceSpare() view): a kernel takes the counter's view by value
// and calls tryAppend(), which returns the next free slot, or accum::npos
// when the declared capacity is used up -- then the counter's DeviceFlag is
// set and no slot at or past the capacity is ever returned. On the host,
// commit(array) reads the count back, clamps it to the capacity, adopts that
// many samples with array.commit(n) and resets the counter for the next
// step; checkOverflow() then turns a set flag into an aether::Error, so an
// overflow does not throw away the samples that did fit.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>

#include "aether/array.h"
#include "aether/device_flag.h"

namespace aether {
namespace accum {

/** The "no slot" value tryAppend() returns on overflow. */
inline constexpr offset_t npos = offset_t(~offset_t(0));

/** What a kernel takes by value: the counter word, the capacity and the
 *  overflow flag. */
class AppendCounterView {
public:
    AppendCounterView() = default;
    AETHER_GB300_HD AppendCounterView(std::uint32_t* counter, std::size_t capacity, DeviceFlagView overflow)
        : counter_(counter), capacity_(capacity), overflow_(overflow) {}

    /** The next slot (< capacity), or npos with the overflow flag set. The
     *  counter itself may climb past the capacity; no slot beyond it is
     *  returned. */
    AETHER_GB300_HD offset_t tryAppend() const {
#if defined(__CUDA_ARCH__)
        const std::uint32_t slot = atomicAdd(counter_, 1u);
#else
        const std::uint32_t slot =
            reinterpret_cast<std::atomic<std::uint32_t>*>(counter_)->fetch_add(1u, std::memory_order_relaxed);
#endif
        if (std::size_t(slot) >= capacity_) {
            overflow_.set();
            return npos;
        }
        return offset_t(slot);
    }
    AETHER_GB300_HD std::size_t capacity() const { return capacity_; }

private:
    std::uint32_t* counter_ = nullptr;
    std::size_t capacity_ = 0;
    DeviceFlagView overflow_{};
};

/** An append counter over `capacity` slots: one 32-bit word on the device
 *  (with a page-locked host copy) and a DeviceFlag for overflow. */
class AppendCounter {
public:
    explicit AppendCounter(std::size_t capacity)
        : capacity_(capacity),
          host_(AETHER_MEM_PINNED, sizeof(std::uint32_t), "host (pinned)"),
          dev_(AETHER_MEM_DEVICE, sizeof(std::uint32_t), "device 0") {
        if (capacity >= std::size_t(npos))
            throw Error::memory("AppendCounter", "device 0", capacity, "capacity must stay below 2^32 - 1 slots");
        reset();
    }
    std::size_t capacity() const { return capacity_; }
    AppendCounterView deviceView() const {
        return AppendCounterView(static_cast<std::uint32_t*>(dev_.get()), capacity_, overflow_.deviceView());
    }
    /** The raw count (may exceed the capacity after an overflow). */
    std::size_t rawCount() const {
        detail::copy(host_.get(), AETHER_MEM_PINNED, dev_.get(), AETHER_MEM_DEVICE, sizeof(std::uint32_t), nullptr,
                     "AppendCounter::rawCount");
        detail::sync(nullptr);
        std::uint32_t v = 0;
        std::memcpy(&v, host_.get(), sizeof v);
        return v;
    }
    bool overflowed() const { return overflow_.isSet(); }
    /** Throws if the flag is set; clears it either way. */
    void checkOverflow(const std::string& context = "AppendCounter::checkOverflow") { overflow_.checkAndClear(context); }
    /** Zero the counter for a fresh step (the overflow flag is left alone). */
    void reset() {
        const std::uint32_t z = 0;
        std::memcpy(host_.get(), &z, sizeof z);
        detail::copy(dev_.get(), AETHER_MEM_DEVICE, host_.get(), AETHER_MEM_PINNED, sizeof z, nullptr,
                     "AppendCounter::reset");
        detail::sync(nullptr);
    }
    /** Adopt min(count, capacity) appended samples into `arr` and reset the
     *  counter; never throws for an overflow. The count committed. */
    template <class T, std::size_t... Es>
    std::size_t commit(Array<T, Es...>& arr) {
        const std::size_t n = std::min(rawCount(), capacity_);
        arr.commit(n);
        reset();
        return n;
    }

private:
    std::size_t capacity_;
    detail::Chunk host_, dev_;
    DeviceFlag overflow_;
};

}  // namespace accum
}  // namespace aether
