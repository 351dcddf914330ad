// aether/device_flag.h -- the device half of the error contract.
//
// DeviceFlag (err/DeviceFlag.h:49-160): a sticky 32-bit word that device code
// sets with atomicOr and the host reads back, clears, or turns into a thrown
// aether::Error (checkAndClear). The word lives in device memory with a
// pinned host copy, both allocated through the C-ABI. DeviceFlagView is what
// a kernel takes by value; its set() is device code when compiled by nvcc and
// a relaxed atomic store on the host.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>

#include "aether/array.h"

#ifdef __CUDACC__
#define AETHER_GB300_HD __host__ __device__
#else
#define AETHER_GB300_HD
#endif

namespace aether {

class DeviceFlagView {
public:
    DeviceFlagView() = default;
    AETHER_GB300_HD explicit DeviceFlagView(std::uint32_t* p) : ptr_(p) {}
    AETHER_GB300_HD void set() const {
#ifdef __CUDA_ARCH__
        atomicOr(ptr_, 1u);
#else
        reinterpret_cast<std::atomic<std::uint32_t>*>(ptr_)->store(1u, std::memory_order_relaxed);
#endif
    }
    AETHER_GB300_HD std::uint32_t* data() const { return ptr_; }

private:
    std::uint32_t* ptr_ = nullptr;
};

class DeviceFlag {
public:
    DeviceFlag()
        : host_(AETHER_MEM_PINNED, sizeof(std::uint32_t), "host (pinned)"),
          dev_(AETHER_MEM_DEVICE, sizeof(std::uint32_t), "device 0") {
        clear();
    }
    DeviceFlagView deviceView() const { return DeviceFlagView(static_cast<std::uint32_t*>(dev_.get())); }
    /** Non-destructive read (downloads the device word). */
    bool isSet() const {
        detail::copy(host_.get(), AETHER_MEM_PINNED, dev_.get(), AETHER_MEM_DEVICE, sizeof(std::uint32_t), nullptr,
                     "DeviceFlag::isSet");
        detail::sync(nullptr);
        std::uint32_t v = 0;
        std::memcpy(&v, host_.get(), sizeof v);
        return v != 0;
    }
    void clear() {
        const std::uint32_t zero = 0;
        std::memcpy(host_.get(), &zero, sizeof zero);
        detail::copy(dev_.get(), AETHER_MEM_DEVICE, host_.get(), AETHER_MEM_PINNED, sizeof zero, nullptr,
                     "DeviceFlag::clear");
        detail::sync(nullptr);
    }
    /** Throws aether::Error naming `what` if the flag was set; clears it either way. */
    void checkAndClear(const std::string& what) {
        const bool was = isSet();
        clear();
        if (was) throw Error(what + ": device flag set");
    }

private:
    detail::Chunk host_, dev_;
};

}  // namespace aether
