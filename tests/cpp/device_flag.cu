// The device half of DeviceFlag (include/aether/device_flag.h): a kernel sets
// the flag for the samples that fail a check, the host sees it, and
// checkAndClear throws once and leaves the flag clear.
#include <aether/aether.h>

#include <cstdio>

__global__ void flag_negative(const double* x, std::size_t n, aether::DeviceFlagView f) {
    const std::size_t i = blockIdx.x * std::size_t(blockDim.x) + threadIdx.x;
    if (i < n && x[i] < 0.0) f.set();
}

int main() {
    const std::size_t n = 1000;
    aether::Array<double> x(n);
    auto xv = x.deviceView();
    xv = aether::random::Generator(3).uniform<double, 1>(0.0, 1.0);
    aether::DeviceFlag flag;
    flag_negative<<<(n + 255) / 256, 256>>>(xv.data(), n, flag.deviceView());
    if (flag.isSet()) {
        std::printf("flag set on non-negative data\n");
        return 1;
    }
    xv = aether::random::Generator(3).uniform<double, 1>(-1.0, 1.0);
    flag_negative<<<(n + 255) / 256, 256>>>(xv.data(), n, flag.deviceView());
    if (!flag.isSet() || !flag.isSet()) {   // sticky: a read does not clear
        std::printf("flag not set\n");
        return 1;
    }
    bool threw = false;
    try {
        flag.checkAndClear("flag_negative");
    } catch (const aether::Error& e) {
        threw = std::string(e.what()).find("flag_negative") != std::string::npos;
    }
    if (!threw || flag.isSet()) {
        std::printf("checkAndClear did not throw once and clear\n");
        return 1;
    }
    flag.checkAndClear("flag_negative");   // clear: no throw
    std::printf("device flag ok\n");
    return 0;
}
