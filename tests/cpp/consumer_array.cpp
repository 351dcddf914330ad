// The Array surface beyond construction (array/Array.h:82-364), on a device:
// push_back of Items on the host, growth through reserve/resize with the
// 32-sample capacity rule kept and every plane's filled samples carried over
// (host and device copies), commit of samples written into the spare tail,
// packed (layout_right) views only for an exactly full array, and a
// whole-view engine assignment on the grown array. Prints "array ok".
#include <aether/aether.h>

#include <cstdio>

#define CHECK(c)                                                  \
    do {                                                          \
        if (!(c)) {                                               \
            std::printf("check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                             \
        }                                                         \
    } while (0)

int main() {
    using aether::Array;
    Array<double, 3> v(0);
    CHECK(v.samples() == 0 && v.capacity() == 0);
    for (int k = 0; k < 40; ++k) v.push_back(aether::Vec3d{double(k), 2.0 * k, -1.0 * k});
    CHECK(v.samples() == 40 && v.capacity() == 64);   // 0 -> 32 -> 64
    {
        auto h = v.hostView();
        for (int k = 0; k < 40; ++k) CHECK(h(0, k) == k && h(1, k) == 2.0 * k && h(2, k) == -1.0 * k);
    }
    v.upload();
    v.reserve(100);   // device copy must survive the reallocation
    CHECK(v.capacity() == 128 && v.samples() == 40);
    {
        auto h = v.hostView();
        for (int k = 0; k < 40; ++k) h(0, k) = h(1, k) = h(2, k) = -7.0;   // clobber the host copy
    }
    v.download();
    {
        auto h = v.hostView();
        for (int k = 0; k < 40; ++k) CHECK(h(0, k) == k && h(1, k) == 2.0 * k && h(2, k) == -1.0 * k);
    }
    // write into the spare tail, then commit it
    {
        auto s = v.hostSpare();
        CHECK(s.samples() == 88);
        for (int k = 0; k < 5; ++k) s(0, k) = s(1, k) = s(2, k) = 100.0 + k;
    }
    v.commit(5);
    CHECK(v.samples() == 45);
    bool threw = false;
    try {
        v.commit(1000);
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        (void)v.devicePacked();   // capacity 128 != samples 45
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    v.upload();
    // an engine assignment over the grown array: w = 2 v + 1
    Array<double, 3> w(45);
    w.deviceView() = v.deviceView() * 2.0 + 1.0;
    w.download();
    {
        auto h = w.hostView();
        auto s = v.hostView();
        for (int k = 0; k < 45; ++k)
            for (int c = 0; c < 3; ++c) CHECK(h(c, k) == 2.0 * s(c, k) + 1.0);
    }
    // exactly full: packed views exist and address the same planes
    Array<double, 3> full(64);
    CHECK(full.capacity() == 64);
    auto p = full.hostPacked();
    auto st = full.hostView();
    CHECK(&p(1, 5) == &st(1, 5) && &p(2, 63) == &st(2, 63));
    full.resize(10);
    CHECK(full.samples() == 10 && full.capacity() == 64);
    full.clear();
    CHECK(full.samples() == 0);
    std::printf("array ok\n");
    return 0;
}
