// aether::interop's DLPack import and export (aether/dlpack.h), the cases of
// the reference's tests/test_DLPackRoundtrip.cu and
// tests/test_DLPackDtypes_common.h over hand-built producers whose deleters
// count their calls.
//
// Built as a host program (no engine, no device): `dlpack_interop` runs every
// check and prints "dlpack ok". Built as a shared library with
// -DDLPACK_WITH_ENGINE and linked to the engine, it exports dlpack_scale(),
// which imports a foreign producer's input and output tensors (any DLPack
// generation) and runs the engine's runtime-typed Scale on them.
#include <aether/aether.h>
#include <aether/dlpack.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#if !defined(DLPACK_WITH_ENGINE)
namespace {

int g_legacy = 0, g_versioned = 0;
void countLegacy(DLManagedTensor*) { ++g_legacy; }
void countVersioned(DLManagedTensorVersioned*) { ++g_versioned; }

int failures = 0;
#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                              \
        }                                                            \
    } while (0)

template <class M>
void fill(M& t, void* data, int ndim, int64_t* shape, int64_t* strides, DLDataType dt, DLDevice dev) {
    t.dl_tensor.data = data;
    t.dl_tensor.device = dev;
    t.dl_tensor.ndim = ndim;
    t.dl_tensor.dtype = dt;
    t.dl_tensor.shape = shape;
    t.dl_tensor.strides = strides;
    t.dl_tensor.byte_offset = 0;
}

constexpr DLDevice kCpu{kDLCPU, 0};
constexpr DLDataType kF64{kDLFloat, 64, 1};

void importLegacy() {
    std::vector<double> buf(3 * 8);
    int64_t shape[2] = {3, 8}, strides[2] = {8, 1};
    DLManagedTensor t{};
    fill(t, buf.data(), 2, shape, strides, kF64, kCpu);
    t.deleter = &countLegacy;
    g_legacy = 0;
    {
        auto imp = aether::interop::fromDLPack(&t);
        CHECK(imp.view.data == buf.data());   // zero copy
        CHECK(imp.view.rank == 2 && imp.view.extents[0] == 3 && imp.view.extents[1] == 8);
        CHECK(imp.view.strides[0] == 8 && imp.view.strides[1] == 1);
        CHECK(imp.view.dtype_code == kDLFloat && imp.view.dtype_bits == 64 && imp.view.dtype_lanes == 1);
        CHECK(imp.view.device == aether::Device(aether::kDLCPU));
        CHECK(imp.owner.owns());
        CHECK(g_legacy == 0);
        aether::interop::DLPackOwner moved = std::move(imp.owner);   // the owner moves, the deleter does not run
        CHECK(!imp.owner.owns() && moved.owns() && g_legacy == 0);
        moved.release();
        moved.release();   // idempotent
        CHECK(g_legacy == 1);
    }
    CHECK(g_legacy == 1);   // exactly once
}

void importVersioned() {
    std::vector<float> buf(4 * 5);
    int64_t shape[2] = {4, 5};
    DLManagedTensorVersioned t{};
    t.version = DLPackVersion{1, 0};
    fill(t, buf.data(), 2, shape, nullptr, DLDataType{kDLFloat, 32, 1}, DLDevice{kDLCUDA, 3});
    t.deleter = &countVersioned;
    g_versioned = 0;
    {
        auto imp = aether::interop::fromDLPack(&t);
        // null strides: compact row-major
        CHECK(imp.view.strides[0] == 5 && imp.view.strides[1] == 1);
        CHECK(imp.view.dtype_bits == 32);
        CHECK(imp.view.device == aether::Device(aether::kDLCUDA, 3));
        CHECK(!aether::interop::hostAccessible(imp.view.device.type));
    }
    CHECK(g_versioned == 1);
}

void importBoolAndRawBits() {
    uint8_t flags[6] = {1, 0, 1, 1, 0, 0};
    int64_t shape[1] = {6};
    DLManagedTensor t{};
    fill(t, flags, 1, shape, nullptr, DLDataType{kDLBool, 8, 1}, kCpu);
    t.deleter = &countLegacy;
    g_legacy = 0;
    {
        auto imp = aether::interop::fromDLPack(&t);
        CHECK(imp.view.dtype_code == kDLBool && imp.view.dtype_bits == 8);
    }
    CHECK(g_legacy == 1);
    // a 64-bit unsigned payload is described, never converted
    uint64_t raw[3] = {0xFFFFFFFFFFFFFFFFull, 0x8000000000000001ull, 42};
    int64_t s3[1] = {3};
    DLManagedTensor u{};
    fill(u, raw, 1, s3, nullptr, DLDataType{kDLUInt, 64, 1}, kCpu);
    u.deleter = &countLegacy;
    auto imp = aether::interop::fromDLPack(&u);
    CHECK(imp.view.data == raw && static_cast<uint64_t*>(imp.view.data)[1] == 0x8000000000000001ull);
}

template <class M>
bool refusedOnce(M& t, int& counter, const char* needle) {
    counter = 0;
    bool threw = false;
    try {
        auto imp = aether::interop::fromDLPack(&t);
    } catch (const aether::Error& e) {
        threw = true;
        const std::string w = e.what();
        if (w.find("aether::interop::fromDLPack failed on DLPack") == std::string::npos ||
            w.find(needle) == std::string::npos) {
            std::printf("unexpected message: %s\n", w.c_str());
            return false;
        }
    }
    return threw && counter == 1;   // the deleter still ran, once
}

void rejections() {
    double d[64] = {};
    int64_t shape[7] = {1, 1, 1, 1, 1, 1, 2};
    DLManagedTensor t{};
    t.deleter = &countLegacy;
    fill(t, d, 1, shape, nullptr, DLDataType{kDLComplex, 64, 1}, kCpu);
    CHECK(refusedOnce(t, g_legacy, "unsupported dtype (code=5, bits=64, lanes=1)"));
    fill(t, d, 7, shape, nullptr, kF64, kCpu);
    CHECK(refusedOnce(t, g_legacy, "rank 7 exceeds RuntimeView's cap of 6"));
    fill(t, d, 1, shape, nullptr, kF64, kCpu);
    t.dl_tensor.byte_offset = 16;
    CHECK(refusedOnce(t, g_legacy, "byte_offset=16 != 0"));
    fill(t, d, 1, shape, nullptr, kF64, DLDevice{kDLOpenCL, 0});
    CHECK(refusedOnce(t, g_legacy, "unknown/unsupported device kind (type=4)"));
    int64_t negShape[1] = {-2};
    fill(t, d, 1, negShape, nullptr, kF64, kCpu);
    CHECK(refusedOnce(t, g_legacy, "shape[0]=-2 is negative"));
    int64_t negStride[1] = {-1}, two[1] = {2};
    fill(t, d, 1, two, negStride, kF64, kCpu);
    CHECK(refusedOnce(t, g_legacy, "strides[0]=-1 is negative"));
    int64_t big[2] = {int64_t(1) << 40, int64_t(1) << 40};
    fill(t, d, 2, big, nullptr, kF64, kCpu);
    CHECK(refusedOnce(t, g_legacy, "exceeds int64"));
    for (DLDataType dt : {DLDataType{kDLComplex, 128, 1}, DLDataType{kDLFloat, 128, 1}, DLDataType{kDLBfloat, 32, 1},
                          DLDataType{kDLFloat, 64, 2}, DLDataType{kDLOpaqueHandle, 64, 1}}) {
        DLManagedTensorVersioned v{};
        v.deleter = &countVersioned;
        fill(v, d, 1, two, nullptr, dt, kCpu);
        CHECK(refusedOnce(v, g_versioned, "unsupported dtype"));
    }
    {
        DLManagedTensorVersioned v{};
        v.version = DLPackVersion{2, 0};
        v.deleter = &countVersioned;
        fill(v, d, 1, two, nullptr, kF64, kCpu);
        CHECK(refusedOnce(v, g_versioned, "DLPack major version 2 is newer than 1"));
        v.version = DLPackVersion{1, 3};   // a later minor version imports
        g_versioned = 0;
        { auto imp = aether::interop::fromDLPack(&v); }
        CHECK(g_versioned == 1);
    }
    // a null tensor pointer: nothing to delete, still an error
    bool threw = false;
    try {
        aether::interop::fromDLPack(static_cast<DLManagedTensor*>(nullptr));
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        aether::interop::fromDLPack(static_cast<DLManagedTensorVersioned*>(nullptr));
    } catch (const aether::Error&) {
        threw = true;
    }
    CHECK(threw);
    // an empty tensor imports (its span check is skipped)
    int64_t empty[2] = {0, int64_t(1) << 62};
    fill(t, d, 2, empty, nullptr, kF64, kCpu);
    g_legacy = 0;
    {
        auto imp = aether::interop::fromDLPack(&t);
        CHECK(imp.view.extents[0] == 0);
    }
    CHECK(g_legacy == 1);
}

// export -> import is the identity, strides verbatim (a padded SoA layout)
void roundTrips() {
    std::vector<double> planes(3 * 16);
    aether::RuntimeView v{};
    v.data = planes.data();
    v.dtype_code = kDLFloat;
    v.dtype_bits = 64;
    v.dtype_lanes = 1;
    v.rank = 2;
    v.extents[0] = 3;
    v.extents[1] = 10;
    v.strides[0] = 16;   // plane pitch larger than the sample count
    v.strides[1] = 1;
    for (const aether::Device dev : {aether::Device(aether::kDLCPU), aether::Device(aether::kDLCUDA, 1)}) {
        v.device = dev;
        DLManagedTensorVersioned* ex = aether::interop::toDLPack(v);
        CHECK(ex->version.major == DLPACK_MAJOR_VERSION && ex->version.minor == DLPACK_MINOR_VERSION);
        CHECK(ex->flags == 0 && ex->dl_tensor.byte_offset == 0);
        CHECK(ex->dl_tensor.device.device_type == DLDeviceType(dev.type) && ex->dl_tensor.device.device_id == dev.id);
        auto back = aether::interop::fromDLPack(ex);   // owns `ex`: its deleter frees the export
        CHECK(back.view.data == v.data && back.view.rank == 2);
        CHECK(std::memcmp(back.view.extents, v.extents, sizeof v.extents) == 0);
        CHECK(std::memcmp(back.view.strides, v.strides, sizeof v.strides) == 0);
        CHECK(back.view.device == dev);
    }
    // every supported dtype survives both directions, both generations
    const DLDataType kinds[] = {{kDLFloat, 64, 1}, {kDLFloat, 32, 1}, {kDLFloat, 16, 1}, {kDLBfloat, 16, 1},
                                {kDLBool, 8, 1},   {kDLInt, 64, 1},   {kDLInt, 32, 1},   {kDLInt, 16, 1},
                                {kDLInt, 8, 1},    {kDLUInt, 64, 1},  {kDLUInt, 32, 1},  {kDLUInt, 16, 1},
                                {kDLUInt, 8, 1}};
    for (const DLDataType dt : kinds) {
        v.dtype_code = dt.code;
        v.dtype_bits = dt.bits;
        v.device = aether::Device(aether::kDLCPU);
        DLManagedTensorVersioned* ex = aether::interop::toDLPack(v);
        CHECK(ex->dl_tensor.dtype.code == dt.code && ex->dl_tensor.dtype.bits == dt.bits);
        {
            auto back = aether::interop::fromDLPack(ex);
            CHECK(back.view.dtype_code == dt.code && back.view.dtype_bits == dt.bits);
        }
        DLManagedTensor* lg = aether::interop::toDLPackLegacy(v);
        // the legacy code table has no bool: it leaves as 8-bit unsigned
        CHECK(lg->dl_tensor.dtype.code == (dt.code == kDLBool ? uint8_t(kDLUInt) : dt.code));
        CHECK(lg->dl_tensor.dtype.bits == dt.bits);
        auto back = aether::interop::fromDLPack(lg);
        CHECK(back.view.strides[0] == 16);
    }
    // exports refuse what imports refuse
    v.dtype_code = kDLComplex;
    bool threw = false;
    try {
        aether::interop::toDLPack(v);
    } catch (const aether::Error& e) {
        threw = std::string(e.what()).find("aether::interop::toDLPack failed") != std::string::npos;
    }
    CHECK(threw);
    v.dtype_code = kDLFloat;
    v.dtype_bits = 64;
    threw = false;
    try {
        v.device = aether::Device(4);
        aether::interop::toDLPackLegacy(v);
    } catch (const aether::Error& e) {
        threw = std::string(e.what()).find("unknown/unsupported device kind") != std::string::npos;
    }
    CHECK(threw);
    // a typed view through fromView: components first, samples last
    std::vector<double> soa(3 * 7);
    auto tv = aether::make_view<double, 3, aether::dyn>(soa.data(), aether::Device(aether::kDLCPU), 7);
    DLManagedTensorVersioned* ex = aether::interop::toDLPack(tv);
    CHECK(ex->dl_tensor.ndim == 2 && ex->dl_tensor.shape[0] == 3 && ex->dl_tensor.shape[1] == 7);
    CHECK(ex->dl_tensor.strides[0] == 7 && ex->dl_tensor.strides[1] == 1);
    ex->deleter(ex);
}

template <class V>
bool promotionRefused(const aether::RuntimeView& r, const char* needle) {
    try {
        (void)r.as<V>();
    } catch (const aether::Error& e) {
        const std::string w = e.what();
        if (w.find("aether::RuntimeView::as failed") != std::string::npos && w.find(needle) != std::string::npos)
            return true;
        std::printf("unexpected message: %s\n", w.c_str());
    }
    return false;
}

// RuntimeView::as<StaticViewT>(): a DLPack import promoted back onto typed
// views (tests/test_DLPackRoundtrip.cu:278-298), and its refusals
void promotions() {
    const std::size_t n = 5;
    std::vector<double> soa(3 * n);
    for (std::size_t i = 0; i < soa.size(); ++i) soa[i] = double(i);
    auto tv = aether::make_view<double, 3, aether::dyn>(soa.data(), aether::Device(aether::kDLCUDA), n);
    auto back = aether::interop::fromDLPack(aether::interop::toDLPack(tv));
    const aether::Vec3dView promoted = back.view.as<aether::Vec3dView>();
    CHECK(promoted.data() == tv.data() && promoted.device() == aether::Device(aether::kDLCUDA));
    CHECK(promoted.extent(1) == n && promoted.mapping().stride(0) == n);
    CHECK(back.view.size() == int64_t(3 * n));

    // a padded plane layout promotes onto a layout_stride view only
    aether::RuntimeView r{};
    r.data = soa.data();
    r.dtype_code = 2;
    r.dtype_bits = 64;
    r.dtype_lanes = 1;
    r.rank = 2;
    r.extents[0] = 2;
    r.extents[1] = 4;
    r.strides[0] = 6;
    r.strides[1] = 1;
    r.device = aether::Device(aether::kDLCPU);
    using Strided = aether::View<double, aether::extents<2, aether::dyn>, aether::layout_stride>;
    const Strided sv = r.as<Strided>();
    CHECK(sv(1, 3) == soa[9] && sv(0, 2) == soa[2]);
    using V2d = aether::VecView<double, 2>;
    using V2f = aether::VecView<float, 2>;
    CHECK(promotionRefused<V2d>(r, "not row-major"));
    CHECK(promotionRefused<aether::Vec3dView>(r, "extent 0 is 2, the view's is 3"));
    CHECK(promotionRefused<V2f>(r, "dtype mismatch"));
    CHECK(promotionRefused<aether::ScalarView<double>>(r, "rank 2 != the view's 1"));
    r.device = aether::Device(4);
    CHECK(promotionRefused<Strided>(r, "unknown/unsupported device kind (type=4)"));
    r.device = aether::Device(aether::kDLCPU);
    r.strides[0] = int64_t(1) << 33;
    CHECK(promotionRefused<Strided>(r, "32-bit offsets"));
    // a const view of floats, rank 1
    std::vector<float> f(7, 1.5f);
    auto fv = aether::make_view<const float, aether::dyn>(f.data(), aether::Device(aether::kDLCPU), f.size());
    const aether::RuntimeView fr = aether::fromView(fv);
    CHECK(fr.dtype_bits == 32 && fr.size() == 7);
    CHECK(fr.as<aether::ScalarView<const float>>()(6) == 1.5f);
}

}  // namespace

int main() {
    importLegacy();
    importVersioned();
    importBoolAndRawBits();
    rejections();
    roundTrips();
    promotions();
    if (failures) return 1;
    std::printf("dlpack ok\n");
    return 0;
}
#else
#include <cuda_runtime.h>

namespace {
template <class M>
aether::interop::DLPackImport take(void* p) {
    return aether::interop::fromDLPack(static_cast<M*>(p));
}
aether::interop::DLPackImport takeAny(void* p, int versioned) {
    return versioned ? take<DLManagedTensorVersioned>(p) : take<DLManagedTensor>(p);
}
}  // namespace

/** out = s * in on the device, both imported from a foreign producer; the
 *  call owns both tensors from its start and runs each deleter once, after a
 *  synchronise. 0 on success, else the error text in `err`. */
extern "C" int dlpack_scale(void* in, int in_versioned, void* out, int out_versioned, double s, char* err, size_t cap) {
    try {
        aether::interop::DLPackImport a;
        try {
            a = takeAny(in, in_versioned);
        } catch (...) {
            // the output was handed over too: release it unimported
            if (out_versioned)
                aether::interop::DLPackOwner::fromVersioned(static_cast<DLManagedTensorVersioned*>(out)).release();
            else
                aether::interop::DLPackOwner::fromLegacy(static_cast<DLManagedTensor*>(out)).release();
            throw;
        }
        auto o = takeAny(out, out_versioned);
        aether::eval::runtimeEval(aether::eval::RuntimeOp::Scale, a.view, aether::RuntimeView{}, o.view, s);
        if (cudaDeviceSynchronize() != cudaSuccess) throw aether::Error("dlpack_scale: synchronize failed");
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, cap, "%s", e.what());
        return 1;
    }
}
#endif
