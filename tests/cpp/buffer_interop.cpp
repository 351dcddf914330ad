// aether::interop's buffer layer (aether/buffer.h), the cases of the
// reference's tests/test_DLPackBuffer_common.h over hand-built producers
// whose deleters count their calls. Host only: device records are described,
// never dereferenced. Prints "buffer ok" when every check holds.
#include <aether/aether.h>
#include <aether/buffer.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

namespace io = aether::interop;

int failures = 0;
#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                              \
        }                                                            \
    } while (0)

int g_v = 0, g_l = 0;
void countV(DLManagedTensorVersioned*) { ++g_v; }
void countL(DLManagedTensor*) { ++g_l; }

double g_data[64];
int64_t g_shape[2] = {4, 8};

DLManagedTensorVersioned versioned(uint64_t flags, DLDevice dev = {kDLCPU, 0}) {
    DLManagedTensorVersioned t{};
    t.version = DLPackVersion{1, 0};
    t.flags = flags;
    t.deleter = &countV;
    t.dl_tensor.data = g_data;
    t.dl_tensor.device = dev;
    t.dl_tensor.ndim = 2;
    t.dl_tensor.dtype = DLDataType{kDLFloat, 64, 1};
    t.dl_tensor.shape = g_shape;
    return t;
}
DLManagedTensor legacy(DLDevice dev = {kDLCPU, 0}) {
    DLManagedTensor t{};
    t.deleter = &countL;
    t.dl_tensor.data = g_data;
    t.dl_tensor.device = dev;
    t.dl_tensor.ndim = 2;
    t.dl_tensor.dtype = DLDataType{kDLFloat, 64, 1};
    t.dl_tensor.shape = g_shape;
    return t;
}

template <class F>
std::string thrown(F f) {
    try {
        f();
    } catch (const aether::Error& e) {
        return e.what();
    }
    return "";
}
bool has(const std::string& s, const char* needle) { return s.find(needle) != std::string::npos; }

void imports() {
    g_v = 0;
    {
        auto t = versioned(0);
        const io::BufferView b = io::importDLPack(&t, "torch.Tensor");
        CHECK(b.access == io::Access::ReadWrite && b.writable() && !b.owned() && b.producer == "torch.Tensor");
        CHECK(b.view.data == g_data && b.view.strides[0] == 8 && b.view.device == aether::Device(aether::kDLCPU));
        auto r = versioned(DLPACK_FLAG_BITMASK_READ_ONLY);
        io::BufferView rb = io::importDLPack(&r);
        CHECK(rb.access == io::Access::ReadOnly && !rb.writable());
        io::assumeWritable(rb);   // an assertion cannot override a declared read-only
        CHECK(!rb.writable());
        CHECK(g_v == 0);
    }
    CHECK(g_v == 2);   // each deleter once, with the last view
    g_l = 0;
    {
        auto t = legacy();
        io::BufferView b = io::importDLPack(&t);
        CHECK(b.access == io::Access::Unknown && !b.writable() && !b.assumedWritable);
        io::assumeWritable(b);
        CHECK(b.writable() && b.assumedWritable && b.access == io::Access::Unknown);
        const io::BufferView copy = b;   // copies share the keep-alive
        b = io::BufferView{};
        CHECK(g_l == 0 && copy.writable());
    }
    CHECK(g_l == 1);
    // CUDA records, both generations: described, never dereferenced
    g_v = g_l = 0;
    {
        auto t = versioned(DLPACK_FLAG_BITMASK_READ_ONLY, DLDevice{kDLCUDA, 1});
        auto l = legacy(DLDevice{kDLCUDA, 0});
        const io::BufferView b = io::importDLPack(&t), c = io::importDLPack(&l);
        CHECK(b.access == io::Access::ReadOnly && b.view.device == aether::Device(aether::kDLCUDA, 1));
        CHECK(c.access == io::Access::Unknown && c.view.device == aether::Device(aether::kDLCUDA, 0));
        CHECK(has(thrown([&] { io::requireHostAccess(b, "sum"); }), "sum: device: host access needs host memory, got cuda"));
        auto h = versioned(0, DLDevice{kDLCUDAHost, 0});
        const io::BufferView hb = io::importDLPack(&h);
        CHECK(thrown([&] { io::requireHostAccess(hb, "sum"); }).empty());   // page-locked host memory
    }
    CHECK(g_v == 2 && g_l == 1);
}

void refusedImports() {
    // kinds this build does not launch on, and codes DLPack does not define:
    // refused, the deleter run once
    for (const int32_t kind : {int32_t(kDLOpenCL), int32_t(kDLVulkan), int32_t(kDLCUDAManaged), int32_t(99)}) {
        g_v = 0;
        auto t = versioned(0);
        std::memcpy(&t.dl_tensor.device.device_type, &kind, sizeof kind);   // 99: no enumerator, as a C producer writes it
        const std::string w = thrown([&] { io::importDLPack(&t); });
        CHECK(has(w, "unknown/unsupported device kind") && g_v == 1);
    }
    g_l = 0;
    auto l = legacy();
    l.dl_tensor.dtype = DLDataType{kDLComplex, 64, 1};
    CHECK(has(thrown([&] { io::importDLPack(&l); }), "unsupported dtype") && g_l == 1);
    g_v = 0;
    auto t = versioned(0);
    t.version.major = 2;
    CHECK(has(thrown([&] { io::importDLPack(&t); }), "major version 2 is newer") && g_v == 1);
    CHECK(has(thrown([&] { io::importDLPack(static_cast<DLManagedTensor*>(nullptr)); }), "null DLManagedTensor*"));
}

void byteOffset() {
    g_v = 0;
    auto t = versioned(0);
    t.dl_tensor.byte_offset = 3 * sizeof(double);
    {
        const io::BufferView b = io::importDLPack(&t);
        CHECK(b.view.data == static_cast<void*>(g_data + 3));
    }
    CHECK(g_v == 1);
}

void names() {
    CHECK(std::string(io::accessName(io::Access::ReadWrite)) == "read-write");
    CHECK(std::string(io::accessName(io::Access::ReadOnly)) == "read-only");
    CHECK(std::string(io::accessName(io::Access::Unknown)) == "unknown");
    CHECK(io::dtypeName(DLDataType{kDLFloat, 64, 1}) == "float64" && io::dtypeName(DLDataType{kDLBool, 8, 1}) == "bool");
    CHECK(io::dtypeName(DLDataType{kDLUInt, 8, 1}) == "uint8" && io::dtypeName(DLDataType{kDLFloat, 32, 4}) ==
                                                                      "dtype(code=2, bits=32, lanes=4)");
    CHECK(io::deviceTypeName(kDLCUDA) == "cuda" && io::deviceTypeName(kDLCUDAHost) == "cuda_host" &&
          io::deviceTypeName(4) == "device_type 4");
}

void exports() {
    g_v = 0;
    {
        auto t = versioned(0);
        const io::BufferView rw = io::importDLPack(&t);
        DLManagedTensorVersioned* e = io::exportDLPack(rw);
        CHECK(e->flags == 0 && e->dl_tensor.data == g_data && e->dl_tensor.strides[0] == 8);
        e->deleter(e);
        auto r = versioned(DLPACK_FLAG_BITMASK_READ_ONLY);
        const io::BufferView ro = io::importDLPack(&r);
        e = io::exportDLPack(ro);
        CHECK(e->flags == DLPACK_FLAG_BITMASK_READ_ONLY);
        e->deleter(e);
        CHECK(has(thrown([&] { io::exportDLPackLegacy(ro); }), "legacy DLPack cannot carry the read-only flag"));
    }
    CHECK(g_v == 2);
    g_l = 0;
    {
        auto l = legacy();
        io::BufferView u = io::importDLPack(&l);
        DLManagedTensorVersioned* e = io::exportDLPack(u);
        CHECK(e->flags == DLPACK_FLAG_BITMASK_READ_ONLY);   // unknown leaves read-only
        e->deleter(e);
        io::assumeWritable(u);
        e = io::exportDLPack(u);
        CHECK(e->flags == 0);
        e->deleter(e);
        DLManagedTensor* le = io::exportDLPackLegacy(u);   // unknown leaves as it came
        const io::BufferView back = io::importDLPack(le);
        CHECK(back.access == io::Access::Unknown && back.view.data == g_data && back.view.extents[1] == 8);
    }
    CHECK(g_l == 1);
    // bool leaves a legacy export as 8-bit unsigned
    uint8_t flags[4] = {1, 0, 1, 1};
    int64_t n4[1] = {4};
    DLManagedTensor bt{};
    bt.dl_tensor.data = flags;
    bt.dl_tensor.device = DLDevice{kDLCPU, 0};
    bt.dl_tensor.ndim = 1;
    bt.dl_tensor.dtype = DLDataType{kDLBool, 8, 1};
    bt.dl_tensor.shape = n4;
    io::BufferView bb = io::importDLPack(&bt);
    io::assumeWritable(bb);
    DLManagedTensor* le = io::exportDLPackLegacy(bb);
    CHECK(le->dl_tensor.dtype.code == kDLUInt && le->dl_tensor.dtype.bits == 8);
    le->deleter(le);
}

// import -> export -> import -> export: the first producer outlives every
// view and tensor of the chain, and its deleter runs once, after the last
void chain() {
    g_v = 0;
    auto t = versioned(0);
    DLManagedTensorVersioned* e2 = nullptr;
    {
        io::BufferView b1 = io::importDLPack(&t, "first");
        DLManagedTensorVersioned* e1 = io::exportDLPack(b1);
        b1 = io::BufferView{};
        CHECK(g_v == 0);
        io::BufferView b2 = io::importDLPack(e1, "second");
        e2 = io::exportDLPack(b2);
    }
    CHECK(g_v == 0);   // e2 still holds the chain
    {
        const io::BufferView b3 = io::importDLPack(e2, "third");
        CHECK(b3.view.data == g_data && g_v == 0);
    }
    CHECK(g_v == 1);
}

void owned() {
    aether::RuntimeView v{};
    v.data = g_data;
    v.dtype_code = kDLFloat;
    v.dtype_bits = 64;
    v.dtype_lanes = 1;
    v.rank = 1;
    v.extents[0] = 64;
    v.strides[0] = 1;
    v.device = aether::Device(aether::kDLCUDA);
    const io::BufferView b = io::ownedBuffer("aether_gb300", v, io::Access::ReadWrite);
    CHECK(b.owned() && b.owner == "aether_gb300" && b.producer.empty() && b.writable());
}

void arrayInterface() {
    io::ArrayInterface ai;
    ai.data = g_data;
    ai.shape = {4, 8};
    ai.strides = {64, 8};
    ai.typestr = "<f8";
    ai.producer = "numpy.ndarray";
    const io::BufferView a = io::fromArrayInterface(ai);
    g_v = 0;
    auto t = versioned(0);
    const io::BufferView d = io::importDLPack(&t, "numpy.ndarray");
    CHECK(a.view.data == d.view.data && a.view.rank == d.view.rank && a.view.strides[0] == d.view.strides[0] &&
          a.view.strides[1] == d.view.strides[1] && a.view.dtype_bits == d.view.dtype_bits);
    CHECK(a.access == io::Access::ReadWrite && a.producer == d.producer);
    ai.strides.clear();   // None: C-contiguous
    ai.readOnly = true;
    ai.device = DLDevice{kDLCUDA, 0};
    const io::BufferView c = io::fromArrayInterface(ai);
    CHECK(c.view.strides[0] == 8 && c.access == io::Access::ReadOnly && c.view.device == aether::Device(aether::kDLCUDA));
    for (const char* ts : {"|b1", "<i4", "<u2", "|u1", "<f4", "<f2"}) {
        ai.typestr = ts;
        CHECK(thrown([&] { io::fromArrayInterface(ai); }).empty());
    }
    ai.typestr = ">f8";
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "is not little-endian"));
    ai.typestr = "<c16";
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "unsupported kind"));
    ai.typestr = "<f";
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "is malformed"));
    ai.typestr = "<u33";
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "unsupported item size"));
    ai.typestr = "<f8";
    ai.strides = {60, 8};
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "byte stride 60 is not a multiple of the item size 8"));
    ai.strides = {8};
    CHECK(has(thrown([&] { io::fromArrayInterface(ai); }), "strides has 1 entries for a rank-2 shape"));
}

void requirements() {
    io::ArrayInterface ai;
    ai.data = g_data;
    ai.shape = {4, 8};
    ai.typestr = "<f8";
    const io::BufferView b = io::fromArrayInterface(ai);
    io::Requirements ok;
    ok.dtype = DLDataType{kDLFloat, 64, 1};
    ok.count = 32;
    ok.shape = std::vector<int64_t>{4, 8};
    ok.contiguous = true;
    ok.alignment = 8;
    ok.deviceType = kDLCPU;
    ok.deviceId = 0;
    ok.writable = true;
    CHECK(io::refusals(b, ok).empty());
    CHECK(thrown([&] { io::require(b, ok); }).empty());

    // a read-only, strided, offset view on the device fails every check
    io::ArrayInterface bad = ai;
    bad.data = reinterpret_cast<char*>(g_data) + 4;
    bad.typestr = "<f4";
    bad.shape = {4, 4};
    bad.strides = {32, 8};
    bad.readOnly = true;
    bad.device = DLDevice{kDLCUDA, 1};
    const io::BufferView w = io::fromArrayInterface(bad);
    const std::vector<std::string> r = io::refusals(w, ok);
    CHECK(r.size() == 8);
    if (r.size() == 8) {
        CHECK(r[0] == "dtype: required float64, got float32");
        CHECK(r[1] == "count: required 32 elements, got 16");
        CHECK(r[2] == "shape: required (4, 8), got (4, 4)");
        CHECK(r[3] == "stride: required C-contiguous with unit stride, got strides (8, 2) for shape (4, 4)");
        CHECK(has(r[4], "alignment: required 8-byte aligned, got address") && has(r[4], "(4 bytes past a boundary)"));
        CHECK(r[5] == "device: required cpu, got cuda");
        CHECK(r[6] == "device id: required 0, got 1");
        CHECK(r[7] == "access: required read-write, got read-only");
    }
    const std::string all = thrown([&] { io::require(w, ok); });
    CHECK(has(all, "aether::interop::require: dtype: required float64") && has(all, "; access: required read-write"));
    // an unknown buffer names the assertion that would accept it
    g_l = 0;
    auto l = legacy();
    const io::BufferView u = io::importDLPack(&l);
    io::Requirements wr;
    wr.writable = true;
    const std::vector<std::string> ru = io::refusals(u, wr);
    CHECK(ru.size() == 1 && ru[0] == "access: required read-write, got unknown (assert writability explicitly to accept it)");
    io::Requirements one;
    one.shape = std::vector<int64_t>{32};
    CHECK(io::refusals(b, one).size() == 1 && io::refusals(b, one)[0] == "shape: required (32,), got (4, 8)");
}

}  // namespace

int main() {
    imports();
    refusedImports();
    byteOffset();
    names();
    exports();
    chain();
    owned();
    arrayInterface();
    requirements();
    if (failures) return 1;
    std::printf("buffer ok\n");
    return 0;
}
