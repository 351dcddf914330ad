// aether/dlpack.h -- DLPack <-> RuntimeView, host side (interop/DLPack.h).
//
// aether::interop::fromDLPack takes either DLPack generation (the legacy
// DLManagedTensor and the versioned DLManagedTensorVersioned of DLPack 1.0)
// and returns a RuntimeView over the producer's memory (no copy), the device
// it lives on, and a DLPackOwner that calls the producer's deleter exactly
// once, when it is destroyed or released. toDLPack exports a RuntimeView or a
// typed View as a versioned tensor whose deleter frees what the export
// allocated (the data stays the caller's); toDLPackLegacy exports the
// pre-1.0 struct (interop/DLPackLegacy.h).
//
// As in the reference (interop/DLPack.h:7-40): DLPack orders nothing around
// the deleter, so work launched on imported memory must be complete before
// the owner runs it. Refused imports -- more than six modes, a nonzero
// byte_offset, an unsupported dtype (float 64/32/16, bfloat16, int and uint of
// 64/32/16/8 bits and bool pass, one lane), a device other than the host,
// CUDA or page-locked host memory, a negative extent or stride, a span past
// int64 -- throw aether::Error after calling the deleter once: the import
// owned the tensor from the moment it was handed over. The imported view
// carries the producer's device; RuntimeView::as<StaticViewT>() promotes it
// to a typed view.
//
// The DLPack structures are the published ABI of the DLPack project (v1.0),
// declared here field for field so that producers and consumers built
// against that header exchange them unchanged; a translation unit that has
// already included the project's dlpack.h uses its declarations instead.
#pragma once

#include <climits>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "aether/layout.h"
#include "aether/runtime.h"

#ifndef DLPACK_DLPACK_H_
#define DLPACK_DLPACK_H_
#define DLPACK_MAJOR_VERSION 1
#define DLPACK_MINOR_VERSION 0
#define DLPACK_FLAG_BITMASK_READ_ONLY (1UL << 0UL)
#define DLPACK_FLAG_BITMASK_IS_COPIED (1UL << 1UL)
extern "C" {
typedef struct {
    uint32_t major;
    uint32_t minor;
} DLPackVersion;
typedef enum {
    kDLCPU = 1,
    kDLCUDA = 2,
    kDLCUDAHost = 3,
    kDLOpenCL = 4,
    kDLVulkan = 7,
    kDLMetal = 8,
    kDLVPI = 9,
    kDLROCM = 10,
    kDLROCMHost = 11,
    kDLExtDev = 12,
    kDLCUDAManaged = 13,
    kDLOneAPI = 14,
    kDLWebGPU = 15,
    kDLHexagon = 16,
    kDLMAIA = 17,
} DLDeviceType;
typedef struct {
    DLDeviceType device_type;
    int32_t device_id;
} DLDevice;
typedef enum {
    kDLInt = 0U,
    kDLUInt = 1U,
    kDLFloat = 2U,
    kDLOpaqueHandle = 3U,
    kDLBfloat = 4U,
    kDLComplex = 5U,
    kDLBool = 6U,
} DLDataTypeCode;
typedef struct {
    uint8_t code;
    uint8_t bits;
    uint16_t lanes;
} DLDataType;
typedef struct {
    void* data;
    DLDevice device;
    int32_t ndim;
    DLDataType dtype;
    int64_t* shape;
    int64_t* strides;
    uint64_t byte_offset;
} DLTensor;
typedef struct DLManagedTensor {
    DLTensor dl_tensor;
    void* manager_ctx;
    void (*deleter)(struct DLManagedTensor* self);
} DLManagedTensor;
typedef struct DLManagedTensorVersioned {
    DLPackVersion version;
    void* manager_ctx;
    void (*deleter)(struct DLManagedTensorVersioned* self);
    uint64_t flags;
    DLTensor dl_tensor;
} DLManagedTensorVersioned;
}
#endif

namespace aether {
namespace interop {

/** Calls the producer's deleter exactly once: on destruction or release().
 *  Move-only. */
class DLPackOwner {
public:
    DLPackOwner() = default;
    static DLPackOwner fromLegacy(DLManagedTensor* t) {
        DLPackOwner o;
        o.legacy_ = t;
        return o;
    }
    static DLPackOwner fromVersioned(DLManagedTensorVersioned* t) {
        DLPackOwner o;
        o.versioned_ = t;
        return o;
    }
    DLPackOwner(const DLPackOwner&) = delete;
    DLPackOwner& operator=(const DLPackOwner&) = delete;
    DLPackOwner(DLPackOwner&& o) noexcept : legacy_(o.legacy_), versioned_(o.versioned_) {
        o.legacy_ = nullptr;
        o.versioned_ = nullptr;
    }
    DLPackOwner& operator=(DLPackOwner&& o) noexcept {
        if (this != &o) {
            release();
            legacy_ = std::exchange(o.legacy_, nullptr);
            versioned_ = std::exchange(o.versioned_, nullptr);
        }
        return *this;
    }
    ~DLPackOwner() { release(); }
    /** Run the deleter now (once); later calls do nothing. */
    void release() {
        if (DLManagedTensor* t = std::exchange(legacy_, nullptr))
            if (t->deleter) t->deleter(t);
        if (DLManagedTensorVersioned* t = std::exchange(versioned_, nullptr))
            if (t->deleter) t->deleter(t);
    }
    bool owns() const { return legacy_ || versioned_; }

private:
    DLManagedTensor* legacy_ = nullptr;
    DLManagedTensorVersioned* versioned_ = nullptr;
};

/** An imported tensor: its descriptor (with its device) and the owner of its
 *  memory. */
struct DLPackImport {
    RuntimeView view{};
    DLPackOwner owner;
};

namespace detail {

inline bool dtypeIsSupported(DLDataType dt) {
    if (dt.lanes != 1) return false;
    switch (dt.code) {
    case kDLFloat: return dt.bits == 64 || dt.bits == 32 || dt.bits == 16;
    case kDLBfloat: return dt.bits == 16;
    case kDLBool: return dt.bits == 8;
    case kDLInt:
    case kDLUInt: return dt.bits == 64 || dt.bits == 32 || dt.bits == 16 || dt.bits == 8;
    default: return false;
    }
}
// The memory kinds this engine launches on or reads: the host, CUDA device
// memory and page-locked host memory (interop/DLPack.h:172-203, a CUDA build).
inline bool deviceIsKnown(int type) {
    return type == ::kDLCPU || type == ::kDLCUDA || type == ::kDLCUDAHost;
}

// The device code as the producer wrote it: read as the int32 it is on the
// wire, since a code outside the enumerators is no valid DLDeviceType value.
inline int rawDeviceType(const DLDevice& d) {
    static_assert(sizeof(d.device_type) == sizeof(int32_t), "DLDeviceType is an int32 on the wire");
    int32_t v;
    std::memcpy(&v, &d.device_type, sizeof v);
    return v;
}

[[noreturn]] inline void refuse(const std::string& op, const std::string& why) {
    throw Error::memory(op, "DLPack", 0, why);
}

/** The descriptor of a DLTensor, or a throw; ownership stays with the caller
 *  (interop/DLPack.h:226-314). A null strides pointer means compact
 *  row-major; every extent and stride must be non-negative and the span the
 *  view addresses, 1 + sum (extent - 1) x stride elements, must fit int64. */
inline RuntimeView viewOf(const DLTensor& t) {
    const std::string op = "aether::interop::fromDLPack";
    if (t.ndim < 0 || t.ndim > AETHER_RT_RANK_CAP)
        refuse(op, "rank " + std::to_string(t.ndim) + " exceeds RuntimeView's cap of " +
                       std::to_string(AETHER_RT_RANK_CAP));
    if (t.byte_offset != 0) refuse(op, "byte_offset=" + std::to_string(t.byte_offset) + " != 0 is not supported");
    if (!dtypeIsSupported(t.dtype))
        refuse(op, "unsupported dtype (code=" + std::to_string(unsigned(t.dtype.code)) +
                       ", bits=" + std::to_string(unsigned(t.dtype.bits)) +
                       ", lanes=" + std::to_string(unsigned(t.dtype.lanes)) + ")");
    const int kind = rawDeviceType(t.device);
    if (!deviceIsKnown(kind)) refuse(op, "unknown/unsupported device kind (type=" + std::to_string(kind) + ")");
    for (int k = 0; k < t.ndim; ++k) {
        if (t.shape[k] < 0) refuse(op, "shape[" + std::to_string(k) + "]=" + std::to_string(t.shape[k]) + " is negative");
        if (t.strides && t.strides[k] < 0)
            refuse(op, "strides[" + std::to_string(k) + "]=" + std::to_string(t.strides[k]) + " is negative");
    }
    RuntimeView r{};
    r.data = t.data;
    r.dtype_code = t.dtype.code;
    r.dtype_bits = t.dtype.bits;
    r.dtype_lanes = t.dtype.lanes;
    r.rank = t.ndim;
    r.device = Device(kind, t.device.device_id);
    const unsigned __int128 lim = uint64_t(INT64_MAX);
    unsigned __int128 step = 1, span = 1;
    bool empty = false;
    for (int k = t.ndim - 1; k >= 0; --k) {
        r.extents[k] = t.shape[k];
        if (t.strides) {
            r.strides[k] = t.strides[k];
        } else {
            if (step > lim) refuse(op, "compact strides exceed int64");
            r.strides[k] = int64_t(step);
        }
        step *= uint64_t(t.shape[k]);   // step <= 2^63 and shape < 2^63: no wrap
        if (step > lim) step = lim + 1;
        empty |= t.shape[k] == 0;
    }
    if (!empty) {
        for (int k = 0; k < t.ndim; ++k) {
            span += (unsigned __int128)uint64_t(r.extents[k] - 1) * uint64_t(r.strides[k]);
            if (span > lim) refuse(op, "required span exceeds int64 elements");
        }
    }
    return r;
}

template <class M>
DLPackImport import_(M* managed, DLPackOwner owner, const char* type) {
    if (!managed) refuse("aether::interop::fromDLPack", std::string("null ") + type + "*");
    DLPackImport im;
    im.owner = std::move(owner);   // owns the tensor from here: a refusal below still deletes it once
    im.view = viewOf(managed->dl_tensor);
    return im;
}

struct ExportCtx {
    std::vector<int64_t> shape, strides;
};
inline void deleteExported(DLManagedTensorVersioned* self) {
    delete static_cast<ExportCtx*>(self->manager_ctx);
    delete self;
}

}  // namespace detail

/** True for memory the host can dereference. */
inline bool hostAccessible(int device_type) {
    return device_type == ::kDLCPU || device_type == ::kDLCUDAHost || device_type == ::kDLROCMHost;
}

/** Import a legacy DLManagedTensor (no copy); the owner runs its deleter. */
inline DLPackImport fromDLPack(DLManagedTensor* managed) {
    return detail::import_(managed, DLPackOwner::fromLegacy(managed), "DLManagedTensor");
}
/** Import a DLPack 1.x DLManagedTensorVersioned (no copy). A major version
 *  above 1 may lay the struct out differently: refused, deleter called, as
 *  the DLPack specification requires of a consumer. */
inline DLPackImport fromDLPack(DLManagedTensorVersioned* managed) {
    if (managed && managed->version.major > 1) {
        const uint32_t major = managed->version.major;
        DLPackOwner::fromVersioned(managed).release();
        detail::refuse("aether::interop::fromDLPack", "DLPack major version " + std::to_string(major) + " is newer than 1");
    }
    return detail::import_(managed, DLPackOwner::fromVersioned(managed), "DLManagedTensorVersioned");
}

namespace detail {
/** The checks both exports share (interop/DLPack.h:383-396); the dtype to write. */
inline DLDataType exportable(const char* op, const RuntimeView& view) {
    if (view.rank < 0 || view.rank > AETHER_RT_RANK_CAP)
        refuse(op, "rank " + std::to_string(view.rank) + " exceeds RuntimeView's cap");
    const DLDataType dt{view.dtype_code, view.dtype_bits, view.dtype_lanes};
    if (!dtypeIsSupported(dt)) refuse(op, "unsupported dtype");
    if (!deviceIsKnown(view.device.type)) refuse(op, "unknown/unsupported device kind");
    return dt;
}
template <class M>
M* exportInto(M* t, const RuntimeView& view, DLDataType dt) {
    auto* ctx = new ExportCtx();
    ctx->shape.assign(view.extents, view.extents + view.rank);
    ctx->strides.assign(view.strides, view.strides + view.rank);
    t->manager_ctx = ctx;
    t->dl_tensor.data = view.data;
    t->dl_tensor.device = DLDevice{DLDeviceType(view.device.type), int32_t(view.device.id)};
    t->dl_tensor.ndim = view.rank;
    t->dl_tensor.dtype = dt;
    t->dl_tensor.shape = ctx->shape.data();
    t->dl_tensor.strides = ctx->strides.data();   // verbatim: any stride pattern round-trips
    t->dl_tensor.byte_offset = 0;
    return t;
}
inline void deleteExportedLegacy(DLManagedTensor* self) {
    delete static_cast<ExportCtx*>(self->manager_ctx);
    delete self;
}
}  // namespace detail

/** Export a descriptor as a DLPack 1.0 tensor on the view's device; the
 *  receiver calls its deleter, which frees the export's own allocations, not
 *  the data (interop/DLPack.h:383-420). */
inline DLManagedTensorVersioned* toDLPack(const RuntimeView& view) {
    const DLDataType dt = detail::exportable("aether::interop::toDLPack", view);
    auto* t = new DLManagedTensorVersioned{};
    t->version = DLPackVersion{DLPACK_MAJOR_VERSION, DLPACK_MINOR_VERSION};
    t->deleter = &detail::deleteExported;
    t->flags = 0;
    return detail::exportInto(t, view, dt);
}
/** A typed view, through fromView. */
template <class T, class X, class L, bool Vo, bool RO>
DLManagedTensorVersioned* toDLPack(const View<T, X, L, Vo, RO>& v) {
    return toDLPack(fromView(v));
}

/** Export as a pre-1.0 DLManagedTensor (interop/DLPackLegacy.h). The legacy
 *  type-code enum has no bool, so a bool view leaves as 8-bit unsigned, the
 *  nearest code a legacy consumer reads. */
inline DLManagedTensor* toDLPackLegacy(const RuntimeView& view) {
    DLDataType dt = detail::exportable("aether::interop::toDLPackLegacy", view);
    if (dt.code == kDLBool) dt.code = kDLUInt;
    auto* t = new DLManagedTensor{};
    t->deleter = &detail::deleteExportedLegacy;
    return detail::exportInto(t, view, dt);
}
template <class T, class X, class L, bool Vo, bool RO>
DLManagedTensor* toDLPackLegacy(const View<T, X, L, Vo, RO>& v) {
    return toDLPackLegacy(fromView(v));
}

}  // namespace interop
}  // namespace aether
