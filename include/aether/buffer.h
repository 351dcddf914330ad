// aether/buffer.h -- foreign buffers with their access, owner and lifetime
// (interop/Buffer.h), host side.
//
// aether::interop::BufferView is a zero-copy RuntimeView of someone's memory
// plus what a consumer of a foreign array needs to know about it:
//
//   access     as the producer declared it -- a versioned DLPack tensor's
//              read-only flag gives ReadOnly or ReadWrite, a legacy DLPack
//              tensor (whose protocol has no flag) gives Unknown, an array
//              interface's data[1] gives ReadOnly or ReadWrite. Unknown is
//              never treated as writable unless a caller asserts it
//              (assumeWritable), and the assertion is kept on the view.
//   owner      the allocating library's name, or "external" when borrowed;
//   producer   the producer's type name ("torch.Tensor", "numpy.ndarray");
//   keepAlive  a shared owner of the producer's memory. A DLPack import
//              puts the producer's deleter there, so it runs once, when the
//              last copy of the view is gone; a re-export stores another
//              share in the exported tensor, so import -> export -> import
//              chains keep the first producer alive to the end.
//
// Requirements states what a consumer needs (dtype, element count, shape,
// C-contiguity, alignment, device, writability); refusals() lists every
// check a buffer fails as "<check>: required <want>, got <have>", and
// require() throws them joined. Nothing here calls CUDA: work queued on
// imported memory must be ordered before the last keep-alive is released.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <string>
#include <utility>
#include <vector>

#include "aether/dlpack.h"

namespace aether {
namespace interop {

/** How a buffer may be accessed, as its producer declared it. */
enum class Access { ReadWrite, ReadOnly, Unknown };

/** "read-write", "read-only" or "unknown". */
inline const char* accessName(Access a) {
    switch (a) {
    case Access::ReadWrite: return "read-write";
    case Access::ReadOnly: return "read-only";
    default: return "unknown";
    }
}

/** The owner name of borrowed memory. */
inline constexpr const char* kExternalOwner = "external";

/** A zero-copy view of a buffer with its access, ownership and lifetime.
 *  view.data already includes any byte offset of the producer; copies share
 *  the keep-alive. */
struct BufferView {
    RuntimeView view{};
    Access access = Access::Unknown;
    bool assumedWritable = false;
    std::string owner = kExternalOwner;
    std::string producer;
    std::shared_ptr<void> keepAlive;

    /** The memory belongs to a library of this family. */
    bool owned() const { return owner != kExternalOwner; }
    /** Writes are allowed: declared read-write, or unknown and asserted. */
    bool writable() const { return access == Access::ReadWrite || (access == Access::Unknown && assumedWritable); }
};

/** Record the caller's assertion that `b` may be written. It changes
 *  nothing for a buffer declared read-only. */
inline void assumeWritable(BufferView& b) { b.assumedWritable = true; }

/** A view of memory that `owner` (a library of this family) allocated. */
inline BufferView ownedBuffer(std::string owner, const RuntimeView& view, Access access,
                              std::shared_ptr<void> keepAlive = {}) {
    BufferView b;
    b.view = view;
    b.access = access;
    b.owner = std::move(owner);
    b.keepAlive = std::move(keepAlive);
    return b;
}

namespace detail {

// A DLTensor with its byte offset moved into the data pointer, validated as
// fromDLPack validates (interop/Buffer.h:93-99).
inline RuntimeView bufferViewOf(const DLTensor& t) {
    DLTensor f = t;
    f.data = static_cast<char*>(t.data) + t.byte_offset;
    f.byte_offset = 0;
    return viewOf(f);
}

template <class M>
std::shared_ptr<void> keepProducer(M* managed) {
    return std::shared_ptr<void>(static_cast<void*>(managed), [](void* p) {
        M* t = static_cast<M*>(p);
        if (t->deleter) t->deleter(t);
    });
}

}  // namespace detail

/** Import a DLPack 1.x tensor; access follows its read-only flag. The view's
 *  keep-alive owns `managed` from the call on, so a refusal runs the deleter
 *  once before the throw (interop/Buffer.h:111-131). Unlike fromDLPack, a
 *  byte offset is accepted (folded into the data pointer). */
inline BufferView importDLPack(DLManagedTensorVersioned* managed, std::string producer = "dlpack") {
    if (!managed) throw Error("aether::interop::importDLPack: null DLManagedTensorVersioned*");
    std::shared_ptr<void> keep = detail::keepProducer(managed);
    if (managed->version.major > 1)
        throw Error("aether::interop::importDLPack: DLPack major version " + std::to_string(managed->version.major) +
                    " is newer than the supported 1");
    BufferView b;
    b.view = detail::bufferViewOf(managed->dl_tensor);
    b.access = (managed->flags & DLPACK_FLAG_BITMASK_READ_ONLY) ? Access::ReadOnly : Access::ReadWrite;
    b.producer = std::move(producer);
    b.keepAlive = std::move(keep);
    return b;
}
/** Import a pre-1.0 DLPack tensor; its protocol carries no access flag, so
 *  access is Unknown. */
inline BufferView importDLPack(DLManagedTensor* managed, std::string producer = "dlpack") {
    if (!managed) throw Error("aether::interop::importDLPack: null DLManagedTensor*");
    std::shared_ptr<void> keep = detail::keepProducer(managed);
    BufferView b;
    b.view = detail::bufferViewOf(managed->dl_tensor);
    b.access = Access::Unknown;
    b.producer = std::move(producer);
    b.keepAlive = std::move(keep);
    return b;
}

/** The fields of a __cuda_array_interface__ (device) or __array_interface__
 *  (host) dictionary, for bindings that build a BufferView without DLPack. */
struct ArrayInterface {
    void* data = nullptr;               // data[0]
    bool readOnly = false;              // data[1]
    std::vector<int64_t> shape;         // elements
    std::vector<int64_t> strides;       // BYTES; empty for C-contiguous (the protocol's None)
    std::string typestr;                // "<f8", "|u1", "|b1", ...
    DLDevice device{::kDLCPU, 0};
    std::string producer;
    std::shared_ptr<void> keepAlive;
};

namespace detail {

[[noreturn]] inline void refuseTypestr(const std::string& ts, const char* why) {
    throw Error("aether::interop::fromArrayInterface: typestr '" + ts + "' " + why);
}

/** A typestr's DLPack dtype: little-endian (or byte-order free) floats,
 *  signed and unsigned integers and bools. */
inline DLDataType dtypeOfTypestr(const std::string& ts) {
    if (ts.size() < 3) refuseTypestr(ts, "is malformed");
    const uint16_t probe = 1;
    const bool nativeLittle = *reinterpret_cast<const uint8_t*>(&probe) == 1;
    const char order = ts[0];
    if (!(order == '<' || order == '|' || (order == '=' && nativeLittle))) refuseTypestr(ts, "is not little-endian");
    int bytes = 0;
    for (std::size_t k = 2; k < ts.size(); ++k) {
        if (ts[k] < '0' || ts[k] > '9' || bytes > 1000) refuseTypestr(ts, "is malformed");
        bytes = bytes * 10 + (ts[k] - '0');
    }
    if (bytes < 1 || bytes > 16) refuseTypestr(ts, "has an unsupported item size");
    const uint8_t bits = uint8_t(bytes * 8);
    switch (ts[1]) {
    case 'f': return DLDataType{kDLFloat, bits, 1};
    case 'i': return DLDataType{kDLInt, bits, 1};
    case 'u': return DLDataType{kDLUInt, bits, 1};
    case 'b': return DLDataType{kDLBool, bits, 1};
    default: refuseTypestr(ts, "has an unsupported kind");
    }
}

}  // namespace detail

/** A BufferView from array-interface fields: byte strides become element
 *  strides (each a multiple of the item size), access follows readOnly, and
 *  the record is validated like a DLPack import (interop/Buffer.h:222-259). */
inline BufferView fromArrayInterface(const ArrayInterface& ai) {
    const DLDataType dt = detail::dtypeOfTypestr(ai.typestr);
    const int64_t item = dt.bits / 8;
    if (!ai.strides.empty() && ai.strides.size() != ai.shape.size())
        throw Error("aether::interop::fromArrayInterface: strides has " + std::to_string(ai.strides.size()) +
                    " entries for a rank-" + std::to_string(ai.shape.size()) + " shape");
    std::vector<int64_t> shape = ai.shape, strides;
    for (const int64_t s : ai.strides) {
        if (item == 0 || s % item != 0)
            throw Error("aether::interop::fromArrayInterface: byte stride " + std::to_string(s) +
                        " is not a multiple of the item size " + std::to_string(item));
        strides.push_back(s / item);
    }
    DLTensor t{};
    t.data = ai.data;
    t.device = ai.device;
    t.ndim = int32_t(shape.size());
    t.dtype = dt;
    t.shape = shape.data();
    t.strides = strides.empty() ? nullptr : strides.data();
    BufferView b;
    b.view = detail::viewOf(t);
    b.access = ai.readOnly ? Access::ReadOnly : Access::ReadWrite;
    b.producer = ai.producer;
    b.keepAlive = ai.keepAlive;
    return b;
}

/** What a consumer needs from a buffer; unset fields are not checked.
 *  `writable` is the switch for a consumer that writes through the buffer. */
struct Requirements {
    std::optional<DLDataType> dtype;
    std::optional<int64_t> count;
    std::optional<std::vector<int64_t>> shape;
    bool contiguous = false;     // C-contiguous, unit innermost stride
    std::size_t alignment = 0;   // bytes; 0 = unchecked
    std::optional<int> deviceType;
    std::optional<int> deviceId;
    bool writable = false;
};

/** "float64", "int32", "bool", ... */
inline std::string dtypeName(DLDataType dt) {
    const std::string b = std::to_string(unsigned(dt.bits));
    if (dt.lanes == 1) {
        switch (dt.code) {
        case kDLFloat: return "float" + b;
        case kDLInt: return "int" + b;
        case kDLUInt: return "uint" + b;
        case kDLBfloat: return "bfloat" + b;
        case kDLBool: return "bool";
        default: break;
        }
    }
    return "dtype(code=" + std::to_string(unsigned(dt.code)) + ", bits=" + b + ", lanes=" + std::to_string(unsigned(dt.lanes)) +
           ")";
}
/** "cpu", "cuda", "cuda_host", "cuda_managed", else "device_type <n>". */
inline std::string deviceTypeName(int t) {
    switch (t) {
    case ::kDLCPU: return "cpu";
    case ::kDLCUDA: return "cuda";
    case ::kDLCUDAHost: return "cuda_host";
    case ::kDLCUDAManaged: return "cuda_managed";
    default: return "device_type " + std::to_string(t);
    }
}

namespace detail {

inline DLDataType dtypeOfView(const RuntimeView& v) { return DLDataType{v.dtype_code, v.dtype_bits, v.dtype_lanes}; }

inline std::string tuple(const std::vector<int64_t>& v) {
    std::string s = "(";
    for (std::size_t k = 0; k < v.size(); ++k) s += (k ? ", " : "") + std::to_string(v[k]);
    return s + (v.size() == 1 ? ",)" : ")");
}

// Row-major compact, modes of extent 1 ignored; an empty view is contiguous.
inline bool cContiguous(const RuntimeView& v) {
    int64_t want = 1;
    for (int k = v.rank - 1; k >= 0; --k) {
        if (v.extents[k] == 0) return true;
        if (v.extents[k] != 1 && v.strides[k] != want) return false;
        want *= v.extents[k];
    }
    return true;
}

}  // namespace detail

/** Every check of `req` that `b` fails, one "<check>: required <want>, got
 *  <have>" message each, in the order of Requirements' fields; empty when
 *  `b` satisfies all of them (interop/Buffer.h:420-470). */
inline std::vector<std::string> refusals(const BufferView& b, const Requirements& req) {
    std::vector<std::string> out;
    const RuntimeView& v = b.view;
    std::vector<int64_t> shape(v.extents, v.extents + v.rank), strides(v.strides, v.strides + v.rank);
    int64_t count = 1;
    for (const int64_t e : shape) count *= e;
    const DLDataType dt = detail::dtypeOfView(v);
    if (req.dtype && !(req.dtype->code == dt.code && req.dtype->bits == dt.bits && req.dtype->lanes == dt.lanes))
        out.push_back("dtype: required " + dtypeName(*req.dtype) + ", got " + dtypeName(dt));
    if (req.count && *req.count != count)
        out.push_back("count: required " + std::to_string(*req.count) + " elements, got " + std::to_string(count));
    if (req.shape && *req.shape != shape)
        out.push_back("shape: required " + detail::tuple(*req.shape) + ", got " + detail::tuple(shape));
    if (req.contiguous && !detail::cContiguous(v))
        out.push_back("stride: required C-contiguous with unit stride, got strides " + detail::tuple(strides) +
                      " for shape " + detail::tuple(shape));
    if (req.alignment) {
        const std::uintptr_t a = reinterpret_cast<std::uintptr_t>(v.data);
        if (a % req.alignment)
            out.push_back("alignment: required " + std::to_string(req.alignment) + "-byte aligned, got address " +
                          std::to_string(a) + " (" + std::to_string(a % req.alignment) + " bytes past a boundary)");
    }
    if (req.deviceType && *req.deviceType != v.device.type)
        out.push_back("device: required " + deviceTypeName(*req.deviceType) + ", got " + deviceTypeName(v.device.type));
    if (req.deviceId && *req.deviceId != v.device.id)
        out.push_back("device id: required " + std::to_string(*req.deviceId) + ", got " + std::to_string(v.device.id));
    if (req.writable && !b.writable())
        out.push_back(std::string("access: required read-write, got ") + accessName(b.access) +
                      (b.access == Access::Unknown ? " (assert writability explicitly to accept it)" : ""));
    return out;
}

/** Throw one aether::Error with every refusal, joined by "; ". */
inline void require(const BufferView& b, const Requirements& req) {
    const std::vector<std::string> r = refusals(b, req);
    if (r.empty()) return;
    std::string msg = "aether::interop::require: ";
    for (std::size_t k = 0; k < r.size(); ++k) msg += (k ? "; " : "") + r[k];
    throw Error(msg);
}

/** Refuse an operation `op` that dereferences `b`'s memory on the host when
 *  that memory is not host-addressable; importing, inspecting and
 *  re-exporting never need this. */
inline void requireHostAccess(const BufferView& b, const char* op) {
    if (hostAccessible(b.view.device.type)) return;
    throw Error(std::string(op) + ": device: host access needs host memory, got " + deviceTypeName(b.view.device.type) +
                " (a record only on the host)");
}

namespace detail {

struct BufferExportCtx {
    std::vector<int64_t> shape, strides;
    std::shared_ptr<void> keepAlive;
};

inline BufferExportCtx* bufferExportCtx(const BufferView& b, const char* op) {
    const RuntimeView& v = b.view;
    if (v.rank < 0 || v.rank > AETHER_RT_RANK_CAP) throw Error(std::string(op) + ": rank " + std::to_string(v.rank) + " exceeds RuntimeView's cap");
    if (!dtypeIsSupported(dtypeOfView(v))) throw Error(std::string(op) + ": unsupported dtype " + dtypeName(dtypeOfView(v)));
    if (!deviceIsKnown(v.device.type)) throw Error(std::string(op) + ": unsupported device " + deviceTypeName(v.device.type));
    auto* ctx = new BufferExportCtx();
    ctx->shape.assign(v.extents, v.extents + v.rank);
    ctx->strides.assign(v.strides, v.strides + v.rank);
    ctx->keepAlive = b.keepAlive;   // the exported tensor keeps the producer alive too
    return ctx;
}

template <class M>
M* fillExport(M* t, const BufferView& b, BufferExportCtx* ctx, DLDataType dt) {
    t->manager_ctx = ctx;
    t->dl_tensor.data = b.view.data;
    t->dl_tensor.device = DLDevice{DLDeviceType(b.view.device.type), int32_t(b.view.device.id)};
    t->dl_tensor.ndim = b.view.rank;
    t->dl_tensor.dtype = dt;
    t->dl_tensor.shape = ctx->shape.data();
    t->dl_tensor.strides = ctx->strides.data();
    t->dl_tensor.byte_offset = 0;
    t->deleter = [](M* self) {
        delete static_cast<BufferExportCtx*>(self->manager_ctx);
        delete self;
    };
    return t;
}

}  // namespace detail

/** Export as a DLPack 1.0 tensor, zero copy: read-only unless the buffer is
 *  writable (so an Unknown buffer leaves read-only unless asserted), with a
 *  share of the keep-alive in its context (interop/Buffer.h:565-582). The
 *  receiver calls its deleter once. */
inline DLManagedTensorVersioned* exportDLPack(const BufferView& b) {
    detail::BufferExportCtx* ctx = detail::bufferExportCtx(b, "aether::interop::exportDLPack");
    auto* t = new DLManagedTensorVersioned{};
    t->version = DLPackVersion{DLPACK_MAJOR_VERSION, DLPACK_MINOR_VERSION};
    t->flags = b.writable() ? 0 : DLPACK_FLAG_BITMASK_READ_ONLY;
    return detail::fillExport(t, b, ctx, detail::dtypeOfView(b.view));
}

/** Export as a pre-1.0 tensor, which cannot say read-only: a read-only
 *  buffer is refused (as numpy refuses it), an Unknown one leaves as it came,
 *  and bool leaves as 8-bit unsigned (interop/Buffer.h:584-600). */
inline DLManagedTensor* exportDLPackLegacy(const BufferView& b) {
    if (b.access == Access::ReadOnly)
        throw Error("aether::interop::exportDLPackLegacy: access: legacy DLPack cannot carry the read-only flag, got "
                    "read-only (export the versioned struct)");
    detail::BufferExportCtx* ctx = detail::bufferExportCtx(b, "aether::interop::exportDLPackLegacy");
    DLDataType dt = detail::dtypeOfView(b.view);
    if (dt.code == kDLBool) dt.code = kDLUInt;
    return detail::fillExport(new DLManagedTensor{}, b, ctx, dt);
}

}  // namespace interop
}  // namespace aether
