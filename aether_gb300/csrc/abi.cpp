// abi.cpp -- the extern "C" surface declared in include/aether_gb300.h.
//
// Memory entry points follow the reference seam (dsc/src/plugin.cpp:20-156):
// status codes, a per-thread last error, device switching around each call.
// Plan entry points own the parsed plan, its compiled module and, for sum
// plans, a default workspace.

#include "aether_gb300.h"

#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.h"
#include "jit.h"
#include "plan.h"

#define AG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

// Kernels of the FP64-grade lowering carry a _tf tag, so profiles and launch
// lists tell them from the double-float kernels of the same expression.
std::string lowering_tag(const ag::Plan& plan, const ag::Lowering& low) {
    return low.math == 3 && plan.dst_dtype == ag::DType::F64 ? "_tf" : "";
}


thread_local std::string g_error;

int fail(const std::string& m) {
    g_error = m;
    return AETHER_FAIL;
}
int cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();
    return fail(std::string(what) + ": " + cudaGetErrorString(e));
}
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
}
template <class F>
int guarded(F&& f) {
    try {
        f();
        return AETHER_OK;
    } catch (const std::exception& e) {
        return fail(e.what());
    }
}

struct OnDevice {
    int prev = 0;
    bool switched = false;
    explicit OnDevice(int dev) {
        cudaGetDevice(&prev);
        switched = prev != dev;
        if (switched) cudaSetDevice(dev);
    }
    ~OnDevice() {
        if (switched) cudaSetDevice(prev);
    }
};

// ---------------------------------------------------------------------------
// Chunks (chunk/Chunk.h:111-260): host, pinned or stream-ordered device bytes.
// ---------------------------------------------------------------------------
struct Chunk {
    int kind = AETHER_MEM_CPU;
    int dev = 0;
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
};

// Pinned host memory from the driver (page-locked, device-mapped). Huge-page
// backed anonymous mappings registered with cudaHostRegister were tried for
// the bulk host<->device streams and measured inconsistent across boxes:
// 36.0 ms per pipelined step on one, 4-8 GB/s copies for seconds on others.
void pinned_alloc(Chunk& c, size_t b) { ck(cudaMallocHost(&c.ptr, b), "cudaMallocHost"); }

std::mutex g_deferred_mu;
std::vector<Chunk*> g_deferred;

void free_now(Chunk* c) {
    if (c->ptr) {
        if (c->kind == AETHER_MEM_CPU) std::free(c->ptr);
        else if (c->kind == AETHER_MEM_PINNED) cudaFreeHost(c->ptr);
        else {
            OnDevice d(c->dev);
            cudaFreeAsync(c->ptr, c->stream);
        }
    }
    delete c;
}

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return st != cudaStreamCaptureStatusNone;
}

// ---------------------------------------------------------------------------
// Plans.
// ---------------------------------------------------------------------------

ag::Lowering default_lowering(const ag::Plan& p) {
    ag::Lowering l;
    l.block = 256;
    l.ipt = 1;
    l.vec = 0;
    l.contract = true;
    l.math = 0;
    (void)p;
    return l;
}

uint64_t ws_needed(const PlanObj& P, uint64_t n) {
    if (!P.plan.wants_sum()) return 0;
    const uint64_t per = chunk_samples(P, false);   // the scalar kernel has the most chunks
    const uint64_t nch = (n + per - 1) / per;
    return 16 + 16 * std::max<uint64_t>(nch, 1);
}

}  // namespace

// ============================================================================
// Memory
// ============================================================================
AG_EXPORT int aether_probe(int* count) {
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (n < 1) return fail("no CUDA device");
    if (count) *count = n;
    return AETHER_OK;
}

AG_EXPORT int aether_runtime_version(int* v) {
    const cudaError_t e = cudaRuntimeGetVersion(v);
    return e == cudaSuccess ? AETHER_OK : cuda_fail(e, "cudaRuntimeGetVersion");
}

AG_EXPORT const char* aether_last_error(void) { return g_error.c_str(); }

AG_EXPORT int aether_chunk_alloc(int kind, int dev, size_t bytes, void* stream, void** chunk, void** ptr) {
    return guarded([&] {
        if (!chunk || !ptr) throw std::runtime_error("chunk_alloc: null output pointer");
        auto c = std::make_unique<Chunk>();
        c->kind = kind;
        c->dev = dev;
        c->bytes = bytes;
        c->stream = static_cast<cudaStream_t>(stream);
        const size_t b = std::max<size_t>(bytes, 1);
        if (kind == AETHER_MEM_CPU) {
            c->ptr = std::aligned_alloc(256, (b + 255) / 256 * 256);
            if (!c->ptr) throw std::runtime_error("chunk_alloc failed on cpu, size=" + std::to_string(bytes) + " bytes");
        } else if (kind == AETHER_MEM_PINNED) {
            pinned_alloc(*c, b);
        } else if (kind == AETHER_MEM_DEVICE) {
            OnDevice d(dev);
            ck(cudaMallocAsync(&c->ptr, b, c->stream), "cudaMallocAsync");
        } else {
            throw std::runtime_error("chunk_alloc: unknown memory kind " + std::to_string(kind));
        }
        *ptr = c->ptr;
        *chunk = c.release();
    });
}

AG_EXPORT void aether_chunk_release(void* chunk) {
    Chunk* c = static_cast<Chunk*>(chunk);
    if (!c) return;
    if (c->kind == AETHER_MEM_DEVICE && capturing(c->stream)) {
        std::lock_guard<std::mutex> lk(g_deferred_mu);
        g_deferred.push_back(c);
        return;
    }
    free_now(c);
}

AG_EXPORT void aether_drain(void) {
    std::vector<Chunk*> keep, now;
    {
        std::lock_guard<std::mutex> lk(g_deferred_mu);
        for (Chunk* c : g_deferred) (capturing(c->stream) ? keep : now).push_back(c);
        g_deferred.swap(keep);
    }
    for (Chunk* c : now) free_now(c);
}

AG_EXPORT int aether_fill(int kind, int dev, void* ptr, size_t bytes, const void* value, size_t width, void* stream) {
    return guarded([&] {
        if (!ptr || (!value && width) || width == 0 || bytes % width)
            throw std::runtime_error("fill: bytes must be a multiple of a non-zero width");
        const unsigned char* v = static_cast<const unsigned char*>(value);
        bool uniform = true;
        for (size_t i = 1; i < width; ++i) uniform = uniform && v[i] == v[0];
        if (kind == AETHER_MEM_CPU || kind == AETHER_MEM_PINNED) {
            if (kind == AETHER_MEM_PINNED && stream) ck(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "sync");
            unsigned char* p = static_cast<unsigned char*>(ptr);
            for (size_t off = 0; off < bytes; off += width) std::memcpy(p + off, v, width);
            return;
        }
        OnDevice d(dev);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (uniform) {
            ck(cudaMemsetAsync(ptr, v[0], bytes, s), "cudaMemsetAsync");
        } else {
            // Non-uniform patterns: seed one copy, then double it with device copies.
            ck(cudaMemcpyAsync(ptr, value, width, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
            size_t done = width;
            unsigned char* p = static_cast<unsigned char*>(ptr);
            while (done < bytes) {
                const size_t n = std::min(done, bytes - done);
                ck(cudaMemcpyAsync(p + done, p, n, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
                done += n;
            }
        }
    });
}

AG_EXPORT int aether_copy(int dst_kind, int dst_dev, void* dst, int src_kind, int src_dev, const void* src,
                          size_t bytes, void* stream) {
    return guarded([&] {
        if (bytes == 0) return;
        if (!dst || !src) throw std::runtime_error("copy: null pointer");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const bool dd = dst_kind == AETHER_MEM_DEVICE, sd = src_kind == AETHER_MEM_DEVICE;
        if (!dd && !sd && dst_kind != AETHER_MEM_PINNED && src_kind != AETHER_MEM_PINNED) {
            std::memcpy(dst, src, bytes);
            return;
        }
        if (dd && sd && dst_dev != src_dev) {
            ck(cudaMemcpyPeerAsync(dst, dst_dev, src, src_dev, bytes, s), "cudaMemcpyPeerAsync");
            return;
        }
        OnDevice d(dd ? dst_dev : src_dev);
        const cudaMemcpyKind k = dd && sd ? cudaMemcpyDeviceToDevice
                                 : dd     ? cudaMemcpyHostToDevice
                                 : sd     ? cudaMemcpyDeviceToHost
                                          : cudaMemcpyHostToHost;
        ck(cudaMemcpyAsync(dst, src, bytes, k, s), "cudaMemcpyAsync");
    });
}

AG_EXPORT int aether_stream_wait(int dev, void* producer, void* consumer) {
    return guarded([&] {
        OnDevice d(dev);
        cudaEvent_t ev;
        ck(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
        cudaError_t e = cudaEventRecord(ev, static_cast<cudaStream_t>(producer));
        if (e == cudaSuccess) e = cudaStreamWaitEvent(static_cast<cudaStream_t>(consumer), ev, 0);
        cudaEventDestroy(ev);
        ck(e, "stream_wait");
    });
}

AG_EXPORT int aether_current_device(int* dev) {
    if (!dev) return fail("current_device: null output pointer");
    const cudaError_t e = cudaGetDevice(dev);
    return e == cudaSuccess ? AETHER_OK : cuda_fail(e, "cudaGetDevice");
}

AG_EXPORT int aether_pointer_device(const void* ptr, int* dev) {
    return guarded([&] {
        if (!ptr || !dev) throw std::runtime_error("pointer_device: null argument");
        cudaPointerAttributes at{};
        ck(cudaPointerGetAttributes(&at, ptr), "cudaPointerGetAttributes");
        if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
            throw std::runtime_error("pointer_device: not a device pointer");
        *dev = at.device;
    });
}

AG_EXPORT int aether_stream_create(int dev, void** stream) {
    return guarded([&] {
        if (!stream) throw std::runtime_error("stream_create: null output pointer");
        OnDevice d(dev);
        cudaStream_t s = nullptr;
        ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        *stream = s;
    });
}

AG_EXPORT void aether_stream_destroy(void* stream) {
    if (stream) cudaStreamDestroy(static_cast<cudaStream_t>(stream));
}

AG_EXPORT int aether_stream_sync(int dev, void* stream) {
    return guarded([&] {
        OnDevice d(dev);
        ck(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
    });
}

// ============================================================================
// Plans
// ============================================================================
AG_EXPORT int aether_plan_create(const char* ir, const AetherLowering* lowering, void** out) {
    return guarded([&] {
        if (!ir || !out) throw std::runtime_error("plan_create: null argument");
        auto P = std::make_unique<PlanObj>();
        P->plan = ag::parse_plan(ir);
        P->low = default_lowering(P->plan);
        if (lowering) {
            if (lowering->block > 0) P->low.block = lowering->block;
            if (lowering->ipt > 0) P->low.ipt = lowering->ipt;
            if (lowering->vec > 0) P->low.vec = lowering->vec;
            if (lowering->contract >= 0) P->low.contract = lowering->contract != 0;
            if (lowering->math >= 0) P->low.math = lowering->math;
            if (lowering->min_blocks > 0) P->low.min_blocks = lowering->min_blocks;
        }
        if (P->low.block % 32 || P->low.block < 32 || P->low.block > 1024)
            throw std::runtime_error("plan_create: block must be a multiple of 32 in [32, 1024]");
        if (P->low.ipt < 1 || P->low.ipt > 8) throw std::runtime_error("plan_create: ipt must be in [1, 8]");
        P->vec = ag::effective_vec(P->plan, P->low);
        if (P->vec != 1 && P->vec != 2 && P->vec != 4) throw std::runtime_error("plan_create: vec must be 1, 2 or 4");
        if (P->low.math == 1 && P->plan.dst_dtype != ag::DType::F64)
            throw std::runtime_error("plan_create: emulated FP64 (math = 1) applies to f64 plans");
        if (P->low.math == 2 && P->plan.dst_dtype == ag::DType::F64)
            throw std::runtime_error("plan_create: the precision form (math = 2) applies to f32 and ff plans");
        if (P->plan.dst_dtype == ag::DType::FF && P->low.math != 2)
            throw std::runtime_error("plan_create: ff destinations are written by the precision form (math = 2)");
        if (P->low.math == 3 && P->plan.dst_dtype != ag::DType::F64)
            throw std::runtime_error("plan_create: FP64-grade triple-float (math = 3) applies to f64 plans");
        if (P->low.math < 0 || P->low.math > 3) throw std::runtime_error("plan_create: math must be 0, 1, 2 or 3");
        P->name = ag::kernel_base(P->plan, ir) + lowering_tag(P->plan, P->low);
        P->source = ag::generate_source(P->plan, P->low, P->name);
        ck(cudaFree(nullptr), "CUDA context");   // make the primary context current
        cudaGetDevice(&P->dev);
        P->compiled = ag::compile_cached(P->source, "plan");
        ck(cudaLibraryLoadData(&P->library, P->compiled.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
           "cudaLibraryLoadData");
        ck(cudaLibraryGetKernel(&P->fv, P->library, (P->name + "_v").c_str()), "cudaLibraryGetKernel");
        ck(cudaLibraryGetKernel(&P->fs, P->library, (P->name + "_s").c_str()), "cudaLibraryGetKernel");
        cudaFuncAttributes fa{};
        ck(cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(P->fv)), "cudaFuncGetAttributes");
        P->registers = fa.numRegs;
        ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&P->blocks_per_sm_v, reinterpret_cast<const void*>(P->fv),
                                                         P->low.block, 0), "occupancy");
        ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&P->blocks_per_sm_s, reinterpret_cast<const void*>(P->fs),
                                                         P->low.block, 0), "occupancy");
        cudaDeviceGetAttribute(&P->sms, cudaDevAttrMultiProcessorCount, P->dev);
        *out = P.release();
    });
}

AG_EXPORT int aether_plan_info(void* plan, AetherPlanInfo* info) {
    return guarded([&] {
        const PlanObj* P = static_cast<const PlanObj*>(plan);
        if (!P || !info) throw std::runtime_error("plan_info: null argument");
        info->hash = P->compiled.hash;
        info->n_operands = P->plan.n_operands;
        info->n_scalars = P->plan.n_scalars;
        info->n_keys = P->plan.n_keys;
        info->dst_comps = P->plan.dst_comps;
        info->dst_dtype = P->plan.dst_dtype == ag::DType::F64 ? 0 : P->plan.dst_dtype == ag::DType::F32 ? 1 : 2;
        info->is_sum = P->plan.wants_sum() ? 1 : 0;
        info->block = P->low.block;
        info->ipt = P->low.ipt;
        info->vec = P->vec;
        info->registers = P->registers;
        info->blocks_per_sm = P->blocks_per_sm_v;
        info->compile_ms = P->compiled.compile_ms;
    });
}

AG_EXPORT int aether_plan_workspace_size(void* plan, uint64_t n, uint64_t* bytes) {
    return guarded([&] {
        const PlanObj* P = static_cast<const PlanObj*>(plan);
        if (!P || !bytes) throw std::runtime_error("plan_workspace_size: null argument");
        *bytes = ws_needed(*P, n);
    });
}

AG_EXPORT int aether_plan_source(void* plan, char* buf, size_t cap, size_t* len) {
    return guarded([&] {
        const PlanObj* P = static_cast<const PlanObj*>(plan);
        if (!P) throw std::runtime_error("plan_source: null plan");
        if (len) *len = P->source.size();
        if (buf && cap) {
            const size_t n = std::min(cap - 1, P->source.size());
            std::memcpy(buf, P->source.data(), n);
            buf[n] = '\0';
        }
    });
}

// Internal (not exported): lets other translation units of the library report
// through aether_last_error.
int ag_internal_fail(const char* message) { return fail(message); }

bool make_args(const PlanObj* P, const AetherLaunch* a, AgArgsHost& k) {
    const ag::Plan& pl = P->plan;
    if (a->n > 0xFFFFFFFFull) throw std::runtime_error("plan_launch: n exceeds the 32-bit sample index");
    if (uint64_t(a->sample_offset) + a->n - 1 > 0xFFFFFFFFull)
        throw std::runtime_error("plan_launch: sample_offset + n exceeds the 32-bit sample index");
    if (int(a->n_operands) < pl.n_operands)
        throw std::runtime_error("plan_launch: plan reads " + std::to_string(pl.n_operands) + " operands, " +
                                 std::to_string(a->n_operands) + " given");
    if (int(a->n_scalars) < pl.n_scalars) throw std::runtime_error("plan_launch: too few scalars");
    if (int(a->n_keys) < pl.n_keys) throw std::runtime_error("plan_launch: too few generator keys");
    k = AgArgsHost{};
    k.n = a->n;
    k.offset = a->sample_offset;
    bool aligned = true;
    if (pl.wants_store()) {
        if (!a->dst) throw std::runtime_error("plan_launch: null destination");
        const int planes = pl.dst_planes();
        if (planes > 1 && a->dst_pitch && a->dst_pitch < a->n)
            throw std::runtime_error("plan_launch: destination pitch smaller than n");
        k.dst = static_cast<char*>(a->dst);
        k.dst_pitch = a->dst_pitch ? a->dst_pitch : a->n;
        const int es = ag::dtype_size(pl.dst_dtype);
        aligned = aligned && (reinterpret_cast<uintptr_t>(a->dst) % 16 == 0) &&
                  (planes == 1 || (k.dst_pitch * es) % 16 == 0);
    }
    for (int i = 0; i < pl.n_operands; ++i) {
        const AetherOperand& o = a->operands[i];
        if (!o.ptr) throw std::runtime_error("plan_launch: operand " + std::to_string(i) + " is null");
        const int comps = pl.operand_comps[size_t(i)];
        const uint64_t pitch = o.pitch ? o.pitch : a->n;
        if (comps > 1 && pitch < a->n)
            throw std::runtime_error("plan_launch: operand " + std::to_string(i) + " pitch smaller than n");
        k.ops[i] = static_cast<const char*>(o.ptr);
        k.pitch[i] = pitch;
        const int es = ag::dtype_size(pl.operand_dtype[size_t(i)]);
        aligned = aligned && (reinterpret_cast<uintptr_t>(o.ptr) % 16 == 0) && (comps == 1 || (pitch * es) % 16 == 0);
    }
    for (int i = 0; i < pl.n_scalars; ++i) {
        if (size_t(i) < pl.scalar_nonneg.size() && pl.scalar_nonneg[size_t(i)] && !(a->scalars[i] >= 0.0))
            throw std::runtime_error("plan_launch: scalar " + std::to_string(i) +
                                     " must be >= 0 (the plan was generated for a non-negative value)");
        k.sc[i] = a->scalars[i];
        k.sch[i] = float(a->scalars[i]);
        k.scl[i] = std::isfinite(k.sch[i]) ? float(a->scalars[i] - double(k.sch[i])) : 0.0f;
    }
    for (int i = 0; i < pl.n_keys; ++i) k.key[i] = a->keys[i];
    return aligned;
}

namespace {

void launch_plan_kernel(const PlanObj& P, AgArgsHost& k, uint64_t n, bool vect, cudaStream_t s) {
    const uint64_t per = chunk_samples(P, vect);
    const uint64_t nch = (n + per - 1) / per;
    const int bps = vect ? P.blocks_per_sm_v : P.blocks_per_sm_s;
    const uint64_t cap = uint64_t(std::max(bps, 1)) * uint64_t(P.sms);
    const unsigned grid = unsigned(std::max<uint64_t>(1, std::min(nch, cap)));
    void* params[] = {&k};
    ck(cudaLaunchKernel(reinterpret_cast<const void*>(vect ? P.fv : P.fs), dim3(grid), dim3(unsigned(P.low.block)),
                        params, 0, s),
       "cudaLaunchKernel");
}

// A default workspace of at least `need` bytes that no launch still running
// on another stream uses (caller holds P.ws_mu). Preference: an entry last
// used on `s` itself, then an idle entry that is large enough, then an idle
// entry grown to `need`, then a new entry. The per-thread default stream is
// one handle for many streams, so it only reuses idle entries.
PlanObj::Workspace& acquire_workspace(PlanObj& P, uint64_t need, cudaStream_t s) {
    auto idle = [](PlanObj::Workspace& w) {
        const cudaError_t e = cudaEventQuery(w.done);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            return false;
        }
        ck(e, "cudaEventQuery(workspace)");
        return true;
    };
    for (PlanObj::Workspace& w : P.ws)
        if (w.ordered && w.last_stream == s && s != cudaStreamPerThread && w.bytes >= need) return w;
    PlanObj::Workspace* grow = nullptr;
    for (PlanObj::Workspace& w : P.ws) {
        if (!idle(w)) continue;
        if (w.bytes >= need) return w;
        if (!grow) grow = &w;
    }
    if (!grow) {
        P.ws.emplace_back();
        grow = &P.ws.back();
        ck(cudaEventCreateWithFlags(&grow->done, cudaEventDisableTiming), "cudaEventCreate(workspace)");
    }
    if (grow->ptr) ck(cudaFree(grow->ptr), "cudaFree(workspace)");
    grow->ptr = nullptr;
    grow->bytes = 0;
    ck(cudaMalloc(&grow->ptr, need), "cudaMalloc(workspace)");
    grow->bytes = need;
    return *grow;
}

}  // namespace

AG_EXPORT int aether_plan_launch(void* plan, const AetherLaunch* a, void* stream) {
    return guarded([&] {
        PlanObj* P = static_cast<PlanObj*>(plan);
        if (!P || !a) throw std::runtime_error("plan_launch: null argument");
        const ag::Plan& pl = P->plan;
        if (a->n == 0) return;
        AgArgsHost k;
        const bool aligned = make_args(P, a, k);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const bool vect = aligned && P->vec > 1;
        if (pl.wants_sum()) {
            if (!a->reduce_out) throw std::runtime_error("plan_launch: sum plan without reduce_out");
            k.red = a->reduce_out;
            const uint64_t need = ws_needed(*P, a->n);
            if (a->workspace) {
                if (a->workspace_bytes < need)
                    throw std::runtime_error("plan_launch: workspace of " + std::to_string(a->workspace_bytes) +
                                             " bytes, " + std::to_string(need) + " needed");
                k.ws = static_cast<char*>(a->workspace);
                k.ws_bytes = a->workspace_bytes;
            } else {
                if (capturing(s))
                    throw std::runtime_error(
                        "plan_launch: a sum plan recorded into a CUDA graph needs its own workspace "
                        "(args->workspace, aether_plan_workspace_size bytes) or aether_plan_launch_noalloc");
                std::unique_lock<std::mutex> lk(P->ws_mu);
                PlanObj::Workspace& w = acquire_workspace(*P, need, s);
                k.ws = static_cast<char*>(w.ptr);
                k.ws_bytes = w.bytes;
                ck(cudaMemsetAsync(k.ws, 0, 16, s), "cudaMemsetAsync(counter)");
                launch_plan_kernel(*P, k, a->n, vect, s);
                // the entry is busy until this event completes, except for
                // later launches on the same stream, which run after it
                ck(cudaEventRecord(w.done, s), "cudaEventRecord(workspace)");
                w.last_stream = s;
                w.ordered = s != cudaStreamPerThread;
                return;
            }
            ck(cudaMemsetAsync(k.ws, 0, 16, s), "cudaMemsetAsync(counter)");
        }
        launch_plan_kernel(*P, k, a->n, vect, s);
    });
}

// ============================================================================
// Batches: many plan launches as one persistent kernel over a device work list
// ============================================================================
namespace {

void batch_enqueue(BatchObj* B, cudaStream_t s) {
    if (B->total_tiles == 0) return;
    const unsigned grid = batch_grid(*B, B->total_tiles);
    void* items = B->dev_items;
    int n = B->n_items;
    uint64_t tiles = B->total_tiles;
    void* params[] = {&items, &n, &tiles};
    ck(cudaLaunchKernel(reinterpret_cast<const void*>(B->kernel), dim3(grid), dim3(unsigned(B->block)), params, 0, s),
       "cudaLaunchKernel(batch)");
}

}  // namespace

AG_EXPORT int aether_batch_create(void* const* plans, int n_plans, const AetherLowering* lowering, void** out) {
    return guarded([&] {
        if (!plans || n_plans <= 0 || !out) throw std::runtime_error("batch_create: no plans");
        auto B = std::make_unique<BatchObj>();
        if (lowering && lowering->block > 0) B->block = lowering->block;
        if (lowering && lowering->ipt > 0) B->ipt = lowering->ipt;
        if (B->block % 32 || B->block < 32 || B->block > 1024)
            throw std::runtime_error("batch_create: block must be a multiple of 32 in [32, 1024]");
        if (B->ipt < 1 || B->ipt > 8) throw std::runtime_error("batch_create: ipt must be in [1, 8]");
        const int min_blocks = lowering && lowering->min_blocks > 0 ? lowering->min_blocks : 0;
        if (min_blocks > 32) throw std::runtime_error("batch_create: min_blocks above 32");
        std::vector<const ag::Plan*> ps;
        std::vector<ag::Lowering> lows;
        std::string key = std::to_string(B->block) + "/" + std::to_string(B->ipt) + "/" + std::to_string(min_blocks);
        for (int p = 0; p < n_plans; ++p) {
            PlanObj* P = static_cast<PlanObj*>(plans[p]);
            if (!P) throw std::runtime_error("batch_create: null plan");
            if (P->plan.wants_sum()) throw std::runtime_error("batch_create: sum plans cannot join a batch");
            B->plans.push_back(P);
            ps.push_back(&P->plan);
            ag::Lowering l = P->low;
            l.block = B->block;
            l.ipt = B->ipt;
            lows.push_back(l);
            B->vecs.push_back(ag::effective_vec(P->plan, l));
            key += "|" + P->name + "/" + std::to_string(l.math) + "/" + std::to_string(l.contract);
        }
        char nm[40];
        std::snprintf(nm, sizeof nm, "ag_batch_%08x", unsigned(ag::fnv1a(key) & 0xffffffffu));
        B->name = nm;
        B->source = ag::generate_batch_source(ps, lows, B->block, B->ipt, B->name, min_blocks);
        ck(cudaFree(nullptr), "CUDA context");
        B->compiled = ag::compile_cached(B->source, "batch");
        ck(cudaLibraryLoadData(&B->library, B->compiled.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
           "cudaLibraryLoadData(batch)");
        ck(cudaLibraryGetKernel(&B->kernel, B->library, B->name.c_str()), "cudaLibraryGetKernel(batch)");
        cudaFuncAttributes fa{};
        ck(cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(B->kernel)), "cudaFuncGetAttributes");
        B->registers = fa.numRegs;
        ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&B->blocks_per_sm, reinterpret_cast<const void*>(B->kernel),
                                                         B->block, 0), "occupancy");
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, dev);
        *out = B.release();
    });
}

AG_EXPORT int aether_batch_set_items(void* batch, const AetherBatchItem* items, int n_items, void* stream) {
    return guarded([&] {
        BatchObj* B = static_cast<BatchObj*>(batch);
        if (!B || (!items && n_items)) throw std::runtime_error("batch_set_items: null argument");
        if (n_items < 0) throw std::runtime_error("batch_set_items: negative item count");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (size_t(n_items) > B->cap_items) {
            size_t cap = std::max<size_t>(size_t(n_items), B->cap_items * 2);
            if (B->host_items) cudaFreeHost(B->host_items);
            if (B->dev_items) cudaFree(B->dev_items);
            B->host_items = nullptr;
            B->dev_items = nullptr;
            B->cap_items = 0;
            void* h = nullptr;
            ck(cudaMallocHost(&h, cap * sizeof(AgItemHost)), "cudaMallocHost(work list)");
            B->host_items = static_cast<AgItemHost*>(h);
            ck(cudaMalloc(&B->dev_items, cap * sizeof(AgItemHost)), "cudaMalloc(work list)");
            B->cap_items = cap;
        }
        uint64_t tiles = 0;
        for (int i = 0; i < n_items; ++i) {
            const AetherBatchItem& it = items[i];
            if (it.plan < 0 || size_t(it.plan) >= B->plans.size())
                throw std::runtime_error("batch_set_items: item " + std::to_string(i) + " names plan " +
                                         std::to_string(it.plan) + " of " + std::to_string(B->plans.size()));
            AgItemHost& h = B->host_items[i];
            h = AgItemHost{};
            if (it.args.n > 0 && !make_args(B->plans[size_t(it.plan)], &it.args, h.a))
                throw std::runtime_error("batch_set_items: item " + std::to_string(i) +
                                         " has a plane that is not 16-byte aligned");
            h.tile0 = tiles;
            h.plan = it.plan;
            const uint64_t per = batch_tile_samples(*B, it.plan);
            tiles += (it.args.n + per - 1) / per;
        }
        B->n_items = n_items;
        B->total_tiles = tiles;
        if (n_items) {
            ck(cudaMemcpyAsync(B->dev_items, B->host_items, size_t(n_items) * sizeof(AgItemHost),
                               cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(work list)");
            ck(cudaStreamSynchronize(s), "cudaStreamSynchronize(work list)");   // the staging buffer is reused
        }
    });
}

AG_EXPORT int aether_batch_launch(void* batch, void* stream) {
    return guarded([&] {
        BatchObj* B = static_cast<BatchObj*>(batch);
        if (!B) throw std::runtime_error("batch_launch: null batch");
        batch_enqueue(B, static_cast<cudaStream_t>(stream));
    });
}

AG_EXPORT int aether_batch_capture(void* batch, void* stream) {
    return guarded([&] {
        BatchObj* B = static_cast<BatchObj*>(batch);
        if (!B) throw std::runtime_error("batch_capture: null batch");
        if (!stream) throw std::runtime_error("batch_capture: capture needs a non-default stream");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (B->exec) cudaGraphExecDestroy(B->exec);
        if (B->graph) cudaGraphDestroy(B->graph);
        B->exec = nullptr;
        B->graph = nullptr;
        ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        try {
            batch_enqueue(B, s);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        ck(cudaStreamEndCapture(s, &B->graph), "cudaStreamEndCapture");
        ck(cudaGraphInstantiate(&B->exec, B->graph, 0), "cudaGraphInstantiate");
        B->graph_tiles = B->total_tiles;
        B->graph_items = B->n_items;
    });
}

AG_EXPORT int aether_batch_replay(void* batch, void* stream) {
    return guarded([&] {
        BatchObj* B = static_cast<BatchObj*>(batch);
        if (!B || !B->exec) throw std::runtime_error("batch_replay: nothing captured");
        if (B->graph_tiles != B->total_tiles || B->graph_items != B->n_items)
            throw std::runtime_error("batch_replay: the work list changed its tiling since the capture; capture again");
        ck(cudaGraphLaunch(B->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch");
    });
}

AG_EXPORT int aether_batch_info(void* batch, AetherBatchInfo* info) {
    return guarded([&] {
        const BatchObj* B = static_cast<const BatchObj*>(batch);
        if (!B || !info) throw std::runtime_error("batch_info: null argument");
        info->hash = B->compiled.hash;
        info->n_plans = int(B->plans.size());
        info->n_items = B->n_items;
        info->total_tiles = B->total_tiles;
        info->block = B->block;
        info->ipt = B->ipt;
        info->registers = B->registers;
        info->blocks_per_sm = B->blocks_per_sm;
        info->compile_ms = B->compiled.compile_ms;
    });
}

AG_EXPORT void aether_batch_release(void* batch) {
    BatchObj* B = static_cast<BatchObj*>(batch);
    if (!B) return;
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    if (B->host_items) cudaFreeHost(B->host_items);
    if (B->dev_items) cudaFree(B->dev_items);
    if (B->library) cudaLibraryUnload(B->library);
    delete B;
}

AG_EXPORT int aether_plan_launch_many(void* const* plans, const AetherLaunch* args, int count, void* stream) {
    if (count < 0 || (count && (!plans || !args))) return fail("plan_launch_many: bad arguments");
    for (int i = 0; i < count; ++i) {
        const int rc = aether_plan_launch(plans[i], &args[i], stream);
        if (rc != AETHER_OK) return rc;
    }
    return AETHER_OK;
}

AG_EXPORT int aether_plan_generate(const char* ir, const AetherLowering* lowering, char* buf, size_t cap,
                                   size_t* len) {
    return guarded([&] {
        if (!ir) throw std::runtime_error("plan_generate: null ir");
        const ag::Plan plan = ag::parse_plan(ir);
        ag::Lowering low = default_lowering(plan);
        if (lowering) {
            if (lowering->block > 0) low.block = lowering->block;
            if (lowering->ipt > 0) low.ipt = lowering->ipt;
            if (lowering->vec > 0) low.vec = lowering->vec;
            if (lowering->contract >= 0) low.contract = lowering->contract != 0;
            if (lowering->math >= 0) low.math = lowering->math;
            if (lowering->min_blocks > 0) low.min_blocks = lowering->min_blocks;
        }
        const std::string src = ag::generate_source(plan, low, ag::kernel_base(plan, ir) + lowering_tag(plan, low));
        if (len) *len = src.size();
        if (buf && cap) {
            const size_t n = std::min(cap - 1, src.size());
            std::memcpy(buf, src.data(), n);
            buf[n] = '\0';
        }
    });
}

AG_EXPORT int aether_rtc_header_count(void) { return ag::payload_count(); }

AG_EXPORT int aether_rtc_header(int index, const char** name, const char** source) {
    return guarded([&] {
        if (!name || !source) throw std::runtime_error("rtc_header: null output pointer");
        if (!ag::payload_header(index, name, source))
            throw std::runtime_error("rtc_header: index " + std::to_string(index) + " of " +
                                     std::to_string(ag::payload_count()));
    });
}

AG_EXPORT uint64_t aether_rtc_digest(void) { return ag::payload_digest(); }

AG_EXPORT int aether_nvrtc_check(const char* source, const char* arch) {
    return guarded([&] {
        if (!source || !arch) throw std::runtime_error("nvrtc_check: null argument");
        ag::compile_for_arch(source, arch);
    });
}

AG_EXPORT int aether_plan_cache_key(const char* source, const char* arch, const char* tag, int header_index,
                                    const char* header_source, uint64_t* key) {
    return guarded([&] {
        if (!source || !arch || !tag || !key) throw std::runtime_error("plan_cache_key: null argument");
        if (header_index >= ag::payload_count())
            throw std::runtime_error("plan_cache_key: header index " + std::to_string(header_index) + " of " +
                                     std::to_string(ag::payload_count()));
        int major = 0, minor = 0;
        nvrtcVersion(&major, &minor);
        *key = ag::cache_key(source, arch, tag, major, minor, header_index, header_source);
    });
}

AG_EXPORT int aether_rtc_compile(const char* source, const char* arch, const char* const* options, int n_options,
                                 void* cubin, size_t cap, size_t* len) {
    return guarded([&] {
        if (!source || !arch || !len || (n_options > 0 && !options))
            throw std::runtime_error("rtc_compile: null argument");
        std::vector<std::string> opts;
        for (int i = 0; i < n_options; ++i) opts.push_back(options[i] ? options[i] : "");
        const std::string bin = ag::compile_with_payload(source, arch, opts);
        *len = bin.size();
        if (cubin) {
            if (cap < bin.size())
                throw std::runtime_error("rtc_compile: buffer of " + std::to_string(cap) + " bytes, " +
                                         std::to_string(bin.size()) + " needed");
            std::memcpy(cubin, bin.data(), bin.size());
        }
    });
}

AG_EXPORT void aether_plan_release(void* plan) {
    PlanObj* P = static_cast<PlanObj*>(plan);
    if (!P) return;
    for (PlanObj::Workspace& w : P->ws) {
        if (w.done) cudaEventSynchronize(w.done);
        if (w.ptr) cudaFree(w.ptr);
        if (w.done) cudaEventDestroy(w.done);
    }
    if (P->library) cudaLibraryUnload(P->library);
    delete P;
}
