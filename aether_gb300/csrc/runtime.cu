// runtime.cu -- aether_runtime_eval: the runtime-typed strided evaluator.
//
// Follows eval/Runtime.h:73-300 of the reference: out = op(a, b, scalar) for
// every element of out's logical shape (rank <= 6, double or float), each
// operand addressed through its own element strides, the flat element index
// running row-major over out's extents. Ops: Assign (copy or double<->float
// cast), Add, Sub, Scale (s*a), AddScaled (a + s*b), SubScaled (a - s*b); the
// scalar is rounded to the input type first (Runtime.h:221). Every add and
// multiply rounds on its own (no contraction), so results equal the
// reference's host loop bit for bit.
//
// Two kernels per (op, input type, output type):
//  * contiguous: all operands row-major with no gaps -> flat indices,
//    four elements per thread with 128-bit accesses when every base is
//    16-byte aligned;
//  * strided: each thread decodes its first flat index into a multi-index
//    with invariant-divisor division (ag_fastdiv.cuh), then walks four
//    consecutive elements by carrying the multi-index.
// Both are grid-stride loops over a grid of a few CTAs per SM.

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "aether_gb300.h"
#include "ag_fastdiv.cuh"

int ag_internal_fail(const char* message);

namespace {

constexpr int kRun = 4;        // elements per thread per step
constexpr int kBlock = 256;

struct RtDesc {
    const void* a;
    const void* b;
    void* o;
    int rank;
    uint32_t total;
    AgFastDiv ext[AETHER_RT_RANK_CAP];
    int64_t sa[AETHER_RT_RANK_CAP], sb[AETHER_RT_RANK_CAP], so[AETHER_RT_RANK_CAP];
    double scalar;
};

__device__ __forceinline__ double rt_add(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ float rt_add(float x, float y) { return __fadd_rn(x, y); }
__device__ __forceinline__ double rt_sub(double x, double y) { return __dsub_rn(x, y); }
__device__ __forceinline__ float rt_sub(float x, float y) { return __fsub_rn(x, y); }
__device__ __forceinline__ double rt_mul(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ float rt_mul(float x, float y) { return __fmul_rn(x, y); }
template <class TO>
__device__ __forceinline__ TO rt_cast(double x);
template <>
__device__ __forceinline__ double rt_cast<double>(double x) { return x; }
template <>
__device__ __forceinline__ float rt_cast<float>(double x) { return __double2float_rn(x); }
template <class TO>
__device__ __forceinline__ TO rt_cast(float x) { return TO(x); }

template <int OP, class TI, class TO>
__device__ __forceinline__ TO rt_apply(TI a, TI b, TI s) {
    if (OP == AETHER_RT_ASSIGN) return rt_cast<TO>(a);
    if (OP == AETHER_RT_ADD) return TO(rt_add(a, b));
    if (OP == AETHER_RT_SUB) return TO(rt_sub(a, b));
    if (OP == AETHER_RT_SCALE) return TO(rt_mul(s, a));
    if (OP == AETHER_RT_ADD_SCALED) return TO(rt_add(a, rt_mul(s, b)));
    return TO(rt_sub(a, rt_mul(s, b)));
}

__host__ __device__ constexpr bool uses_b(int op) {
    return op == AETHER_RT_ADD || op == AETHER_RT_SUB || op == AETHER_RT_ADD_SCALED || op == AETHER_RT_SUB_SCALED;
}

// 4 consecutive elements at 16-byte aligned addresses.
template <class T>
struct Quad;
template <>
struct Quad<double> {
    static __device__ __forceinline__ void load(const double* p, double v[4]) {
        const double2 x = __ldcs(reinterpret_cast<const double2*>(p));
        const double2 y = __ldcs(reinterpret_cast<const double2*>(p) + 1);
        v[0] = x.x, v[1] = x.y, v[2] = y.x, v[3] = y.y;
    }
    static __device__ __forceinline__ void store(double* p, const double v[4]) {
        __stcs(reinterpret_cast<double2*>(p), make_double2(v[0], v[1]));
        __stcs(reinterpret_cast<double2*>(p) + 1, make_double2(v[2], v[3]));
    }
};
template <>
struct Quad<float> {
    static __device__ __forceinline__ void load(const float* p, float v[4]) {
        const float4 x = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w;
    }
    static __device__ __forceinline__ void store(float* p, const float v[4]) {
        __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    }
};

template <int OP, class TI, class TO, bool VEC>
__global__ void __launch_bounds__(kBlock) rt_contiguous(RtDesc d) {
    const TI* A = static_cast<const TI*>(d.a);
    const TI* B = static_cast<const TI*>(d.b);
    TO* O = static_cast<TO*>(d.o);
    const TI s = TI(d.scalar);
    const uint64_t total = d.total;
    const uint64_t step = uint64_t(gridDim.x) * kBlock * kRun;
    for (uint64_t base = (uint64_t(blockIdx.x) * kBlock + threadIdx.x) * kRun; base < total; base += step) {
        if (VEC && base + kRun <= total) {
            TI va[4], vb[4] = {TI(0), TI(0), TI(0), TI(0)};
            TO vo[4];
            Quad<TI>::load(A + base, va);
            if (uses_b(OP)) Quad<TI>::load(B + base, vb);
#pragma unroll
            for (int j = 0; j < 4; ++j) vo[j] = rt_apply<OP, TI, TO>(va[j], vb[j], s);
            Quad<TO>::store(O + base, vo);
        } else {
            for (int j = 0; j < kRun && base + j < total; ++j) {
                const TI x = A[base + j];
                const TI y = uses_b(OP) ? B[base + j] : TI(0);
                O[base + j] = rt_apply<OP, TI, TO>(x, y, s);
            }
        }
    }
}

template <int OP, class TI, class TO>
__global__ void __launch_bounds__(kBlock) rt_strided(RtDesc d) {
    const TI* A = static_cast<const TI*>(d.a);
    const TI* B = static_cast<const TI*>(d.b);
    TO* O = static_cast<TO*>(d.o);
    const TI s = TI(d.scalar);
    const int rank = d.rank;
    const uint64_t total = d.total;
    const uint64_t step = uint64_t(gridDim.x) * kBlock * kRun;
    for (uint64_t base = (uint64_t(blockIdx.x) * kBlock + threadIdx.x) * kRun; base < total; base += step) {
        uint32_t idx[AETHER_RT_RANK_CAP];
        int64_t oa = 0, ob = 0, oo = 0;
        uint32_t rem = uint32_t(base);
        for (int k = rank - 1; k >= 0; --k) {
            uint32_t q, r;
            ag_fastdiv_divmod(rem, d.ext[k], q, r);
            idx[k] = r;
            rem = q;
            oa += int64_t(r) * d.sa[k];
            if (uses_b(OP)) ob += int64_t(r) * d.sb[k];
            oo += int64_t(r) * d.so[k];
        }
        for (int j = 0; j < kRun && base + j < total; ++j) {
            const TI x = A[oa];
            const TI y = uses_b(OP) ? B[ob] : TI(0);
            O[oo] = rt_apply<OP, TI, TO>(x, y, s);
            // next flat index: carry the multi-index
            for (int k = rank - 1; k >= 0; --k) {
                oa += d.sa[k];
                if (uses_b(OP)) ob += d.sb[k];
                oo += d.so[k];
                if (++idx[k] < d.ext[k].d) break;
                idx[k] = 0;
                oa -= int64_t(d.ext[k].d) * d.sa[k];
                if (uses_b(OP)) ob -= int64_t(d.ext[k].d) * d.sb[k];
                oo -= int64_t(d.ext[k].d) * d.so[k];
            }
        }
    }
}

template <int OP, class TI, class TO>
cudaError_t rt_launch(const RtDesc& d, bool contiguous, bool vec, cudaStream_t s) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t threads = (uint64_t(d.total) + kRun - 1) / kRun;
    const uint64_t want = (threads + kBlock - 1) / kBlock;
    const unsigned grid = unsigned(want < uint64_t(sms) * 8 ? (want ? want : 1) : uint64_t(sms) * 8);
    if (contiguous && vec) rt_contiguous<OP, TI, TO, true><<<grid, kBlock, 0, s>>>(d);
    else if (contiguous) rt_contiguous<OP, TI, TO, false><<<grid, kBlock, 0, s>>>(d);
    else rt_strided<OP, TI, TO><<<grid, kBlock, 0, s>>>(d);
    return cudaGetLastError();
}

template <class TI, class TO>
cudaError_t rt_dispatch_op(int op, const RtDesc& d, bool contiguous, bool vec, cudaStream_t s) {
    switch (op) {
    case AETHER_RT_ASSIGN: return rt_launch<AETHER_RT_ASSIGN, TI, TO>(d, contiguous, vec, s);
    case AETHER_RT_ADD: return rt_launch<AETHER_RT_ADD, TI, TO>(d, contiguous, vec, s);
    case AETHER_RT_SUB: return rt_launch<AETHER_RT_SUB, TI, TO>(d, contiguous, vec, s);
    case AETHER_RT_SCALE: return rt_launch<AETHER_RT_SCALE, TI, TO>(d, contiguous, vec, s);
    case AETHER_RT_ADD_SCALED: return rt_launch<AETHER_RT_ADD_SCALED, TI, TO>(d, contiguous, vec, s);
    default: return rt_launch<AETHER_RT_SUB_SCALED, TI, TO>(d, contiguous, vec, s);
    }
}

bool is_f64(const AetherRuntimeView& v) { return v.dtype_code == 2 && v.dtype_bits == 64 && v.dtype_lanes == 1; }
bool is_f32(const AetherRuntimeView& v) { return v.dtype_code == 2 && v.dtype_bits == 32 && v.dtype_lanes == 1; }
bool same_dtype(const AetherRuntimeView& x, const AetherRuntimeView& y) {
    return x.dtype_code == y.dtype_code && x.dtype_bits == y.dtype_bits && x.dtype_lanes == y.dtype_lanes;
}
bool same_shape(const AetherRuntimeView& x, const AetherRuntimeView& y) {
    if (x.rank != y.rank) return false;
    for (int k = 0; k < x.rank; ++k)
        if (x.extents[k] != y.extents[k]) return false;
    return true;
}
bool row_major(const AetherRuntimeView& v) {
    int64_t want = 1;
    for (int k = v.rank - 1; k >= 0; --k) {
        if (v.extents[k] != 1 && v.strides[k] != want) return false;
        want *= v.extents[k];
    }
    return true;
}
bool on_device(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int rt_fail(uint64_t size, const std::string& detail) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) cudaGetLastError();
    const std::string m = "aether::eval::runtimeEval failed on cuda:" + std::to_string(dev) + ", size=" +
                          std::to_string(size) + " bytes (" + detail + ")";
    return ag_internal_fail(m.c_str());
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int aether_runtime_eval(int op, const AetherRuntimeView* a,
                                                                         const AetherRuntimeView* b,
                                                                         const AetherRuntimeView* out, double scalar,
                                                                         void* stream) {
    if (op < AETHER_RT_ASSIGN || op > AETHER_RT_SUB_SCALED) return rt_fail(0, "unknown op");
    if (!a || !out) return rt_fail(0, "null view");
    const bool ub = uses_b(op);
    if (ub && !b) return rt_fail(0, "the op reads b but b is null");
    for (const AetherRuntimeView* v : {a, ub ? b : a, out})
        if (v->rank < 0 || v->rank > AETHER_RT_RANK_CAP) return rt_fail(0, "rank above the cap of 6");
    if (!same_shape(*a, *out)) return rt_fail(0, "shape mismatch: a vs out");
    if (ub && !same_shape(*b, *out)) return rt_fail(0, "shape mismatch: b vs out");
    if (!is_f32(*a) && !is_f64(*a)) return rt_fail(0, "unsupported input dtype (v1: double/float only)");
    if (!is_f32(*out) && !is_f64(*out)) return rt_fail(0, "unsupported output dtype (v1: double/float only)");
    if (op != AETHER_RT_ASSIGN) {
        if (!same_dtype(*a, *out)) return rt_fail(0, "dtype mismatch: a vs out (only Assign performs a cast)");
        if (ub && !same_dtype(*b, *out)) return rt_fail(0, "dtype mismatch: b vs out");
    }
    uint64_t total = 1;
    for (int k = 0; k < out->rank; ++k) {
        if (out->extents[k] < 0) return rt_fail(0, "negative extent");
        total *= uint64_t(out->extents[k]);
        if (total > 0xFFFFFFFFull) break;
    }
    for (const AetherRuntimeView* v : {a, ub ? b : a, out})
        for (int k = 0; k < v->rank; ++k)
            if (v->strides[k] < 0) return rt_fail(0, "negative strides are not addressable");
    if (total == 0) return AETHER_OK;
    if (total > 0xFFFFFFFFull) return rt_fail(total, "flat element count exceeds the offset_t addressable maximum");
    if (!a->data || !out->data || (ub && !b->data)) return rt_fail(0, "null data pointer");
    if (!on_device(a->data) || !on_device(out->data) || (ub && !on_device(b->data)))
        return rt_fail(0, "operands must be device memory (this engine has no host path)");

    RtDesc d{};
    d.a = a->data;
    d.b = ub ? b->data : nullptr;
    d.o = out->data;
    d.rank = out->rank;
    d.total = uint32_t(total);
    d.scalar = scalar;
    for (int k = 0; k < d.rank; ++k) {
        d.ext[k] = ag_fastdiv_make(uint32_t(out->extents[k]));
        d.sa[k] = a->strides[k];
        d.sb[k] = ub ? b->strides[k] : 0;
        d.so[k] = out->strides[k];
    }
    const bool contiguous = row_major(*a) && row_major(*out) && (!ub || row_major(*b));
    auto aligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    const bool vec = contiguous && aligned(d.a) && aligned(d.o) && (!ub || aligned(d.b));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (is_f64(*a) && is_f64(*out)) e = rt_dispatch_op<double, double>(op, d, contiguous, vec, s);
    else if (is_f32(*a) && is_f32(*out)) e = rt_dispatch_op<float, float>(op, d, contiguous, vec, s);
    else if (is_f64(*a)) e = rt_launch<AETHER_RT_ASSIGN, double, float>(d, contiguous, vec, s);
    else e = rt_launch<AETHER_RT_ASSIGN, float, double>(d, contiguous, vec, s);
    if (e != cudaSuccess) return rt_fail(total, std::string("launch: ") + cudaGetErrorString(e));
    return AETHER_OK;
}
