// ag_device.cuh -- device runtime of the generated plan kernels.
//
// Self-contained (no CUDA or C++ standard headers) so the same text compiles
// under NVRTC for the generated kernels and under nvcc for the prebuilt ones.
// Contents: the launch argument block, Philox4x32-10 and the distribution
// conversions (random/detail/Philox.h:95-133, random/detail/Backend.h:75-236),
// the math facade the generated code calls (math/detail/MathDispatch.h:54-112),
// vector loads/stores per component plane, and the compensated-sum primitives
// (accum/TwoSum.h:86-155, accum/atomic.h:141-258).
#pragma once

typedef unsigned int ag_u32;
typedef unsigned long long ag_u64;
typedef long long ag_i64;

#define AG_MAX_OPS 16
#define AG_MAX_SC 16
#define AG_MAX_KEYS 8

// Launch argument block, passed by value. Mirrors AetherLaunch in
// include/aether_gb300.h after host-side validation.
struct AgArgs {
    ag_u64 n;                     // samples
    ag_u32 offset;                // global sample id of sample 0 (Philox position)
    ag_u32 flags;
    char* dst;                    // plane 0 of the destination
    ag_u64 dst_pitch;             // elements between planes
    const char* ops[AG_MAX_OPS];  // plane 0 of each operand
    ag_u64 pitch[AG_MAX_OPS];
    double sc[AG_MAX_SC];         // runtime scalars
    float sch[AG_MAX_SC];         // the same scalars split as double-float (hi, lo) pairs,
    float scl[AG_MAX_SC];         // for plans lowered to emulated FP64
    ag_u64 key[AG_MAX_KEYS];      // generator keys of random leaves
    double* red;                  // sum plans: (hi, comp) result
    char* ws;                     // sum plans: counter + per-chunk partials
    ag_u64 ws_bytes;
};
static_assert(sizeof(AgArgs) == 632, "AgArgs layout must match the host image in abi.cpp");

namespace ag {

// ---------------------------------------------------------------------------
// Philox4x32-10, cuRAND block layout (random/detail/Philox.h:95-133).
// ---------------------------------------------------------------------------
struct q4 {
    ag_u32 x, y, z, w;
};

__device__ __forceinline__ q4 philox(q4 c, ag_u32 kx, ag_u32 ky) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            kx += 0x9E3779B9u;
            ky += 0xBB67AE85u;
        }
        const ag_u32 hi0 = __umulhi(0xD2511F53u, c.x);
        const ag_u32 lo0 = 0xD2511F53u * c.x;
        const ag_u32 hi1 = __umulhi(0xCD9E8D57u, c.z);
        const ag_u32 lo1 = 0xCD9E8D57u * c.z;
        c = q4{hi1 ^ c.y ^ kx, lo1, hi0 ^ c.w ^ ky, lo0};
    }
    return c;
}

// The block owned by (seed, global, counter) (random/detail/Backend.h:136-150).
__device__ __forceinline__ q4 philox_block(ag_u64 seed, ag_u32 global, ag_u32 counter) {
    return philox(q4{counter, 0u, global, 0u}, (ag_u32)seed, (ag_u32)(seed >> 32));
}

// Word -> real conversions (Backend.h:123-157). Each is an exact scaling plus
// at most one rounding, spelled with explicit round-to-nearest operations so
// no contraction can change them.
__device__ __forceinline__ double u01_f64(ag_u32 w) {
    return __dadd_rn(__dmul_rn((double)w, 2.3283064365386963e-10), 1.1641532182693481e-10);
}
__device__ __forceinline__ float u01_f32(ag_u32 w) {
    return __fmul_rn((float)(((w >> 9) << 1) | 1u), 5.9604645e-8f);
}
__device__ __forceinline__ double u01hq_f64(ag_u32 x, ag_u32 y) {
    const ag_u64 z = (ag_u64)x ^ ((ag_u64)y << 21);
    return __dadd_rn(__dmul_rn((double)z, 1.1102230246251565e-16), 5.5511151231257827e-17);
}

// Distribution salts (random/detail/DistributionLeaf.h:117,184,249,313,373).
#define AG_SALT_UNIFORM 0x243F6A8885A308D3ULL
#define AG_SALT_NORMAL 0x13198A2E03707344ULL
#define AG_SALT_LOGNORMAL 0xA4093822299F31D0ULL
#define AG_SALT_EXPONENTIAL 0x082EFA98EC4E6C89ULL
#define AG_SALT_BERNOULLI 0x452821E638D01377ULL

// ---------------------------------------------------------------------------
// Math facade, native pipes. Double: CUDA's correctly rounded sqrt/division
// and its FP64 library functions; rsqrt is 1/sqrt(x) with both steps correctly
// rounded, the host spelling of math/root.h:64-76, so it is bit-exact with the
// reference's CPU path. Float: the full-precision float functions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f_sqrt(double x) { return __dsqrt_rn(x); }
__device__ __forceinline__ float f_sqrt(float x) { return __fsqrt_rn(x); }
__device__ __forceinline__ double f_rsqrt(double x) { return __ddiv_rn(1.0, __dsqrt_rn(x)); }
__device__ __forceinline__ float f_rsqrt(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }
__device__ __forceinline__ double f_abs(double x) { return fabs(x); }
__device__ __forceinline__ float f_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double f_sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
__device__ __forceinline__ float f_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ double f_neg(double x) { return -x; }
__device__ __forceinline__ float f_neg(float x) { return -x; }

#define AG_UNARY(NAME, DFN, FFN)                                              \
    __device__ __forceinline__ double f_##NAME(double x) { return DFN(x); } \
    __device__ __forceinline__ float f_##NAME(float x) { return FFN(x); }
AG_UNARY(exp, exp, expf)
AG_UNARY(expm1, expm1, expm1f)
AG_UNARY(exp2, exp2, exp2f)
AG_UNARY(log, log, logf)
AG_UNARY(log1p, log1p, log1pf)
AG_UNARY(log2, log2, log2f)
AG_UNARY(log10, log10, log10f)
AG_UNARY(sin, sin, sinf)
AG_UNARY(cos, cos, cosf)
AG_UNARY(tan, tan, tanf)
AG_UNARY(asin, asin, asinf)
AG_UNARY(acos, acos, acosf)
AG_UNARY(atan, atan, atanf)
AG_UNARY(tanh, tanh, tanhf)
AG_UNARY(sinh, sinh, sinhf)
AG_UNARY(cosh, cosh, coshf)
AG_UNARY(floor, floor, floorf)
AG_UNARY(ceil, ceil, ceilf)
AG_UNARY(trunc, trunc, truncf)
AG_UNARY(cbrt, cbrt, cbrtf)
AG_UNARY(erf, erf, erff)
#undef AG_UNARY

#define AG_BINARY(NAME, DFN, FFN)                                                               \
    __device__ __forceinline__ double f_##NAME(double a, double b) { return DFN(a, b); }      \
    __device__ __forceinline__ float f_##NAME(float a, float b) { return FFN(a, b); }
AG_BINARY(pow, pow, powf)
AG_BINARY(min, fmin, fminf)
AG_BINARY(max, fmax, fmaxf)
AG_BINARY(atan2, atan2, atan2f)
AG_BINARY(hypot, hypot, hypotf)
#undef AG_BINARY

// Exact-rounding arithmetic (the -fmad=false spelling the reference's bit
// identity builds use) and the contracted spelling.
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }

// Box-Muller, first normal only (Backend.h:209-236): all four words for
// double, two for float.
__device__ __forceinline__ double normal_f64(ag_u64 seed, ag_u32 g, ag_u32 c) {
    const q4 x = philox_block(seed, g, c);
    const double u = u01hq_f64(x.x, x.y);
    const ag_u64 zy = (ag_u64)x.z ^ ((ag_u64)x.w << 21);
    const double v = __dadd_rn(__dmul_rn((double)zy, 2.2204460492503131e-16), 1.1102230246251565e-16);
    const double s = __dsqrt_rn(__dmul_rn(-2.0, log(u)));
    double sv, cv;
    sincos(__dmul_rn(v, 3.1415926535897932), &sv, &cv);
    return __dmul_rn(s, sv);
}
__device__ __forceinline__ float normal_f32(ag_u64 seed, ag_u32 g, ag_u32 c) {
    const q4 x = philox_block(seed, g, c);
    const float u = u01_f32(x.x);
    const float k = 2.3283064e-10f * 6.2831855f;
    const float v = __fadd_rn(__fmul_rn((float)x.y, k), k / 2.0f);
    const float s = __fsqrt_rn(__fmul_rn(-2.0f, logf(u)));
    float sv, cv;
    sincosf(v, &sv, &cv);
    return __fmul_rn(s, sv);
}
__device__ __forceinline__ double draw01(double*, ag_u64 seed, ag_u32 g, ag_u32 c) {
    return u01_f64(philox_block(seed, g, c).x);
}
__device__ __forceinline__ float draw01(float*, ag_u64 seed, ag_u32 g, ag_u32 c) {
    return u01_f32(philox_block(seed, g, c).x);
}
__device__ __forceinline__ double drawn(double*, ag_u64 seed, ag_u32 g, ag_u32 c) { return normal_f64(seed, g, c); }
__device__ __forceinline__ float drawn(float*, ag_u64 seed, ag_u32 g, ag_u32 c) { return normal_f32(seed, g, c); }

// ---------------------------------------------------------------------------
// Per-plane loads and stores: one 128-bit access per thread per plane when
// the lane group is complete, scalar accesses with a bound check otherwise.
// ---------------------------------------------------------------------------
template <int VEC, class T>
struct vec_io;
template <class T>
struct vec_io<1, T> {
    static __device__ __forceinline__ void load(const T* p, ag_u64 s, ag_u64 n, T* x) { x[0] = s < n ? __ldcs(p + s) : T(0); }
    static __device__ __forceinline__ void store(T* p, ag_u64 s, ag_u64 n, const T* x) {
        if (s < n) __stcs(p + s, x[0]);
    }
    static __device__ __forceinline__ void load_rw(const T* p, ag_u64 s, ag_u64 n, T* x) { x[0] = s < n ? p[s] : T(0); }
    // the whole lane group is inside the range (checked once by the caller)
    static __device__ __forceinline__ void load_full(const T* p, ag_u64 s, T* x) { x[0] = __ldcs(p + s); }
    static __device__ __forceinline__ void store_full(T* p, ag_u64 s, const T* x) { __stcs(p + s, x[0]); }
};
template <>
struct vec_io<2, double> {
    static __device__ __forceinline__ void load(const double* p, ag_u64 s, ag_u64 n, double* x) {
        if (s + 2 <= n) {
            const double2 v = __ldcs(reinterpret_cast<const double2*>(p + s));
            x[0] = v.x;
            x[1] = v.y;
        } else {
            x[0] = s < n ? p[s] : 0.0;
            x[1] = s + 1 < n ? p[s + 1] : 0.0;
        }
    }
    static __device__ __forceinline__ void load_rw(const double* p, ag_u64 s, ag_u64 n, double* x) {
        if (s + 2 <= n) {
            const double2 v = *reinterpret_cast<const double2*>(p + s);
            x[0] = v.x;
            x[1] = v.y;
        } else {
            x[0] = s < n ? p[s] : 0.0;
            x[1] = s + 1 < n ? p[s + 1] : 0.0;
        }
    }
    static __device__ __forceinline__ void store(double* p, ag_u64 s, ag_u64 n, const double* x) {
        if (s + 2 <= n) {
            __stcs(reinterpret_cast<double2*>(p + s), make_double2(x[0], x[1]));
        } else {
            if (s < n) p[s] = x[0];
            if (s + 1 < n) p[s + 1] = x[1];
        }
    }
    static __device__ __forceinline__ void load_full(const double* p, ag_u64 s, double* x) {
        const double2 v = __ldcs(reinterpret_cast<const double2*>(p + s));
        x[0] = v.x;
        x[1] = v.y;
    }
    static __device__ __forceinline__ void store_full(double* p, ag_u64 s, const double* x) {
        __stcs(reinterpret_cast<double2*>(p + s), make_double2(x[0], x[1]));
    }
};
template <>
struct vec_io<4, float> {
    static __device__ __forceinline__ void load(const float* p, ag_u64 s, ag_u64 n, float* x) {
        if (s + 4 <= n) {
            const float4 v = __ldcs(reinterpret_cast<const float4*>(p + s));
            x[0] = v.x;
            x[1] = v.y;
            x[2] = v.z;
            x[3] = v.w;
        } else {
#pragma unroll
            for (int v = 0; v < 4; ++v) x[v] = s + v < n ? p[s + v] : 0.0f;
        }
    }
    static __device__ __forceinline__ void load_rw(const float* p, ag_u64 s, ag_u64 n, float* x) {
        if (s + 4 <= n) {
            const float4 v = *reinterpret_cast<const float4*>(p + s);
            x[0] = v.x;
            x[1] = v.y;
            x[2] = v.z;
            x[3] = v.w;
        } else {
#pragma unroll
            for (int v = 0; v < 4; ++v) x[v] = s + v < n ? p[s + v] : 0.0f;
        }
    }
    static __device__ __forceinline__ void store(float* p, ag_u64 s, ag_u64 n, const float* x) {
        if (s + 4 <= n) {
            __stcs(reinterpret_cast<float4*>(p + s), make_float4(x[0], x[1], x[2], x[3]));
        } else {
#pragma unroll
            for (int v = 0; v < 4; ++v)
                if (s + v < n) p[s + v] = x[v];
        }
    }
    static __device__ __forceinline__ void load_full(const float* p, ag_u64 s, float* x) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(p + s));
        x[0] = v.x;
        x[1] = v.y;
        x[2] = v.z;
        x[3] = v.w;
    }
    static __device__ __forceinline__ void store_full(float* p, ag_u64 s, const float* x) {
        __stcs(reinterpret_cast<float4*>(p + s), make_float4(x[0], x[1], x[2], x[3]));
    }
};
// Mixed widths: a float plane inside a double-width lane group, and the
// reverse, fall back to two/four scalar accesses.
template <>
struct vec_io<2, float> {
    static __device__ __forceinline__ void load(const float* p, ag_u64 s, ag_u64 n, float* x) {
        if (s + 2 <= n) {
            const float2 v = __ldcs(reinterpret_cast<const float2*>(p + s));
            x[0] = v.x;
            x[1] = v.y;
        } else {
            x[0] = s < n ? p[s] : 0.0f;
            x[1] = s + 1 < n ? p[s + 1] : 0.0f;
        }
    }
    static __device__ __forceinline__ void load_rw(const float* p, ag_u64 s, ag_u64 n, float* x) { load(p, s, n, x); }
    static __device__ __forceinline__ void store(float* p, ag_u64 s, ag_u64 n, const float* x) {
        if (s < n) p[s] = x[0];
        if (s + 1 < n) p[s + 1] = x[1];
    }
    static __device__ __forceinline__ void load_full(const float* p, ag_u64 s, float* x) {
        const float2 v = __ldcs(reinterpret_cast<const float2*>(p + s));
        x[0] = v.x;
        x[1] = v.y;
    }
    static __device__ __forceinline__ void store_full(float* p, ag_u64 s, const float* x) {
        p[s] = x[0];
        p[s + 1] = x[1];
    }
};
template <>
struct vec_io<4, double> {
    static __device__ __forceinline__ void load(const double* p, ag_u64 s, ag_u64 n, double* x) {
        vec_io<2, double>::load(p, s, n, x);
        vec_io<2, double>::load(p, s + 2, n, x + 2);
    }
    static __device__ __forceinline__ void load_rw(const double* p, ag_u64 s, ag_u64 n, double* x) {
        vec_io<2, double>::load_rw(p, s, n, x);
        vec_io<2, double>::load_rw(p, s + 2, n, x + 2);
    }
    static __device__ __forceinline__ void store(double* p, ag_u64 s, ag_u64 n, const double* x) {
        vec_io<2, double>::store(p, s, n, x);
        vec_io<2, double>::store(p, s + 2, n, x + 2);
    }
    static __device__ __forceinline__ void load_full(const double* p, ag_u64 s, double* x) {
        vec_io<2, double>::load_full(p, s, x);
        vec_io<2, double>::load_full(p, s + 2, x + 2);
    }
    static __device__ __forceinline__ void store_full(double* p, ag_u64 s, const double* x) {
        vec_io<2, double>::store_full(p, s, x);
        vec_io<2, double>::store_full(p, s + 2, x + 2);
    }
};

// ---------------------------------------------------------------------------
// Compensated sums. two_sum_err is Knuth's exact residual; pair_combine and
// the xor-16..1 butterfly are the reference's (hi, comp) tree
// (accum/atomic.h:141-258), so a warp's 32 pairs reduce exactly as the host
// twin reduce32Host_ does.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double two_sum_err(double a, double b, double s) {
    const double bb = __dsub_rn(s, a);
    return __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
template <class T>
__device__ __forceinline__ bool finite_(T x) {
    return isfinite(x);
}
template <class T>
__device__ __forceinline__ void pair_combine(T ah, T ac, T bh, T bc, T& oh, T& oc) {
    const T s = rn_add(ah, bh);
    const T e = two_sum_err(ah, bh, s);
    oh = s;
    oc = finite_(s) ? rn_add(rn_add(ac, bc), e) : T(0);
}
template <class T>
__device__ __forceinline__ void neumaier_add(T& hi, T& comp, T term) {
    const T s = rn_add(hi, term);
    const T e = two_sum_err(hi, term, s);
    hi = s;
    comp = finite_(s) ? rn_add(comp, e) : T(0);
}
template <class T>
__device__ __forceinline__ void butterfly32(T& h, T& c) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const T rh = __shfl_xor_sync(0xffffffffu, h, off);
        const T rc = __shfl_xor_sync(0xffffffffu, c, off);
        pair_combine(h, c, rh, rc, h, c);
    }
}

}  // namespace ag

namespace ag {

// Finish one chunk of a sum plan: reduce the CTA's (hi, comp) pairs with the
// warp butterfly and a fixed cross-warp order, publish the chunk's partial,
// and let the CTA that completes the last chunk combine all partials in a
// fixed order (so the result does not depend on scheduling) and reset the
// counter for the next launch. Workspace layout: [u32 counter, pad to 16 B]
// then one double2 (hi, comp) per chunk. No CTA ever waits on another.
template <int BLOCK>
__device__ __forceinline__ void sum_chunk_finish(const AgArgs& a, ag_u64 ch, ag_u64 nchunks, double h, double c) {
    __shared__ double sh_h[BLOCK / 32], sh_c[BLOCK / 32];
    __shared__ int sh_last;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    butterfly32(h, c);
    if (lane == 0) {
        sh_h[warp] = h;
        sh_c[warp] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double H = sh_h[0], C = sh_c[0];
        for (int w = 1; w < BLOCK / 32; ++w) pair_combine(H, C, sh_h[w], sh_c[w], H, C);
        double2* part = reinterpret_cast<double2*>(a.ws + 16);
        __stcg(part + ch, make_double2(H, C));
        __threadfence();
        const unsigned ticket = atomicAdd(reinterpret_cast<unsigned*>(a.ws), 1u);
        sh_last = ticket == (unsigned)(nchunks - 1);
    }
    __syncthreads();
    if (sh_last) {
        __threadfence();
        const double2* part = reinterpret_cast<const double2*>(a.ws + 16);
        double H = 0.0, C = 0.0;
        for (ag_u64 k = threadIdx.x; k < nchunks; k += BLOCK) {
            const double2 q = __ldcg(part + k);
            pair_combine(H, C, q.x, q.y, H, C);
        }
        butterfly32(H, C);
        __syncthreads();
        if (lane == 0) {
            sh_h[warp] = H;
            sh_c[warp] = C;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double RH = sh_h[0], RC = sh_c[0];
            for (int w = 1; w < BLOCK / 32; ++w) pair_combine(RH, RC, sh_h[w], sh_c[w], RH, RC);
            a.red[0] = RH;
            a.red[1] = RC;
            *reinterpret_cast<volatile unsigned*>(a.ws) = 0u;
        }
    }
    __syncthreads();
}

}  // namespace ag
