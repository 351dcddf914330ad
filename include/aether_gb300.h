/*
 * aether_gb300.h -- the C-ABI boundary of the GB300 fused-expression engine.
 *
 * Plain C: pointers, sizes and status codes only. Every entry point returns 0
 * on success, 1 on failure (the message is in aether_last_error(), kept per
 * thread) and 2 when an optional feature is missing, the convention of the
 * reference's plugin seam (dsc/src/seam.h:16-53, dsc/src/plugin.cpp:22-39).
 * Nothing throws across this boundary. Streams are raw cudaStream_t values
 * passed as void*; NULL is the legacy default stream.
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef AETHER_GB300_H
#define AETHER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AETHER_GB300_ABI 1

enum { AETHER_OK = 0, AETHER_FAIL = 1, AETHER_MISSING = 2 };
/* Memory kinds, as in the reference seam (dsc/src/seam.h:10). */
enum { AETHER_MEM_CPU = 0, AETHER_MEM_DEVICE = 1, AETHER_MEM_PINNED = 2 };

/* ------------------------------------------------------------------------- *
 * Memory. Replaces the AetherMemoryV1 table of dsc/src/seam.h:22-53
 * (probe, runtime_version, last_error, chunk_alloc, chunk_release, drain,
 * fill, copy, stream_wait, stream_sync), backed on the reference side by
 * aether/chunk/Chunk.h:111-260 and aether/chunk/Copy.h:87-192.
 * ------------------------------------------------------------------------- */

/* dsc/src/seam.h:24 probe: 0 only if a driver answers and >= 1 device exists. */
int aether_probe(int* device_count);
/* dsc/src/seam.h:25 runtime_version. */
int aether_runtime_version(int* version);
/* dsc/src/seam.h:27 last_error: the calling thread's last failure message. */
const char* aether_last_error(void);
/* dsc/src/seam.h:28 chunk_alloc: `bytes` of `kind` memory on `dev`; device
 * memory is stream-ordered on `stream` (chunk/Chunk.h:217-260). */
int aether_chunk_alloc(int kind, int dev, size_t bytes, void* stream, void** chunk, void** ptr);
/* dsc/src/seam.h:29 chunk_release: frees on the chunk's stream; deferred while
 * that stream is capturing (chunk/StreamOrdered.h:141-286). */
void aether_chunk_release(void* chunk);
/* dsc/src/seam.h:30 drain: release deferred frees whose capture has ended. */
void aether_drain(void);
/* dsc/src/seam.h:31 fill: repeat the `width`-byte `value` over `bytes`
 * (chunk/Fill.h:33). */
int aether_fill(int kind, int dev, void* ptr, size_t bytes, const void* value, size_t width, void* stream);
/* dsc/src/seam.h:32 copy: any legal (dst kind, src kind) pair, stream-ordered
 * (chunk/Copy.h:87-192). */
int aether_copy(int dst_kind, int dst_dev, void* dst, int src_kind, int src_dev, const void* src, size_t bytes,
                void* stream);
/* dsc/src/seam.h:34 stream_wait: `consumer` waits for work queued on `producer`. */
int aether_stream_wait(int dev, void* producer, void* consumer);
/* dsc/src/seam.h:35 stream_sync. */
int aether_stream_sync(int dev, void* stream);
/* dsc/src/seam.h:26 current_device. */
int aether_current_device(int* dev);
/* dsc/src/seam.h:36 pointer_device: the device that owns a device pointer. */
int aether_pointer_device(const void* ptr, int* dev);
/* No counterpart in the seam, whose callers make cudaStream_t handles with the
 * CUDA runtime (chunk/StreamOrdered.h:38): a non-blocking stream on `dev` for
 * callers that include no CUDA header (graph capture needs one). */
int aether_stream_create(int dev, void** stream);
void aether_stream_destroy(void* stream);

/* ------------------------------------------------------------------------- *
 * Plans: one fused assignment `dst <op>= expr` lowered to one sm_103a kernel.
 * Replaces the consumer-written __global__ that evaluates `view[i] = expr`
 * (expr/Assign.h:191-231 RecursiveAssign/SampleRef, view/View.h:385-418) and
 * its launch (backend/cuda/Launch.h:53-74 launchConfig, :84-88
 * checkLastLaunch), and the bundle variant (backend/cuda/bundle/Assign.h:55-268,
 * bundle/LoadStore.h:149-318). The expression is the aether-ir/1 text that
 * the C++ front end (the headers under include/aether) serialises from the
 * expression tree's type; the kernel is compiled once per (text, lowering)
 * and cached in memory and on disk by hash.
 * ------------------------------------------------------------------------- */

/* One SoA operand: plane c of the array starts at ptr + c * pitch elements
 * (array/Array.h:288-304: pitch = capacity, a multiple of 32 samples). */
typedef struct AetherOperand {
    const void* ptr;
    uint64_t pitch;
} AetherOperand;

typedef struct AetherLaunch {
    uint64_t n;                   /* samples to evaluate */
    uint32_t sample_offset;       /* global sample id of sample 0 (SampleIndex::global) */
    uint32_t flags;               /* 0 */
    void* dst;                    /* destination planes (device memory) */
    uint64_t dst_pitch;           /* elements between destination planes */
    const AetherOperand* operands;
    uint32_t n_operands;
    const double* scalars;        /* runtime scalars (host memory), e.g. CWiseScale factors */
    uint32_t n_scalars;
    const uint64_t* keys;         /* Generator keys of random leaves (random/Generator.h:183) */
    uint32_t n_keys;
    double* reduce_out;           /* sum plans: device pointer to (hi, comp) */
    /* Sum plans: device scratch of aether_plan_workspace_size bytes, or NULL
     * for one of the plan's own. Own workspaces form a pool: a launch reuses
     * an entry last used on the same stream or one whose last launch has
     * finished, and allocates a new entry otherwise, so concurrent launches
     * of one plan on different streams never share scratch. A caller-given
     * workspace is the caller's to keep private to one launch at a time. A
     * launch recorded into a CUDA graph needs a caller-given workspace (or
     * aether_plan_launch_noalloc); without one it is refused. */
    void* workspace;
    uint64_t workspace_bytes;
} AetherLaunch;

/* Lowering options; any field <= 0 takes the tuned default. */
typedef struct AetherLowering {
    int block;        /* threads per CTA */
    int ipt;          /* lane groups per thread per chunk */
    int vec;          /* samples per lane group (vector width) */
    int contract;     /* 1: FMA contraction allowed, 0: every add/mul rounds (-fmad=false), -1: default (1) */
    int math;         /* 0: FP64 on the FP64 pipe; 1: FP64 emulated on the FP32/INT pipes (double-float);
                         2: the precision form -- f32 or float-float storage evaluated in double-float
                         arithmetic, exact products of f32 operands, FP64 only in the final stage of sums;
                         3: FP64-grade on the FP32/INT pipes (triple-float, f64 plans): doubles split exactly
                         into three floats, results within an ulp or so of the native pipe's */
    int min_blocks;   /* __launch_bounds__ min blocks per SM */
} AetherLowering;

typedef struct AetherPlanInfo {
    uint64_t hash;            /* cache key of the compiled kernel */
    int n_operands, n_scalars, n_keys;
    int dst_comps;
    int dst_dtype;            /* 0 f64, 1 f32, 2 ff */
    int is_sum;               /* writes a (hi, comp) global sum */
    int block, ipt, vec;
    int registers;            /* per thread, of the vectorized kernel */
    int blocks_per_sm;        /* occupancy of the vectorized kernel */
    double compile_ms;        /* 0 when the kernel came from a cache */
} AetherPlanInfo;

/* Parse, check and compile `ir` (aether-ir/1). `lowering` may be NULL. */
int aether_plan_create(const char* ir, const AetherLowering* lowering, void** plan);
int aether_plan_info(void* plan, AetherPlanInfo* info);
/* Device scratch a sum plan needs for `n` samples (0 for other plans). */
int aether_plan_workspace_size(void* plan, uint64_t n, uint64_t* bytes);
/* Enqueue the plan on `stream`. Never synchronises. */
int aether_plan_launch(void* plan, const AetherLaunch* args, void* stream);
/* The generated CUDA source (for inspection); `len` receives its length. */
int aether_plan_source(void* plan, char* buf, size_t cap, size_t* len);
void aether_plan_release(void* plan);

/* ------------------------------------------------------------------------- *
 * Batches: many independent assignments (arrays of uneven sizes, several
 * expression kinds) as one persistent kernel over a device work list, and
 * that launch captured into a CUDA graph. Replaces a host loop of
 * consumer-written kernel launches, one per array (backend/cuda/Launch.h:53-88,
 * the pattern of tests/test_GraphCapture.cu:50-57), whose capture rules
 * (tests/test_GraphCapture.cu:17-25) the capture below follows. Sum plans
 * cannot join a batch.
 * ------------------------------------------------------------------------- */
typedef struct AetherBatchItem {
    int plan;          /* index into the plans given to aether_batch_create */
    int reserved;
    AetherLaunch args; /* as for aether_plan_launch; every plane 16-byte aligned */
} AetherBatchItem;

typedef struct AetherBatchInfo {
    uint64_t hash;
    int n_plans, n_items;
    uint64_t total_tiles;
    int block, ipt;
    int registers, blocks_per_sm;
    double compile_ms;
} AetherBatchInfo;

/* Compile one persistent kernel for `plans` (block/ipt from `lowering`). */
int aether_batch_create(void* const* plans, int n_plans, const AetherLowering* lowering, void** batch);
/* Replace the work list; items are cut into equal tiles the CTAs take
 * round-robin. Returns once the list is on the device. */
int aether_batch_set_items(void* batch, const AetherBatchItem* items, int n_items, void* stream);
/* One launch over the whole work list. */
int aether_batch_launch(void* batch, void* stream);
/* Capture one launch into a CUDA graph held by the batch (non-default stream);
 * aether_batch_replay launches it. A work list with a different tiling needs a
 * new capture; new contents with the same tiling do not. */
int aether_batch_capture(void* batch, void* stream);
int aether_batch_replay(void* batch, void* stream);
int aether_batch_info(void* batch, AetherBatchInfo* info);
void aether_batch_release(void* batch);
/* `count` plain launches from one host loop: the per-call baseline a batch is
 * measured against. */
int aether_plan_launch_many(void* const* plans, const AetherLaunch* args, int count, void* stream);

/* Launch a sum plan without allocating anything on the device. No counterpart
 * in the reference: it exists for callers that cannot call cudaMalloc where
 * they launch -- hosts that run under a fixed device-memory budget,
 * latency-critical loops. The plan's scratch (a counter and one partial per
 * chunk, 16 + 16 * chunks bytes) comes from a 1 MiB array compiled into the
 * library that every GPU which loads it holds until exit; sizes that need more
 * are refused with an error naming the limit. `args->workspace` must be NULL.
 * The first call on a device resolves the array's address (a first call on a
 * stream that is capturing is refused with an error saying so); the address
 * is kept for the process, so the entry point is not usable after a
 * cudaDeviceReset. Calls share the array (the counter is cleared at each
 * call), so calls whose kernels overlap on the GPU race and must be
 * serialised by the caller. */
int aether_plan_launch_noalloc(void* plan, const AetherLaunch* args, void* stream);

/* ------------------------------------------------------------------------- *
 * Serving: a request loop with continuous batching. No single counterpart in
 * the reference: it serves, from one process, what a reference user gets
 * from one assignment per call (expr/Assign.h:251-346 through
 * backend/cuda/Launch.h:53-88, synchronised per call) on arrays kept on the
 * device (a device copy of host bytes, residency/Replica.h:56-100, filled by
 * chunk/Copy.h:87-192).
 *
 * The server owns one device arena of `hbm_budget_bytes`. Every request names
 * its operands by a residency id: an id already on the device is reused, a
 * new one is copied in from its host bytes, and idle operands are evicted
 * least recently used first when the arena is full. A request is admitted
 * when its output and its missing operands fit in the arena; requests wait in
 * arrival order until they do. Admitted requests that arrive while others run
 * are launched as soon as one of `max_inflight` launch slots frees up, up to
 * `max_items` requests per launch in one persistent batched kernel
 * (AETHER_SERVE_BATCHED), or one plain plan launch each
 * (AETHER_SERVE_PLAIN, the per-call baseline). Results do not depend on the
 * mode or on the mix: each request runs its plan's own arithmetic.
 * ------------------------------------------------------------------------- */
enum { AETHER_SERVE_BATCHED = 0, AETHER_SERVE_PLAIN = 1 };
/* request flags */
enum { AETHER_SERVE_KEEP_OUTPUT = 1 };
/* request states */
enum { AETHER_SERVE_QUEUED = 0, AETHER_SERVE_RUNNING = 1, AETHER_SERVE_DONE = 2, AETHER_SERVE_FAILED = 3 };

typedef struct AetherServeConfig {
    uint64_t hbm_budget_bytes; /* size of the device arena (operands + outputs) */
    int mode;                  /* AETHER_SERVE_BATCHED or AETHER_SERVE_PLAIN */
    int max_inflight;          /* launches on the device at once; 0 = 4 */
    int max_items;             /* requests per batched launch; 0 = 256 */
    int block, ipt;            /* lowering of the batched kernel; 0 = 512, 1 */
    int idle_spin_us;          /* the loop polls this long after its last work before it sleeps; 0 = 2000 */
    int upload_engine;         /* 0: SMs read mapped pinned host operands in one gather kernel per launch
                                  (other memory: copy engine); 1: copy engine only */
    int grouping;              /* batched mode: 0 = the requests of a launch grouped by plan, one work-list
                                  kernel compiled for each plan (a lone request runs its plan's own kernel);
                                  1 = one work-list kernel holding every plan behind a switch */
} AetherServeConfig;

typedef struct AetherServeOperand {
    uint64_t id;      /* residency key: equal ids name equal bytes */
    const void* host; /* the bytes (pinned memory copies fastest); may be NULL if the id is resident */
    uint64_t pitch;   /* samples per plane (0 = n); pitch * element size a multiple of 16 */
} AetherServeOperand;

typedef struct AetherServeRequest {
    int plan;                            /* index into the plans given to aether_serve_open */
    int flags;                           /* AETHER_SERVE_KEEP_OUTPUT */
    uint64_t n;                          /* samples */
    const AetherServeOperand* operands;  /* one per plan operand, in plan order */
    uint32_t n_operands;
    uint32_t n_scalars;
    const double* scalars;
    const uint64_t* keys;
    uint32_t n_keys;
    uint32_t reserved;
    void* host_out;       /* optional: the output planes are copied here (comps * out_pitch elements) */
    uint64_t arrival_ns;  /* aether_serve_feed: arrival time after the feed starts */
} AetherServeRequest;

typedef struct AetherServeStatus {
    int state;            /* AETHER_SERVE_* state */
    int launch_items;     /* requests in the launch that ran this one */
    uint64_t t_arrival_ns, t_dispatch_ns, t_done_ns; /* since aether_serve_open */
    const void* output;   /* device output while kept (AETHER_SERVE_KEEP_OUTPUT) */
    uint64_t out_pitch;   /* samples per output plane */
    uint64_t bytes;       /* algorithmic bytes: operand planes read + output planes written */
    uint64_t uploaded_bytes; /* operand bytes this request copied in */
} AetherServeStatus;

typedef struct AetherServeStats {
    uint64_t submitted, completed, failed;
    uint64_t launches, launched_items;
    uint64_t bytes, uploaded_bytes;
    uint64_t resident_hits, resident_misses, evictions;
    uint64_t arena_bytes, arena_peak_bytes, resident_bytes;
    uint64_t first_arrival_ns, last_done_ns;
    uint64_t enqueue_ns;      /* host time the loop spent issuing copies and launches */
    uint64_t admit_ns;        /* host time the loop spent admitting (arena, residency) */
} AetherServeStats;

/* Compile the batched kernel for `plans` (none may be a sum plan), allocate the
 * arena and start the loop's thread on the calling thread's device. */
int aether_serve_open(void* const* plans, int n_plans, const AetherServeConfig* config, void** server);
/* Queue one request now; its ticket identifies it until aether_serve_release
 * (kept outputs) or aether_serve_close. Requests that can never fit the arena
 * or do not match their plan are refused here. */
int aether_serve_submit(void* server, const AetherServeRequest* request, uint64_t* ticket);
/* Queue `count` requests, each at its arrival_ns after the call starts
 * (sleeping or spinning in between on the calling thread); the arrival time
 * recorded is the scheduled one. tickets[i] receives request i's ticket. */
int aether_serve_feed(void* server, const AetherServeRequest* requests, int count, uint64_t* tickets);
int aether_serve_status(void* server, uint64_t ticket, AetherServeStatus* status);
/* Wait until the request is done or failed, or `timeout_s` passes (status 1). */
int aether_serve_wait(void* server, uint64_t ticket, double timeout_s, AetherServeStatus* status);
/* Free a kept output. */
int aether_serve_release(void* server, uint64_t ticket);
int aether_serve_stats(void* server, AetherServeStats* stats);
/* Finish the work on the device, stop the loop and free the arena. */
void aether_serve_close(void* server);

/* ------------------------------------------------------------------------- *
 * Runtime-typed strided evaluation. Replaces aether::eval::runtimeEval
 * (eval/Runtime.h:73-300) over RuntimeView descriptors (view/RuntimeView.h:
 * 71-110): out = op(a, b, scalar) for every element of out's logical shape,
 * row-major over out's extents, each operand addressed through its own
 * element strides. Assign copies or casts (double <-> float); the other ops
 * need one dtype throughout; the scalar is rounded to the input type first.
 * Every add and multiply rounds on its own. Errors are reported before any
 * launch, worded as the reference's "<op> failed on <where>, size=<n> bytes
 * (<detail>)". Operands must be device memory: there is no host path.
 * ------------------------------------------------------------------------- */
enum {
    AETHER_RT_ASSIGN = 0,
    AETHER_RT_ADD = 1,
    AETHER_RT_SUB = 2,
    AETHER_RT_SCALE = 3,
    AETHER_RT_ADD_SCALED = 4,
    AETHER_RT_SUB_SCALED = 5
};
#define AETHER_RT_RANK_CAP 6

typedef struct AetherRuntimeView {
    void* data;
    uint8_t dtype_code;     /* DLPack type code: 2 = float */
    uint8_t dtype_bits;     /* 32 or 64 */
    uint16_t dtype_lanes;   /* 1 */
    int32_t rank;           /* <= AETHER_RT_RANK_CAP */
    int64_t extents[AETHER_RT_RANK_CAP];
    int64_t strides[AETHER_RT_RANK_CAP];  /* element units, >= 0 */
} AetherRuntimeView;

/* `b` is read only by Add, Sub, AddScaled and SubScaled (may be NULL otherwise). */
int aether_runtime_eval(int op, const AetherRuntimeView* a, const AetherRuntimeView* b, const AetherRuntimeView* out,
                        double scalar, void* stream);

/* Offline lowering, no device needed: parse and check `ir`, write the CUDA
 * source of its kernel into `buf` (up to `cap` bytes, NUL-terminated) and its
 * length into `len`. Stands in for the reference's compile-time type check of
 * an expression (the static_asserts of the expr/nodes headers and expr/Assign.h:205-231). */
int aether_plan_generate(const char* ir, const AetherLowering* lowering, char* buf, size_t cap, size_t* len);
/* The NVRTC payload, for kernels a code generator compiles with NVRTC.
 * Replaces the sealed header payload of dsc/aether_dsc/_core.py:132-200
 * (names, bytes and a content digest) over the NVRTC-parseable surface of
 * aether/device.h (aether/device.h:1-30). It holds, each under its include
 * name: the device-safe consumer headers "aether/device.h" and everything it
 * includes (views, SampleIndex, Items, expressions, aether::math, Philox
 * leaves), and the engine's device runtime (ag_device.cuh: Philox streams,
 * word conversions, native math facade, compensated sums; ag_emu64.cuh and
 * its tables: double-float arithmetic and functions; the Box-Muller draw),
 * under its bare names and again under "aether/gb300/". Sources are
 * NUL-terminated, owned by the library, valid until unload. The digest covers
 * every name and byte. */
int aether_rtc_header_count(void);
int aether_rtc_header(int index, const char** name, const char** source);
uint64_t aether_rtc_digest(void);
/* Compile `source` for `arch` (e.g. "sm_103a") with NVRTC against the whole
 * payload, plus `n_options` extra NVRTC options (for aether/device.h under
 * NVRTC: --include-path=<CUDA>/include/cccl, where the toolkit keeps libcu++;
 * -DAETHER_GB300_EMULATED_FP64 for the double-float math facade). Writes the
 * CUBIN into `cubin` (`cap` bytes) and its size into `len`; with cubin NULL
 * only the size. On failure the NVRTC log is the last error. */
int aether_rtc_compile(const char* source, const char* arch, const char* const* options, int n_options, void* cubin,
                       size_t cap, size_t* len);
/* The in-memory and on-disk cache key of a generated kernel: `source` compiled
 * for `arch` under option tag `tag` by this library's NVRTC, hashed with the
 * name and text of every payload header above, so a kernel cached before any
 * of those headers changed is never served after the change. With
 * header_index >= 0 the key is computed as if payload header `header_index`
 * held `header_source` instead (no device needed; used to check that every
 * header reaches the key). No counterpart in the reference, which compiles
 * consumer kernels ahead of time with nvcc. */
int aether_plan_cache_key(const char* source, const char* arch, const char* tag, int header_index,
                          const char* header_source, uint64_t* key);
/* Compile `source` with NVRTC for `arch` (e.g. "sm_103a") without loading it;
 * on failure the compiler log is the last error. */
int aether_nvrtc_check(const char* source, const char* arch);

/* ------------------------------------------------------------------------- *
 * Function tables.
 *
 * aether_memory_v1 returns the seam table of dsc/src/seam.h:22-53 with its
 * exact layout (ABI 2), so the reference's Python loader can open this library
 * in place of its CUDA plugin. The FFT entries (cuFFT, outside the fused
 * expression path) answer AETHER_MISSING with a message, the seam's
 * optional-feature convention.
 *
 * aether_gb300_v1 returns the same table plus every entry point of the fused
 * expression path: one versioned symbol a loader can bind in one call.
 * ------------------------------------------------------------------------- */
#define AETHER_MEMORY_ABI 2
typedef struct AetherMemoryV1 {
    uint32_t abi;
    int (*probe)(int* device_count);
    int (*runtime_version)(int* version);
    int (*current_device)(int* dev);
    const char* (*last_error)(void);
    int (*chunk_alloc)(int kind, int dev, size_t bytes, void* stream, void** chunk, void** ptr);
    void (*chunk_release)(void* chunk);
    void (*drain)(void);
    int (*fill)(int kind, int dev, void* ptr, size_t bytes, const void* value, size_t width, void* stream);
    int (*copy)(int dst_kind, int dst_dev, void* dst, int src_kind, int src_dev, const void* src, size_t bytes,
                void* stream);
    int (*stream_wait)(int dev, void* producer, void* consumer);
    int (*stream_sync)(int dev, void* stream);
    int (*pointer_device)(const void* ptr, int* dev);
    int (*fft_plan)(int dev, int kind, int is_double, int norm, int forward, int ndim, const int64_t* shape, int naxes,
                    const int32_t* axes, void* stream, void** plan);
    int (*fft_exec)(void* plan, const void* in, void* out, void* stream);
    void (*fft_destroy)(void* plan);
} AetherMemoryV1;
const AetherMemoryV1* aether_memory_v1(void);

typedef struct AetherGB300V1 {
    uint32_t abi;   /* AETHER_GB300_ABI */
    const AetherMemoryV1* memory;
    int (*stream_create)(int dev, void** stream);
    void (*stream_destroy)(void* stream);
    int (*plan_create)(const char* ir, const AetherLowering* lowering, void** plan);
    int (*plan_info)(void* plan, AetherPlanInfo* info);
    int (*plan_workspace_size)(void* plan, uint64_t n, uint64_t* bytes);
    int (*plan_launch)(void* plan, const AetherLaunch* args, void* stream);
    int (*plan_source)(void* plan, char* buf, size_t cap, size_t* len);
    void (*plan_release)(void* plan);
    int (*plan_launch_noalloc)(void* plan, const AetherLaunch* args, void* stream);
    int (*plan_launch_many)(void* const* plans, const AetherLaunch* args, int count, void* stream);
    int (*batch_create)(void* const* plans, int n_plans, const AetherLowering* lowering, void** batch);
    int (*batch_set_items)(void* batch, const AetherBatchItem* items, int n_items, void* stream);
    int (*batch_launch)(void* batch, void* stream);
    int (*batch_capture)(void* batch, void* stream);
    int (*batch_replay)(void* batch, void* stream);
    int (*batch_info)(void* batch, AetherBatchInfo* info);
    void (*batch_release)(void* batch);
    int (*serve_open)(void* const* plans, int n_plans, const AetherServeConfig* config, void** server);
    int (*serve_submit)(void* server, const AetherServeRequest* request, uint64_t* ticket);
    int (*serve_feed)(void* server, const AetherServeRequest* requests, int count, uint64_t* tickets);
    int (*serve_status)(void* server, uint64_t ticket, AetherServeStatus* status);
    int (*serve_wait)(void* server, uint64_t ticket, double timeout_s, AetherServeStatus* status);
    int (*serve_release)(void* server, uint64_t ticket);
    int (*serve_stats)(void* server, AetherServeStats* stats);
    void (*serve_close)(void* server);
    int (*runtime_eval)(int op, const AetherRuntimeView* a, const AetherRuntimeView* b, const AetherRuntimeView* out,
                        double scalar, void* stream);
    int (*rtc_header_count)(void);
    int (*rtc_header)(int index, const char** name, const char** source);
    uint64_t (*rtc_digest)(void);
    int (*plan_generate)(const char* ir, const AetherLowering* lowering, char* buf, size_t cap, size_t* len);
    int (*nvrtc_check)(const char* source, const char* arch);
    int (*plan_cache_key)(const char* source, const char* arch, const char* tag, int header_index,
                          const char* header_source, uint64_t* key);
    int (*rtc_compile)(const char* source, const char* arch, const char* const* options, int n_options, void* cubin,
                       size_t cap, size_t* len);
} AetherGB300V1;
const AetherGB300V1* aether_gb300_v1(void);

#ifdef __cplusplus
}
#endif
#endif
