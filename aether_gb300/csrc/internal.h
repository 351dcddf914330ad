// internal.h -- types shared by the translation units of libaether_gb300.so.
//
// Nothing here is exported: the C-ABI in include/aether_gb300.h hands these
// objects out as opaque handles. abi.cpp owns plans and batches; serve.cpp
// drives the same compiled kernels from its request loop.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "aether_gb300.h"
#include "jit.h"
#include "plan.h"

// Host image of the device's AgArgs (csrc/device/ag_device.cuh); the kernel
// receives it by value.
struct AgArgsHost {
    uint64_t n;
    uint32_t offset, flags;
    char* dst;
    uint64_t dst_pitch;
    const char* ops[16];
    uint64_t pitch[16];
    double sc[16];
    float sch[16];
    float scl[16];
    uint64_t key[8];
    double* red;
    char* ws;
    uint64_t ws_bytes;
};
static_assert(sizeof(AgArgsHost) == 632, "AgArgs layout");

struct PlanObj {
    ag::Plan plan;
    ag::Lowering low;
    std::string name;
    std::string source;
    ag::Compiled compiled;
    cudaLibrary_t library = nullptr;
    cudaKernel_t fv = nullptr, fs = nullptr;
    int vec = 2;
    int registers = 0;
    int blocks_per_sm_v = 1, blocks_per_sm_s = 1;
    int sms = 1;
    int dev = 0;
    // Default workspaces of sum plans (launches with args->workspace == NULL):
    // a pool, so launches on different streams never share scratch. An entry
    // is reused by a later launch on the same stream (stream order) or once
    // the event recorded after its last launch has completed.
    struct Workspace {
        void* ptr = nullptr;
        size_t bytes = 0;
        cudaStream_t last_stream = nullptr;
        bool ordered = false;          // last_stream orders later launches on it
        cudaEvent_t done = nullptr;    // recorded after the last launch
    };
    std::mutex ws_mu;
    std::vector<Workspace> ws;
};

// One work-list entry of a batched kernel (the AgItem of the generated source).
struct AgItemHost {
    AgArgsHost a;
    uint64_t tile0;
    int plan;
    int pad;
};
static_assert(sizeof(AgItemHost) == 648, "AgItem layout");

struct BatchObj {
    std::vector<PlanObj*> plans;
    std::vector<int> vecs;
    int block = 256, ipt = 1;
    std::string name, source;
    ag::Compiled compiled;
    cudaLibrary_t library = nullptr;
    cudaKernel_t kernel = nullptr;
    int blocks_per_sm = 1, sms = 1, registers = 0;
    AgItemHost* host_items = nullptr;   // pinned staging of the work list
    void* dev_items = nullptr;
    size_t cap_items = 0;
    int n_items = 0;
    uint64_t total_tiles = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_tiles = 0;
    int graph_items = 0;
};

inline void ag_ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Samples one CTA pass of a plan's kernel covers.
inline uint64_t chunk_samples(const PlanObj& P, bool vectorized) {
    return uint64_t(P.low.block) * uint64_t(P.low.ipt) * uint64_t(vectorized ? P.vec : 1);
}

// Samples one tile of plan p of a batch covers.
inline uint64_t batch_tile_samples(const BatchObj& B, int p) {
    return uint64_t(B.block) * uint64_t(B.ipt) * uint64_t(B.vecs[size_t(p)]);
}

// Validate a launch against its plan and build the kernel's argument block.
// Returns whether every plane is 16-byte aligned (the vectorized kernel).
bool make_args(const PlanObj* P, const AetherLaunch* a, AgArgsHost& k);

// Grid of a batched kernel over `tiles` tiles.
inline unsigned batch_grid(const BatchObj& B, uint64_t tiles) {
    const uint64_t cap = uint64_t(B.blocks_per_sm > 1 ? B.blocks_per_sm : 1) * uint64_t(B.sms);
    return unsigned(tiles < cap ? (tiles ? tiles : 1) : cap);
}

// Reports through aether_last_error; returns AETHER_FAIL.
int ag_internal_fail(const char* message);
