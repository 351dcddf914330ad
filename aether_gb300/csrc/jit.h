// jit.h -- NVRTC compilation of generated plan kernels, cached by hash in
// memory and on disk, loaded through the driver API.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ag {

struct Compiled {
    std::string cubin;
    double compile_ms = 0.0;   // 0 when served from a cache
    uint64_t hash = 0;
};

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ULL);

// Compile `source` (which may include "ag_device.cuh" / "ag_emu64.cuh") for
// the current device's architecture. Throws std::runtime_error with the NVRTC
// log on failure.
Compiled compile_cached(const std::string& source, const std::string& tag);

// The architecture string of the current device, e.g. "sm_103a".
std::string current_arch();

// Compile for `arch` without caching or loading (offline checks).
std::string compile_for_arch(const std::string& source, const std::string& arch);

// The device headers generated kernels include (the NVRTC payload) and a
// digest of their names and contents.
int payload_count();
bool payload_header(int i, const char** name, const char** src);
uint64_t payload_digest();

// Compile a code generator's `source` for `arch` against the whole payload
// (the consumer headers included), with extra NVRTC `options`; returns the
// CUBIN or throws with the NVRTC log.
std::string compile_with_payload(const std::string& source, const std::string& arch,
                                 const std::vector<std::string>& options);

// The cache key of `source` compiled for `arch` with option tag `tag` by
// NVRTC major.minor: the source, the options and every payload header's name
// and text. With override_index >= 0, header override_index is taken as
// `override_src` instead of its embedded text (to show that a header edit
// changes the key).
uint64_t cache_key(const std::string& source, const std::string& arch, const std::string& tag, int nvrtc_major,
                   int nvrtc_minor, int override_index, const char* override_src);

}  // namespace ag
