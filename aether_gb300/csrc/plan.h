// plan.h -- the aether-ir/1 plan: parser, type checker and CUDA code generator.
//
// A plan is one fused assignment `dst <op>= expr` over the sample axis of SoA
// arrays, the statement a consumer of the reference writes inside its own
// kernel (`d[i] = a + b*exp(c)`, expr/Assign.h:251-346). The tree's text is its
// type signature; the generated kernel is cached by the hash of that text and
// the lowering options.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ag {

enum class DType { F64, F32, FF, I32, U8 };

struct Node {
    std::string op;
    std::vector<int> kids;
    std::vector<int> shape;   // element extents, row-major; empty = rank 0
    int comps = 1;
    bool is_bool = false;
    int k = 0;                // operand / scalar / key slot, or the first integer argument
    std::vector<int> ints;    // further integer arguments
    double lit = 0.0;
    DType dtype = DType::F64; // storage type of an `in` leaf
    bool nonneg_hint = false; // `(sc K +)`: the launch promises a value >= 0
};

struct Plan {
    DType dst_dtype = DType::F64;
    std::vector<int> dst_shape;
    int dst_comps = 1;
    std::string op;           // set | add | sub | sum | setsum
    std::vector<Node> nodes;  // topological: every kid precedes its parent
    int root = -1;
    int n_operands = 0;       // 1 + highest operand slot used
    int n_scalars = 0;
    int n_keys = 0;
    std::vector<DType> operand_dtype;
    std::vector<int> operand_comps;
    std::vector<char> scalar_nonneg;   // per scalar slot: launches must pass a value >= 0
    bool has_random = false;
    bool wants_sum() const { return op == "sum" || op == "setsum"; }
    bool wants_store() const { return op != "sum"; }
    // compensated per-sample accumulation: value planes, then compensation planes
    bool wants_acc() const { return op == "acc" || op == "accat"; }
    // planes of the destination: float-float and accumulation planes are pairs
    int dst_planes() const { return dst_comps * ((dst_dtype == DType::FF || wants_acc()) ? 2 : 1); }
};

// Lowering options (part of the cache key).
struct Lowering {
    int block = 256;          // threads per CTA
    int ipt = 1;              // lane groups per thread per chunk
    int vec = 0;              // samples per lane group (0 = 16 bytes of the widest storage type)
    bool contract = true;     // allow FMA contraction of arithmetic nodes
    int math = 0;             // 0 = native FP64 pipe, 1 = emulated FP64 on FP32/INT pipes (double-float),
                              // 2 = precision form (f32/ff storage), 3 = FP64-grade triple-float
    int min_blocks = 0;       // __launch_bounds__ second argument (0 = none)
};

Plan parse_plan(const std::string& text);
const char* dtype_name(DType d);
int dtype_size(DType d);

// Generated CUDA source for the plan: kernels `<base>_v` (vectorized lane
// groups) and `<base>_s` (one sample per lane group). With chunk_only, only
// the per-chunk device function `ag_chunk<suffix>` (and its fallback) is
// emitted, for inclusion in a batch module.
std::string generate_source(const Plan& plan, const Lowering& low, const std::string& base = "ag_plan",
                            const std::string& suffix = "", bool chunk_only = false);

// One persistent kernel `<base>` over a device work list of items, each an
// argument block plus the plan it runs; items are cut into tiles of
// block*ipt*vec_p samples that CTAs take round-robin. All plans share block
// and ipt; each keeps its own math mode and vector width.
std::string generate_batch_source(const std::vector<const Plan*>& plans, const std::vector<Lowering>& lows,
                                  int block, int ipt, const std::string& base,
                                  int min_blocks = 0);

// Kernel base name of a plan: ag_<expr|fill|sum>_<8 hex digits of the text hash>,
// so profiles and launch lists tell plans apart.
std::string kernel_base(const Plan& plan, const std::string& text);

// Chunk = samples one CTA covers per pass = block * ipt * vec.
int effective_vec(const Plan& plan, const Lowering& low);

}  // namespace ag
