// aether/batch.h -- batches and the serving loop for C++ callers.
//
// gb300::Batch gathers assignments (dst, expr) over arrays of any sizes and
// runs them as one persistent kernel over a device work list, or replays that
// launch from a CUDA graph (aether_batch_*). gb300::Server wraps the request
// loop with continuous batching (aether_serve_*): plans are given as
// expression templates over placeholder views, requests name their operands
// by residency id and host bytes. Both are RAII owners of their C handles;
// failures throw aether::Error.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "aether/array.h"
#include "aether/eval.h"
#include "aether/expr.h"
#include "aether_gb300.h"

namespace aether {
namespace gb300 {

namespace detail {
inline void check(int rc, const char* what) {
    if (rc != AETHER_OK) throw Error(std::string(what) + " failed (" + aether::detail::last_error() + ")");
}
}  // namespace detail

/** Assignments collected into one launch. Every plane must be 16-byte
 *  aligned (arrays and their partitions are). */
class Batch {
public:
    explicit Batch(const Lowering& low = default_lowering()) : low_(low) {}
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;
    ~Batch() {
        if (handle_) aether_batch_release(handle_);
    }

    /** dst = e, joined to the batch (evaluated at launch()). */
    template <class V>
    void add(const V& dst, const Expr& e) {
        using T = typename V::value_type;
        if (handle_) throw Error("aether Batch: add after the first launch");
        const ir::Shape shape = dst_shape(ir::shape_of(typename V::element_extents{}), e);
        Expr ee = e;
        if (e.shape() != shape) {
            if (!e.shape().empty()) throw Error("aether Batch: expression shape does not match the view");
            ee = Expr(ir::bcast(e.node(), shape));
        }
        Item it;
        const std::string dtype = aether::detail::dtype_name<T>();
        it.text = plan_text(dtype, shape, "set", ee, it.ctx);
        it.plan = gb300::detail::plan_for(it.text, dtype, low_);
        it.n = dst.samples();
        it.dst = const_cast<T*>(dst.data());
        it.pitch = aether::detail::plane_pitch(dst);
        items_.push_back(std::move(it));
    }

    /** One launch over every item on `s` (the work list is built and
     *  uploaded on the first call). */
    void launch(Stream s = nullptr) {
        build_(s);
        detail::check(aether_batch_launch(handle_, s), "batch_launch");
    }
    /** Capture one launch into a CUDA graph (a non-default stream), then
     *  replay it; array contents may change between replays. */
    void capture(Stream s) {
        build_(s);
        detail::check(aether_batch_capture(handle_, s), "batch_capture");
    }
    void replay(Stream s) { detail::check(aether_batch_replay(handle_, s), "batch_replay"); }
    AetherBatchInfo info() const {
        AetherBatchInfo i{};
        detail::check(aether_batch_info(handle_, &i), "batch_info");
        return i;
    }

private:
    struct Item {
        std::string text;
        ir::Context ctx;
        void* plan = nullptr;
        std::size_t n = 0;
        void* dst = nullptr;
        std::size_t pitch = 0;
        std::vector<AetherOperand> ops;
    };
    void build_(Stream s) {
        if (handle_) return;
        std::vector<void*> plans;
        std::map<void*, int> index;
        for (const Item& it : items_)
            if (index.emplace(it.plan, int(plans.size())).second) plans.push_back(it.plan);
        AetherLowering l{low_.block, low_.ipt, 0, -1, 0, 0};
        detail::check(aether_batch_create(plans.data(), int(plans.size()), &l, &handle_), "batch_create");
        std::vector<AetherBatchItem> list(items_.size());
        for (std::size_t i = 0; i < items_.size(); ++i) {
            Item& it = items_[i];
            for (const ir::OperandSlot& o : it.ctx.operands) it.ops.push_back(AetherOperand{o.ptr, o.pitch});
            AetherBatchItem& b = list[i];
            b = AetherBatchItem{};
            b.plan = index[it.plan];
            b.args.n = it.n;
            b.args.dst = it.dst;
            b.args.dst_pitch = it.pitch;
            b.args.operands = it.ops.data();
            b.args.n_operands = uint32_t(it.ops.size());
            b.args.scalars = it.ctx.scalars.data();
            b.args.n_scalars = uint32_t(it.ctx.scalars.size());
            b.args.keys = it.ctx.keys.data();
            b.args.n_keys = uint32_t(it.ctx.keys.size());
        }
        detail::check(aether_batch_set_items(handle_, list.data(), int(list.size()), s), "batch_set_items");
    }
    Lowering low_;
    std::vector<Item> items_;
    void* handle_ = nullptr;
};

/** The serving loop (continuous batching, HBM-budget arena, resident operands). */
class Server {
public:
    /** One served expression: built from placeholder views by `build`. */
    struct Shape {
        void* plan;
        std::vector<double> scalars;
        std::vector<uint64_t> keys;
        std::vector<int> order;   // the plan's operand k is template operand order[k]
    };

    explicit Server(uint64_t budget_bytes, int mode = AETHER_SERVE_BATCHED, int max_inflight = 0, int max_items = 0)
        : budget_(budget_bytes), mode_(mode), inflight_(max_inflight), items_(max_items) {}
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;
    ~Server() { close(); }

    /** Register a shape before open(): `leaves` are placeholder views (any
     *  distinct addresses, pitch 0) in template order, `e` the expression
     *  over them, `dst_dtype`/`dst_shape` the output. Returns its index. */
    int add_shape(const std::vector<Expr>& leaves, const Expr& e, const std::string& dst_dtype,
                  const ir::Shape& dst_shape, const Lowering& low = default_lowering()) {
        if (handle_) throw Error("aether Server: add_shape after open");
        ir::Context ctx;
        const std::string text = plan_text(dst_dtype, dst_shape, "set", e, ctx);
        Shape s;
        s.plan = gb300::detail::plan_for(text, dst_dtype, low);
        s.scalars = ctx.scalars;
        s.keys = ctx.keys;
        for (const ir::OperandSlot& o : ctx.operands) {
            int t = -1;
            for (std::size_t k = 0; k < leaves.size(); ++k) {
                const auto* leaf = dynamic_cast<const ir::Leaf*>(leaves[k].node().get());
                if (leaf && leaf->ptr == o.ptr) t = int(k);
            }
            if (t < 0) throw Error("aether Server: an operand of the expression is not one of the leaves");
            s.order.push_back(t);
        }
        shapes_.push_back(std::move(s));
        return int(shapes_.size()) - 1;
    }

    void open() {
        std::vector<void*> plans;
        for (const Shape& s : shapes_) plans.push_back(s.plan);
        AetherServeConfig cfg{};
        cfg.hbm_budget_bytes = budget_;
        cfg.mode = mode_;
        cfg.max_inflight = inflight_;
        cfg.max_items = items_;
        detail::check(aether_serve_open(plans.data(), int(plans.size()), &cfg, &handle_), "serve_open");
    }

    /** Queue a request of shape `shape` over n samples; `ids[k]`/`hosts[k]`
     *  are template operand k's residency id and host bytes (pitch = the
     *  32-sample capacity of n). `host_out` (optional) receives the output. */
    uint64_t submit(int shape, std::size_t n, const std::vector<uint64_t>& ids, const std::vector<const void*>& hosts,
                    void* host_out = nullptr, bool keep_output = false) {
        const Shape& s = shapes_.at(std::size_t(shape));
        std::vector<AetherServeOperand> ops(s.order.size());
        for (std::size_t k = 0; k < s.order.size(); ++k)
            ops[k] = AetherServeOperand{ids.at(std::size_t(s.order[k])), hosts.at(std::size_t(s.order[k])),
                                        quantized_capacity(n)};
        AetherServeRequest r{};
        r.plan = shape;
        r.flags = keep_output ? AETHER_SERVE_KEEP_OUTPUT : 0;
        r.n = n;
        r.operands = ops.data();
        r.n_operands = uint32_t(ops.size());
        r.scalars = s.scalars.data();
        r.n_scalars = uint32_t(s.scalars.size());
        r.keys = s.keys.data();
        r.n_keys = uint32_t(s.keys.size());
        r.host_out = host_out;
        uint64_t t = 0;
        detail::check(aether_serve_submit(handle_, &r, &t), "serve_submit");
        return t;
    }
    AetherServeStatus wait(uint64_t ticket, double timeout_s = 60.0) {
        AetherServeStatus st{};
        detail::check(aether_serve_wait(handle_, ticket, timeout_s, &st), "serve_wait");
        return st;
    }
    void release(uint64_t ticket) { detail::check(aether_serve_release(handle_, ticket), "serve_release"); }
    AetherServeStats stats() const {
        AetherServeStats s{};
        detail::check(aether_serve_stats(handle_, &s), "serve_stats");
        return s;
    }
    void close() {
        if (handle_) aether_serve_close(handle_);
        handle_ = nullptr;
    }

private:
    uint64_t budget_;
    int mode_, inflight_, items_;
    std::vector<Shape> shapes_;
    void* handle_ = nullptr;
};

}  // namespace gb300
}  // namespace aether
