// serve.cpp -- the request loop behind aether_serve_* (include/aether_gb300.h).
//
// One thread per server owns every device-side decision: it admits queued
// requests in arrival order while their output and missing operands fit in
// the arena (evicting idle operands, least recently used first), copies the
// missing operands in on one copy stream, and launches the admitted requests
// on the first free launch slot -- as one persistent batched kernel over a
// work list (continuous batching) or as one plain plan launch each. It polls
// the slots' completion events and retires their requests. Submitting threads
// only append to the queue.
//
// A launch slot is a stream, a work-list buffer and its pinned staging, and
// checkpoint events: one after each plan's run (its kernel and its requests'
// output copies), so a request retires -- and frees its arena bytes -- as soon
// as its own run has finished, not when the whole launch has. A slot is reused
// only after its last checkpoint has fired, so its staging and its work list
// are no longer read by the device when they are written again.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <thread>
#include <unordered_map>

#include "internal.h"
#include "serve_copy.h"

#define AG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kArenaAlign = 256;

uint64_t round_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

// Best-fit allocator over one device allocation: free ranges indexed by
// offset (to merge neighbours on release) and by size (to find the smallest
// range that fits in O(log n), whatever the fragmentation).
class Arena {
public:
    void init(uint64_t bytes) {
        size_ = bytes;
        by_off_.clear();
        by_size_.clear();
        insert_(0, bytes);
        used_ = peak_ = 0;
    }
    static uint64_t span(uint64_t bytes) { return round_up(bytes ? bytes : 1, kArenaAlign); }
    bool alloc(uint64_t bytes, uint64_t* off) {
        const uint64_t b = span(bytes);
        auto it = by_size_.lower_bound(b);
        if (it == by_size_.end()) return false;
        const uint64_t o = it->second, len = it->first;
        erase_(o, len);
        if (len > b) insert_(o + b, len - b);
        *off = o;
        used_ += b;
        peak_ = std::max(peak_, used_);
        return true;
    }
    void release(uint64_t off, uint64_t bytes) {
        const uint64_t b = span(bytes);
        used_ -= b;
        uint64_t start = off, len = b;
        auto next = by_off_.lower_bound(off);
        if (next != by_off_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                start = prev->first;
                len += prev->second;
                erase_(prev->first, prev->second);
            }
        }
        next = by_off_.lower_bound(off);
        if (next != by_off_.end() && off + b == next->first) {
            len += next->second;
            erase_(next->first, next->second);
        }
        insert_(start, len);
    }
    uint64_t size() const { return size_; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }
    size_t holes() const { return by_off_.size(); }

private:
    void insert_(uint64_t off, uint64_t len) {
        by_off_[off] = len;
        by_size_.emplace(len, off);
    }
    void erase_(uint64_t off, uint64_t len) {
        by_off_.erase(off);
        auto range = by_size_.equal_range(len);
        for (auto it = range.first; it != range.second; ++it)
            if (it->second == off) {
                by_size_.erase(it);
                break;
            }
    }
    std::map<uint64_t, uint64_t> by_off_;
    std::multimap<uint64_t, uint64_t> by_size_;
    uint64_t size_ = 0, used_ = 0, peak_ = 0;
};

// An operand kept on the device under its residency id.
struct Resident {
    uint64_t off = 0, bytes = 0;
    int refs = 0;                     // admitted requests that read it
    uint64_t upload_seq = 0;          // position of its copy on the copy stream
    std::list<uint64_t>::iterator lru;
    bool idle = false;                // in the idle list (refs == 0)
};

struct Request {
    int plan = 0, flags = 0;
    uint64_t n = 0;
    std::vector<AetherServeOperand> ops;
    std::vector<uint64_t> op_bytes;   // bytes of each operand's planes
    std::vector<uint64_t> op_off;     // arena offsets once admitted
    std::vector<char> op_direct;      // host bytes the SMs can read in place (mapped pinned memory)
    std::vector<double> sc;
    std::vector<uint64_t> keys;
    void* host_out = nullptr;
    uint64_t out_pitch = 0, out_bytes = 0, out_off = 0;
    bool out_live = false;
    bool wait_upload = false;         // reads an operand whose copy may still be in flight
    int state = AETHER_SERVE_QUEUED;
    int launch_items = 0;
    uint64_t t_arrival = 0, t_dispatch = 0, t_done = 0;
    uint64_t bytes = 0, uploaded = 0;
    std::string error;
};

struct Upload {
    const void* host;
    uint64_t off, bytes;
    bool direct;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t copied = nullptr;
    AgItemHost* staging = nullptr;
    void* dev_items = nullptr;
    std::vector<Request*> rs;         // the slot's requests (stable: the request deque only grows)
    // When some requests read only resident operands and others wait for
    // copies, the first n_first of rs run in a launch of their own that does
    // not wait for them.
    size_t n_first = 0;
    // Checkpoints in stream order: after each run of one plan (its kernel and
    // its requests' output copies) an event; requests [previous end, cp_end[k])
    // retire when event k completes, so a request does not wait for the
    // other plans of its launch.
    std::vector<cudaEvent_t> cp_ev;   // created on first need, reused
    std::vector<size_t> cp_end;
    size_t cp_next = 0;               // the first checkpoint not yet seen complete
    size_t retired = 0;               // requests of rs retired so far
    uint64_t upload_seq = 0;
    bool busy = false;
};

// A completion seen by the loop: checkpoint `cp` of slot `s`, or the rest of
// the slot (cp = SIZE_MAX) when an error ends it.
struct Fin {
    Slot* s;
    cudaError_t e;
    size_t cp;
};

struct Server {
    int dev = 0, sms = 1;
    AetherServeConfig cfg{};
    std::vector<PlanObj*> plans;
    BatchObj* batch = nullptr;              // every plan behind a switch (grouping 1)
    std::vector<BatchObj*> plan_batch;      // one work-list kernel per plan (grouping 0)
    char* base = nullptr;
    Arena arena;
    cudaStream_t copy_stream = nullptr;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> reqs;         // ticket = index; references stay valid as it grows
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, Resident> residents;
    std::list<uint64_t> idle_lru;     // front = least recently used
    uint64_t resident_bytes = 0;
    uint64_t upload_seq = 0, uploads_done_seq = 0;
    AetherServeStats st{};
    std::string fatal;
    bool stop = false;
    std::thread loop;
    Clock::time_point t0;

    uint64_t now() const {
        return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count());
    }

    // --- arena and residency (called with mu held) -----------------------
    bool alloc_evicting(uint64_t bytes, uint64_t* off) {
        while (!arena.alloc(bytes, off)) {
            if (idle_lru.empty()) return false;
            const uint64_t id = idle_lru.front();
            idle_lru.pop_front();
            auto it = residents.find(id);
            arena.release(it->second.off, it->second.bytes);
            resident_bytes -= it->second.bytes;
            residents.erase(it);
            ++st.evictions;
        }
        return true;
    }
    void unref(uint64_t id) {
        auto it = residents.find(id);
        if (it == residents.end()) return;
        Resident& R = it->second;
        if (--R.refs == 0) {
            R.lru = idle_lru.insert(idle_lru.end(), id);
            R.idle = true;
        }
    }
    void fail_request(Request& r, const std::string& why) {
        r.state = AETHER_SERVE_FAILED;
        r.error = why;
        r.t_done = now();
        ++st.failed;
    }

    enum Admit { ADMITTED, BLOCKED, REFUSED };

    Admit try_admit(Request& r, std::vector<Upload>& ups) {
        const size_t ups0 = ups.size();
        std::vector<uint64_t> refd, created;
        auto rollback = [&] {
            for (uint64_t id : created) {
                auto it = residents.find(id);
                arena.release(it->second.off, it->second.bytes);
                resident_bytes -= it->second.bytes;
                residents.erase(it);
            }
            for (uint64_t id : refd) unref(id);
            ups.resize(ups0);
            if (r.out_live) arena.release(r.out_off, r.out_bytes);
            r.out_live = false;
            r.uploaded = 0;
            r.wait_upload = false;
        };
        if (!alloc_evicting(r.out_bytes, &r.out_off)) return BLOCKED;
        r.out_live = true;
        r.op_off.assign(r.ops.size(), 0);
        for (size_t i = 0; i < r.ops.size(); ++i) {
            const AetherServeOperand& o = r.ops[i];
            auto it = residents.find(o.id);
            if (it != residents.end()) {
                Resident& R = it->second;
                if (R.bytes != r.op_bytes[i]) {
                    rollback();
                    fail_request(r, "serve: operand id " + std::to_string(o.id) + " is resident with " +
                                        std::to_string(R.bytes) + " bytes, the request needs " +
                                        std::to_string(r.op_bytes[i]));
                    return REFUSED;
                }
                if (R.idle) {
                    idle_lru.erase(R.lru);
                    R.idle = false;
                }
                ++R.refs;
                refd.push_back(o.id);
                if (R.upload_seq > uploads_done_seq) r.wait_upload = true;
                r.op_off[i] = R.off;
                ++st.resident_hits;
                continue;
            }
            if (!o.host) {
                rollback();
                fail_request(r, "serve: operand id " + std::to_string(o.id) + " is not resident and has no host bytes");
                return REFUSED;
            }
            uint64_t off = 0;
            if (!alloc_evicting(r.op_bytes[i], &off)) {
                rollback();
                return BLOCKED;
            }
            Resident R;
            R.off = off;
            R.bytes = r.op_bytes[i];
            R.refs = 1;
            R.upload_seq = ++upload_seq;
            residents.emplace(o.id, R);
            resident_bytes += R.bytes;
            created.push_back(o.id);
            refd.push_back(o.id);
            ups.push_back(Upload{o.host, off, R.bytes, cfg.upload_engine == 0 && r.op_direct[i] != 0});
            r.uploaded += R.bytes;
            r.op_off[i] = off;
            ++st.resident_misses;
        }
        return ADMITTED;
    }

    AetherLaunch launch_of(const Request& r, std::vector<AetherOperand>& ops) const {
        ops.resize(std::max<size_t>(1, r.ops.size()));
        for (size_t i = 0; i < r.ops.size(); ++i) ops[i] = AetherOperand{base + r.op_off[i], r.ops[i].pitch};
        AetherLaunch a{};
        a.n = r.n;
        a.dst = base + r.out_off;
        a.dst_pitch = r.out_pitch;
        a.operands = ops.data();
        a.n_operands = uint32_t(r.ops.size());
        a.scalars = r.sc.data();
        a.n_scalars = uint32_t(r.sc.size());
        a.keys = r.keys.data();
        a.n_keys = uint32_t(r.keys.size());
        return a;
    }

    // Enqueue the copies, the launch and the output copies of one slot (mu not held).
    void enqueue(Slot& S, const std::vector<Upload>& ups, bool wait_uploads) {
        // Mapped pinned sources go through one gather kernel per slot (in
        // launches of up to kAgCopyMaxSegments); the rest through the copy engine.
        AgCopyBatch gb;
        gb.n = 0;
        for (const Upload& u : ups) {
            if (!u.direct) {
                ag_ck(cudaMemcpyAsync(base + u.off, u.host, u.bytes, cudaMemcpyHostToDevice, copy_stream),
                      "cudaMemcpyAsync(operand)");
                continue;
            }
            gb.seg[gb.n++] = AgCopySegment{u.host, base + u.off, u.bytes};
            if (gb.n == kAgCopyMaxSegments) {
                ag_ck(ag_gather_copy(gb, sms, copy_stream), "gather copy");
                gb.n = 0;
            }
        }
        if (gb.n) ag_ck(ag_gather_copy(gb, sms, copy_stream), "gather copy");
        const bool need_wait = !ups.empty() || wait_uploads;
        if (!need_wait) S.n_first = 0;
        S.cp_end.clear();
        S.cp_next = 0;
        S.retired = 0;
        // requests on resident operands only: launched before the wait
        if (S.n_first) launch_group(S, 0, S.n_first);
        if (need_wait) {
            ag_ck(cudaEventRecord(S.copied, copy_stream), "cudaEventRecord(copied)");
            ag_ck(cudaStreamWaitEvent(S.stream, S.copied, 0), "cudaStreamWaitEvent(copied)");
        }
        launch_group(S, S.n_first, S.rs.size() - S.n_first);
    }

    // Mark on the slot's stream the end of requests [.., end): they retire
    // when this event completes.
    void checkpoint(Slot& S, size_t end) {
        const size_t k = S.cp_end.size();
        if (k == S.cp_ev.size()) {
            cudaEvent_t e = nullptr;
            ag_ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate(checkpoint)");
            S.cp_ev.push_back(e);
        }
        ag_ck(cudaEventRecord(S.cp_ev[k], S.stream), "cudaEventRecord(checkpoint)");
        S.cp_end.push_back(end);
    }

    // The host output copies of requests [b, e) of a slot.
    void copy_outputs(Slot& S, size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            const Request& r = *S.rs[i];
            if (r.host_out)
                ag_ck(cudaMemcpyAsync(r.host_out, base + r.out_off, r.out_bytes, cudaMemcpyDeviceToHost, S.stream),
                      "cudaMemcpyAsync(output)");
        }
    }

    // Launch requests [first, first + count) of a slot on its stream, then
    // their host output copies. One request runs its plan's own kernel (no
    // work list, same arithmetic); several run as one batched kernel.
    // One request through its plan's own kernel.
    void launch_plain(const Request& r, cudaStream_t stream, std::vector<AetherOperand>& ops) {
        PlanObj* P = plans[size_t(r.plan)];
        AetherLaunch a = launch_of(r, ops);
        AgArgsHost k;
        const bool vect = make_args(P, &a, k) && P->vec > 1;
        const uint64_t per = chunk_samples(*P, vect);
        const int bps = vect ? P->blocks_per_sm_v : P->blocks_per_sm_s;
        const uint64_t cap = uint64_t(std::max(bps, 1)) * uint64_t(P->sms);
        const unsigned grid = unsigned(std::max<uint64_t>(1, std::min((r.n + per - 1) / per, cap)));
        void* params[] = {&k};
        ag_ck(cudaLaunchKernel(reinterpret_cast<const void*>(vect ? P->fv : P->fs), dim3(grid),
                               dim3(unsigned(P->low.block)), params, 0, stream),
              "cudaLaunchKernel(plain)");
    }

    void launch_group(Slot& S, size_t first, size_t count) {
        if (!count) return;
        std::vector<AetherOperand> ops;
        if (count == 1) {
            launch_plain(*S.rs[first], S.stream, ops);
            copy_outputs(S, first, first + 1);
            checkpoint(S, first + 1);
        } else if (!plan_batch.empty()) {
            // grouped by plan (the caller sorted the range): one work list,
            // copied once, and one launch per plan -- its own kernel for a
            // lone request, the plan's work-list kernel for several
            size_t b = 0;
            std::vector<std::pair<size_t, uint64_t>> runs;   // (end of run, tiles)
            while (b < count) {
                const int plan = S.rs[first + b]->plan;
                const BatchObj& B = *plan_batch[size_t(plan)];
                size_t e = b;
                uint64_t tiles = 0;
                while (e < count && S.rs[first + e]->plan == plan) {
                    const Request& r = *S.rs[first + e];
                    AgItemHost& h = S.staging[first + e];
                    h = AgItemHost{};
                    AetherLaunch a = launch_of(r, ops);
                    make_args(B.plans[0], &a, h.a);   // alignment was checked at submit
                    h.tile0 = tiles;
                    h.plan = 0;
                    const uint64_t per = batch_tile_samples(B, 0);
                    tiles += (r.n + per - 1) / per;
                    ++e;
                }
                runs.push_back({e, tiles});
                b = e;
            }
            AgItemHost* dev = static_cast<AgItemHost*>(S.dev_items) + first;
            if (runs.size() < count)
                ag_ck(cudaMemcpyAsync(dev, S.staging + first, count * sizeof(AgItemHost), cudaMemcpyHostToDevice,
                                      S.stream),
                      "cudaMemcpyAsync(work list)");
            b = 0;
            for (const auto& run : runs) {
                const size_t e = run.first;
                if (e - b == 1) {
                    launch_plain(*S.rs[first + b], S.stream, ops);
                } else {
                    const BatchObj& B = *plan_batch[size_t(S.rs[first + b]->plan)];
                    void* items = dev + b;
                    int n = int(e - b);
                    uint64_t t = run.second;
                    void* params[] = {&items, &n, &t};
                    ag_ck(cudaLaunchKernel(reinterpret_cast<const void*>(B.kernel), dim3(batch_grid(B, t)),
                                           dim3(unsigned(B.block)), params, 0, S.stream),
                          "cudaLaunchKernel(batch)");
                }
                // this plan's requests finish here, before the runs after it
                copy_outputs(S, first + b, first + e);
                checkpoint(S, first + e);
                b = e;
            }
        } else {
            uint64_t tiles = 0;
            for (size_t i = 0; i < count; ++i) {
                const Request& r = *S.rs[first + i];
                AgItemHost& h = S.staging[first + i];
                h = AgItemHost{};
                AetherLaunch a = launch_of(r, ops);
                make_args(batch->plans[size_t(r.plan)], &a, h.a);   // alignment was checked at submit
                h.tile0 = tiles;
                h.plan = r.plan;
                const uint64_t per = batch_tile_samples(*batch, r.plan);
                tiles += (r.n + per - 1) / per;
            }
            AgItemHost* dev = static_cast<AgItemHost*>(S.dev_items) + first;
            ag_ck(cudaMemcpyAsync(dev, S.staging + first, count * sizeof(AgItemHost), cudaMemcpyHostToDevice, S.stream),
                  "cudaMemcpyAsync(work list)");
            void* items = dev;
            int n = int(count);
            uint64_t t = tiles;
            void* params[] = {&items, &n, &t};
            ag_ck(cudaLaunchKernel(reinterpret_cast<const void*>(batch->kernel), dim3(batch_grid(*batch, tiles)),
                                   dim3(unsigned(batch->block)), params, 0, S.stream),
                  "cudaLaunchKernel(batch)");
            copy_outputs(S, first, first + count);
            checkpoint(S, first + count);
        }
    }

    // Retire requests [b, e) of a slot that finished with status `err` (mu held).
    void retire_range(Slot& S, size_t b, size_t e, cudaError_t err, uint64_t t) {
        if (err != cudaSuccess && fatal.empty()) fatal = std::string("serve: launch failed: ") + cudaGetErrorString(err);
        for (size_t i = b; i < e; ++i) {
            Request& r = *S.rs[i];
            for (const AetherServeOperand& o : r.ops) unref(o.id);
            if (err != cudaSuccess) {
                fail_request(r, fatal);
            } else {
                r.state = AETHER_SERVE_DONE;
                r.t_done = t;
                ++st.completed;
                st.bytes += r.bytes;
                st.uploaded_bytes += r.uploaded;
                st.last_done_ns = std::max(st.last_done_ns, t);
            }
            if (!(r.flags & AETHER_SERVE_KEEP_OUTPUT) || err != cudaSuccess) {
                arena.release(r.out_off, r.out_bytes);
                r.out_live = false;
            }
        }
    }

    // Retire what the completion events say finished (mu held).
    void retire(const std::vector<Fin>& fin, uint64_t t) {
        for (const Fin& f : fin) {
            Slot& S = *f.s;
            const size_t end = f.cp == SIZE_MAX ? S.rs.size() : S.cp_end[f.cp];
            retire_range(S, S.retired, end, f.e, t);
            S.retired = end;
            if (S.retired < S.rs.size()) continue;
            uploads_done_seq = std::max(uploads_done_seq, S.upload_seq);
            S.rs.clear();
            S.n_first = 0;
            S.cp_end.clear();
            S.cp_next = 0;
            S.retired = 0;
            S.busy = false;
        }
        if (!fin.empty()) cv_done.notify_all();
    }

    bool any_busy() const {
        for (const Slot& S : slots)
            if (S.busy) return true;
        return false;
    }

    // Admit queued requests into slot S (mu held). Returns whether the head of
    // the queue is blocked on arena bytes.
    bool admit(Slot& S, size_t limit, std::vector<Upload>& ups, bool& wait_uploads) {
        while (!queue.empty() && S.rs.size() < limit) {
            Request& r = reqs[queue.front()];
            const Admit a = try_admit(r, ups);
            if (a == BLOCKED) return true;
            if (a == ADMITTED) {
                S.rs.push_back(&r);
                wait_uploads = wait_uploads || r.wait_upload;
            }
            queue.pop_front();
        }
        return false;
    }

    // The loop. Slots belong to this thread: it polls their events without
    // the lock and takes the lock only to retire, admit and record.
    void run() {
        cudaSetDevice(dev);
        const size_t limit = cfg.mode == AETHER_SERVE_PLAIN ? 1 : size_t(cfg.max_items);
        std::vector<Fin> fin;
        std::unique_lock<std::mutex> lk(mu, std::defer_lock);
        const uint64_t spin_ns = uint64_t(cfg.idle_spin_us) * 1000u;
        uint64_t last_work = now();
        while (true) {
            fin.clear();
            for (Slot& S : slots) {
                if (!S.busy) continue;
                // checkpoints complete in stream order
                while (S.cp_next < S.cp_end.size()) {
                    const cudaError_t e = cudaEventQuery(S.cp_ev[S.cp_next]);
                    if (e == cudaErrorNotReady) break;
                    if (e != cudaSuccess) {
                        cudaGetLastError();
                        fin.push_back(Fin{&S, e, SIZE_MAX});   // the rest of the slot fails
                        S.cp_next = S.cp_end.size();
                        break;
                    }
                    fin.push_back(Fin{&S, e, S.cp_next});
                    ++S.cp_next;
                }
            }
            const uint64_t t_fin = fin.empty() ? 0 : now();
            lk.lock();
            retire(fin, t_fin);
            Slot* S = nullptr;
            size_t free_slots = 0;
            for (Slot& sl : slots)
                if (!sl.busy) {
                    if (!S) S = &sl;
                    ++free_slots;
                }
            bool blocked = false;
            if (S && !queue.empty() && fatal.empty()) {
                std::vector<Upload> ups;
                bool wait_uploads = false;
                const uint64_t ta = now();
                // Spread what waits over the free slots: requests run side by
                // side on separate streams while slots are free (a light load
                // launches them one by one, as plain mode does), and share
                // launches only once the queue outgrows the free slots.
                const size_t share = (queue.size() + free_slots - 1) / free_slots;
                blocked = admit(*S, std::min(limit, std::max<size_t>(1, share)), ups, wait_uploads);
                st.admit_ns += now() - ta;
                if (!S->rs.empty()) {
                    // requests that read resident operands only go first
                    auto mid = std::stable_partition(S->rs.begin(), S->rs.end(), [](const Request* r) {
                        return r->uploaded == 0 && !r->wait_upload;
                    });
                    const size_t ready = size_t(mid - S->rs.begin());
                    S->n_first = (ready > 0 && ready < S->rs.size()) ? ready : 0;
                    if (!plan_batch.empty()) {
                        // each launch group ordered by plan, one run per plan,
                        // the plan with the least work first: its requests
                        // retire at their own checkpoint, before larger runs
                        std::vector<uint64_t> work(plans.size());
                        auto order = [&](std::vector<Request*>::iterator b, std::vector<Request*>::iterator e) {
                            std::fill(work.begin(), work.end(), 0);
                            for (auto it = b; it != e; ++it) work[size_t((*it)->plan)] += (*it)->n;
                            std::stable_sort(b, e, [&](const Request* x, const Request* y) {
                                const uint64_t wx = work[size_t(x->plan)], wy = work[size_t(y->plan)];
                                return wx != wy ? wx < wy : x->plan < y->plan;
                            });
                        };
                        order(S->rs.begin(), mid);
                        order(mid, S->rs.end());
                    }
                    S->busy = true;
                    // The completion of a slot that waited for the copy stream
                    // proves every copy enqueued before its wait has landed.
                    S->upload_seq = (wait_uploads || !ups.empty()) ? upload_seq : 0;
                    const uint64_t td = now();
                    for (Request* rp : S->rs) {
                        rp->state = AETHER_SERVE_RUNNING;
                        rp->t_dispatch = td;
                        rp->launch_items = int(S->rs.size());
                    }
                    ++st.launches;
                    st.launched_items += S->rs.size();
                    lk.unlock();
                    std::string err;
                    try {
                        enqueue(*S, ups, wait_uploads);
                    } catch (const std::exception& ex) {
                        err = ex.what();
                    }
                    const uint64_t t_enq = now() - td;
                    lk.lock();
                    st.enqueue_ns += t_enq;
                    if (!err.empty()) {
                        // Nothing of this slot may still be queued behind a
                        // failed call; wait for what was enqueued, then fail it.
                        cudaStreamSynchronize(S->stream);
                        cudaStreamSynchronize(copy_stream);
                        cudaGetLastError();
                        if (fatal.empty()) fatal = err;
                        for (Request* rp : S->rs) {
                            Request& r = *rp;
                            for (const AetherServeOperand& o : r.ops) unref(o.id);
                            arena.release(r.out_off, r.out_bytes);
                            r.out_live = false;
                            fail_request(r, err);
                        }
                        S->rs.clear();
                        S->n_first = 0;
                        S->cp_end.clear();
                        S->cp_next = 0;
                        S->retired = 0;
                        S->busy = false;
                        cv_done.notify_all();
                    }
                    lk.unlock();
                    continue;
                }
            }
            if (!fatal.empty() && !queue.empty()) {
                // A device error ends the server: fail what waits.
                while (!queue.empty()) {
                    fail_request(reqs[queue.front()], fatal);
                    queue.pop_front();
                }
                cv_done.notify_all();
            }
            const bool busy = any_busy();
            if (stop && queue.empty() && !busy) break;
            if (busy || !fin.empty()) last_work = now();
            if (!busy && (queue.empty() || blocked) && now() - last_work >= spin_ns) {
                // Idle for the spin window, or blocked behind kept outputs
                // only the client can free: sleep until a submit or release.
                cv_work.wait_for(lk, std::chrono::milliseconds(blocked ? 1 : 50));
                lk.unlock();
                last_work = now() - spin_ns;
                continue;
            }
            lk.unlock();
            if (fin.empty()) std::this_thread::yield();
        }
    }
};

uint64_t planes_of(ag::DType d, int comps) { return uint64_t(comps) * (d == ag::DType::FF ? 2u : 1u); }

// Whether [p, p + bytes) is pinned host memory the device reads at the same
// address (16-byte aligned at the start): checked at both ends.
bool mapped_host(const void* p, uint64_t bytes) {
    if (!bytes || (reinterpret_cast<uintptr_t>(p) & 15u)) return false;
    const char* ends[2] = {static_cast<const char*>(p), static_cast<const char*>(p) + bytes - 1};
    for (const char* q : ends) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (at.type != cudaMemoryTypeHost || at.devicePointer != q) return false;
    }
    return true;
}

int serve_fail(const std::string& m) { return ag_internal_fail(m.c_str()); }

template <class F>
int serve_guarded(F&& f) {
    try {
        f();
        return AETHER_OK;
    } catch (const std::exception& e) {
        return serve_fail(e.what());
    }
}

// Validate one request and build its record (no lock needed).
Request build_request(Server* S, const AetherServeRequest* q) {
    if (!q) throw std::runtime_error("serve_submit: null request");
    if (q->plan < 0 || size_t(q->plan) >= S->plans.size())
        throw std::runtime_error("serve_submit: plan index " + std::to_string(q->plan) + " of " +
                                 std::to_string(S->plans.size()));
    const PlanObj* P = S->plans[size_t(q->plan)];
    const ag::Plan& pl = P->plan;
    if (q->n == 0 || q->n > 0xFFFFFFFFull) throw std::runtime_error("serve_submit: n must be in [1, 2^32 - 1]");
    if (int(q->n_operands) != pl.n_operands)
        throw std::runtime_error("serve_submit: plan reads " + std::to_string(pl.n_operands) + " operands, " +
                                 std::to_string(q->n_operands) + " given");
    if (int(q->n_scalars) < pl.n_scalars) throw std::runtime_error("serve_submit: too few scalars");
    if (int(q->n_keys) < pl.n_keys) throw std::runtime_error("serve_submit: too few generator keys");
    if (q->n_operands && !q->operands) throw std::runtime_error("serve_submit: null operand list");
    Request r;
    r.plan = q->plan;
    r.flags = q->flags;
    r.n = q->n;
    r.host_out = q->host_out;
    uint64_t need = 0;
    for (uint32_t i = 0; i < q->n_operands; ++i) {
        AetherServeOperand o = q->operands[i];
        const int comps = pl.operand_comps[i];
        const int es = ag::dtype_size(pl.operand_dtype[i]);
        if (!o.pitch) o.pitch = q->n;
        if (comps > 1 && o.pitch < q->n)
            throw std::runtime_error("serve_submit: operand " + std::to_string(i) + " pitch smaller than n");
        if (comps > 1 && (o.pitch * uint64_t(es)) % 16)
            throw std::runtime_error("serve_submit: operand " + std::to_string(i) +
                                     " planes are not 16-byte aligned (pitch * element size)");
        const uint64_t b = planes_of(pl.operand_dtype[i], comps) * o.pitch * uint64_t(es);
        r.ops.push_back(o);
        r.op_bytes.push_back(b);
        r.op_direct.push_back(o.host && mapped_host(o.host, b) ? 1 : 0);
        need += Arena::span(b);
        r.bytes += q->n * planes_of(pl.operand_dtype[i], comps) * uint64_t(es);
    }
    r.sc.assign(q->scalars, q->scalars + q->n_scalars);
    if (q->n_keys) r.keys.assign(q->keys, q->keys + q->n_keys);
    const int oes = ag::dtype_size(pl.dst_dtype);
    const uint64_t oplanes = planes_of(pl.dst_dtype, pl.dst_comps);
    r.out_pitch = round_up(q->n, 32);
    r.out_bytes = oplanes * r.out_pitch * uint64_t(oes);
    r.bytes += q->n * oplanes * uint64_t(oes);
    need += Arena::span(r.out_bytes);
    if (need > S->arena.size())
        throw std::runtime_error("serve_submit: the request needs " + std::to_string(need) +
                                 " bytes of arena, the budget is " + std::to_string(S->arena.size()));
    return r;
}

// Queue `count` built requests under one lock; request i arrived at arrivals[i].
void queue_requests(Server* S, Request* rs, size_t count, const uint64_t* arrivals, uint64_t* tickets) {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) throw std::runtime_error("serve_submit: the server is closing");
    for (size_t i = 0; i < count; ++i) {
        rs[i].t_arrival = arrivals[i];
        tickets[i] = S->reqs.size();
        S->reqs.push_back(std::move(rs[i]));
        S->queue.push_back(tickets[i]);
        if (++S->st.submitted == 1) S->st.first_arrival_ns = arrivals[i];
    }
    S->cv_work.notify_one();
}

void fill_status(const Server* S, const Request& r, AetherServeStatus* o) {
    *o = AetherServeStatus{};
    o->state = r.state;
    o->launch_items = r.launch_items;
    o->t_arrival_ns = r.t_arrival;
    o->t_dispatch_ns = r.t_dispatch;
    o->t_done_ns = r.t_done;
    o->output = (r.out_live && r.state == AETHER_SERVE_DONE) ? S->base + r.out_off : nullptr;
    o->out_pitch = r.out_pitch;
    o->bytes = r.bytes;
    o->uploaded_bytes = r.uploaded;
}

void destroy(Server* S) {
    if (S->loop.joinable()) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
        }
        S->cv_work.notify_all();
        S->loop.join();
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(S->dev);
    for (Slot& sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        for (cudaEvent_t e : sl.cp_ev) cudaEventDestroy(e);
        if (sl.copied) cudaEventDestroy(sl.copied);
        if (sl.staging) cudaFreeHost(sl.staging);
        if (sl.dev_items) cudaFree(sl.dev_items);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (S->copy_stream) {
        cudaStreamSynchronize(S->copy_stream);
        cudaStreamDestroy(S->copy_stream);
    }
    if (S->base) cudaFree(S->base);
    if (S->batch) aether_batch_release(S->batch);
    for (BatchObj* b : S->plan_batch) aether_batch_release(b);
    cudaGetLastError();
    cudaSetDevice(prev);
    delete S;
}

}  // namespace

AG_EXPORT int aether_serve_open(void* const* plans, int n_plans, const AetherServeConfig* config, void** out) {
    return serve_guarded([&] {
        if (!plans || n_plans <= 0 || !config || !out) throw std::runtime_error("serve_open: null argument");
        std::unique_ptr<Server, void (*)(Server*)> S(new Server, destroy);
        S->cfg = *config;
        if (S->cfg.mode != AETHER_SERVE_BATCHED && S->cfg.mode != AETHER_SERVE_PLAIN)
            throw std::runtime_error("serve_open: mode must be AETHER_SERVE_BATCHED or AETHER_SERVE_PLAIN");
        if (S->cfg.max_inflight <= 0) S->cfg.max_inflight = 4;
        if (S->cfg.max_items <= 0) S->cfg.max_items = 256;
        if (S->cfg.block <= 0) S->cfg.block = 512;
        if (S->cfg.ipt <= 0) S->cfg.ipt = 1;
        if (S->cfg.idle_spin_us < 0) S->cfg.idle_spin_us = 0;
        if (S->cfg.idle_spin_us == 0) S->cfg.idle_spin_us = 2000;
        if (S->cfg.max_inflight > 64) throw std::runtime_error("serve_open: max_inflight above 64");
        if (S->cfg.max_items > 65536) throw std::runtime_error("serve_open: max_items above 65536");
        if (S->cfg.hbm_budget_bytes < (1u << 20)) throw std::runtime_error("serve_open: budget below 1 MiB");
        for (int p = 0; p < n_plans; ++p) {
            PlanObj* P = static_cast<PlanObj*>(plans[p]);
            if (!P) throw std::runtime_error("serve_open: null plan");
            if (P->plan.wants_sum()) throw std::runtime_error("serve_open: sum plans cannot be served");
            if (P->plan.op != "set") throw std::runtime_error("serve_open: served plans overwrite their output (op set)");
            S->plans.push_back(P);
        }
        ag_ck(cudaGetDevice(&S->dev), "cudaGetDevice");
        ag_ck(cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->dev), "cudaDeviceGetAttribute");
        AetherLowering low{};
        low.block = S->cfg.block;
        low.ipt = S->cfg.ipt;
        if (S->cfg.grouping != 0 && S->cfg.grouping != 1) throw std::runtime_error("serve_open: grouping must be 0 or 1");
        if (S->cfg.mode == AETHER_SERVE_BATCHED && S->cfg.grouping == 0) {
            for (int p = 0; p < n_plans; ++p) {
                // each plan's work-list kernel takes the plan's own block shape
                // and occupancy bound (its tuned lowering) unless the server sets one
                const PlanObj* P = S->plans[size_t(p)];
                AetherLowering lp{};
                lp.block = config->block > 0 ? config->block : P->low.block;
                lp.ipt = config->ipt > 0 ? config->ipt : P->low.ipt;
                lp.min_blocks = config->block > 0 ? 0 : P->low.min_blocks;
                void* b = nullptr;
                if (aether_batch_create(&plans[p], 1, &lp, &b) != AETHER_OK)
                    throw std::runtime_error(aether_last_error());
                S->plan_batch.push_back(static_cast<BatchObj*>(b));
            }
        } else {
            void* b = nullptr;
            if (aether_batch_create(plans, n_plans, &low, &b) != AETHER_OK) throw std::runtime_error(aether_last_error());
            S->batch = static_cast<BatchObj*>(b);
        }
        void* base = nullptr;
        ag_ck(cudaMalloc(&base, S->cfg.hbm_budget_bytes), "cudaMalloc(serving arena)");
        S->base = static_cast<char*>(base);
        S->arena.init(S->cfg.hbm_budget_bytes);
        S->st.arena_bytes = S->cfg.hbm_budget_bytes;
        ag_ck(cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(copy)");
        S->slots.resize(size_t(S->cfg.max_inflight));
        const size_t items = S->cfg.mode == AETHER_SERVE_PLAIN ? 1 : size_t(S->cfg.max_items);
        for (Slot& sl : S->slots) {
            ag_ck(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "cudaStreamCreate(slot)");
            ag_ck(cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming), "cudaEventCreate");
            void* h = nullptr;
            ag_ck(cudaMallocHost(&h, items * sizeof(AgItemHost)), "cudaMallocHost(work list)");
            sl.staging = static_cast<AgItemHost*>(h);
            ag_ck(cudaMalloc(&sl.dev_items, items * sizeof(AgItemHost)), "cudaMalloc(work list)");
        }
        S->t0 = Clock::now();
        Server* raw = S.get();
        S->loop = std::thread([raw] { raw->run(); });
        *out = S.release();
    });
}

AG_EXPORT int aether_serve_submit(void* server, const AetherServeRequest* request, uint64_t* ticket) {
    return serve_guarded([&] {
        Server* S = static_cast<Server*>(server);
        if (!S || !ticket) throw std::runtime_error("serve_submit: null argument");
        Request r = build_request(S, request);
        const uint64_t t = S->now();
        queue_requests(S, &r, 1, &t, ticket);
    });
}

AG_EXPORT int aether_serve_feed(void* server, const AetherServeRequest* requests, int count, uint64_t* tickets) {
    return serve_guarded([&] {
        Server* S = static_cast<Server*>(server);
        if (!S || (count > 0 && (!requests || !tickets))) throw std::runtime_error("serve_feed: null argument");
        // Build every record first, so the timed loop only queues them.
        std::vector<Request> rs;
        rs.reserve(size_t(std::max(count, 0)));
        for (int i = 0; i < count; ++i) rs.push_back(build_request(S, &requests[i]));
        std::vector<uint64_t> due(rs.size());
        const uint64_t start = S->now();
        for (size_t i = 0; i < rs.size(); ++i) due[i] = start + requests[i].arrival_ns;
        size_t i = 0;
        while (i < rs.size()) {
            uint64_t t = S->now();
            while (t < due[i]) {
                if (due[i] - t > 200000) std::this_thread::sleep_for(std::chrono::nanoseconds(due[i] - t - 100000));
                else std::this_thread::yield();
                t = S->now();
            }
            // everything due by now goes in under one lock
            size_t j = i + 1;
            while (j < rs.size() && due[j] <= t) ++j;
            queue_requests(S, &rs[i], j - i, &due[i], &tickets[i]);
            i = j;
        }
    });
}

AG_EXPORT int aether_serve_status(void* server, uint64_t ticket, AetherServeStatus* status) {
    return serve_guarded([&] {
        Server* S = static_cast<Server*>(server);
        if (!S || !status) throw std::runtime_error("serve_status: null argument");
        std::lock_guard<std::mutex> lk(S->mu);
        if (ticket >= S->reqs.size()) throw std::runtime_error("serve_status: unknown ticket");
        fill_status(S, S->reqs[ticket], status);
    });
}

AG_EXPORT int aether_serve_wait(void* server, uint64_t ticket, double timeout_s, AetherServeStatus* status) {
    Server* S = static_cast<Server*>(server);
    if (!S) return serve_fail("serve_wait: null server");
    std::unique_lock<std::mutex> lk(S->mu);
    if (ticket >= S->reqs.size()) return serve_fail("serve_wait: unknown ticket");
    const Request& r = S->reqs[ticket];
    const auto until = Clock::now() + std::chrono::nanoseconds(int64_t(std::min(std::max(0.0, timeout_s), 1e6) * 1e9));
    while (r.state != AETHER_SERVE_DONE && r.state != AETHER_SERVE_FAILED) {
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout &&
            r.state != AETHER_SERVE_DONE && r.state != AETHER_SERVE_FAILED)
            return serve_fail("serve_wait: timed out");
    }
    if (status) fill_status(S, r, status);
    if (r.state == AETHER_SERVE_FAILED) return serve_fail(r.error);
    return AETHER_OK;
}

AG_EXPORT int aether_serve_release(void* server, uint64_t ticket) {
    return serve_guarded([&] {
        Server* S = static_cast<Server*>(server);
        if (!S) throw std::runtime_error("serve_release: null server");
        std::lock_guard<std::mutex> lk(S->mu);
        if (ticket >= S->reqs.size()) throw std::runtime_error("serve_release: unknown ticket");
        Request& r = S->reqs[ticket];
        if (r.state != AETHER_SERVE_DONE) throw std::runtime_error("serve_release: the request has not finished");
        if (r.out_live) {
            S->arena.release(r.out_off, r.out_bytes);
            r.out_live = false;
        }
        S->cv_work.notify_one();
    });
}

AG_EXPORT int aether_serve_stats(void* server, AetherServeStats* stats) {
    return serve_guarded([&] {
        Server* S = static_cast<Server*>(server);
        if (!S || !stats) throw std::runtime_error("serve_stats: null argument");
        std::lock_guard<std::mutex> lk(S->mu);
        *stats = S->st;
        stats->arena_peak_bytes = S->arena.peak();
        stats->resident_bytes = S->resident_bytes;
    });
}

AG_EXPORT void aether_serve_close(void* server) {
    if (server) destroy(static_cast<Server*>(server));
}
