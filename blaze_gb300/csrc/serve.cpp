// serve.cpp — request loop with continuous batching for dense products on one GB300.
//
// Blaze has no server; this is the serving form of the same C = alpha*op(A)*op(B) + beta*C path
// (one request = one product, CBLAS argument conventions, device-resident operands).
//
// Model:
//   * Requests arrive at any time (gb300_server_submit) and wait in a queue.
//   * A scheduler thread admits them while a stream slot is free and the device memory the
//     request needs (its scratch, from device_product_footprint) fits the server's budget next to
//     what running requests hold; a request that cannot fit even on an idle server is rejected.
//     Admission is FIFO with backfill: a smaller request may pass a head request that does not fit
//     yet, unless the head has waited longer than the aging limit.
//   * Each slot owns a stream and a grow-only workspace, so admitted requests run concurrently
//     and their kernels overlap on the device.  Large requests (max(m, n) >= large_threshold) run
//     only on the first `large_slots` slots, whose streams have the lowest priority; the other
//     slots take the rest at a higher priority and the batch lanes at the highest.  The block
//     scheduler dispatches pending blocks of higher-priority streams first, so a large native
//     product with hundreds of waiting CTAs does not hold back the kernels of small and medium
//     requests launched after it (without priorities their p99 was that product's time).  A large
//     request waiting for a large slot does not stop others from passing it, and while a large
//     tensor-core product runs a share of the SMs is also kept out of its persistent grid.
//   * Large native requests run as a chain of k-panels (native_panels), which keeps each CTA of
//     theirs short.
//   * The scheduler thread never waits for the device: slot workspaces are stream-ordered (growing
//     one frees and allocates on the slot's stream) and lanes keep outgrown staging buffers, since
//     cudaFree / cudaFreeHost would wait for every stream, large products included.
//   * Small requests (every dimension at most `batch_threshold`) do not take a slot: at each
//     scheduling step the queued ones are coalesced into one persistent grouped launch (grouped.cu,
//     FP64) on one of two batch lanes, up to `batch_max` per launch, while the previous launch may
//     still run on the other lane.  FP64 meets the bound of every accuracy class (k * 2^-53 for
//     the native and split classes, well below the BF16 classes' bounds), so a small request's
//     class only decides its reported bound.
//   * Completion is detected with a CUDA event per request; latency = completion - submission.
//   * Results do not depend on the mix: the split form accumulates exact integers (its k-segments
//     depend only on the shape), BF16 forms have a fixed accumulation order per tile, the native
//     kernel's split-k choice depends only on the shape, and a grouped launch gives each product
//     the warp-tile shape of its own (m, n, k) with a fixed k order per tile, whatever else is in
//     the batch (a small request alone is a batch of one).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gb300_blas.h"
#include "gb300_internal.h"
#include "ptx.cuh"
#include "runtime.h"
#include "split_api.h"

namespace gb {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct ServeRequest {
    uint64_t id = 0;
    gb300_serve_request req{};
    Gemm g;
    SplitRequest sreq;
    size_t footprint = 0;
    size_t need[kSlotCount] = {};
    bool large = false;       // a large tensor-core product (reserve_sms applies)
    int cls = 1;              // size class: 0 small (grouped launches), 1 medium, 2 large
    Clock::time_point t_submit, t_start, t_end;
    int slot = -1;
    int state = 0;  // 0 queued, 1 running, 2 done
    gb300_serve_result res{};
    cudaEvent_t done = nullptr;
    const void* info_dev = nullptr;
};

struct ServeSlot {
    cudaStream_t stream = nullptr;
    Workspace ws;
    ServeRequest* cur = nullptr;
    // page-locked landing place of the running request's status word and accuracy record, copied
    // behind the product on the slot's stream (read once its completion event has fired)
    uint8_t* host = nullptr;
};
constexpr size_t kHostStatus = 0, kHostInfo = 64, kHostBytes = 512;

// A batch lane: a stream, the grouped-launch buffers and the requests of the launch in flight.
struct BatchLane {
    cudaStream_t stream = nullptr;
    GroupedLane* lane = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<ServeRequest*> batch;
    Clock::time_point t_start;
};
constexpr int kBatchLanes = 2;

enum Admit : int { kAdmitted = 0, kNoSlot, kNoMemory, kLargeLimit };

// Large native FP64 requests run as a chain of k-panels, C = alpha A_p B_p + C (the first panel
// with the request's beta), so that a CTA of the native kernel holds its SM for one panel's k loop
// (about 4 ms at n = 8192 instead of 33 ms): priority decides which stream's blocks take an SM as
// it frees up, and running CTAs are never preempted.  The panel order is fixed, so the result is
// the same alone and in the mix; the bound stays k 2^-53.
constexpr int64_t kServeNativePanel = 1024;

int native_panels(const Gemm& g, const SplitRequest& sreq, const LaunchCtl& ctl, cudaStream_t st, Workspace& ws,
                  SplitResult* res, std::string* err) {
    int rc = GB300_OK;
    for (int64_t k0 = 0; k0 < g.k && rc == GB300_OK; k0 += kServeNativePanel) {
        Gemm q = g;
        q.k = std::min(kServeNativePanel, g.k - k0);
        q.A = static_cast<const double*>(g.A) + (g.ta ? k0 * g.lda : k0);
        q.B = static_cast<const double*>(g.B) + (g.tb ? k0 : k0 * g.ldb);
        if (k0 > 0) q.beta = 1.0;
        rc = device_product(q, sreq, ctl, st, ws, res, err);
    }
    res->error_bound = double(g.k) * 0x1p-53;
    return rc;
}

double percentile(std::vector<double> l, double p) {
    if (l.empty()) return 0.0;
    std::sort(l.begin(), l.end());
    const double pos = p * double(l.size() - 1);
    const size_t lo = size_t(pos);
    const size_t hi = std::min(lo + 1, l.size() - 1);
    return l[lo] + (l[hi] - l[lo]) * (pos - double(lo));
}

}  // namespace

class Server {
  public:
    gb300_server_config cfg{};
    std::vector<ServeSlot> slots;
    std::vector<BatchLane> lanes;
    std::vector<gb300_gemm_problem> batch_probs;
    std::deque<ServeRequest*> queue;
    std::unordered_map<uint64_t, ServeRequest*> reqs;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    uint64_t next_id = 1;
    size_t budget = 0;
    int num_sms = 0;
    // statistics
    std::vector<double> latencies;
    std::vector<double> class_lat[3];
    int64_t grouped_launches = 0, grouped_requests = 0;
    int64_t submitted = 0, completed = 0, rejected = 0, failed = 0;
    double useful_flops = 0;
    Clock::time_point t_first;
    bool any = false;
    size_t peak_bytes = 0;

    size_t bytes_held() const {
        size_t t = 0;
        for (const auto& s : slots) t += s.ws.total();
        return t;
    }

    // Slots [0, n_large) take large requests, the others everything else.
    int n_large = 1;

    // Try to start `r` on a free slot of its kind.
    Admit try_admit(ServeRequest* r) {
        int free_slot = -1;
        const size_t lo = r->cls == 2 ? 0 : size_t(n_large), hi = r->cls == 2 ? size_t(n_large) : slots.size();
        for (size_t i = lo; i < hi; ++i)
            if (!slots[i].cur) { free_slot = int(i); break; }
        if (free_slot < 0) return r->cls == 2 ? kLargeLimit : kNoSlot;
        ServeSlot& sl = slots[size_t(free_slot)];
        // projected bytes of the slot after running r: each buffer grows to the larger of what it
        // holds and what r needs
        auto projected = [&](const ServeSlot& x) {
            size_t t = 0;
            for (int s = 0; s < kSlotCount; ++s) t += std::max(x.ws.bytes[s], r->need[s]);
            return t;
        };
        size_t others = 0;
        for (size_t i = 0; i < slots.size(); ++i)
            if (int(i) != free_slot) others += slots[i].ws.total();
        if (others + projected(sl) > budget) {
            // give back memory of idle slots (this one included) before refusing
            for (size_t i = 0; i < slots.size(); ++i)
                if (!slots[i].cur && slots[i].ws.total() > 0) slots[i].ws.release();
            others = 0;
            for (size_t i = 0; i < slots.size(); ++i)
                if (int(i) != free_slot) others += slots[i].ws.total();
            if (others + projected(sl) > budget) return kNoMemory;
        }
        launch(r, free_slot);
        return kAdmitted;
    }

    // Coalesce queued small requests into one grouped launch on an idle lane.
    bool launch_batch(BatchLane& ln) {
        batch_probs.clear();
        ln.batch.clear();
        const size_t cap = size_t(std::max(1, cfg.batch_max));
        for (auto it = queue.begin(); it != queue.end() && ln.batch.size() < cap;) {
            ServeRequest* r = *it;
            if (r->cls != 0) {
                ++it;
                continue;
            }
            gb300_gemm_problem p;
            p.order = r->req.order; p.transA = r->req.transA; p.transB = r->req.transB;
            p.m = r->req.m; p.n = r->req.n; p.k = r->req.k;
            p.alpha = r->req.alpha; p.beta = r->req.beta;
            p.A = r->req.A; p.lda = r->req.lda; p.B = r->req.B; p.ldb = r->req.ldb;
            p.C = r->req.C; p.ldc = r->req.ldc;
            batch_probs.push_back(p);
            ln.batch.push_back(r);
            it = queue.erase(it);
        }
        if (ln.batch.empty()) return false;
        ln.t_start = Clock::now();
        std::string err;
        const int st = grouped_lane_launch(ln.lane, batch_probs.data(), int64_t(batch_probs.size()), nullptr, &err);
        for (ServeRequest* r : ln.batch) {
            r->state = 1;
            r->t_start = ln.t_start;
            r->res.status = st;
            r->res.method_used = GB300_METHOD_NATIVE;
            r->res.slices = 0;
            r->res.error_bound = double(std::max<int64_t>(r->req.k, 1)) * 0x1p-53;
        }
        cudaEventRecord(ln.done, ln.stream);
        ++grouped_launches;
        grouped_requests += int64_t(ln.batch.size());
        return true;
    }

    void finish(ServeRequest* r) {
        r->t_end = Clock::now();
        r->res.queue_ms = ms_between(r->t_submit, r->t_start);
        r->res.latency_ms = ms_between(r->t_submit, r->t_end);
        r->res.run_ms = ms_between(r->t_start, r->t_end);
        r->state = 2;
        if (r->res.status == GB300_OK) {
            ++completed;
            latencies.push_back(r->res.latency_ms);
            class_lat[r->cls].push_back(r->res.latency_ms);
            useful_flops += 2.0 * double(r->g.m) * double(r->g.n) * double(r->g.k);
        } else {
            ++failed;
        }
    }

    void complete_batch(BatchLane& ln) {
        for (ServeRequest* r : ln.batch) finish(r);
        ln.batch.clear();
    }

    void launch(ServeRequest* r, int si) {
        ServeSlot& sl = slots[size_t(si)];
        r->slot = si;
        r->state = 1;
        r->t_start = Clock::now();
        sl.cur = r;
        LaunchCtl ctl;
        ctl.status = sl.ws.d_status;
        SplitRequest sreq = r->sreq;
        // keep SMs for small requests while a large tensor-core product runs
        if (r->large && cfg.reserve_sms > 0) sreq.max_sms = std::max(1, num_sms - cfg.reserve_sms);
        std::string err;
        cudaMemsetAsync(sl.ws.d_status, 0, sizeof(int), sl.stream);
        SplitResult res;
        const bool panels = r->cls == 2 && sreq.method == GB300_METHOD_NATIVE && r->g.k > kServeNativePanel;
        const int st = panels ? native_panels(r->g, sreq, ctl, sl.stream, sl.ws, &res, &err)
                              : device_product(r->g, sreq, ctl, sl.stream, sl.ws, &res, &err);
        r->res.status = st;
        r->res.method_used = res.method_used;
        r->res.slices = res.slices;
        r->res.error_bound = res.error_bound;
        r->info_dev = res.info_dev;
        cudaMemcpyAsync(sl.host + kHostStatus, sl.ws.d_status, sizeof(int), cudaMemcpyDeviceToHost, sl.stream);
        if (r->info_dev && split_info_bytes() <= kHostBytes - kHostInfo)
            cudaMemcpyAsync(sl.host + kHostInfo, r->info_dev, split_info_bytes(), cudaMemcpyDeviceToHost, sl.stream);
        cudaEventRecord(r->done, sl.stream);
        peak_bytes = std::max(peak_bytes, bytes_held());
        if (st != GB300_OK) r->res.status = st;
    }

    void complete(ServeSlot& sl) {
        ServeRequest* r = sl.cur;
        int status = 0;
        std::memcpy(&status, sl.host + kHostStatus, sizeof(int));
        if (r->res.status == GB300_OK && status != 0) r->res.status = GB300_ERR_DEVICE_TIMEOUT;
        if (r->info_dev && split_info_bytes() <= kHostBytes - kHostInfo) {
            int sl_ = 0;
            double bd = 0;
            split_decode_info(sl.host + kHostInfo, &sl_, &bd);
            r->res.slices = sl_;
            r->res.error_bound = bd;
        }
        finish(r);
        sl.cur = nullptr;
    }

    void loop() {
        std::unique_lock<std::mutex> lock(mu);
        while (!stop) {
            bool progressed = false;
            // completions
            for (auto& sl : slots) {
                if (sl.cur && cudaEventQuery(sl.cur->done) == cudaSuccess) {
                    complete(sl);
                    progressed = true;
                }
            }
            for (auto& ln : lanes) {
                if (!ln.batch.empty() && cudaEventQuery(ln.done) == cudaSuccess) {
                    complete_batch(ln);
                    progressed = true;
                }
            }
            if (progressed) cv_done.notify_all();
            // small requests: one grouped launch per idle lane with everything queued
            for (auto& ln : lanes)
                if (ln.batch.empty() && launch_batch(ln)) progressed = true;
            // admissions: FIFO with backfill, unless the head has aged past the limit; a large
            // request waiting for a large slot lets the others pass
            const auto now = Clock::now();
            bool head_blocked = false;
            bool first = true;
            for (auto it = queue.begin(); it != queue.end();) {
                ServeRequest* r = *it;
                if (head_blocked) break;
                if (r->cls == 0) {  // waits for a lane
                    ++it;
                    continue;
                }
                const Admit a = try_admit(r);
                if (a == kAdmitted) {
                    it = queue.erase(it);
                    progressed = true;
                } else {
                    if (first && a != kLargeLimit && ms_between(r->t_submit, now) > cfg.aging_ms) head_blocked = true;
                    ++it;
                }
                first = false;
            }
            bool busy = false;
            for (const auto& sl : slots) busy |= (sl.cur != nullptr);
            for (const auto& ln : lanes) busy |= !ln.batch.empty();
            if (!progressed) {
                // running work is polled every 20 us; an idle server sleeps until a submission
                if (busy) cv_work.wait_for(lock, std::chrono::microseconds(20));
                else cv_work.wait(lock, [&] { return stop || !queue.empty(); });
            }
        }
    }
};

}  // namespace gb

// ============================================================================================
//  C-ABI
// ============================================================================================
extern "C" {

void gb300_server_config_init(gb300_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->memory_budget_bytes = int64_t(150) << 30;
    c->slots = 8;
    c->reserve_sms = 16;
    c->aging_ms = 50.0;
    c->large_threshold = 2048;
    c->batch_threshold = 256;
    c->batch_max = 2048;
    c->large_slots = 2;
}

int gb300_server_create(const gb300_server_config* cfg, gb300_server** out) {
    if (!out) return GB300_ERR_INVALID_ARG;
    gb::Runtime& r = gb::runtime();
    std::string err;
    {
        std::lock_guard<std::mutex> lock(r.mu);
        const int st = gb::ensure_init(&err);
        if (st != GB300_OK) {
            gb::set_error(st, "gb300_server_create: " + err);
            return st;
        }
    }
    auto* s = new gb::Server();
    if (cfg) s->cfg = *cfg;
    else gb300_server_config_init(&s->cfg);
    if (s->cfg.slots <= 0) s->cfg.slots = 1;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    s->budget = size_t(std::max<int64_t>(s->cfg.memory_budget_bytes, 0));
    s->budget = std::min(s->budget, size_t(double(fr) * 0.95));
    s->num_sms = r.num_sms;
    // at least one slot of each kind
    if (s->cfg.slots < 2) s->cfg.slots = 2;
    s->n_large = std::min(std::max(1, s->cfg.large_slots), s->cfg.slots - 1);
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    const int prio_mid = prio_greatest < prio_least ? prio_greatest + 1 : prio_greatest;
    s->slots.resize(size_t(s->cfg.slots));
    for (size_t i = 0; i < s->slots.size(); ++i) {
        auto& sl = s->slots[i];
        const int prio = int(i) < s->n_large ? prio_least : std::min(prio_mid, prio_least);
        cudaError_t e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, prio);
        if (e == cudaSuccess) e = cudaMalloc(&sl.ws.d_status, 64);
        if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&sl.host), gb::kHostBytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            gb::set_error(GB300_ERR_CUDA, std::string("gb300_server_create: ") + cudaGetErrorString(e));
            delete s;
            return GB300_ERR_CUDA;
        }
        cudaMemset(sl.ws.d_status, 0, 64);
        sl.ws.stream = sl.stream;
        // a slot's buffers are only used on its stream: growing them must not wait for the device
        sl.ws.stream_ordered = true;
    }
    s->lanes.resize(gb::kBatchLanes);
    for (auto& ln : s->lanes) {
        cudaError_t e = cudaStreamCreateWithPriority(&ln.stream, cudaStreamNonBlocking, prio_greatest);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.done, cudaEventDisableTiming);
        if (e == cudaSuccess) ln.lane = gb::grouped_lane_create(ln.stream, &err);
        if (e != cudaSuccess || !ln.lane) {
            gb::set_error(GB300_ERR_CUDA, "gb300_server_create: batch lane set-up failed " + err);
            s->worker = std::thread();
            gb300_server_destroy(reinterpret_cast<gb300_server*>(s));
            return GB300_ERR_CUDA;
        }
    }
    s->worker = std::thread([s] { s->loop(); });
    *out = reinterpret_cast<gb300_server*>(s);
    return GB300_OK;
}

int gb300_server_submit(gb300_server* srv, const gb300_serve_request* q, uint64_t* ticket) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s || !q || !ticket) return GB300_ERR_INVALID_ARG;
    const bool rm = q->order == 101;
    const bool tA = q->transA != 111, tB = q->transB != 111;
    if ((q->order != 101 && q->order != 102) || q->m < 0 || q->n < 0 || q->k < 0 ||
        q->lda < std::max<int64_t>(1, rm ? (tA ? q->m : q->k) : (tA ? q->k : q->m)) ||
        q->ldb < std::max<int64_t>(1, rm ? (tB ? q->k : q->n) : (tB ? q->n : q->k)) ||
        q->ldc < std::max<int64_t>(1, rm ? q->n : q->m) || q->accuracy < GB300_METHOD_AUTO ||
        q->accuracy > GB300_METHOD_SPLIT_CRT) {
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_server_submit: invalid request");
        return GB300_ERR_INVALID_ARG;
    }
    auto* r = new gb::ServeRequest();
    r->req = *q;
    gb::Gemm& g = r->g;
    if (rm) {
        g.m = q->m; g.n = q->n; g.ta = tA; g.tb = tB; g.A = q->A; g.lda = q->lda; g.B = q->B; g.ldb = q->ldb;
    } else {
        g.m = q->n; g.n = q->m; g.ta = tB; g.tb = tA; g.A = q->B; g.lda = q->ldb; g.B = q->A; g.ldb = q->lda;
    }
    g.k = (q->alpha == 0.0) ? 0 : q->k;
    g.C = q->C;
    g.ldc = q->ldc;
    g.alpha = q->alpha;
    g.beta = q->beta;
    r->sreq.method = q->accuracy;
    r->sreq.target_error = q->target_error;
    r->sreq.slices = 0;
    r->large = std::max(q->m, q->n) >= s->cfg.large_threshold && q->accuracy != GB300_METHOD_NATIVE;
    // small requests of any class run in FP64 grouped launches, unless a split request asks for a
    // bound below FP64's k * 2^-53
    const int64_t mx = std::max(q->m, std::max(q->n, q->k));
    const bool fp64_meets = !(q->accuracy == GB300_METHOD_SPLIT || q->accuracy == GB300_METHOD_SPLIT_CRT) ||
                            q->target_error <= 0.0 || q->target_error >= double(std::max<int64_t>(q->k, 1)) * 0x1p-53;
    r->cls = (s->cfg.batch_threshold > 0 && mx <= s->cfg.batch_threshold && fp64_meets)
                 ? 0
                 : (std::max(q->m, q->n) >= s->cfg.large_threshold ? 2 : 1);
    if (g.m > 0 && g.n > 0 && r->cls != 0) gb::device_product_slot_needs(g, r->sreq, r->need);
    r->footprint = 0;
    for (int s_ = 0; s_ < gb::kSlotCount; ++s_) r->footprint += r->need[s_];
    if (cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming) != cudaSuccess) {
        delete r;
        gb::set_error(GB300_ERR_CUDA, "gb300_server_submit: event creation failed");
        return GB300_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    r->id = s->next_id++;
    r->t_submit = gb::Clock::now();
    if (!s->any) {
        s->any = true;
        s->t_first = r->t_submit;
    }
    ++s->submitted;
    s->reqs[r->id] = r;
    *ticket = r->id;
    if (r->footprint > s->budget) {
        r->state = 2;
        r->res.status = GB300_ERR_ADMISSION;
        r->t_start = r->t_end = r->t_submit;
        ++s->rejected;
        s->cv_done.notify_all();
        gb::set_error(GB300_ERR_ADMISSION, "gb300_server_submit: the request needs " + std::to_string(r->footprint) +
                                               " bytes of device memory, above the server budget of " +
                                               std::to_string(s->budget));
        return GB300_ERR_ADMISSION;
    }
    if (g.m == 0 || g.n == 0) {
        r->state = 2;
        r->res.status = GB300_OK;
        r->t_start = r->t_end = r->t_submit;
        ++s->completed;
        s->cv_done.notify_all();
        return GB300_OK;
    }
    s->queue.push_back(r);
    s->cv_work.notify_one();
    return GB300_OK;
}

int gb300_server_wait(gb300_server* srv, uint64_t ticket, double timeout_ms, gb300_serve_result* res) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s) return GB300_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) {
        gb::set_error(GB300_ERR_INVALID_ARG, "gb300_server_wait: unknown ticket");
        return GB300_ERR_INVALID_ARG;
    }
    gb::ServeRequest* r = it->second;
    const auto pred = [&] { return r->state == 2; };
    if (timeout_ms < 0) s->cv_done.wait(lock, pred);
    else if (!s->cv_done.wait_for(lock, std::chrono::duration<double, std::milli>(timeout_ms), pred)) {
        gb::set_error(GB300_ERR_DEVICE_TIMEOUT, "gb300_server_wait: the request has not finished yet");
        return GB300_ERR_DEVICE_TIMEOUT;
    }
    if (res) *res = r->res;
    cudaEventDestroy(r->done);
    s->reqs.erase(it);
    const int st = r->res.status;
    delete r;
    return st;
}

int gb300_server_poll(gb300_server* srv, uint64_t ticket, int* done) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s || !done) return GB300_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return GB300_ERR_INVALID_ARG;
    *done = it->second->state == 2;
    return GB300_OK;
}

int gb300_server_get_stats(gb300_server* srv, gb300_server_stats* out) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s || !out) return GB300_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rejected = s->rejected;
    out->failed = s->failed;
    out->queued = int64_t(s->queue.size());
    const std::vector<double>& l = s->latencies;
    if (!l.empty()) {
        out->p50_ms = gb::percentile(l, 0.50);
        out->p99_ms = gb::percentile(l, 0.99);
        out->max_ms = *std::max_element(l.begin(), l.end());
        double sum = 0;
        for (double v : l) sum += v;
        out->mean_ms = sum / double(l.size());
    }
    for (int c = 0; c < 3; ++c) {
        out->class_completed[c] = int64_t(s->class_lat[c].size());
        out->class_p50_ms[c] = gb::percentile(s->class_lat[c], 0.50);
        out->class_p99_ms[c] = gb::percentile(s->class_lat[c], 0.99);
    }
    out->grouped_launches = s->grouped_launches;
    out->grouped_mean_batch = s->grouped_launches ? double(s->grouped_requests) / double(s->grouped_launches) : 0.0;
    if (s->any) {
        const double wall = gb::ms_between(s->t_first, gb::Clock::now()) * 1e-3;
        out->wall_s = wall;
        out->tflops = wall > 0 ? s->useful_flops / wall / 1e12 : 0.0;
    }
    out->bytes_in_use = int64_t(s->bytes_held());
    out->peak_bytes = int64_t(s->peak_bytes);
    out->budget_bytes = int64_t(s->budget);
    return GB300_OK;
}

void gb300_server_reset_stats(gb300_server* srv) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s) return;
    std::lock_guard<std::mutex> lock(s->mu);
    s->latencies.clear();
    for (auto& v : s->class_lat) v.clear();
    s->grouped_launches = s->grouped_requests = 0;
    s->submitted = s->completed = s->rejected = s->failed = 0;
    s->useful_flops = 0;
    s->any = false;
    s->peak_bytes = s->bytes_held();
}

void gb300_server_destroy(gb300_server* srv) {
    auto* s = reinterpret_cast<gb::Server*>(srv);
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto& ln : s->lanes) {
        gb::grouped_lane_destroy(ln.lane);
        if (ln.done) cudaEventDestroy(ln.done);
        if (ln.stream) cudaStreamDestroy(ln.stream);
    }
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        sl.ws.release();
        if (sl.ws.d_status) cudaFree(sl.ws.d_status);
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (auto& kv : s->reqs) {
        if (kv.second->done) cudaEventDestroy(kv.second->done);
        delete kv.second;
    }
    delete s;
}

}  // extern "C"
