// Serving loop: continuous batching of decode requests on one GPU.
//
// The reference decodes one stream per blocking call on the legacy default
// stream (src/multians_gpu_decoder.cu:575-687, called once from
// src/main.cc:111-116); a service built on it pays the whole launch sequence
// and a device synchronisation per request.  Here a worker thread owns the
// GPU side:
//
//   submit ──► mailbox ──► pending (arrival order)
//                              │ admission: the request's units, output and
//                              │ decode workspace fit in the device range
//                              ▼
//                           ready ──(H2D of inputs on the copy stream)
//                              │ a launch slot is free
//                              ▼
//            one batch = everything ready of the slot's size class, on
//            the slot's stream (small requests have a slot of their own,
//            on a high-priority stream):
//            wait(copies) → upload params → 4 batch kernels → D2H outputs
//                              │ host callback at the end of the stream work
//                              ▼
//            reap: device status, overflow fix-up, completions, release
//
// Device memory: one range allocated at creation (the budget), carved by a
// first-fit arena.  Tables live there for the server's lifetime; every
// request holds one block [workspace slice | units | output] from admission
// to completion; each launch slot keeps a preallocated header buffer
// (parameters, work items, status and scan flags of one batch).  Nothing on
// the request path calls cudaMalloc or cudaFree.
#include <cuda_runtime.h>
#include <time.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <thread>
#include <vector>

#include "mans_arena.h"
#include "multians_gb300.h"

namespace {

constexpr uint64_t kDefaultBudget = 16ull << 30;
constexpr uint64_t kHeadroom = 1ull << 30;      // left to other users of the device
constexpr uint64_t kHeaderCap = 8ull << 20;     // preallocated header per slot
constexpr uint64_t kSmallHeaderCap = 1ull << 20;   // ... of the small-request slot
constexpr uint32_t kDefaultSmall = 1u << 20;    // small request: n_out <= 1 MiB
constexpr uint64_t kNone = ~0ull;

uint64_t clock_ns() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t) ts.tv_sec * 1000000000ull + (uint64_t) ts.tv_nsec;
}

uint64_t align256(uint64_t x) { return (x + 255) & ~255ull; }

bool is_pinned_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

struct Table {
    uint64_t off;
    uint32_t L;
    uint64_t hash;                 // FNV-1a of the words, for container lookups
    std::vector<uint32_t> words;   // host copy
};

uint64_t table_hash(const uint32_t* t, uint32_t L) {
    uint64_t h = 1469598103934665603ull ^ L;
    for (uint32_t j = 0; j < L; ++j) {
        h ^= t[j];
        h *= 1099511628211ull;
    }
    return h;
}

struct Req {
    mans_request r;
    uint64_t arrival = 0, admit = 0;
    uint64_t off = kNone;          // arena block
    uint64_t slice_bytes = 0, bytes = 0;
    bool checked = false;
    int check_rc = 0;
    bool host_in = false, host_out = false, pinned_out = false;
    bool taken = false;            // chosen for the batch being built
    mans_stream_desc d{};
    char* slice = nullptr;
};

struct Slot {
    cudaStream_t stream = nullptr;
    uint64_t header_off = kNone;   // preallocated header
    uint64_t extra_off = kNone;    // larger header for this batch, if needed
    uint64_t header_cap = kHeaderCap;
    bool small = false;            // takes small requests only
    mans_batch* b = nullptr;
    std::vector<Req*> reqs;
    uint64_t seq = 0;
    bool busy = false;
    std::atomic<bool> done{false};
    mans_server* srv = nullptr;
};

}  // namespace

struct mans_server {
    int device = 0;
    uint32_t max_inflight = 2, max_batch = 4096;
    uint64_t small_bytes = 0;      // 0: no small-request slot
    char* base = nullptr;
    mans::Arena arena;
    std::mutex arena_mu;
    std::vector<Table> tables;
    std::unordered_multimap<uint64_t, uint32_t> table_ids;   // hash -> id
    std::mutex tables_mu;

    // Adds a table (or finds the identical one already resident).
    int add_table(const uint32_t* host_table, uint32_t L, uint32_t* id) {
        if (mans_table_check(host_table, L) < 0) return MANS_ERR_TABLE;
        const uint64_t h = table_hash(host_table, L);
        {
            std::lock_guard<std::mutex> lk(tables_mu);
            auto range = table_ids.equal_range(h);
            for (auto it = range.first; it != range.second; ++it) {
                const Table& t = tables[it->second];
                if (t.L == L && std::memcmp(t.words.data(), host_table, (size_t) L * 4) == 0) {
                    *id = it->second;
                    return MANS_OK;
                }
            }
        }
        uint64_t off;
        {
            std::lock_guard<std::mutex> lk(arena_mu);
            if (!arena.alloc((uint64_t) L * 4, &off)) return MANS_ERR_NOMEM;
        }
        if (cudaMemcpy(base + off, host_table, (size_t) L * 4, cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            std::lock_guard<std::mutex> lk(arena_mu);
            arena.release(off);
            return MANS_ERR_CUDA;
        }
        std::lock_guard<std::mutex> lk(tables_mu);
        *id = (uint32_t) tables.size();
        tables.push_back({off, L, h, std::vector<uint32_t>(host_table, host_table + L)});
        table_ids.emplace(h, *id);
        return MANS_OK;
    }

    // input copies, one in-order stream per size class (a small request's
    // copy does not queue behind a large one's), and the event a batch of
    // that class waits on
    cudaStream_t copy_stream[2] = {nullptr, nullptr};
    cudaEvent_t copy_ev[2] = {nullptr, nullptr};
    int size_class(const Req* q) const { return small_bytes && q->r.n_out <= small_bytes; }
    std::vector<std::unique_ptr<Slot>> slots;

    // mailbox + worker wake-up
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req*> mailbox;
    bool stop = false;

    // worker-private queues
    std::deque<Req*> pending, ready;
    bool head_waiting = false;
    uint64_t next_seq = 0;

    // completions + statistics
    std::mutex cq_mu;
    std::condition_variable cq_cv;
    std::deque<mans_completion> done;
    mans_server_stats st{};

    std::thread worker;

    void complete(Req* q, int status, uint32_t dev_status, uint64_t seq) {
        mans_completion c;
        c.tag = q->r.tag;
        c.status = status;
        c.dev_status = dev_status;
        c.arrival_ns = q->arrival;
        c.admit_ns = q->admit;
        c.done_ns = clock_ns();
        c.batch = seq;
        if (q->off != kNone) {
            std::lock_guard<std::mutex> lk(arena_mu);
            arena.release(q->off);
        }
        {
            std::lock_guard<std::mutex> lk(cq_mu);
            done.push_back(c);
            ++st.completed;
            if (status != MANS_OK) ++st.failed;
            else {
                st.bytes_out += q->r.n_out;
                st.bytes_in += q->r.n_units * 4;
            }
        }
        cq_cv.notify_all();
        delete q;
    }

    // Checks a request and sizes its device block.  A container request
    // gets its stream fields (and table) from the container header.
    int validate(Req* q) {
        if (q->r.flags & MANS_REQ_CONTAINER) {
            if (q->r.flags & MANS_REQ_DEVICE_IO) return MANS_ERR_ARG;
            mans_container_info ci;
            const int rc = mans_container_parse(q->r.units, q->r.n_units, &ci);
            if (rc != MANS_OK) return rc;
            if (ci.n_symbols > q->r.n_out) return MANS_ERR_ARG;
            const unsigned char* c = (const unsigned char*) q->r.units;
            uint32_t tid = 0;
            const int tr = add_table((const uint32_t*) (c + ci.table_offset), ci.L, &tid);
            if (tr != MANS_OK) return tr;
            q->r.units = (const uint32_t*) (c + ci.units_offset);
            q->r.n_units = ci.n_units;
            q->r.n_out = ci.n_symbols;
            q->r.table = tid;
            q->r.first_state = ci.first_state;
            q->r.first_bit = ci.first_bit;
        }
        const mans_request& r = q->r;
        uint32_t L;
        uint64_t toff;
        {
            std::lock_guard<std::mutex> lk(tables_mu);
            if (r.table >= tables.size()) return MANS_ERR_ARG;
            L = tables[r.table].L;
            toff = tables[r.table].off;
        }
        if (r.n_out == 0) return MANS_OK;
        if (!r.units || !r.out || r.n_units == 0 || r.n_units > 0xffffffffull ||
            r.first_state < L || r.first_state >= 2 * L || r.first_bit > 32)
            return MANS_ERR_ARG;
        const bool dev = (r.flags & MANS_REQ_DEVICE_IO) != 0;
        if (dev && ((uintptr_t) r.units & 15) != 0) return MANS_ERR_ARG;
        q->host_in = q->host_out = !dev;
        q->pinned_out = q->host_out && is_pinned_host(r.out);
        mans_stream_desc d{};
        d.d_units = dev ? r.units : (const uint32_t*) (uintptr_t) 256;   // sizing only
        d.n_units = r.n_units;
        d.d_out = dev ? r.out : (uint8_t*) (uintptr_t) 256;
        d.n_out = r.n_out;
        d.d_table = (const uint32_t*) (base + toff);
        d.L = L;
        d.first_state = r.first_state;
        d.first_bit = r.first_bit;
        d.flags = ((r.flags & MANS_REQ_SOURCE_ORDER) ? MANS_DECODE_SOURCE_ORDER : 0u) |
                  ((r.flags & MANS_REQ_NO_CAPTURE) ? MANS_DECODE_NO_CAPTURE : 0u);
        size_t slice = 0;
        const int rc = mans_batch_slice_size(&d, nullptr, &slice);
        if (rc != MANS_OK) return rc;
        q->d = d;
        q->slice_bytes = align256(slice);
        q->bytes = q->slice_bytes + (q->host_in ? align256(r.n_units * 4) : 0) +
                   (q->host_out ? align256(r.n_out) : 0);
        return MANS_OK;
    }

    bool any_busy() const {
        for (const auto& s : slots)
            if (s->busy) return true;
        return false;
    }

    // Admits queued requests in arrival order while their blocks fit.
    bool admit() {
        bool progress = false;
        while (!pending.empty()) {
            Req* q = pending.front();
            if (!q->checked) {
                q->check_rc = validate(q);
                q->checked = true;
            }
            const int rc = q->check_rc;
            if (rc != MANS_OK || q->r.n_out == 0) {
                pending.pop_front();
                complete(q, rc, 0, 0);
                progress = true;
                continue;
            }
            uint64_t off;
            bool ok;
            {
                std::lock_guard<std::mutex> lk(arena_mu);
                ok = arena.alloc(q->bytes, &off);
            }
            if (!ok) {
                if (!any_busy() && ready.empty()) {
                    // nothing will be released: it can never fit
                    pending.pop_front();
                    complete(q, MANS_ERR_NOMEM, 0, 0);
                    progress = true;
                    continue;
                }
                if (!head_waiting) {
                    std::lock_guard<std::mutex> lk(cq_mu);
                    ++st.admission_waits;
                }
                head_waiting = true;
                break;
            }
            head_waiting = false;
            pending.pop_front();
            q->off = off;
            char* blk = base + off;
            q->slice = blk;
            char* p = blk + q->slice_bytes;
            if (q->host_in) {
                q->d.d_units = (const uint32_t*) p;
                p += align256(q->r.n_units * 4);
                if (cudaMemcpyAsync((void*) q->d.d_units, q->r.units, q->r.n_units * 4,
                                    cudaMemcpyHostToDevice, copy_stream[size_class(q)]) !=
                    cudaSuccess) {
                    cudaGetLastError();
                    complete(q, MANS_ERR_CUDA, 0, 0);
                    progress = true;
                    continue;
                }
            }
            if (q->host_out) q->d.d_out = (uint8_t*) p;
            q->admit = clock_ns();
            ready.push_back(q);
            progress = true;
        }
        return progress;
    }

    static void CUDART_CB on_done(void* arg) {
        Slot* s = (Slot*) arg;
        {
            std::lock_guard<std::mutex> lk(s->srv->mu);
            s->done.store(true);
        }
        s->srv->cv.notify_all();
    }

    // Takes q out of the ready queue and completes it with rc.
    void drop_ready(Req* q, int rc) {
        ready.erase(std::find(ready.begin(), ready.end(), q));
        complete(q, rc, 0, 0);
    }

    // Launches one batch on a free slot, in arrival order, up to max_batch
    // requests: the small-request slot (offered first) takes the small
    // requests that are ready; any other slot the larger ones, or, when none
    // is ready, the small ones the busy small-request slot has left.
    bool launch() {
        if (ready.empty()) return false;
        Slot* s = nullptr;
        std::vector<Req*> take;
        for (auto& c : slots) {
            if (c->busy) continue;
            for (int want = c->small; want <= 1 && take.empty(); ++want)
                for (Req* q : ready) {
                    if (take.size() >= max_batch) break;
                    if (size_class(q) == want) take.push_back(q);
                }
            if (!take.empty()) {
                s = c.get();
                break;
            }
        }
        if (!s) return false;
        size_t n = take.size();
        std::vector<mans_stream_desc> descs(n);
        std::vector<void*> slices(n);
        size_t hbytes = 0;
        uint64_t hoff = s->header_off;
        for (;;) {
            for (size_t i = 0; i < n; ++i) {
                descs[i] = take[i]->d;
                slices[i] = take[i]->slice;
            }
            if (mans_batch_header_size(descs.data(), (uint32_t) n, nullptr, &hbytes) != MANS_OK) {
                drop_ready(take[0], MANS_ERR_ARG);   // cannot happen for validated requests
                return true;
            }
            if (hbytes <= s->header_cap) break;
            if (n > 1) { n = (n + 1) / 2; continue; }
            uint64_t off;
            bool ok;
            {
                std::lock_guard<std::mutex> lk(arena_mu);
                ok = arena.alloc(hbytes, &off);
            }
            if (ok) { s->extra_off = hoff = off; break; }
            if (any_busy()) return false;   // wait for memory to come back
            drop_ready(take[0], MANS_ERR_NOMEM);
            return true;
        }
        // a copy stream is in order: one event covers every input of the
        // taken requests' size class (they are all of one) copied so far
        const int cls = size_class(take[0]);
        cudaEventRecord(copy_ev[cls], copy_stream[cls]);
        cudaStreamWaitEvent(s->stream, copy_ev[cls], 0);
        mans_batch* b = nullptr;
        int rc = mans_batch_create_split(descs.data(), (uint32_t) n, nullptr, base + hoff,
                                         hbytes, slices.data(), s->stream, &b);
        if (rc == MANS_OK) rc = mans_batch_decode(b, s->stream);
        if (rc == MANS_OK) {
            for (size_t i = 0; i < n; ++i) {
                Req* q = take[i];
                if (q->pinned_out &&
                    cudaMemcpyAsync(q->r.out, q->d.d_out, q->r.n_out, cudaMemcpyDeviceToHost,
                                    s->stream) != cudaSuccess) {
                    rc = MANS_ERR_CUDA;
                    break;
                }
            }
        }
        s->reqs.assign(take.begin(), take.begin() + n);
        for (size_t i = 0; i < n; ++i) take[i]->taken = true;
        ready.erase(std::remove_if(ready.begin(), ready.end(), [](const Req* q) { return q->taken; }),
                    ready.end());
        s->b = b;
        s->seq = ++next_seq;
        s->done.store(false);
        if (rc == MANS_OK && cudaLaunchHostFunc(s->stream, on_done, s) != cudaSuccess)
            rc = MANS_ERR_CUDA;
        if (rc != MANS_OK) {
            cudaGetLastError();
            cudaStreamSynchronize(s->stream);
            finish(s, rc);
            return true;
        }
        s->busy = true;
        std::lock_guard<std::mutex> lk(cq_mu);
        ++st.batches;
        st.kernel_launches += mans_last_launch_count();
        st.largest_batch = std::max<uint64_t>(st.largest_batch, n);
        return true;
    }

    // Completes every request of a slot (status rc if nonzero, else each
    // stream's device status) and frees the slot.
    void finish(Slot* s, int rc) {
        const size_t n = s->reqs.size();
        std::vector<uint32_t> dev(n, 0);
        if (rc == MANS_OK && s->b) {
            uint32_t acc = 0;
            rc = mans_batch_status(s->b, s->stream, &acc, dev.data());
            if (rc == MANS_OK && (acc & MANS_DEV_SYNC_OVERFLOW)) {
                // re-decode overflowed streams with longer regions, then
                // copy their outputs again
                uint32_t redone = 0;
                std::vector<uint32_t> before = dev;
                rc = mans_batch_fixup(s->b, s->stream, &redone);
                if (rc == MANS_OK) rc = mans_batch_status(s->b, s->stream, &acc, dev.data());
                for (size_t i = 0; rc == MANS_OK && i < n; ++i) {
                    Req* q = s->reqs[i];
                    if ((before[i] & MANS_DEV_SYNC_OVERFLOW) && q->pinned_out &&
                        cudaMemcpyAsync(q->r.out, q->d.d_out, q->r.n_out,
                                        cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
                        rc = MANS_ERR_CUDA;
                }
                if (cudaStreamSynchronize(s->stream) != cudaSuccess) rc = MANS_ERR_CUDA;
                std::lock_guard<std::mutex> lk(cq_mu);
                st.streams_redone += redone;
            }
            // pageable outputs: copied now that the batch is done
            for (size_t i = 0; rc == MANS_OK && i < n; ++i) {
                Req* q = s->reqs[i];
                if (q->host_out && !q->pinned_out &&
                    cudaMemcpy(q->r.out, q->d.d_out, q->r.n_out, cudaMemcpyDeviceToHost) !=
                        cudaSuccess)
                    rc = MANS_ERR_CUDA;
            }
        }
        for (size_t i = 0; i < n; ++i) {
            const int qs = rc != MANS_OK ? rc : mans_status_code(dev[i]);
            complete(s->reqs[i], qs, dev[i], s->seq);
        }
        s->reqs.clear();
        if (s->b) mans_batch_destroy(s->b);
        s->b = nullptr;
        if (s->extra_off != kNone) {
            std::lock_guard<std::mutex> lk(arena_mu);
            arena.release(s->extra_off);
            s->extra_off = kNone;
        }
        s->busy = false;
    }

    bool reap() {
        bool progress = false;
        for (auto& s : slots) {
            if (s->busy && s->done.load()) {
                finish(s.get(), MANS_OK);
                progress = true;
            }
        }
        return progress;
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            while (!mailbox.empty()) {
                pending.push_back(mailbox.front());
                mailbox.pop_front();
            }
            const bool stopping = stop;
            lk.unlock();
            bool progress = reap();
            if (!stopping) {
                progress |= admit();
                progress |= launch();
            }
            lk.lock();
            if (stopping && !any_busy()) break;
            if (progress || !mailbox.empty()) continue;
            bool fired = false;
            for (auto& s : slots) fired |= s->busy && s->done.load();
            if (!fired) cv.wait_for(lk, std::chrono::milliseconds(2));
        }
        lk.unlock();
        // requests admitted but not launched may still have input copies in
        // flight from the caller's memory: let them end before returning
        for (cudaStream_t cs : copy_stream) cudaStreamSynchronize(cs);
        for (Req* q : pending) delete q;
        for (Req* q : ready) delete q;
        pending.clear();
        ready.clear();
    }
};

extern "C" {

uint64_t mans_server_now_ns(void) { return clock_ns(); }

int mans_server_create(const mans_server_cfg* cfg, mans_server** out) {
    if (!out) return MANS_ERR_ARG;
    *out = nullptr;
    mans_server_cfg c{};
    if (cfg) c = *cfg;
    auto s = std::make_unique<mans_server>();
    if (cudaGetDevice(&s->device) != cudaSuccess) return MANS_ERR_CUDA;
    s->max_inflight = c.max_inflight ? std::min<uint32_t>(c.max_inflight, 8) : 2;
    s->max_batch = c.max_batch ? std::min<uint32_t>(c.max_batch, 1u << 20) : 4096;
    s->small_bytes = c.small_bytes == 0xffffffffu ? 0 : (c.small_bytes ? c.small_bytes : kDefaultSmall);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return MANS_ERR_CUDA;
    uint64_t budget = c.budget_bytes ? c.budget_bytes : kDefaultBudget;
    if (free_b > kHeadroom) budget = std::min<uint64_t>(budget, free_b - kHeadroom);
    else budget = 0;
    budget &= ~255ull;
    const uint64_t headers =
        (uint64_t) s->max_inflight * kHeaderCap + (s->small_bytes ? kSmallHeaderCap : 0);
    if (budget < headers + (1ull << 20)) return MANS_ERR_NOMEM;
    if (cudaMalloc(&s->base, budget) != cudaSuccess) {
        cudaGetLastError();
        return MANS_ERR_NOMEM;
    }
    s->arena.reset(budget);
    auto fail = [&](int rc) {
        for (auto& sl : s->slots)
            if (sl->stream) cudaStreamDestroy(sl->stream);
        for (int i = 0; i < 2; ++i) {
            if (s->copy_ev[i]) cudaEventDestroy(s->copy_ev[i]);
            if (s->copy_stream[i]) cudaStreamDestroy(s->copy_stream[i]);
        }
        cudaFree(s->base);
        return rc;
    };
    for (int i = 0; i < 2; ++i)
        if (cudaStreamCreateWithFlags(&s->copy_stream[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->copy_ev[i], cudaEventDisableTiming) != cudaSuccess)
            return fail(MANS_ERR_CUDA);
    // the small-request slot first (it is offered the ready requests first),
    // on a stream of the highest priority: its blocks are scheduled ahead of
    // the waiting blocks of the larger batches' kernels
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return fail(MANS_ERR_CUDA);
    for (uint32_t i = s->small_bytes ? 0 : 1; i <= s->max_inflight; ++i) {
        auto sl = std::make_unique<Slot>();
        sl->srv = s.get();
        sl->small = i == 0;
        sl->header_cap = sl->small ? kSmallHeaderCap : kHeaderCap;
        if (cudaStreamCreateWithPriority(&sl->stream, cudaStreamNonBlocking,
                                         sl->small ? greatest : least) != cudaSuccess)
            return fail(MANS_ERR_CUDA);
        if (!s->arena.alloc(sl->header_cap, &sl->header_off)) return fail(MANS_ERR_NOMEM);
        s->slots.push_back(std::move(sl));
    }
    s->st.range_bytes = budget;
    mans_server* raw = s.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return MANS_OK;
}

int mans_server_add_table(mans_server* s, const uint32_t* host_table, uint32_t L, uint32_t* id) {
    if (!s || !host_table || !id || L < 2 || L > 8192) return MANS_ERR_ARG;
    return s->add_table(host_table, L, id);
}

int mans_server_submit(mans_server* s, const mans_request* reqs, size_t n) {
    if (!s || (!reqs && n)) return MANS_ERR_ARG;
    const uint64_t now = clock_ns();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return MANS_ERR_BUSY;
        for (size_t i = 0; i < n; ++i) {
            Req* q = new Req();
            q->r = reqs[i];
            q->arrival = reqs[i].arrival_ns ? reqs[i].arrival_ns : now;
            s->mailbox.push_back(q);
        }
    }
    {
        std::lock_guard<std::mutex> lk(s->cq_mu);
        s->st.submitted += n;
    }
    s->cv.notify_all();
    return MANS_OK;
}

int mans_server_poll(mans_server* s, mans_completion* out, size_t cap, size_t* n_out,
                     uint32_t wait_us) {
    if (!s || !n_out || (!out && cap)) return MANS_ERR_ARG;
    *n_out = 0;
    std::unique_lock<std::mutex> lk(s->cq_mu);
    if (s->done.empty() && wait_us)
        s->cq_cv.wait_for(lk, std::chrono::microseconds(wait_us),
                          [s] { return !s->done.empty(); });
    size_t k = 0;
    while (k < cap && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n_out = k;
    return MANS_OK;
}

int mans_server_stats_get(mans_server* s, mans_server_stats* out) {
    if (!s || !out) return MANS_ERR_ARG;
    mans_server_stats v;
    {
        std::lock_guard<std::mutex> lk(s->cq_mu);
        v = s->st;
    }
    {
        std::lock_guard<std::mutex> lk(s->arena_mu);
        v.range_in_use = s->arena.in_use();
        v.range_peak = s->arena.peak();
    }
    *out = v;
    return MANS_OK;
}

int mans_server_destroy(mans_server* s) {
    if (!s) return MANS_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (Req* q : s->mailbox) delete q;
    for (auto& sl : s->slots)
        if (sl->stream) cudaStreamDestroy(sl->stream);
    for (int i = 0; i < 2; ++i) {
        if (s->copy_ev[i]) cudaEventDestroy(s->copy_ev[i]);
        if (s->copy_stream[i]) cudaStreamDestroy(s->copy_stream[i]);
    }
    if (s->base) cudaFree(s->base);
    delete s;
    return MANS_OK;
}

}  // extern "C"
