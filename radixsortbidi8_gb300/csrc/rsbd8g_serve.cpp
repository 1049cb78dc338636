// rsbd8g_serve.cpp - serving loop: continuous batching of sort requests on one GPU.
//
// Requests (a descriptor, a count, a device input and a device output array) arrive from any host
// thread.  A dispatcher thread admits pending requests in arrival order while the device-memory
// budget and the in-flight slots allow, coalesces the admitted requests that share a key size and
// resolved filter (any direction) into one batched launch (rsbd8g_segmented_sortcopy_ptrs_dirs:
// every request one segment, each in its own arrays, with its own direction), and launches each
// batch on its own stream, so batches overlap on the device while new requests keep arriving.  A
// request large enough to run alone goes through the plain sort (rsbd8g_radixsortcopynoalloc),
// which is 13-18 % faster than the segmented launch on one large array.  The budget is one device
// arena allocated up front: the ping-pong buffers, the batch scratch and the batch's pointer tables
// are carved out of it and given back when the batch completes, so keys and scratch stay resident
// and nothing is allocated per request.  Creating a server loads every kernel a request can need
// (rsbd8g_prepare), so no request waits for the CUDA runtime to load one.
// Completion is observed with a host function queued behind each batch on its stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "rsbd8g.h"

namespace rsbd8g {
bool device_memory(const void *p);            // rsbd8g_api.cu
int filter_class(const rsbd8g_desc *d);       // rsbd8g_api.cu
}

namespace {

constexpr size_t kAlignArena = 256;
size_t aup(size_t x) { return (x + kAlignArena - 1) & ~(kAlignArena - 1); }

// first-fit allocator over [0, size) of the arena; host bookkeeping only
class Arena {
public:
    void init(size_t size) { free_[0] = size; }
    bool alloc(size_t bytes, size_t *off) {
        bytes = aup(bytes ? bytes : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = aup(bytes ? bytes : 1);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }
    size_t largest_free() const {
        size_t m = 0;
        for (auto &kv : free_) m = std::max(m, kv.second);
        return m;
    }

private:
    std::map<size_t, size_t> free_;   // offset -> length
    size_t used_ = 0;
};

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id;
    rsbd8g_desc desc;
    uint64_t count;
    const void *in;
    void *out;
    size_t buf_off = 0, buf_bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int state = 0;   // 0 pending, 1 running, 2 done
    bool device = false;   // input and output are device memory
    int group = 0;         // requests of one group sort alike but for direction (same_group)
    rsbd8g_status status = RSBD8G_OK;
};

struct Server;

struct Batch {
    Server *srv = nullptr;
    std::vector<Request *> reqs;
    int slot = -1;
    size_t scratch_off = 0, scratch_bytes = 0, tables_off = 0, tables_bytes = 0;
    unsigned char *host_tables = nullptr;   // pinned: offsets, in, out, buf, directions (device layout)
    uint32_t *host_err = nullptr;      // pinned: the device status word after the batch
    uint64_t keys = 0;
    double t_done = 0;
    bool launch_failed = false;
    bool big = false;                  // one request that fills the GPU on its own
};

// Batch shapes.  A request of more than kAloneKeys keys fills the GPU by itself and runs as a batch
// of its own; smaller requests are coalesced up to kBatchKeys keys, so a small request never waits
// for a large one it was batched with.  Large batches leave one in-flight slot to small ones.
constexpr uint64_t kAloneKeys = uint64_t(1) << 22;
constexpr uint64_t kBatchKeys = uint64_t(1) << 24;

// requests that one segmented launch can sort: the same key size, resolved filter (the kernels'
// template mode) and flags; the direction is per segment (an unsigned key under "native" and under
// "nativeabs" resolves to the same filter, so those share a launch too)
bool same_group(const Request &a, const Request &b) {
    return a.desc.key_bytes == b.desc.key_bytes && a.group == b.group && a.desc.flags == b.desc.flags;
}

struct Server {
    int device = 0;
    unsigned char *arena_base = nullptr;
    size_t budget = 0;
    Arena arena;
    std::vector<cudaStream_t> streams;
    std::vector<bool> slot_busy;
    std::vector<unsigned char *> slot_tables;   // pinned staging per slot, in the arena's table layout
    std::vector<uint32_t *> slot_err;
    size_t slot_table_cap = 0;
    uint32_t max_batch_requests = 4096;

    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request *> pending;
    std::vector<Request *> all;            // by id
    std::mutex done_mu;                    // only guards `finished`; never held across a CUDA call
    std::vector<Batch *> finished;         // completed on the device, to be retired
    bool stop = false;
    std::thread dispatcher;

    // statistics
    uint64_t completed = 0, keys_done = 0, batches = 0, max_coalesced = 0, max_inflight = 0;
    uint64_t inflight = 0, inflight_big = 0;

    ~Server() {
        {
            std::lock_guard<std::mutex> g(mu);
            stop = true;
        }
        cv.notify_all();
        if (dispatcher.joinable()) dispatcher.join();
        cudaSetDevice(device);
        for (auto s : streams) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
        for (auto p : slot_tables) cudaFreeHost(p);
        for (auto p : slot_err) cudaFreeHost(p);
        if (arena_base) cudaFree(arena_base);
        for (auto r : all) delete r;
    }

    // runs on the CUDA callback thread once the batch's work is done: it must not call CUDA and
    // must not wait on `mu` (the dispatcher may hold it), so it only queues the batch
    static void CUDART_CB on_done(void *p) {
        Batch *b = static_cast<Batch *>(p);
        b->t_done = now_s();
        Server *s = b->srv;
        {
            std::lock_guard<std::mutex> g(s->done_mu);
            s->finished.push_back(b);
        }
        s->cv.notify_all();
    }

    // retire completed batches: statuses, statistics, memory back to the arena (`mu` held)
    void retire_locked() {
        std::vector<Batch *> done;
        {
            std::lock_guard<std::mutex> g(done_mu);
            done.swap(finished);
        }
        for (Batch *b : done) {
            const uint32_t err = *b->host_err;
            const rsbd8g_status st = b->launch_failed ? RSBD8G_ERR_CUDA
                                     : (err & 1u)     ? RSBD8G_ERR_TIMEOUT
                                     : err            ? RSBD8G_ERR_DEVICE_FAULT
                                                      : RSBD8G_OK;
            for (auto r : b->reqs) {
                r->state = 2;
                r->status = st;
                r->t_done = b->t_done;
                arena.release(r->buf_off, r->buf_bytes);
                ++completed;
                keys_done += r->count;
            }
            arena.release(b->scratch_off, b->scratch_bytes);
            arena.release(b->tables_off, b->tables_bytes);
            slot_busy[size_t(b->slot)] = false;
            --inflight;
            if (b->big) --inflight_big;
            delete b;
        }
        if (!done.empty()) cv.notify_all();
    }

    // admit the next batch if a slot and memory allow (`mu` held); nullptr when nothing to do
    Batch *form_locked() {
        for (;;) {
            if (pending.empty()) return nullptr;
            int slot = -1;
            for (size_t i = 0; i < slot_busy.size(); ++i)
                if (!slot_busy[i]) {
                    slot = int(i);
                    break;
                }
            if (slot < 0) return nullptr;
            // the head: the oldest pending request that may start now (a large one only while a slot
            // stays free for small requests).  It decides the group of the batch; a small head takes
            // the pending small requests of its group, in arrival order, while the batch stays within
            // kBatchKeys and their buffers fit the budget.
            Request *head = nullptr;
            const bool keep_slot = slot_busy.size() > 1 && inflight_big + 1 >= slot_busy.size();
            for (Request *r : pending)
                if (r->count <= kAloneKeys || !keep_slot) {
                    head = r;
                    break;
                }
            if (!head) return nullptr;
            const bool big = head->count > kAloneKeys;
            const rsbd8g_desc key = head->desc;
            std::vector<Request *> take;
            uint64_t total = 0;
            for (Request *r : pending) {
                if (take.size() >= max_batch_requests) break;
                if (r != head) {
                    if (big || take.empty()) {   // a large head runs alone; nothing goes before the head
                        if (big && !take.empty()) break;
                        continue;
                    }
                    if (!same_group(*r, *head) || r->count > kAloneKeys || total + r->count > kBatchKeys) continue;
                }
                size_t off;
                r->buf_bytes = size_t(r->count) * key.key_bytes;
                if (!arena.alloc(r->buf_bytes, &off)) break;
                r->buf_off = off;
                take.push_back(r);
                total += r->count;
            }
            if (take.empty()) return nullptr;    // memory is full: wait for a batch to finish
            size_t sb = 0;
            rsbd8g_segtuning tun{1, 0, 0, 0};
            const size_t n = take.size();
            const size_t tb = aup((n + 1) * 8) + 3 * aup(n * 8) + aup(n);
            size_t soff = 0, toff = 0;
            // a large request alone: the plain sort's scratch; otherwise the segmented launch's
            const rsbd8g_status ss = big ? rsbd8g_scratch_bytes(&key, total, &sb)
                                         : rsbd8g_segmented_scratch_bytes(&key, total, n, &tun, &sb);
            bool ok = ss == RSBD8G_OK && n + 1 <= slot_table_cap && arena.alloc(sb, &soff);
            if (ok && !arena.alloc(tb, &toff)) {
                arena.release(soff, sb);
                ok = false;
            }
            if (!ok) {   // give the buffers back and retry when memory frees up
                for (Request *r : take) arena.release(r->buf_off, r->buf_bytes);
                if (inflight == 0) {   // nothing will free memory: fail the head request
                    pending.erase(std::find(pending.begin(), pending.end(), head));
                    head->state = 2;
                    head->status = RSBD8G_ERR_BUSY;
                    head->t_done = now_s();
                    cv.notify_all();
                    continue;
                }
                return nullptr;
            }
            for (Request *r : take) r->state = 1;
            pending.erase(std::remove_if(pending.begin(), pending.end(), [](const Request *r) { return r->state == 1; }),
                          pending.end());
            Batch *b = new Batch;
            b->srv = this;
            b->reqs = take;
            b->slot = slot;
            b->scratch_off = soff;
            b->scratch_bytes = sb;
            b->tables_off = toff;
            b->tables_bytes = tb;
            b->host_tables = slot_tables[size_t(slot)];
            b->host_err = slot_err[size_t(slot)];
            b->keys = total;
            b->big = big;
            const double t = now_s();
            for (auto r : take) {
                r->state = 1;
                r->t_start = t;
            }
            slot_busy[size_t(slot)] = true;
            ++inflight;
            if (big) ++inflight_big;
            ++batches;
            max_coalesced = std::max<uint64_t>(max_coalesced, n);
            max_inflight = std::max(max_inflight, inflight);
            return b;
        }
    }

    // issue a formed batch on its stream (`mu` NOT held: CUDA calls only)
    void issue(Batch *b) {
        const size_t n = b->reqs.size();
        rsbd8g_desc key = b->reqs.front()->desc;
        // the tables in the pinned slot buffer laid out as in the arena, so one copy moves them all
        const size_t o_in = aup((n + 1) * 8), o_out = o_in + aup(n * 8), o_buf = o_out + aup(n * 8),
                     o_dir = o_buf + aup(n * 8);
        unsigned char *ht = b->host_tables;
        uint64_t *ho = reinterpret_cast<uint64_t *>(ht), *hi = reinterpret_cast<uint64_t *>(ht + o_in),
                 *hout = reinterpret_cast<uint64_t *>(ht + o_out), *hbuf = reinterpret_cast<uint64_t *>(ht + o_buf);
        uint8_t *hdir = ht + o_dir;
        ho[0] = 0;
        // the buffers are in the arena (device memory): the batch may prefetch tiles into L2 when
        // every request's arrays are device memory too
        bool device = true;
        for (size_t i = 0; i < n; ++i) device = device && b->reqs[i]->device;
        if (device) key.flags |= RSBD8G_FLAG_DEVICE_ARRAYS;
        for (size_t i = 0; i < n; ++i) {
            ho[i + 1] = ho[i] + b->reqs[i]->count;
            hi[i] = reinterpret_cast<uint64_t>(b->reqs[i]->in);
            hout[i] = reinterpret_cast<uint64_t>(b->reqs[i]->out);
            hbuf[i] = reinterpret_cast<uint64_t>(arena_base + b->reqs[i]->buf_off);
            hdir[i] = uint8_t(b->reqs[i]->desc.direction);
        }
        unsigned char *dt = arena_base + b->tables_off;
        uint64_t *d_off = reinterpret_cast<uint64_t *>(dt);
        uint64_t *d_in = reinterpret_cast<uint64_t *>(dt + o_in);
        uint64_t *d_out = reinterpret_cast<uint64_t *>(dt + o_out);
        uint64_t *d_buf = reinterpret_cast<uint64_t *>(dt + o_buf);
        uint8_t *d_dir = dt + o_dir;
        cudaStream_t s = streams[size_t(b->slot)];
        rsbd8g_segtuning tun{1, 0, 0, 0};
        rsbd8g_status st = RSBD8G_OK;
        *b->host_err = 0;
        if (b->big) {   // one request alone: the plain sort (its status word is at the scratch start too)
            Request *r = b->reqs.front();
            rsbd8g_desc d = r->desc;
            if (device) d.flags |= RSBD8G_FLAG_DEVICE_ARRAYS;
            st = rsbd8g_radixsortcopynoalloc(&d, r->count, arena_base + b->scratch_off, b->scratch_bytes, r->in, r->out,
                                             arena_base + r->buf_off, reinterpret_cast<rsbd8g_stream>(s));
        } else if (cudaMemcpyAsync(dt, ht, o_dir + n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            st = RSBD8G_ERR_CUDA;
        }
        else
            st = rsbd8g_segmented_sortcopy_ptrs_dirs(&key, b->keys, n, d_off, d_in, d_out, d_buf, d_dir,
                                                     arena_base + b->scratch_off, b->scratch_bytes, &tun,
                                                     reinterpret_cast<rsbd8g_stream>(s));
        if (st == RSBD8G_OK &&
            cudaMemcpyAsync(b->host_err, arena_base + b->scratch_off, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            st = RSBD8G_ERR_CUDA;
        if (st != RSBD8G_OK || cudaLaunchHostFunc(s, on_done, b) != cudaSuccess) {
            cudaGetLastError();
            b->launch_failed = true;
            cudaStreamSynchronize(s);
            on_done(b);
        }
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        while (!stop) {
            retire_locked();
            Batch *b = form_locked();
            if (b) {
                lk.unlock();
                issue(b);
                lk.lock();
                continue;
            }
            cv.wait_for(lk, std::chrono::microseconds(200));
        }
        // finish what is in flight
        while (inflight > 0) {
            retire_locked();
            if (inflight == 0) break;
            cv.wait_for(lk, std::chrono::milliseconds(1));
        }
    }
};

}  // namespace

struct rsbd8g_server {
    Server s;
};

extern "C" {

RSBD8G_API rsbd8g_status rsbd8g_server_create(size_t budget_bytes, uint32_t max_inflight, rsbd8g_server **out) {
    if (!out || budget_bytes < (size_t(1) << 20) || max_inflight == 0 || max_inflight > 64) return RSBD8G_ERR_BAD_ARG;
    *out = nullptr;
    rsbd8g_server *h = new rsbd8g_server;
    Server &s = h->s;
    cudaGetDevice(&s.device);
    s.budget = budget_bytes;
    if (cudaMalloc(&s.arena_base, budget_bytes) != cudaSuccess) {
        cudaGetLastError();
        s.arena_base = nullptr;
        delete h;
        return RSBD8G_ERR_NO_MEMORY;
    }
    s.arena.init(budget_bytes);
    s.slot_table_cap = s.max_batch_requests + 1;
    for (uint32_t i = 0; i < max_inflight; ++i) {
        cudaStream_t st;
        unsigned char *tab = nullptr;
        uint32_t *err = nullptr;
        // a batch of n < slot_table_cap requests: offsets, three pointer tables and the directions,
        // each starting on a 256-byte boundary as in the arena
        const size_t tab_bytes = 4 * aup(s.slot_table_cap * 8) + aup(s.slot_table_cap);
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void **>(&tab), tab_bytes) != cudaSuccess ||
            cudaMallocHost(reinterpret_cast<void **>(&err), 64) != cudaSuccess) {
            cudaGetLastError();
            delete h;
            return RSBD8G_ERR_NO_MEMORY;
        }
        s.streams.push_back(st);
        s.slot_tables.push_back(tab);
        s.slot_err.push_back(err);
        s.slot_busy.push_back(false);
    }
    // load every kernel a request can need now, so that no request waits for one to load
    for (uint32_t kb : {1u, 2u, 4u, 8u, 16u})
        for (uint32_t kind : {uint32_t(RSBD8G_KIND_UNSIGNED), uint32_t(RSBD8G_KIND_SIGNED), uint32_t(RSBD8G_KIND_FLOAT)})
            for (uint32_t mode : {0u, 1u, 2u, 3u, 4u, 5u, 6u, 7u}) {
                const rsbd8g_desc d{kb, kind, mode, uint32_t(RSBD8G_ASCFWDORDER), uint32_t(RSBD8G_DIRECT), 0u, 0, 0};
                (void)rsbd8g_prepare(&d);     // combinations the resolver refuses are never submitted
            }
    s.dispatcher = std::thread([&s] { s.run(); });
    *out = h;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_server_submit(rsbd8g_server *h, const rsbd8g_desc *desc, size_t count,
                                              const void *input, void *output, uint64_t *request_id) {
    if (!h || !desc || !request_id) return RSBD8G_ERR_BAD_ARG;
    size_t probe = 0;
    rsbd8g_segtuning tun{1, 0, 0, 0};
    rsbd8g_status st = rsbd8g_segmented_scratch_bytes(desc, count ? count : 1, 1, &tun, &probe);
    if (st != RSBD8G_OK) return st;
    if (count >= (size_t(1) << 30)) return RSBD8G_ERR_TOO_LARGE;
    if (count > 0 && (!input || !output || input == output)) return RSBD8G_ERR_BAD_ARG;
    Server &s = h->s;
    if (probe + size_t(count) * desc->key_bytes + 4096 > s.budget) return RSBD8G_ERR_BUSY;   // can never fit
    Request *r = new Request;
    r->desc = *desc;
    r->count = count;
    r->in = input;
    r->out = output;
    r->device = rsbd8g::device_memory(input) && rsbd8g::device_memory(output);
    r->group = rsbd8g::filter_class(desc);
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> g(s.mu);
        r->id = s.all.size();
        s.all.push_back(r);
        if (count == 0) {
            r->state = 2;
            r->t_done = r->t_submit;
        } else {
            s.pending.push_back(r);
        }
    }
    s.cv.notify_all();
    *request_id = r->id;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_server_wait(rsbd8g_server *h, uint64_t request_id, double timeout_s,
                                            rsbd8g_request_info *info) {
    if (!h) return RSBD8G_ERR_BAD_ARG;
    Server &s = h->s;
    std::unique_lock<std::mutex> lk(s.mu);
    if (request_id >= s.all.size()) return RSBD8G_ERR_BAD_ARG;
    Request *r = s.all[request_id];
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (r->state != 2) {
        if (s.cv.wait_until(lk, deadline) == std::cv_status::timeout && r->state != 2) return RSBD8G_ERR_TIMEOUT;
    }
    if (info) {
        info->status = r->status;
        info->count = r->count;
        info->submit_s = r->t_submit;
        info->start_s = r->t_start;
        info->done_s = r->t_done;
    }
    return r->status;
}

RSBD8G_API rsbd8g_status rsbd8g_server_drain(rsbd8g_server *h, double timeout_s) {
    if (!h) return RSBD8G_ERR_BAD_ARG;
    Server &s = h->s;
    std::unique_lock<std::mutex> lk(s.mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (!s.pending.empty() || s.inflight > 0) {
        if (s.cv.wait_until(lk, deadline) == std::cv_status::timeout && (!s.pending.empty() || s.inflight > 0))
            return RSBD8G_ERR_TIMEOUT;
    }
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_server_stats(rsbd8g_server *h, rsbd8g_server_counters *out) {
    if (!h || !out) return RSBD8G_ERR_BAD_ARG;
    Server &s = h->s;
    std::lock_guard<std::mutex> g(s.mu);
    out->submitted = s.all.size();
    out->completed = s.completed;
    out->keys_completed = s.keys_done;
    out->batches = s.batches;
    out->max_coalesced = s.max_coalesced;
    out->max_inflight_batches = s.max_inflight;
    out->pending = s.pending.size();
    out->arena_used = s.arena.used();
    out->budget = s.budget;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_server_destroy(rsbd8g_server *h) {
    if (!h) return RSBD8G_ERR_BAD_ARG;
    delete h;
    return RSBD8G_OK;
}

}  // extern "C"
