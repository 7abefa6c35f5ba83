// wrs_server.cu -- served request loop (host code): continuous batching of build+sample
// requests over wrs_batch slots, with resident alias tables under a device memory budget.
//
// Scheduling step (wrs_server_progress):
//   1. reap   -- every slot whose completion event has fired hands its requests back as
//                completions, unpins their tables and marks the tables it built as ready;
//   2. admit  -- for each free slot, requests are taken from the head of the arrival-order
//                queue while the batch limits hold: a request whose table is resident only
//                samples (waiting on the building slot's event if that table is still being
//                built by another slot); otherwise its table is allocated in the table arena,
//                evicting least-recently-used unpinned tables if needed.  A request that
//                does not fit stays at the head (arrival order is kept);
//   3. launch -- wrs_batch_set / wrs_batch_build / (cross-slot waits) / wrs_batch_sample on
//                the slot's stream, then the device status word is copied back and the
//                slot's completion event recorded.
// Slots run on separate non-blocking streams, so a new batch overlaps with those in flight.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <new>
#include <random>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/wrs.h"
#include "wrs_internal.cuh"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

constexpr uint64_t kArenaUnit = 256;

// Best-fit allocator over [0, size) with coalescing of free neighbours.  The free blocks are
// indexed twice -- by offset (to merge a released block with its neighbours) and by (size,
// offset) (the smallest block that fits, the lowest such offset first) -- so an allocation, a
// release and each retry of the eviction loop cost O(log free blocks), however many tables are
// resident.
class Arena {
  public:
    void reset(uint64_t size) {
        by_off_.clear();
        by_size_.clear();
        if (size) insert(0, size);
        used_ = 0;
    }
    bool alloc(uint64_t bytes, uint64_t& off) {
        bytes = (bytes + kArenaUnit - 1) / kArenaUnit * kArenaUnit;
        const auto it = by_size_.lower_bound({bytes, 0});
        if (it == by_size_.end()) return false;
        const uint64_t size = it->first;
        off = it->second;
        erase(off, size);
        if (size > bytes) insert(off + bytes, size - bytes);
        used_ += bytes;
        return true;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = (bytes + kArenaUnit - 1) / kArenaUnit * kArenaUnit;
        used_ -= bytes;
        auto next = by_off_.lower_bound(off);
        if (next != by_off_.end() && off + bytes == next->first) {
            bytes += next->second;
            by_size_.erase({next->second, next->first});
            next = by_off_.erase(next);
        }
        if (next != by_off_.begin()) {
            const auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                bytes += prev->second;
                by_size_.erase({prev->second, prev->first});
                by_off_.erase(prev);
            }
        }
        insert(off, bytes);
    }
    uint64_t used() const { return used_; }

  private:
    void insert(uint64_t off, uint64_t size) {
        by_off_[off] = size;
        by_size_.insert({size, off});
    }
    void erase(uint64_t off, uint64_t size) {
        by_off_.erase(off);
        by_size_.erase({size, off});
    }
    std::map<uint64_t, uint64_t> by_off_;                 // offset -> size
    std::set<std::pair<uint64_t, uint64_t>> by_size_;     // (size, offset)
    uint64_t used_ = 0;
};

struct Table {
    uint64_t id = 0;
    uint32_t n = 0;
    uint64_t off = 0;
    uint32_t pins = 0;       // requests in flight that use the table
    int building_slot = -1;  // slot whose batch in flight builds it, -1 when ready
    bool in_lru = false;
    std::list<uint64_t>::iterator lru;
};

struct Pending {
    uint64_t ticket;
    wrs_request r;
    double submit;
};

struct InFlight {
    uint64_t ticket;
    double submit;
    uint64_t table_id;
    uint32_t built;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    wrs_batch* batch = nullptr;
    uint32_t* status_host = nullptr;  // pinned copy of the batch's device status word
    bool busy = false;
    std::vector<InFlight> reqs;
    std::vector<uint64_t> built_ids;
};

}  // namespace

struct wrs_server {
    const wrs_handle* h = nullptr;
    wrs_server_config cfg{};
    void* arena_base = nullptr;
    uint64_t arena_bytes = 0;
    uint64_t scratch_bytes = 0;
    Arena arena;
    std::unordered_map<uint64_t, Table> tables;
    std::list<uint64_t> lru;  // unpinned resident tables, least recently used first
    std::deque<Pending> queue;
    std::vector<Slot> slots;
    std::deque<wrs_completion> done;
    uint64_t next_ticket = 0;
    uint64_t outstanding = 0;
    wrs_server_stats stats{};
};

namespace {

wrs_status sfail(wrs_status s, const std::string& msg) {
    wrs::set_last_error(s, msg.c_str());
    return s;
}

wrs_status scuda(cudaError_t e, const char* where) {
    return sfail(WRS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define SRV_CUDA(call, where)                        \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return scuda(e_, where); \
    } while (0)

void unpin(wrs_server* s, uint64_t id) {
    auto it = s->tables.find(id);
    if (it == s->tables.end()) return;
    Table& t = it->second;
    if (t.pins && --t.pins == 0) {
        s->lru.push_back(id);
        t.lru = std::prev(s->lru.end());
        t.in_lru = true;
    }
}

void pin(wrs_server* s, Table& t) {
    if (t.in_lru) {
        s->lru.erase(t.lru);
        t.in_lru = false;
    }
    ++t.pins;
}

void drop_table(wrs_server* s, uint64_t id) {
    auto it = s->tables.find(id);
    if (it == s->tables.end()) return;
    if (it->second.in_lru) s->lru.erase(it->second.lru);
    s->arena.release(it->second.off, 8ull * it->second.n);
    s->tables.erase(it);
}

// Allocates 8n bytes for a table, evicting unpinned tables (least recently used first).
bool alloc_table(wrs_server* s, uint32_t n, uint64_t& off) {
    while (!s->arena.alloc(8ull * n, off)) {
        if (s->lru.empty()) return false;
        const uint64_t victim = s->lru.front();
        drop_table(s, victim);
        ++s->stats.evictions;
    }
    s->stats.table_bytes_peak = std::max<uint64_t>(s->stats.table_bytes_peak, s->arena.used());
    return true;
}

wrs_status reap(wrs_server* s) {
    const double t = now_s();
    for (size_t k = 0; k < s->slots.size(); ++k) {
        Slot& sl = s->slots[k];
        if (!sl.busy) continue;
        const cudaError_t q = cudaEventQuery(sl.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return scuda(q, "batch completion");
        const uint32_t st = *sl.status_host;
        s->stats.device_status |= st;
        for (uint64_t id : sl.built_ids) {
            auto it = s->tables.find(id);
            if (it != s->tables.end() && it->second.building_slot == static_cast<int>(k))
                it->second.building_slot = -1;
        }
        for (const InFlight& r : sl.reqs) {
            unpin(s, r.table_id);
            wrs_completion c{};
            c.ticket = r.ticket;
            c.submit_s = r.submit;
            c.done_s = t;
            c.built = r.built;
            c.status = (st & wrs::kStatusTimeout) ? WRS_ERR_TIMEOUT : WRS_OK;
            s->done.push_back(c);
            ++s->stats.completed;
        }
        sl.reqs.clear();
        sl.built_ids.clear();
        sl.busy = false;
    }
    return WRS_OK;
}

// Forms and launches one batch on free slot k; returns false in `launched` if nothing
// could be admitted.
wrs_status admit_and_launch(wrs_server* s, size_t k, bool& launched) {
    launched = false;
    Slot& sl = s->slots[k];
    std::vector<wrs_dist_desc> descs;
    std::vector<int> waits;
    uint64_t weights = 0, samples = 0;
    char* base = static_cast<char*>(s->arena_base);
    while (!s->queue.empty() && descs.size() < s->cfg.max_batch_dists) {
        Pending& p = s->queue.front();
        const wrs_request& r = p.r;
        auto it = s->tables.find(r.table_id);
        if (it != s->tables.end() && it->second.n != r.n) {
            if (it->second.pins) {
                // the id names a table of another size that is in use: reject the request
                wrs_completion c{};
                c.ticket = p.ticket;
                c.submit_s = p.submit;
                c.done_s = now_s();
                c.status = WRS_ERR_INVALID_ARG;
                s->done.push_back(c);
                ++s->stats.completed;
                s->queue.pop_front();
                continue;
            }
            drop_table(s, r.table_id);
            it = s->tables.end();
        }
        if (samples + r.s > s->cfg.max_batch_samples) break;
        wrs_dist_desc d{};
        d.samples = r.samples;
        d.s = r.s;
        d.seed = r.seed;
        d.n = r.n;
        uint32_t built = 0;
        if (it != s->tables.end()) {
            Table& t = it->second;
            if (t.building_slot >= 0 && t.building_slot != static_cast<int>(k) &&
                std::find(waits.begin(), waits.end(), t.building_slot) == waits.end())
                waits.push_back(t.building_slot);
            pin(s, t);
            d.table = reinterpret_cast<wrs_alias_entry*>(base + t.off);
            ++s->stats.reuses;
        } else {
            if (weights + r.n > s->cfg.max_batch_weights) break;
            uint64_t off = 0;
            if (!alloc_table(s, r.n, off)) break;  // waits for memory, keeps arrival order
            Table t;
            t.id = r.table_id;
            t.n = r.n;
            t.off = off;
            t.building_slot = static_cast<int>(k);
            Table& ins = s->tables.emplace(r.table_id, t).first->second;
            pin(s, ins);
            d.weights = r.weights;
            d.table = reinterpret_cast<wrs_alias_entry*>(base + off);
            weights += r.n;
            built = 1;
            sl.built_ids.push_back(r.table_id);
            ++s->stats.builds;
        }
        samples += r.s;
        descs.push_back(d);
        sl.reqs.push_back(InFlight{p.ticket, p.submit, r.table_id, built});
        s->queue.pop_front();
    }
    if (descs.empty()) return WRS_OK;
    wrs_status st = wrs_batch_set(sl.batch, sl.stream, descs.data(),
                                  static_cast<uint32_t>(descs.size()));
    if (st == WRS_OK) st = wrs_batch_build(s->h, sl.stream, sl.batch);
    if (st != WRS_OK) return st;
    for (int w : waits) SRV_CUDA(cudaStreamWaitEvent(sl.stream, s->slots[w].done, 0), "slot wait");
    st = wrs_batch_sample(s->h, sl.stream, sl.batch);
    if (st != WRS_OK) return st;
    uint32_t* dev_status = wrs::batch_status_word(sl.batch);
    SRV_CUDA(cudaMemcpyAsync(sl.status_host, dev_status, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             sl.stream),
             "status copy");
    SRV_CUDA(cudaMemsetAsync(dev_status, 0, sizeof(uint32_t), sl.stream), "status clear");
    SRV_CUDA(cudaEventRecord(sl.done, sl.stream), "slot event");
    sl.busy = true;
    ++s->stats.batches;
    launched = true;
    return WRS_OK;
}

uint32_t take_completions(wrs_server* s, wrs_completion* out, uint32_t max_out) {
    uint32_t c = 0;
    while (c < max_out && !s->done.empty()) {
        out[c++] = s->done.front();
        s->done.pop_front();
        --s->outstanding;
    }
    return c;
}

void destroy_slots(wrs_server* s) {
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.batch) wrs_batch_destroy(sl.batch);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.status_host) cudaFreeHost(sl.status_host);
    }
    s->slots.clear();
}

}  // namespace

extern "C" {

wrs_status wrs_server_config_init(wrs_server_config* c) {
    if (!c) return sfail(WRS_ERR_INVALID_ARG, "config is NULL");
    std::memset(c, 0, sizeof(*c));
    c->memory_budget = 16ull << 30;
    c->slots = 3;
    c->max_batch_dists = 1024;
    c->max_batch_weights = 1ull << 25;
    c->max_batch_samples = 1ull << 24;
    return WRS_OK;
}

wrs_status wrs_server_create(const wrs_handle* h, const wrs_server_config* c, wrs_server** out) {
    if (!h || !c || !out) return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (c->slots == 0 || c->slots > 16) return sfail(WRS_ERR_INVALID_ARG, "slots must be 1..16");
    if (c->max_batch_dists == 0 || c->max_batch_weights == 0 || c->max_batch_samples == 0)
        return sfail(WRS_ERR_INVALID_ARG, "batch limits must be >= 1");
    const size_t per = wrs_batch_bytes(h, c->max_batch_dists, c->max_batch_weights,
                                       c->max_batch_samples);
    if (per == 0) return sfail(WRS_ERR_INVALID_ARG, "batch limits out of range (alias method only)");
    const uint64_t scratch = static_cast<uint64_t>(per) * c->slots;
    if (scratch + (1ull << 20) > c->memory_budget)
        return sfail(WRS_ERR_INVALID_ARG, "memory_budget does not cover the batch scratch");
    wrs_server* s = new (std::nothrow) wrs_server;
    if (!s) return sfail(WRS_ERR_OOM, "host allocation failed");
    s->h = h;
    s->cfg = *c;
    s->scratch_bytes = scratch;
    s->arena_bytes = (c->memory_budget - scratch) / kArenaUnit * kArenaUnit;
    cudaError_t e = cudaMalloc(&s->arena_base, s->arena_bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        delete s;
        return e == cudaErrorMemoryAllocation ? sfail(WRS_ERR_OOM, "table arena allocation failed")
                                              : scuda(e, "cudaMalloc");
    }
    s->arena.reset(s->arena_bytes);
    s->slots.resize(c->slots);
    for (Slot& sl : s->slots) {
        wrs_status st = wrs_batch_create(h, c->max_batch_dists, c->max_batch_weights,
                                         c->max_batch_samples, &sl.batch);
        if (st == WRS_OK) {
            e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
            if (e == cudaSuccess)
                e = cudaHostAlloc(reinterpret_cast<void**>(&sl.status_host), sizeof(uint32_t),
                                  cudaHostAllocDefault);
            if (e != cudaSuccess) st = scuda(e, "slot setup");
            else *sl.status_host = 0;
        }
        if (st != WRS_OK) {
            destroy_slots(s);
            cudaFree(s->arena_base);
            delete s;
            return st;
        }
    }
    s->stats.table_arena_bytes = s->arena_bytes;
    s->stats.scratch_bytes = scratch;
    *out = s;
    return WRS_OK;
}

void wrs_server_destroy(wrs_server* s) {
    if (!s) return;
    destroy_slots(s);
    if (s->arena_base) cudaFree(s->arena_base);
    delete s;
}

wrs_status wrs_server_submit(wrs_server* s, const wrs_request* r, uint64_t* ticket) {
    if (!s || !r) return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (r->n == 0 || r->n > s->cfg.max_batch_weights || r->n > 0x7fffffffu)
        return sfail(WRS_ERR_INVALID_ARG, "request n out of range");
    if (r->s > s->cfg.max_batch_samples) return sfail(WRS_ERR_INVALID_ARG, "request s out of range");
    if (!r->weights) return sfail(WRS_ERR_INVALID_ARG, "request weights is NULL");
    if (r->s && !r->samples) return sfail(WRS_ERR_INVALID_ARG, "request samples is NULL");
    if (8ull * r->n > s->arena_bytes)
        return sfail(WRS_ERR_CAPACITY, "the request's table exceeds the table arena");
    Pending p{s->next_ticket++, *r, now_s()};
    s->queue.push_back(p);
    ++s->outstanding;
    ++s->stats.submitted;
    if (ticket) *ticket = p.ticket;
    return WRS_OK;
}

wrs_status wrs_server_progress(wrs_server* s, wrs_completion* out, uint32_t max_out,
                               uint32_t* count) {
    if (!s) return sfail(WRS_ERR_INVALID_ARG, "server is NULL");
    if (count) *count = 0;
    wrs_status st = reap(s);
    if (st != WRS_OK) return st;
    for (size_t k = 0; k < s->slots.size() && !s->queue.empty(); ++k) {
        if (s->slots[k].busy) continue;
        bool launched = false;
        st = admit_and_launch(s, k, launched);
        if (st != WRS_OK) return st;
        if (!launched) break;  // the head request waits for memory
    }
    const uint32_t c = out ? take_completions(s, out, max_out) : 0;
    if (count) *count = c;
    return WRS_OK;
}

uint64_t wrs_server_pending(const wrs_server* s) { return s ? s->outstanding : 0; }

wrs_status wrs_server_get_stats(const wrs_server* s, wrs_server_stats* st) {
    if (!s || !st) return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    *st = s->stats;
    return WRS_OK;
}

wrs_status wrs_server_run_trace(wrs_server* s, const wrs_request* reqs, const double* arrival_s,
                                uint32_t count, wrs_completion* out) {
    if (!s || (count && (!reqs || !arrival_s || !out)))
        return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (s->outstanding) return sfail(WRS_ERR_INVALID_ARG, "the server has requests pending");
    const uint64_t base = s->next_ticket;
    const double t0 = now_s();
    uint32_t next = 0, completed = 0;
    std::vector<wrs_completion> buf(256);
    while (completed < count) {
        const double t = now_s() - t0;
        bool busy = false;
        while (next < count && arrival_s[next] <= t) {
            uint64_t ticket = 0;
            wrs_status st = wrs_server_submit(s, &reqs[next], &ticket);
            if (st != WRS_OK) return st;
            s->queue.back().submit = t0 + arrival_s[next];
            ++next;
            busy = true;
        }
        uint32_t c = 0;
        wrs_status st = wrs_server_progress(s, buf.data(), static_cast<uint32_t>(buf.size()), &c);
        if (st != WRS_OK) return st;
        for (uint32_t i = 0; i < c; ++i) out[buf[i].ticket - base] = buf[i];
        completed += c;
        if (!busy && c == 0) std::this_thread::yield();
    }
    return WRS_OK;
}

}  // extern "C"

int wrs_test_arena(uint64_t seed, uint32_t iterations) {
    constexpr uint64_t kSize = 1ull << 30;
    Arena ar;
    ar.reset(kSize);
    std::mt19937_64 rng(seed);
    std::map<uint64_t, uint64_t> live;  // offset -> rounded bytes
    uint64_t used = 0;
    for (uint32_t it = 0; it < iterations; ++it) {
        if (live.empty() || rng() % 3u) {
            const uint64_t bytes = 1u + rng() % (4ull << 20);
            uint64_t off = 0;
            if (!ar.alloc(bytes, off)) continue;
            const uint64_t rb = (bytes + kArenaUnit - 1) / kArenaUnit * kArenaUnit;
            if (off % kArenaUnit || off + rb > kSize) return 1;
            const auto nx = live.lower_bound(off);
            if (nx != live.end() && nx->first < off + rb) return 2;
            if (nx != live.begin() && std::prev(nx)->first + std::prev(nx)->second > off) return 3;
            live[off] = rb;
            used += rb;
        } else {
            auto victim = live.begin();
            std::advance(victim, static_cast<long>(rng() % live.size()));
            ar.release(victim->first, victim->second);
            used -= victim->second;
            live.erase(victim);
        }
        if (ar.used() != used) return 4;
    }
    for (const auto& kv : live) ar.release(kv.first, kv.second);
    uint64_t off = 1;
    if (!ar.alloc(kSize, off) || off != 0) return 5;
    return 0;
}
