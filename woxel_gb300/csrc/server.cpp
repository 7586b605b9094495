// server.cpp — continuous-batching render server (wx_server_*).
//
// A scheduler thread owns the GPU side: it admits queued requests in arrival
// order while their output buffers fit the budget (a device arena carved by a
// first-fit allocator, so serving never calls cudaMalloc/cudaFree), forms
// time-sliced batches of 8x4 tiles across all admitted requests (a large
// request spans several slices through the jobs' tile offsets) and launches
// them on up to max_inflight streams with the batched persistent kernel.
// Requests that arrive while launches are on the GPU join the next slice, so
// their work overlaps with the earlier requests'. Per-pixel results equal
// wx_render's: a tile is rendered by the same lane code whichever launch it
// lands in.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "wx_alloc.h"
#include "wx_common.h"
#include "wx_kernels.h"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over one device allocation, 256-byte granules, with
// coalescing of neighbouring free ranges.
class Arena {
  public:
    cudaError_t init(size_t bytes) {
        size_ = bytes & ~(size_t)255;
        if (size_ == 0) return cudaSuccess;
        cudaError_t e = wx::dev_alloc(&base_, size_);
        if (e == cudaSuccess) free_[0] = size_;
        return e;
    }
    void destroy() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
    }
    bool alloc(size_t n, size_t *off) {
        n = (n + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const size_t rest = it->second - n, at = it->first + n;
            free_.erase(it);
            if (rest) free_[at] = rest;
            in_use_ += n;
            peak_ = std::max(peak_, in_use_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = (n + 255) & ~(size_t)255;
        in_use_ -= n;
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + n == next->first) {
            n += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += n;
                return;
            }
        }
        free_[off] = n;
    }
    char *base() const { return static_cast<char *>(base_); }
    size_t size() const { return size_; }
    size_t in_use() const { return in_use_; }
    size_t peak() const { return peak_; }

  private:
    void *base_ = nullptr;
    size_t size_ = 0, in_use_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_;
};

enum class RState { Pending, Active, Done, Polled };

struct Req {
    uint64_t ticket = 0;
    wx_request r{};
    wxk::DevGrid g{};
    uint32_t tiles = 0, next = 0, done_tiles = 0;
    size_t off = 0, bytes = 0;
    bool has_buf = false;
    uint8_t *rgba = nullptr;
    wx_hit *hits = nullptr;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = WX_OK;
    RState state = RState::Pending;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    wxk::Job *jobs_host = nullptr;
    wxk::Job *jobs_dev = nullptr;
    uint32_t *counter = nullptr;   // [0] tile queue, [1] tiles skipped for cancelled requests
    uint32_t *skipped_host = nullptr;  // page-locked copy of counter[1] after the launch
    bool busy = false;
    std::vector<std::pair<Req *, uint32_t>> parts;
};

constexpr uint32_t kTileW = 8, kTileH = 4;
// Cancel table: a request's tiles in launches already on the GPU are skipped
// once its ticket (low 32 bits) is written at ticket % kCancelSlots.
constexpr uint32_t kCancelSlots = 65536;

}  // namespace

struct wx_server {
    wx_ctx *ctx = nullptr;
    int device = 0, num_sms = 0;
    wx_server_config cfg{};
    std::vector<wxk::DevGrid> grids;
    uint64_t grid_bytes = 0;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> pending, active, done_q;
    std::unordered_map<uint64_t, Req *> reqs;
    std::vector<Slot> slots;
    uint32_t *cancel_dev = nullptr, *cancel_host = nullptr;  // the cancel table and its page-locked source
    cudaStream_t ctl = nullptr;                             // carries cancel writes while launches run
    std::thread th;
    bool stop = false, arena_ready = false, broken = false;
    uint64_t next_ticket = 1;
    wx_server_stats st{};

    void finish(Req *q, int status) {
        q->status = status;
        q->state = RState::Done;
        q->t_done = now_s();
        done_q.push_back(q);
        if (status == WX_ERR_CANCELLED) st.cancelled++;
        else {
            st.completed++;
            st.rays_done += (uint64_t)q->tiles * 32;
        }
        cv_done.notify_all();
    }

    // Tiles of q are retired (rendered, or given up after an error); the
    // request finishes once every tile is, so no launch still refers to it.
    void retire_tiles(Req *q, uint32_t n, bool ok) {
        if (!ok && q->status == WX_OK) q->status = WX_ERR_CUDA;
        q->done_tiles += n;
        if (q->done_tiles == q->tiles && q->state == RState::Active) finish(q, q->status);
    }

    // Completed launches -> request progress. Called with mu held.
    bool retire() {
        bool any = false;
        for (Slot &s : slots) {
            if (!s.busy) continue;
            const cudaError_t e = cudaEventQuery(s.ev);
            if (e == cudaErrorNotReady) continue;
            if (e != cudaSuccess) cudaGetLastError();
            else st.tiles_cancelled_launched += *s.skipped_host;
            for (auto &p : s.parts) retire_tiles(p.first, p.second, e == cudaSuccess);
            s.parts.clear();
            s.busy = false;
            any = true;
        }
        return any;
    }

    // Pending -> active while the arena has room (arrival order). Called with mu held.
    void admit() {
        while (!pending.empty()) {
            Req *q = pending.front();
            if (q->bytes && !arena.alloc(q->bytes, &q->off)) break;
            pending.pop_front();
            q->has_buf = q->bytes != 0;
            q->rgba = reinterpret_cast<uint8_t *>(arena.base() + q->off);
            q->hits = q->r.want_hits
                          ? reinterpret_cast<wx_hit *>(arena.base() + q->off +
                                                       (((size_t)q->r.width * q->r.height * 4 + 255) & ~(size_t)255))
                          : nullptr;
            q->t_admit = now_s();
            q->state = RState::Active;
            if (q->tiles == 0) finish(q, WX_OK);
            else active.push_back(q);
        }
    }

    // One time slice of tiles into a free slot. Called with mu held.
    bool launch(Slot &s) {
        const bool fifo = cfg.flags & WX_SERVE_FIFO;
        uint32_t budget = fifo ? UINT32_MAX : cfg.slice_tiles, tiles = 0, n = 0;
        for (Req *q : active) {
            if (q->next < q->tiles && q->status != WX_OK) {  // failed or cancelled: give up its remaining tiles
                const uint32_t rest = q->tiles - q->next;
                q->next = q->tiles;
                if (q->status == WX_ERR_CANCELLED) st.tiles_cancelled_queued += rest;
                retire_tiles(q, rest, false);
            }
            if (q->next >= q->tiles) continue;
            if (n >= cfg.max_frames || budget == 0) break;
            const uint32_t take = std::min(q->tiles - q->next, budget);
            wxk::Job &j = s.jobs_host[n++];
            memset(&j, 0, sizeof j);
            j.g = q->g;
            j.width = q->r.width;
            j.height = q->r.height;
            j.tile_w = kTileW;
            j.tile_h = kTileH;
            j.order = (uint32_t)wxk::Tuning().order;
            j.tiles_x = (q->r.width & ~7u) / kTileW;
            j.tiles = q->tiles;
            j.tile_begin = tiles;
            j.tile_off = q->next;
            j.rgba = reinterpret_cast<uint32_t *>(q->rgba);
            j.hits = q->hits;
            j.s = q->r.state;
            j.cancel_slot = (uint32_t)(q->ticket % kCancelSlots);
            j.cancel_id = (uint32_t)q->ticket;
            s.parts.emplace_back(q, take);
            q->next += take;
            tiles += take;
            budget -= take;
            if (fifo) break;
        }
        while (!active.empty() && active.front()->next >= active.front()->tiles) active.pop_front();
        if (n == 0) return false;
        wxk::Tuning t;
        cudaError_t e = cudaMemcpyAsync(s.jobs_dev, s.jobs_host, n * sizeof(wxk::Job), cudaMemcpyHostToDevice, s.stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s.counter, 0, 2 * sizeof(uint32_t), s.stream);
        if (e == cudaSuccess)
            e = wxk::launch_batched(s.jobs_dev, n, tiles, s.counter, t, num_sms, wxk::all_modes(s.jobs_host, n),
                                    s.stream, cancel_dev, s.counter + 1);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s.skipped_host, s.counter + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s.stream);
        if (e == cudaSuccess) e = cudaEventRecord(s.ev, s.stream);
        if (e != cudaSuccess) {
            cudaGetLastError();
            for (auto &p : s.parts) retire_tiles(p.first, p.second, false);
            s.parts.clear();
            return false;
        }
        s.busy = true;
        st.launches++;
        return true;
    }

    void loop() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        try {
            schedule(lk);
        } catch (...) {
            // A host allocation failed inside the scheduler: stop scheduling, let the
            // launches in flight finish (their outputs stay valid until destroy), and
            // refuse new submissions (WX_ERR_OOM).
            broken = true;
            for (Slot &sl : slots)
                if (sl.busy) {
                    cudaEventSynchronize(sl.ev);
                    sl.busy = false;
                }
            cv_done.notify_all();
        }
    }

    void schedule(std::unique_lock<std::mutex> &lk) {
        for (;;) {
            retire();
            admit();
            const uint32_t usable = (cfg.flags & WX_SERVE_FIFO) ? 1u : cfg.max_inflight;
            for (uint32_t i = 0; i < usable; i++)
                if (!slots[i].busy && !launch(slots[i])) break;
            const bool busy = std::any_of(slots.begin(), slots.end(), [](const Slot &s) { return s.busy; });
            if (stop && !busy) break;
            // Poll the launches' events every 20 us while any is in flight; otherwise
            // sleep until a submission, release, cancel or stop notifies (or 50 ms).
            if (busy) cv_work.wait_for(lk, std::chrono::microseconds(20));
            else cv_work.wait_for(lk, std::chrono::milliseconds(50));
        }
    }
};

namespace {
int sfail(int code, const std::string &msg) {
    wx::set_thread_error(msg);
    return code;
}
void fill_result(const Req *q, wx_result *o) {
    o->ticket = q->ticket;
    o->user = q->r.user;
    o->status = q->status;
    o->width = q->r.width;
    o->height = q->r.height;
    o->rgba8 = q->status == WX_OK ? q->rgba : nullptr;
    o->hits = q->status == WX_OK ? q->hits : nullptr;
    o->t_submit = q->t_submit;
    o->t_admit = q->t_admit;
    o->t_done = q->t_done;
}
}  // namespace

extern "C" {

int wx_server_create(wx_ctx *ctx, const wx_server_config *cfg, wx_server **out) {
    return wx::guard("wx_server_create", [&]() -> int {
        if (!ctx || !cfg || !out) return sfail(WX_ERR_INVALID, "wx_server_create: null argument");
        wx_server_config c = *cfg;
        if (c.max_inflight == 0) c.max_inflight = 2;
        // Default slice: four 1080p frames. Measured at saturation (5000 req/s over the 8
        // benchmark grids): 3.58 Grays/s at 16,384 tiles per launch, 5.62 at 65,536, 5.90 at
        // 262,144 and 5.94 at 1,048,576, with p50/p99 at 200-2000 req/s unchanged or better.
        if (c.slice_tiles == 0) c.slice_tiles = 262144;
        if (c.max_frames == 0) c.max_frames = 256;
        if (c.max_inflight > 8 || c.max_frames > 1024)
            return sfail(WX_ERR_INVALID, "wx_server_create: max_inflight must be <= 8 and max_frames <= 1024");
        auto *s = new (std::nothrow) wx_server();
        if (!s) return sfail(WX_ERR_OOM, "host allocation failed");
        s->ctx = ctx;
        s->cfg = c;
        wxk::ctx_device_info(ctx, &s->device, &s->num_sms);
        cudaSetDevice(s->device);
        cudaError_t e;
        auto bail = [&](cudaError_t err, const char *what) {
            s->stop = true;
            wx_server_destroy(s);
            return sfail(err == cudaErrorMemoryAllocation ? WX_ERR_OOM : WX_ERR_CUDA,
                         std::string(what) + ": " + cudaGetErrorString(err));
        };
        try {  // host containers first; the scheduler then never grows a slot's parts list
            s->slots.resize(c.max_inflight);
            for (Slot &sl : s->slots) sl.parts.reserve(c.max_frames);
        } catch (...) {
            delete s;
            throw;
        }
        for (Slot &sl : s->slots) {
            if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
            if ((e = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
            if ((e = wx::pinned_alloc(&sl.jobs_host, c.max_frames * sizeof(wxk::Job))) != cudaSuccess) return bail(e, "jobs");
            if ((e = wx::dev_alloc(&sl.jobs_dev, c.max_frames * sizeof(wxk::Job))) != cudaSuccess) return bail(e, "jobs");
            if ((e = wx::dev_alloc(&sl.counter, 256)) != cudaSuccess) return bail(e, "counter");
            if ((e = wx::pinned_alloc(&sl.skipped_host, sizeof(uint32_t))) != cudaSuccess) return bail(e, "counter");
            *sl.skipped_host = 0;
        }
        if ((e = wx::dev_alloc(&s->cancel_dev, kCancelSlots * sizeof(uint32_t))) != cudaSuccess) return bail(e, "cancel");
        if ((e = wx::pinned_alloc(&s->cancel_host, kCancelSlots * sizeof(uint32_t))) != cudaSuccess)
            return bail(e, "cancel");
        if ((e = cudaMemset(s->cancel_dev, 0, kCancelSlots * sizeof(uint32_t))) != cudaSuccess) return bail(e, "cancel");
        if ((e = cudaStreamCreateWithFlags(&s->ctl, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
        try {
            s->th = std::thread([s] { s->loop(); });
        } catch (...) {
            s->stop = true;
            wx_server_destroy(s);
            throw;
        }
        *out = s;
        return WX_OK;
    });
}

int wx_server_add_grid(wx_server *s, const wx_grid *grid, uint32_t *grid_id) {
    return wx::guard("wx_server_add_grid", [&]() -> int {
        if (!s || !grid || !grid_id) return sfail(WX_ERR_INVALID, "wx_server_add_grid: null argument");
        wxk::DevGrid g;
        int dev = -1;
        wxk::grid_device_view(grid, &g, &dev);
        if (dev != s->device) return sfail(WX_ERR_INVALID, "wx_server_add_grid: grid is on another device");
        wx_grid_info info;
        wx_grid_get_info(grid, &info);
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->arena_ready) return sfail(WX_ERR_INVALID, "wx_server_add_grid: add grids before the first request");
        if (s->grid_bytes + info.device_bytes > s->cfg.budget_bytes)
            return sfail(WX_ERR_BUDGET, "wx_server_add_grid: resident grids exceed the budget");
        s->grids.push_back(g);
        s->grid_bytes += info.device_bytes;
        *grid_id = (uint32_t)s->grids.size() - 1;
        return WX_OK;
    });
}

int wx_server_submit(wx_server *s, const wx_request *r, uint64_t *ticket) {
    return wx::guard("wx_server_submit", [&]() -> int {
        if (!s || !r) return sfail(WX_ERR_INVALID, "wx_server_submit: null argument");
        if ((uint64_t)r->width * r->height >= (1ull << 32)) return sfail(WX_ERR_UNSUPPORTED, "wx_server_submit: too large");
        auto *q = new (std::nothrow) Req();
        if (!q) return sfail(WX_ERR_OOM, "host allocation failed");
        q->r = *r;
        q->tiles = ((r->width & ~7u) / kTileW) * ((r->height & ~3u) / kTileH);
        q->bytes = q->tiles ? (((size_t)r->width * r->height * 4 + 255) & ~(size_t)255) +
                                  (r->want_hits ? (size_t)r->width * r->height * sizeof(wx_hit) : 0)
                            : 0;
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->broken) {
            delete q;
            return sfail(WX_ERR_OOM, "wx_server_submit: the server stopped after a host allocation failure");
        }
        if (r->grid_id >= s->grids.size()) {
            delete q;
            return sfail(WX_ERR_INVALID, "wx_server_submit: unknown grid_id");
        }
        if (!s->arena_ready) {
            // The output arena takes the budget left after the resident grids,
            // keeping 1 GiB of the device's free memory untouched.
            cudaSetDevice(s->device);
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            const size_t margin = (size_t)1 << 30;
            size_t bytes = s->cfg.budget_bytes - s->grid_bytes;
            if (free_b > margin && bytes > free_b - margin) bytes = free_b - margin;
            const cudaError_t e = s->arena.init(bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                delete q;
                return sfail(WX_ERR_OOM, std::string("wx_server_submit: output arena: ") + cudaGetErrorString(e));
            }
            s->arena_ready = true;
        }
        if (q->bytes > s->arena.size()) {
            delete q;
            return sfail(WX_ERR_BUDGET, "wx_server_submit: request larger than the output arena");
        }
        q->g = s->grids[r->grid_id];
        q->ticket = s->next_ticket++;
        q->t_submit = now_s();
        try {  // a failed insertion leaves neither container holding q
            s->reqs.emplace(q->ticket, q);
        } catch (...) {
            delete q;
            throw;
        }
        try {
            s->pending.push_back(q);
        } catch (...) {
            s->reqs.erase(q->ticket);
            delete q;
            throw;
        }
        s->st.submitted++;
        if (ticket) *ticket = q->ticket;
        s->cv_work.notify_one();
        return WX_OK;
    });
}

int wx_server_cancel(wx_server *s, uint64_t ticket) {
    return wx::guard("wx_server_cancel", [&]() -> int {
        if (!s) return WX_ERR_INVALID;
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return sfail(WX_ERR_INVALID, "wx_server_cancel: unknown ticket");
        Req *q = it->second;
        if (q->state == RState::Pending) {
            s->pending.erase(std::find(s->pending.begin(), s->pending.end(), q));
            s->finish(q, WX_ERR_CANCELLED);
            return WX_OK;
        }
        if (q->state != RState::Active) return sfail(WX_ERR_INVALID, "wx_server_cancel: request already finished");
        if (q->status == WX_OK) {
            // Tiles not yet launched are dropped by the scheduler; launches on the GPU
            // skip the rest once the ticket lands in the cancel table (copied on the
            // control stream, concurrently with them). The request finishes with
            // WX_ERR_CANCELLED when no launch refers to it any more.
            q->status = WX_ERR_CANCELLED;
            const uint32_t slot = (uint32_t)(q->ticket % kCancelSlots);
            s->cancel_host[slot] = (uint32_t)q->ticket;
            int prev = -1;
            cudaGetDevice(&prev);
            if (prev != s->device) cudaSetDevice(s->device);
            const cudaError_t e = cudaMemcpyAsync(s->cancel_dev + slot, s->cancel_host + slot, sizeof(uint32_t),
                                                  cudaMemcpyHostToDevice, s->ctl);
            if (prev != s->device && prev >= 0) cudaSetDevice(prev);
            if (e != cudaSuccess) cudaGetLastError();  // the launched tiles then just render
        }
        s->cv_work.notify_one();
        return WX_OK;
    });
}

int wx_server_poll(wx_server *s, wx_result *out, uint32_t max, uint32_t *n, int wait_ms) {
    return wx::guard("wx_server_poll", [&]() -> int {
        if (!s || !n || (max && !out)) return sfail(WX_ERR_INVALID, "wx_server_poll: null argument");
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->done_q.empty() && wait_ms > 0)
            s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done_q.empty(); });
        uint32_t k = 0;
        while (k < max && !s->done_q.empty()) {
            Req *q = s->done_q.front();
            s->done_q.pop_front();
            q->state = RState::Polled;
            fill_result(q, &out[k++]);
        }
        *n = k;
        return WX_OK;
    });
}

int wx_server_copy_result(wx_server *s, uint64_t ticket, uint8_t *rgba8_host, wx_hit *hits_host) {
    return wx::guard("wx_server_copy_result", [&]() -> int {
        if (!s) return WX_ERR_INVALID;
        const Req *q;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->reqs.find(ticket);
            if (it == s->reqs.end()) return sfail(WX_ERR_INVALID, "wx_server_copy_result: unknown ticket");
            q = it->second;
            if (q->state != RState::Polled) return sfail(WX_ERR_INVALID, "wx_server_copy_result: result not polled yet");
            if (q->status != WX_OK) return sfail(WX_ERR_INVALID, "wx_server_copy_result: request did not complete");
        }
        // A polled request is only freed by wx_server_release on the caller's thread.
        cudaSetDevice(s->device);
        const size_t npix = (size_t)q->r.width * q->r.height;
        if (rgba8_host && q->rgba && cudaMemcpy(rgba8_host, q->rgba, npix * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return sfail(WX_ERR_CUDA, "wx_server_copy_result: copy failed");
        if (hits_host && q->hits &&
            cudaMemcpy(hits_host, q->hits, npix * sizeof(wx_hit), cudaMemcpyDeviceToHost) != cudaSuccess)
            return sfail(WX_ERR_CUDA, "wx_server_copy_result: copy failed");
        return WX_OK;
    });
}

int wx_server_release(wx_server *s, uint64_t ticket) {
    return wx::guard("wx_server_release", [&]() -> int {
        if (!s) return WX_ERR_INVALID;
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return sfail(WX_ERR_INVALID, "wx_server_release: unknown ticket");
        Req *q = it->second;
        if (q->state != RState::Polled) return sfail(WX_ERR_INVALID, "wx_server_release: result not polled yet");
        if (q->has_buf) s->arena.release(q->off, q->bytes);
        s->reqs.erase(it);
        delete q;
        s->cv_work.notify_one();
        return WX_OK;
    });
}

int wx_server_get_stats(wx_server *s, wx_server_stats *o) {
    return wx::guard("wx_server_get_stats", [&]() -> int {
        if (!s || !o) return WX_ERR_INVALID;
        std::lock_guard<std::mutex> lk(s->mu);
        *o = s->st;
        o->arena_bytes = s->arena.size();
        o->arena_in_use = s->arena.in_use();
        o->arena_peak = s->arena.peak();
        o->pending = s->pending.size();
        o->active = s->active.size();
        return WX_OK;
    });
}

int wx_server_replay(wx_server *s, const wx_request *reqs, const double *arrival_s, uint32_t n, wx_result *results,
                     int release, double timeout_s) {
    return wx::guard("wx_server_replay", [&]() -> int {
        if (!s || (n && (!reqs || !arrival_s || !results))) return sfail(WX_ERR_INVALID, "wx_server_replay: null argument");
        std::unordered_map<uint64_t, uint32_t> index;
        index.reserve(n * 2);
        const double t0 = now_s();
        uint32_t submitted = 0, collected = 0;
        std::vector<wx_result> buf(64);
        auto collect = [&](int wait_ms) {
            uint32_t got = 0;
            wx_server_poll(s, buf.data(), (uint32_t)buf.size(), &got, wait_ms);
            for (uint32_t k = 0; k < got; k++) {
                auto it = index.find(buf[k].ticket);
                if (it == index.end()) continue;  // not ours
                results[it->second] = buf[k];
                collected++;
                if (release) {
                    wx_server_release(s, buf[k].ticket);
                    results[it->second].rgba8 = nullptr;
                    results[it->second].hits = nullptr;
                }
            }
        };
        while (submitted < n) {
            const double due = t0 + arrival_s[submitted];
            for (;;) {
                const double left = due - now_s();
                if (left <= 0) break;
                if (left > 200e-6) {
                    collect(0);
                    std::this_thread::sleep_for(std::chrono::duration<double>(std::min(left - 100e-6, 1e-3)));
                }
            }
            uint64_t ticket = 0;
            const int rc = wx_server_submit(s, &reqs[submitted], &ticket);
            if (rc != WX_OK) return rc;
            index[ticket] = submitted++;
            if (now_s() - t0 > timeout_s) return sfail(WX_ERR_TIMEOUT, "wx_server_replay: timed out while submitting");
        }
        while (collected < n) {
            if (now_s() - t0 > timeout_s) return sfail(WX_ERR_TIMEOUT, "wx_server_replay: timed out waiting for results");
            collect(5);
        }
        return WX_OK;
    });
}

int wx_server_destroy(wx_server *s) {
    return wx::guard("wx_server_destroy", [&]() -> int {
        if (!s) return WX_OK;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            // Unadmitted requests will never run.
            while (!s->pending.empty()) {
                s->finish(s->pending.front(), WX_ERR_CANCELLED);
                s->pending.pop_front();
            }
            s->cv_work.notify_all();
        }
        if (s->th.joinable()) s->th.join();
        cudaSetDevice(s->device);
        for (Slot &sl : s->slots) {
            if (sl.stream) cudaStreamSynchronize(sl.stream);
            if (sl.ev) cudaEventDestroy(sl.ev);
            if (sl.stream) cudaStreamDestroy(sl.stream);
            if (sl.jobs_host) cudaFreeHost(sl.jobs_host);
            if (sl.jobs_dev) cudaFree(sl.jobs_dev);
            if (sl.counter) cudaFree(sl.counter);
            if (sl.skipped_host) cudaFreeHost(sl.skipped_host);
        }
        if (s->ctl) {
            cudaStreamSynchronize(s->ctl);
            cudaStreamDestroy(s->ctl);
        }
        if (s->cancel_dev) cudaFree(s->cancel_dev);
        if (s->cancel_host) cudaFreeHost(s->cancel_host);
        s->arena.destroy();
        for (auto &kv : s->reqs) delete kv.second;
        delete s;
        return WX_OK;
    });
}

}  // extern "C"
