// api.cpp — the C ABI (include/woxel_gb300.h): contexts, grid upload/build,
// per-frame render, batched render (one-shot and CUDA-graph plans), tuning.
//
// Device layout of a grid (uploaded once, immutable afterwards):
//   root   2 x int4          header: {lo.x, lo.y, lo.z, dim.x}, {dim.y, dim.z, 0, use table}
//          n5 x int4         N5 origins (root keys) in DFS order
//          dim.x*dim.y*dim.z u32  dense root-key table over the box of N5 keys
//                            (origin >> 12) starting at lo: N5 index + 1, 0 = none
//   slot5  n5 x 32768 u32    per N4-sized slot: child flag|N4 index, or skip distance
//   slot4  n4 x  4096 u32    per N3-sized slot: child flag|N3 index, or skip distance
//   leaf   n3 x   512 u8     per voxel: 0 for an active voxel (a hit), else the skip
//                            distance, 255 meaning "at least 255: look it up in ovf"
//   ovf    n_ovf x (u32,u32) (voxel key = leaf << 9 | offset, exact distance), sorted
// A slot word folds the reference's three reads per level (child-mask word,
// value-mask word, atlas texel; raycast.comp.wgsl:422-429, :453-461,
// :483-489) into one load that decides hit / descend / skip. Leaf distances
// produced by compute_sdf are small (bounded by the extent of a cluster of
// leaves), so one byte per voxel keeps the leaf pool at a quarter of the
// reference's texel bytes while the overflow table keeps any u32 exact.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "wx_alloc.h"
#include "wx_common.h"
#include "wx_kernels.h"

namespace {
constexpr uint32_t kCounterSlots = 1u << 16;  // one work counter per in-flight launch (ring)
}

struct wx_ctx {
    int device = 0;
    int num_sms = 0;
    std::string err;
    wxk::Tuning tuning;
    uint32_t *counters = nullptr;       // kCounterSlots device counters
    uint32_t next_counter = 0;
    unsigned long long *check = nullptr;  // division self-check results
    void *stage = nullptr;              // device staging for host-memory outputs
    size_t stage_bytes = 0;
    wxk::Job *jobs_dev = nullptr;       // job table of the one-shot batch entry point
    size_t jobs_cap = 0;
    wxk::Job *jobs_host = nullptr;      // pinned staging for that table
    cudaEvent_t jobs_done = nullptr;    // last one-shot batch's table copy
    uint32_t sdf_spins = wxk::kSdfSpinLimit;  // bound of the GPU SDF sweeps' dependency waits
    uint32_t *take_counter() {
        uint32_t *c = counters + next_counter;
        next_counter = (next_counter + 1) % kCounterSlots;
        return c;
    }
};

struct wx_grid {
    int device = 0;
    void *dev = nullptr;
    size_t bytes = 0;
    float *values = nullptr;  // level-set values (zero-crossing mode), own allocation
    wxk::DevGrid g{};
    wx_grid_info info{};
};

struct wx_batch {
    wx_ctx *ctx = nullptr;
    wxk::Job *jobs_dev = nullptr;
    uint32_t njobs = 0, total_tiles = 0;
    uint64_t rays = 0;
    uint32_t *counter = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace wx {
// Injected allocation failures (wx_inject_alloc_failures), taken one per allocation.
static std::atomic<uint32_t> g_alloc_failures{0};
bool take_injected_alloc_failure() {
    uint32_t n = g_alloc_failures.load(std::memory_order_relaxed);
    while (n != 0 && !g_alloc_failures.compare_exchange_weak(n, n - 1, std::memory_order_relaxed)) {
    }
    return n != 0;
}
}  // namespace wx

namespace {

int fail(wx_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    wx::set_thread_error(msg);
    return code;
}
int cuda_fail(wx_ctx *ctx, cudaError_t e, const char *what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? WX_ERR_OOM : WX_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define WX_CUDA(ctx, call)                                       \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// Output byte ranges [lo, hi) (rgba8, hit records) of the last k_pixel launched
// on each (device, stream). A k_pixel launch's predecessor on its stream is
// either the k_pixel recorded here (the only kernel of this library that lets
// its dependents start early) or work after which nothing overlaps; k_pixel
// itself keeps frames older than the predecessor finished (kernels.cu). So a
// frame whose outputs are disjoint from the record's need not wait before its
// stores. A stream without a record counts as overlapping.
struct PixelOutputs {
    int device;
    cudaStream_t stream;
    uintptr_t lo[2], hi[2];
};
constexpr size_t kPixelStreams = 256;  // records kept, oldest dropped first
std::mutex g_pixel_mu;
std::vector<PixelOutputs> g_pixel_outputs;

// Launches k_pixel for cur's outputs and records cur as its stream's last
// k_pixel, both under g_pixel_mu, so a stream's record always names the k_pixel
// enqueued on it last even when several host threads launch on one stream. The
// frame stores without waiting when its outputs are disjoint from the record's.
// cudaStreamPerThread is one handle for a different stream in every host thread,
// so no record can name its predecessor: frames on it always wait. NULL and
// cudaStreamLegacy name the same stream.
cudaError_t launch_pixel_tracked(const wxk::Job &job, const wxk::Tuning &t, PixelOutputs cur) {
    if (cur.stream == cudaStreamPerThread) return wxk::launch_pixel(job, t, false, cur.stream);
    if (cur.stream == cudaStreamLegacy) cur.stream = nullptr;
    auto meet = [](uintptr_t a0, uintptr_t a1, uintptr_t b0, uintptr_t b1) {
        return a0 < a1 && b0 < b1 && a0 < b1 && b0 < a1;
    };
    std::lock_guard<std::mutex> lock(g_pixel_mu);
    auto &v = g_pixel_outputs;
    bool disjoint = false;
    size_t i = 0;
    while (i < v.size() && !(v[i].device == cur.device && v[i].stream == cur.stream)) i++;
    if (i < v.size()) {
        disjoint = true;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                if (meet(cur.lo[a], cur.hi[a], v[i].lo[b], v[i].hi[b])) disjoint = false;
        v.erase(v.begin() + (long)i);
    } else if (v.size() >= kPixelStreams) {
        v.erase(v.begin());
    }
    const cudaError_t e = wxk::launch_pixel(job, t, disjoint, cur.stream);
    if (e == cudaSuccess) v.push_back(cur);  // after a failed launch the stream's last kernel is unknown
    return e;
}

bool device_accessible(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The device-side address of page-locked host memory (cudaMallocHost,
// cudaHostAlloc, cudaHostRegister), through which a kernel writes to the host
// buffer directly; nullptr for pageable memory.
void *pinned_device_alias(void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// A device allocation freed on scope exit (temporaries of wx_grid_build_gpu).
struct DevBuf {
    void *p = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

template <class F>
void parallel_chunks(size_t n, F f) {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 4096 || nt == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    const size_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        const size_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo < hi) th.emplace_back([=] { f(lo, hi); });
    }
    for (auto &x : th) x.join();
}

// The root block: header, origins and the dense table of root keys, which
// replaces the linear scan of get_vdb_leaf_from_nothing
// (raycast.comp.wgsl:398-413) with one load. The scan compares
// floor(p) & ~4095 with each origin, so only origins that are multiples of
// 4096 can match; the table holds those, the first of equal origins winning as
// in the scan. Boxes of more than 2^20 keys keep the scan (use table = 0).
std::vector<int4> root_block(const std::vector<int4> &o5, uint64_t n5) {
    constexpr uint64_t kMaxKeys = 1u << 20;
    int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};
    bool any = false;
    for (uint64_t i = 0; i < n5; i++) {
        const int v[3] = {o5[i].x, o5[i].y, o5[i].z};
        if ((v[0] & 4095) || (v[1] & 4095) || (v[2] & 4095)) continue;
        for (int a = 0; a < 3; a++) {
            const int k = v[a] >> 12;
            lo[a] = any ? std::min(lo[a], k) : k;
            hi[a] = any ? std::max(hi[a], k) : k;
        }
        any = true;
    }
    uint64_t dim[3], keys = 1;
    for (int a = 0; a < 3; a++) {
        dim[a] = any ? (uint64_t)((int64_t)hi[a] - lo[a] + 1) : 0;
        keys *= dim[a];
    }
    const bool use = keys <= kMaxKeys;
    const uint64_t tab = use ? keys : 0;
    std::vector<int4> b(2 + n5 + (tab + 3) / 4, make_int4(0, 0, 0, 0));
    b[0] = make_int4(lo[0], lo[1], lo[2], (int)(use ? dim[0] : 0));
    b[1] = make_int4((int)(use ? dim[1] : 0), (int)(use ? dim[2] : 0), 0, use ? 1 : 0);
    for (uint64_t i = 0; i < n5; i++) b[2 + i] = o5[i];
    auto *t = reinterpret_cast<uint32_t *>(b.data() + 2 + n5);
    for (uint64_t i = 0; use && i < n5; i++) {
        const int v[3] = {o5[i].x, o5[i].y, o5[i].z};
        if ((v[0] & 4095) || (v[1] & 4095) || (v[2] & 4095)) continue;
        const uint64_t e = ((uint64_t)((v[2] >> 12) - lo[2]) * dim[1] + (uint64_t)((v[1] >> 12) - lo[1])) * dim[0] +
                           (uint64_t)((v[0] >> 12) - lo[0]);
        if (!t[e]) t[e] = (uint32_t)i + 1u;
    }
    return b;
}

// The kernels address each pool with a 32-bit element index (node << log2 slots | slot).
int check_pool_limits(wx_ctx *ctx, uint64_t n5, uint64_t n4, uint64_t n3) {
    if (n5 > (1u << 17) || n4 > (1u << 20) || n3 > (1u << 23))
        return fail(ctx, WX_ERR_UNSUPPORTED,
                    "grid too large: at most 131072 N5, 1048576 N4 and 8388608 N3 nodes");
    return WX_OK;
}

// One device block for all pools of a grid (layout at the top of this file);
// the root block is copied in, the other pools are left for the caller.
int alloc_grid(wx_ctx *ctx, const std::vector<int4> &o5, uint64_t n5, uint64_t n4, uint64_t n3, uint64_t n_ovf,
               wx_grid **out) {
    auto *gr = new (std::nothrow) wx_grid();
    if (!gr) return fail(ctx, WX_ERR_OOM, "host allocation failed");
    std::vector<int4> root;
    try {
        root = root_block(o5, n5);
    } catch (...) {
        delete gr;
        return fail(ctx, WX_ERR_OOM, "host allocation failed");
    }
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_o5 = align(root.size() * 16), b5 = align(n5 * 32768ull * 4),
                 b4 = align(n4 * 4096ull * 4), b3 = align(n3 * 512ull), bo = align(n_ovf * 8);
    gr->bytes = b_o5 + b5 + b4 + b3 + bo;
    gr->device = ctx->device;
    cudaError_t e = wx::dev_alloc(&gr->dev, gr->bytes);
    if (e != cudaSuccess) {
        delete gr;
        return cuda_fail(ctx, e, "cudaMalloc(node pools)");
    }
    char *b = static_cast<char *>(gr->dev);
    gr->g.root = reinterpret_cast<const int4 *>(b);
    gr->g.slot5 = reinterpret_cast<const uint32_t *>(b + b_o5);
    gr->g.slot4 = reinterpret_cast<const uint32_t *>(b + b_o5 + b5);
    gr->g.leaf = reinterpret_cast<const uint8_t *>(b + b_o5 + b5 + b4);
    gr->g.ovf = reinterpret_cast<const uint2 *>(b + b_o5 + b5 + b4 + b3);
    gr->g.n5 = (uint32_t)n5;
    gr->g.n4 = (uint32_t)n4;
    gr->g.n3 = (uint32_t)n3;
    gr->g.n_ovf = (uint32_t)n_ovf;
    gr->g.inside = 1u;
    for (uint64_t i = 0; i < n5; i++)
        for (int c : {o5[i].x, o5[i].y, o5[i].z})
            if (c != -4096 && c != 0) gr->g.inside = 0u;
    gr->info.n5 = n5;
    gr->info.n4 = n4;
    gr->info.n3 = n3;
    gr->info.device_bytes = gr->bytes;
    e = cudaMemcpy((void *)gr->g.root, root.data(), root.size() * 16, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(gr->dev);
        delete gr;
        return cuda_fail(ctx, e, "cudaMemcpy(root block)");
    }
    *out = gr;
    return WX_OK;
}

void free_grid(wx_grid *gr) {
    if (!gr) return;
    cudaFree(gr->dev);
    if (gr->values) cudaFree(gr->values);
    delete gr;
}

// Pack the per-voxel u32 leaf distances into bytes plus the overflow table,
// allocate one device block for all pools and upload them.
int upload_pools(wx_ctx *ctx, const std::vector<int4> &o5, const uint32_t *s5, const uint32_t *s4, const uint32_t *s3,
                 uint64_t n5, uint64_t n4, uint64_t n3, wx_grid **out) {
    int rc = check_pool_limits(ctx, n5, n4, n3);
    if (rc != WX_OK) return rc;
    std::vector<uint8_t> leaf;
    std::vector<uint2> ovf;
    try {
        leaf.resize(n3 * wx::kN3Slots);
        const unsigned np = n3 < 4096 ? 1u : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::vector<uint2>> parts(np);
        const size_t chunk = (n3 + np - 1) / np;
        auto pack = [&](unsigned p) {
            for (size_t k = p * chunk; k < std::min<size_t>(n3, (p + 1) * chunk); k++)
                for (uint32_t s = 0; s < wx::kN3Slots; s++) {
                    const uint32_t d = s3[k * wx::kN3Slots + s];
                    leaf[k * wx::kN3Slots + s] = (uint8_t)std::min<uint32_t>(d, 255u);
                    if (d >= 255u) parts[p].push_back(make_uint2((uint32_t)(k << 9) | s, d));
                }
        };
        std::vector<std::thread> th;
        for (unsigned p = 1; p < np; p++) th.emplace_back(pack, p);
        pack(0);
        for (auto &t : th) t.join();
        for (auto &p : parts) ovf.insert(ovf.end(), p.begin(), p.end());  // ascending keys
    } catch (...) {
        return fail(ctx, WX_ERR_OOM, "host allocation failed while packing leaves");
    }
    wx_grid *gr = nullptr;
    if ((rc = alloc_grid(ctx, o5, n5, n4, n3, ovf.size(), &gr)) != WX_OK) return rc;
    cudaError_t e = cudaSuccess;
    if (n5) e = cudaMemcpy((void *)gr->g.slot5, s5, n5 * 32768ull * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n4) e = cudaMemcpy((void *)gr->g.slot4, s4, n4 * 4096ull * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n3) e = cudaMemcpy((void *)gr->g.leaf, leaf.data(), leaf.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !ovf.empty())
        e = cudaMemcpy((void *)gr->g.ovf, ovf.data(), ovf.size() * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_grid(gr);
        return cuda_fail(ctx, e, "cudaMemcpy(node pools)");
    }
    *out = gr;
    return WX_OK;
}

// Tiles of tile_w x (32 / tile_w) pixels over the dispatched region
// 8*floor(w/8) x 4*floor(h/4) (wgpu_context.rs:281).
wxk::Job make_job(const wx_grid *grid, const wx_state_uniform &s, uint32_t width, uint32_t height, uint32_t *rgba,
                  wx_hit *hits, uint32_t tile_begin, const wxk::Tuning &t) {
    wxk::Job j;
    memset(&j, 0, sizeof j);
    j.g = grid->g;
    j.width = width;
    j.height = height;
    j.tile_w = (uint16_t)t.tile_w;
    j.order = (uint32_t)t.order;
    j.tile_h = (uint16_t)(32u / j.tile_w);
    const uint32_t wd = width & ~7u, hd = height & ~3u;
    j.tiles_x = (wd + j.tile_w - 1) / j.tile_w;
    j.tiles = j.tiles_x * ((hd + j.tile_h - 1) / j.tile_h);
    j.tile_begin = tile_begin;
    j.rgba = rgba;
    j.hits = hits;
    j.s = s;
    return j;
}

}  // namespace

void wxk::ctx_device_info(const wx_ctx *ctx, int *device, int *num_sms) {
    *device = ctx->device;
    *num_sms = ctx->num_sms;
}

bool wxk::grid_device_view(const wx_grid *grid, wxk::DevGrid *out, int *device) {
    if (!grid) return false;
    *out = grid->g;
    *device = grid->device;
    return true;
}

extern "C" {

const char *wx_status_string(int status) {
    switch (status) {
        case WX_OK: return "ok";
        case WX_ERR_INVALID: return "invalid argument";
        case WX_ERR_CUDA: return "CUDA error";
        case WX_ERR_OOM: return "out of memory";
        case WX_ERR_UNSUPPORTED: return "unsupported";
        case WX_ERR_BUDGET: return "over memory budget";
        case WX_ERR_TIMEOUT: return "timed out";
        case WX_ERR_CANCELLED: return "cancelled";
        default: return "unknown status";
    }
}

int wx_ctx_create(int device, wx_ctx **out) {
    return wx::guard("wx_ctx_create", [&]() -> int {
        if (!out) return fail(nullptr, WX_ERR_INVALID, "wx_ctx_create: out is NULL");
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceCount");
        if (device < 0 || device >= n) return fail(nullptr, WX_ERR_INVALID, "wx_ctx_create: no such device");
        WX_CUDA(nullptr, cudaSetDevice(device));
        auto *c = new (std::nothrow) wx_ctx();
        if (!c) return fail(nullptr, WX_ERR_OOM, "host allocation failed");
        c->device = device;
        auto cleanup = [&](cudaError_t err, const char *what) {
            wx_ctx_destroy(c);
            return cuda_fail(nullptr, err, what);
        };
        if ((e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
            return cleanup(e, "cudaDeviceGetAttribute");
        if ((e = wxk::init_device_tables()) != cudaSuccess) return cleanup(e, "init_device_tables");
        if ((e = wx::dev_alloc(&c->counters, kCounterSlots * sizeof(uint32_t))) != cudaSuccess)
            return cleanup(e, "cudaMalloc(counters)");
        if ((e = cudaMemset(c->counters, 0, kCounterSlots * sizeof(uint32_t))) != cudaSuccess)
            return cleanup(e, "cudaMemset(counters)");
        if ((e = wx::dev_alloc(&c->check, 4 * sizeof(unsigned long long))) != cudaSuccess)
            return cleanup(e, "cudaMalloc(check)");
        if ((e = cudaEventCreateWithFlags(&c->jobs_done, cudaEventDisableTiming)) != cudaSuccess)
            return cleanup(e, "cudaEventCreate");
        *out = c;
        return WX_OK;
    });
}

int wx_ctx_destroy(wx_ctx *ctx) {
    return wx::guard("wx_ctx_destroy", [&]() -> int {
        if (!ctx) return WX_OK;
        cudaSetDevice(ctx->device);
        if (ctx->jobs_done) {
            cudaEventSynchronize(ctx->jobs_done);
            cudaEventDestroy(ctx->jobs_done);
        }
        if (ctx->stage) cudaFree(ctx->stage);
        if (ctx->counters) cudaFree(ctx->counters);
        if (ctx->check) cudaFree(ctx->check);
        if (ctx->jobs_dev) cudaFree(ctx->jobs_dev);
        if (ctx->jobs_host) cudaFreeHost(ctx->jobs_host);
        delete ctx;
        return WX_OK;
    });
}

const char *wx_last_error(const wx_ctx *ctx) { return ctx ? ctx->err.c_str() : wx_thread_last_error(); }

int wx_ctx_set_tuning(wx_ctx *ctx, const wx_tuning *t) {
    return wx::guard("wx_ctx_set_tuning", [&]() -> int {
        if (!ctx || !t) return fail(ctx, WX_ERR_INVALID, "wx_ctx_set_tuning: null argument");
        const bool tw_ok = t->tile_width == 4 || t->tile_width == 8 || t->tile_width == 16 || t->tile_width == 32;
        if (t->kernel < 0 || t->kernel > 1 || t->warps_per_block < 1 || t->warps_per_block > 8 || t->blocks_per_sm < 0 ||
            t->blocks_per_sm > 64 || !tw_ok || t->tile_order < 0 || t->tile_order > 1 ||
            !(t->rays_per_lane == 1 || t->rays_per_lane == 2 || t->rays_per_lane == 4 || t->rays_per_lane == 8))
            return fail(ctx, WX_ERR_INVALID, "wx_ctx_set_tuning: value out of range");
        ctx->tuning.kernel = t->kernel;
        ctx->tuning.warps_per_block = t->warps_per_block;
        ctx->tuning.blocks_per_sm = t->blocks_per_sm;
        ctx->tuning.tile_w = t->tile_width;
        ctx->tuning.order = t->tile_order;
        ctx->tuning.rays = t->rays_per_lane;
        return WX_OK;
    });
}

int wx_inject_alloc_failures(uint32_t count) {
    return wx::guard("wx_inject_alloc_failures", [&]() -> int {
        wx::g_alloc_failures.store(count, std::memory_order_relaxed);
        return WX_OK;
    });
}

int wx_ctx_set_sdf_wait_limit(wx_ctx *ctx, uint32_t polls) {
    return wx::guard("wx_ctx_set_sdf_wait_limit", [&]() -> int {
        if (!ctx) return WX_ERR_INVALID;
        ctx->sdf_spins = polls ? polls : wxk::kSdfSpinLimit;
        return WX_OK;
    });
}

int wx_ctx_get_tuning(const wx_ctx *ctx, wx_tuning *t) {
    return wx::guard("wx_ctx_get_tuning", [&]() -> int {
        if (!ctx || !t) return WX_ERR_INVALID;
        t->kernel = ctx->tuning.kernel;
        t->warps_per_block = ctx->tuning.warps_per_block;
        t->blocks_per_sm = ctx->tuning.blocks_per_sm;
        t->tile_width = ctx->tuning.tile_w;
        t->tile_order = ctx->tuning.order;
        t->rays_per_lane = ctx->tuning.rays;
        return WX_OK;
    });
}

int wx_autotune(wx_ctx *ctx, const wx_frame *frames, uint32_t n, const wx_tuning *candidates, uint32_t ncand,
                uint32_t reps, wx_tuning *best, double *times_ms) {
    return wx::guard("wx_autotune", [&]() -> int {
        if (!ctx || !frames || n == 0 || !best) return fail(ctx, WX_ERR_INVALID, "wx_autotune: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        std::vector<wx_tuning> cand;
        if (candidates) {
            cand.assign(candidates, candidates + ncand);
        } else {
            for (int order : {1, 0}) {
                for (int kernel : {0, 1})
                    for (int tw : {4, 8, 16})
                        for (int wpb : {2, 4, 8}) cand.push_back(wx_tuning{kernel, wpb, 0, tw, order, 1});
                // Occupancy of the persistent kernel: fewer resident warps than fit (16 per SM).
                for (int tw : {4, 8}) cand.push_back(wx_tuning{0, 4, 4, tw, order, 1});
                // Rays per lane: warps of several tiles whose lanes refill.
                for (int rays : {2, 4, 8})
                    for (int tw : {4, 8})
                        for (int wpb : {2, 4}) cand.push_back(wx_tuning{1, wpb, 0, tw, order, rays});
            }
            if (cand.size() != WX_AUTOTUNE_BUILTIN) return fail(ctx, WX_ERR_INVALID, "wx_autotune: built-in set size");
        }
        if (cand.empty()) return fail(ctx, WX_ERR_INVALID, "wx_autotune: no candidates");
        for (uint32_t i = 0; i < n; i++)
            if (!frames[i].grid || !frames[i].rgba8 || !device_accessible(frames[i].rgba8))
                return fail(ctx, WX_ERR_INVALID, "wx_autotune: frames need a grid and device rgba8");
        const wxk::Tuning saved = ctx->tuning;
        cudaEvent_t e0, e1;
        WX_CUDA(ctx, cudaEventCreate(&e0));
        WX_CUDA(ctx, cudaEventCreate(&e1));
        cudaStream_t st;
        WX_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        double best_ms = 1e300;
        size_t best_i = 0;
        int rc = WX_OK;
        for (size_t c = 0; c < cand.size() && rc == WX_OK; c++) {
            rc = wx_ctx_set_tuning(ctx, &cand[c]);
            if (rc != WX_OK) break;
            double total = 0;
            for (uint32_t rep = 0; rep <= reps && rc == WX_OK; rep++) {  // pass 0 warms up
                cudaEventRecord(e0, st);
                for (uint32_t i = 0; i < n && rc == WX_OK; i++)
                    rc = wx_render(ctx, frames[i].grid, &frames[i].state, frames[i].width, frames[i].height,
                                   frames[i].rgba8, frames[i].hits, st);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) total += ms;
            }
            const double mean = total / (reps ? reps : 1);
            if (times_ms) times_ms[c] = mean;
            if (rc == WX_OK && mean < best_ms) {
                best_ms = mean;
                best_i = c;
            }
        }
        cudaStreamDestroy(st);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != WX_OK) {
            ctx->tuning = saved;
            return rc;
        }
        *best = cand[best_i];
        return wx_ctx_set_tuning(ctx, best);
    });
}

int wx_check_division(wx_ctx *ctx, uint32_t max_m, uint64_t out[3]) {
    return wx::guard("wx_check_division", [&]() -> int {
        if (!ctx || !out) return fail(ctx, WX_ERR_INVALID, "wx_check_division: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        WX_CUDA(ctx, wxk::check_division(max_m, ctx->check, nullptr));
        unsigned long long h[3];
        WX_CUDA(ctx, cudaMemcpy(h, ctx->check, sizeof h, cudaMemcpyDeviceToHost));
        for (int i = 0; i < 3; i++) out[i] = h[i];
        return WX_OK;
    });
}

int wx_bounds_violations(wx_ctx *ctx, uint64_t *count) {
    return wx::guard("wx_bounds_violations", [&]() -> int {
        if (!ctx || !count) return fail(ctx, WX_ERR_INVALID, "wx_bounds_violations: null argument");
    #ifdef WX_BOUNDS_CHECK
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        WX_CUDA(ctx, cudaDeviceSynchronize());
        unsigned long long n = 0;
        WX_CUDA(ctx, wxk::take_bounds_violations(&n));
        *count = n;
        return WX_OK;
    #else
        *count = 0;
        return fail(ctx, WX_ERR_UNSUPPORTED, "wx_bounds_violations: not a bounds-checked build");
    #endif
    });
}

int wx_grid_build(wx_ctx *ctx, wx_topology *t, wx_grid **out) {
    return wx::guard("wx_grid_build", [&]() -> int {
        if (!ctx || !t || !out) return fail(ctx, WX_ERR_INVALID, "wx_grid_build: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        int rc = wx_topology_sdf(t, 0);
        if (rc != WX_OK) return fail(ctx, rc, wx_thread_last_error());
        const uint64_t n5 = t->n5(), n4 = t->n4(), n3 = t->n3();
        if (n4 >= wx::kChildFlag || n3 >= wx::kChildFlag)
            return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_build: more than 2^31 nodes in a level");
        std::vector<uint32_t> s5, s4;
        std::vector<int4> o5(std::max<uint64_t>(n5, 1));
        try {
            s5.resize(n5 * wx::kN5Slots);
            s4.resize(n4 * wx::kN4Slots);
        } catch (...) {
            return fail(ctx, WX_ERR_OOM, "wx_grid_build: host allocation failed");
        }
        bool too_far = false;
        for (uint64_t i = 0; i < n5; i++) {
            o5[i] = make_int4(t->o5[i][0], t->o5[i][1], t->o5[i][2], 0);
            uint32_t next = t->first4[i];
            for (uint32_t s = 0; s < wx::kN5Slots; s++) {
                const bool kid = wx::test_bit(&t->kid5[i * wx::kN5Words], s);
                const bool val = wx::test_bit(&t->val5[i * wx::kN5Words], s);
                const uint32_t d = t->d5[i * wx::kN5Slots + s];
                if (kid) {
                    const uint32_t c = next++;
                    s5[i * wx::kN5Slots + s] = val ? 0u : (wx::kChildFlag | c);
                } else {
                    too_far |= !val && d >= wx::kChildFlag;
                    s5[i * wx::kN5Slots + s] = val ? 0u : d;
                }
            }
        }
        for (uint64_t j = 0; j < n4; j++) {
            uint32_t next = t->first3[j];
            for (uint32_t s = 0; s < wx::kN4Slots; s++) {
                const bool kid = wx::test_bit(&t->kid4[j * wx::kN4Words], s);
                const bool val = wx::test_bit(&t->val4[j * wx::kN4Words], s);
                const uint32_t d = t->d4[j * wx::kN4Slots + s];
                if (kid) {
                    const uint32_t c = next++;
                    s4[j * wx::kN4Slots + s] = val ? 0u : (wx::kChildFlag | c);
                } else {
                    too_far |= !val && d >= wx::kChildFlag;
                    s4[j * wx::kN4Slots + s] = val ? 0u : d;
                }
            }
        }
        if (too_far) return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_build: tile distance >= 2^31");
        wx_grid *gr = nullptr;
        rc = upload_pools(ctx, o5, s5.data(), s4.data(), t->slot3.data(), n5, n4, n3, &gr);
        if (rc != WX_OK) return rc;
        gr->info.active_voxels = wx_topology_active_voxels(t);
        *out = gr;
        return WX_OK;
    });
}

// The same pools as wx_grid_build, with compute_sdf and the packing on the
// GPU (sdf.cu). The host uploads only the masks, the N5 origins and per-word
// child-count prefixes; child tables, child origins, neighbour tables, the
// three sweeps and the packing run on the device.
int wx_grid_build_gpu(wx_ctx *ctx, const wx_topology *t, wx_grid **out) {
    return wx::guard("wx_grid_build_gpu", [&]() -> int {
        if (!ctx || !t || !out) return fail(ctx, WX_ERR_INVALID, "wx_grid_build_gpu: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        using namespace wx;
        const uint64_t n5 = t->n5(), n4 = t->n4(), n3 = t->n3();
        int rc = check_pool_limits(ctx, n5, n4, n3);
        if (rc != WX_OK) return rc;
        if (t->kid5.size() != n5 * kN5Words || t->val5.size() != n5 * kN5Words || t->kid4.size() != n4 * kN4Words ||
            t->val4.size() != n4 * kN4Words || t->val3.size() != n3 * kN3Words || t->first4.size() != n5 ||
            t->first3.size() != n4)
            return fail(ctx, WX_ERR_INVALID, "wx_grid_build_gpu: masks and node counts disagree");
        std::vector<int4> o5(std::max<uint64_t>(n5, 1));
        std::vector<uint32_t> pre5, pre4;
        try {
            pre5.resize(n5 * kN5Words);
            pre4.resize(n4 * kN4Words);
        } catch (...) {
            return fail(ctx, WX_ERR_OOM, "wx_grid_build_gpu: host allocation failed");
        }
        for (uint64_t i = 0; i < n5; i++) {
            o5[i] = make_int4(t->o5[i][0], t->o5[i][1], t->o5[i][2], 0);
            if ((o5[i].x & 4095) || (o5[i].y & 4095) || (o5[i].z & 4095))
                return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_build_gpu: N5 origins must be multiples of 4096");
        }
        auto prefix = [](const std::vector<uint64_t> &kid, uint64_t nodes, uint32_t words, std::vector<uint32_t> &pre) {
            for (uint64_t n = 0; n < nodes; n++) {
                uint32_t acc = 0;
                for (uint32_t w = 0; w < words; w++) {
                    pre[n * words + w] = acc;
                    acc += (uint32_t)__builtin_popcountll(kid[n * words + w]);
                }
            }
        };
        prefix(t->kid5, n5, kN5Words, pre5);
        prefix(t->kid4, n4, kN4Words, pre4);
        std::vector<int4> root;
        try {
            root = root_block(o5, n5);
        } catch (...) {
            return fail(ctx, WX_ERR_OOM, "wx_grid_build_gpu: host allocation failed");
        }

        const uint64_t nmax = std::max<uint64_t>({n5, n4, n3, 1});
        DevBuf kid5, val5, kid4, val4, val3, dpre5, dpre4, first4, first3, droot, c5, c4, org5, org4, org3, d5, d4, d3,
            nb, indeg, queue, ctr;
        struct Alloc {
            DevBuf *b;
            size_t bytes;
        } allocs[] = {{&kid5, n5 * kN5Words * 8},  {&val5, n5 * kN5Words * 8}, {&kid4, n4 * kN4Words * 8},
                      {&val4, n4 * kN4Words * 8},  {&val3, n3 * kN3Words * 8}, {&dpre5, n5 * kN5Words * 4},
                      {&dpre4, n4 * kN4Words * 4}, {&first4, n5 * 4},          {&first3, n4 * 4},
                      {&droot, root.size() * 16},  {&c5, n5 * kN5Slots * 4},   {&c4, n4 * kN4Slots * 4},
                      {&org5, n5 * 16},            {&org4, n4 * 16},           {&org3, n3 * 16},
                      {&d5, n5 * kN5Slots * 4},    {&d4, n4 * kN4Slots * 4},   {&d3, n3 * kN3Slots * 4},
                      {&nb, nmax * 27 * 4},        {&indeg, nmax * 4},         {&queue, nmax * 4},
                      {&ctr, 8 * 4}};
        for (auto &a : allocs)
            if (a.bytes) WX_CUDA(ctx, wx::dev_alloc(&a.b->p, a.bytes));
        struct Up {
            DevBuf *b;
            const void *src;
            size_t bytes;
        } ups[] = {{&kid5, t->kid5.data(), n5 * kN5Words * 8}, {&val5, t->val5.data(), n5 * kN5Words * 8},
                   {&kid4, t->kid4.data(), n4 * kN4Words * 8}, {&val4, t->val4.data(), n4 * kN4Words * 8},
                   {&val3, t->val3.data(), n3 * kN3Words * 8}, {&dpre5, pre5.data(), n5 * kN5Words * 4},
                   {&dpre4, pre4.data(), n4 * kN4Words * 4},   {&first4, t->first4.data(), n5 * 4},
                   {&first3, t->first3.data(), n4 * 4},        {&droot, root.data(), root.size() * 16},
                   {&org5, o5.data(), n5 * 16}};
        for (auto &u : ups)
            if (u.bytes) WX_CUDA(ctx, cudaMemcpy(u.b->p, u.src, u.bytes, cudaMemcpyHostToDevice));
        const cudaStream_t st = nullptr;
        WX_CUDA(ctx, cudaMemsetAsync(ctr.p, 0, 8 * 4, st));
        WX_CUDA(ctx, wxk::sdf_child_table(kid5.as<uint64_t>(), dpre5.as<uint32_t>(), first4.as<uint32_t>(), n5, 15,
                                          c5.as<uint32_t>(), st));
        WX_CUDA(ctx, wxk::sdf_child_table(kid4.as<uint64_t>(), dpre4.as<uint32_t>(), first3.as<uint32_t>(), n4, 12,
                                          c4.as<uint32_t>(), st));
        WX_CUDA(ctx, wxk::sdf_child_origins(c5.as<uint32_t>(), org5.as<int4>(), n5, 5, 7, org4.as<int4>(), st));
        WX_CUDA(ctx, wxk::sdf_child_origins(c4.as<uint32_t>(), org4.as<int4>(), n4, 4, 3, org3.as<int4>(), st));
        WX_CUDA(ctx, wxk::sdf_init(kid5.as<uint64_t>(), n5 * kN5Slots, d5.as<uint32_t>(), st));
        WX_CUDA(ctx, wxk::sdf_init(kid4.as<uint64_t>(), n4 * kN4Slots, d4.as<uint32_t>(), st));
        WX_CUDA(ctx, wxk::sdf_init(val3.as<uint64_t>(), n3 * kN3Slots, d3.as<uint32_t>(), st));
        const wxk::SdfTree tree{droot.as<int4>(), (uint32_t)n5, c5.as<uint32_t>(), c4.as<uint32_t>()};
        struct Level {
            int L;
            DevBuf *org, *d;
            uint64_t nc;
        } levels[] = {{5, &org5, &d5, n5}, {4, &org4, &d4, n4}, {3, &org3, &d3, n3}};
        for (auto &lv : levels) {
            WX_CUDA(ctx, wxk::sdf_neighbours(lv.L, lv.org->as<int4>(), (uint32_t)lv.nc, tree, nb.as<uint32_t>(), st));
            WX_CUDA(ctx, wxk::sdf_sweep(lv.L, lv.d->as<uint32_t>(), nb.as<uint32_t>(), (uint32_t)lv.nc,
                                        indeg.as<uint32_t>(), queue.as<uint32_t>(), ctr.as<uint32_t>(), ctx->num_sms,
                                        ctx->sdf_spins, st));
        }
        // Count the leaf overflow entries (ctr[3]) to size the grid block.
        uint32_t *flags = ctr.as<uint32_t>();
        WX_CUDA(ctx, wxk::sdf_pack_leaves(d3.as<uint32_t>(), n3 * kN3Slots, nullptr, nullptr, 0, flags + 3, st));
        uint32_t h[8];
        WX_CUDA(ctx, cudaMemcpy(h, flags, sizeof h, cudaMemcpyDeviceToHost));
        if (h[2]) return fail(ctx, WX_ERR_TIMEOUT, "wx_grid_build_gpu: a sweep's dependency wait hit its bound");
        const uint64_t n_ovf = h[3];
        wx_grid *gr = nullptr;
        if ((rc = alloc_grid(ctx, o5, n5, n4, n3, n_ovf, &gr)) != WX_OK) return rc;
        cudaError_t e = cudaMemsetAsync(flags + 3, 0, 2 * 4, st);  // ctr[3] overflow count, ctr[4] distance error
        if (e == cudaSuccess)
            e = wxk::sdf_pack_internal(kid5.as<uint64_t>(), val5.as<uint64_t>(), c5.as<uint32_t>(), d5.as<uint32_t>(),
                                       n5 * kN5Slots, const_cast<uint32_t *>(gr->g.slot5), flags + 4, st);
        if (e == cudaSuccess)
            e = wxk::sdf_pack_internal(kid4.as<uint64_t>(), val4.as<uint64_t>(), c4.as<uint32_t>(), d4.as<uint32_t>(),
                                       n4 * kN4Slots, const_cast<uint32_t *>(gr->g.slot4), flags + 4, st);
        if (e == cudaSuccess)
            e = wxk::sdf_pack_leaves(d3.as<uint32_t>(), n3 * kN3Slots, const_cast<uint8_t *>(gr->g.leaf),
                                     const_cast<uint2 *>(gr->g.ovf), (uint32_t)n_ovf, flags + 3, st);
        if (e == cudaSuccess) e = cudaMemcpy(h, flags, sizeof h, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            free_grid(gr);
            return cuda_fail(ctx, e, "wx_grid_build_gpu: packing");
        }
        if (h[4]) {
            free_grid(gr);
            return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_build_gpu: tile distance >= 2^31");
        }
        if (n_ovf) {  // entries arrive in any order; the kernels binary-search them by key
            std::vector<uint2> ov(n_ovf);
            e = cudaMemcpy(ov.data(), gr->g.ovf, n_ovf * 8, cudaMemcpyDeviceToHost);
            std::sort(ov.begin(), ov.end(), [](const uint2 &a, const uint2 &b) { return a.x < b.x; });
            if (e == cudaSuccess) e = cudaMemcpy((void *)gr->g.ovf, ov.data(), n_ovf * 8, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                free_grid(gr);
                return cuda_fail(ctx, e, "wx_grid_build_gpu: overflow table");
            }
        }
        gr->info.active_voxels = wx_topology_active_voxels(t);
        *out = gr;
        return WX_OK;
    });
}

int wx_grid_read_pools(wx_ctx *ctx, const wx_grid *grid, uint32_t *slot5, uint32_t *slot4, uint8_t *leaf,
                       uint32_t *ovf, uint64_t *n_ovf) {
    return wx::guard("wx_grid_read_pools", [&]() -> int {
        if (!ctx || !grid) return fail(ctx, WX_ERR_INVALID, "wx_grid_read_pools: null argument");
        WX_CUDA(ctx, cudaSetDevice(grid->device));
        if (n_ovf) *n_ovf = grid->g.n_ovf;
        const uint64_t n5 = grid->info.n5, n4 = grid->info.n4, n3 = grid->info.n3;
        if (slot5 && n5) WX_CUDA(ctx, cudaMemcpy(slot5, grid->g.slot5, n5 * wx::kN5Slots * 4, cudaMemcpyDeviceToHost));
        if (slot4 && n4) WX_CUDA(ctx, cudaMemcpy(slot4, grid->g.slot4, n4 * wx::kN4Slots * 4, cudaMemcpyDeviceToHost));
        if (leaf && n3) WX_CUDA(ctx, cudaMemcpy(leaf, grid->g.leaf, n3 * wx::kN3Slots, cudaMemcpyDeviceToHost));
        if (ovf && grid->g.n_ovf)
            WX_CUDA(ctx, cudaMemcpy(ovf, grid->g.ovf, (size_t)grid->g.n_ovf * 8, cudaMemcpyDeviceToHost));
        return WX_OK;
    });
}

int wx_grid_upload(wx_ctx *ctx, const wx_vdb345_view *v, wx_grid **out) {
    return wx::guard("wx_grid_upload", [&]() -> int {
        if (!ctx || !v || !out) return fail(ctx, WX_ERR_INVALID, "wx_grid_upload: null argument");
        if (v->origin_stride < 3) return fail(ctx, WX_ERR_INVALID, "wx_grid_upload: origin_stride < 3");
        const uint64_t n5 = v->n5, n4 = v->n4, n3 = v->n3;
        if ((n5 && (!v->kids5 || !v->vals5 || !v->origins || !v->atlas[0])) ||
            (n4 && (!v->kids4 || !v->vals4 || !v->atlas[1])) || (n3 && (!v->vals3 || !v->atlas[2])))
            return fail(ctx, WX_ERR_INVALID, "wx_grid_upload: missing mask/atlas arrays");
        if (n4 >= wx::kChildFlag || n3 >= wx::kChildFlag || n5 >= wx::kChildFlag)
            return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_upload: more than 2^31 nodes in a level");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        // Atlas block placement as the shader computes it: dim = textureDimensions
        // (.y for N5, .x for N4/N3) >> log2(node dim); block (idx%d, (idx/d)%d, idx/d^2).
        const uint32_t d5 = v->dims[0][1] >> 5, d4 = v->dims[1][0] >> 4, d3 = v->dims[2][0] >> 3;
        auto block_ok = [&](int lvl, uint64_t n, uint32_t d, uint32_t nd) {
            if (n == 0) return true;
            if (d == 0) return false;
            const uint64_t dd = (uint64_t)d * d;
            const uint64_t need_x = nd * std::min<uint64_t>(n, d), need_y = nd * std::min<uint64_t>((n + d - 1) / d, d),
                           need_z = nd * ((n + dd - 1) / dd);
            return need_x <= v->dims[lvl][0] && need_y <= v->dims[lvl][1] && need_z <= v->dims[lvl][2];
        };
        if (!block_ok(0, n5, d5, 32) || !block_ok(1, n4, d4, 16) || !block_ok(2, n3, d3, 8))
            return fail(ctx, WX_ERR_INVALID, "wx_grid_upload: atlas dimensions too small for the node counts");
        auto texel = [&](int lvl, uint64_t idx, uint32_t d, uint32_t nd, uint32_t cx, uint32_t cy, uint32_t cz) {
            const uint64_t x = nd * (idx % d) + cx, y = nd * ((idx / d) % d) + cy, z = nd * (idx / ((uint64_t)d * d)) + cz;
            return v->atlas[lvl][(z * v->dims[lvl][1] + y) * v->dims[lvl][0] + x];
        };
        std::vector<uint32_t> s5, s4, s3;
        std::vector<int4> o5(std::max<uint64_t>(n5, 1));
        try {
            s5.resize(n5 * wx::kN5Slots);
            s4.resize(n4 * wx::kN4Slots);
            s3.resize(n3 * wx::kN3Slots);
        } catch (...) {
            return fail(ctx, WX_ERR_OOM, "wx_grid_upload: host allocation failed");
        }
        std::atomic<int> bad{0};
        for (uint64_t i = 0; i < n5; i++) {
            const int32_t *o = v->origins + i * v->origin_stride;
            o5[i] = make_int4(o[0], o[1], o[2], 0);
        }
        parallel_chunks(n5, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++)
                for (uint32_t s = 0; s < wx::kN5Slots; s++) {
                    const uint32_t w = s >> 5, b = 1u << (s & 31);
                    const bool kid = v->kids5[i * 1024 + w] & b, val = v->vals5[i * 1024 + w] & b;
                    uint32_t c[3];
                    wx::offset_child(s, 5, c);
                    const uint32_t tx = texel(0, i, d5, 32, c[0], c[1], c[2]);
                    uint32_t word;
                    if (val) word = 0;
                    else if (kid) { word = wx::kChildFlag | tx; if (tx >= n4) bad = 1; }
                    else { word = tx; if (tx >= wx::kChildFlag) bad = 2; }
                    s5[i * wx::kN5Slots + s] = word;
                }
        });
        parallel_chunks(n4, [&](size_t lo, size_t hi) {
            for (size_t j = lo; j < hi; j++)
                for (uint32_t s = 0; s < wx::kN4Slots; s++) {
                    const uint32_t w = s >> 5, b = 1u << (s & 31);
                    const bool kid = v->kids4[j * 128 + w] & b, val = v->vals4[j * 128 + w] & b;
                    uint32_t c[3];
                    wx::offset_child(s, 4, c);
                    const uint32_t tx = texel(1, j, d4, 16, c[0], c[1], c[2]);
                    uint32_t word;
                    if (val) word = 0;
                    else if (kid) { word = wx::kChildFlag | tx; if (tx >= n3) bad = 1; }
                    else { word = tx; if (tx >= wx::kChildFlag) bad = 2; }
                    s4[j * wx::kN4Slots + s] = word;
                }
        });
        parallel_chunks(n3, [&](size_t lo, size_t hi) {
            for (size_t k = lo; k < hi; k++)
                for (uint32_t s = 0; s < wx::kN3Slots; s++) {
                    const bool val = v->vals3[k * 16 + (s >> 5)] & (1u << (s & 31));
                    uint32_t c[3];
                    wx::offset_child(s, 3, c);
                    s3[k * wx::kN3Slots + s] = val ? 0u : texel(2, k, d3, 8, c[0], c[1], c[2]);
                }
        });
        if (bad == 1) return fail(ctx, WX_ERR_INVALID, "wx_grid_upload: child index in atlas out of range");
        if (bad == 2) return fail(ctx, WX_ERR_UNSUPPORTED, "wx_grid_upload: internal tile distance >= 2^31");
        wx_grid *gr = nullptr;
        int rc = upload_pools(ctx, o5, s5.data(), s4.data(), s3.data(), n5, n4, n3, &gr);
        if (rc != WX_OK) return rc;
        uint64_t act = 0;
        for (uint64_t w = 0; w < n3 * 16; w++) act += (uint64_t)__builtin_popcount(v->vals3[w]);
        gr->info.active_voxels = act;
        *out = gr;
        return WX_OK;
    });
}

int wx_grid_release(wx_ctx *ctx, wx_grid *grid) {
    return wx::guard("wx_grid_release", [&]() -> int {
        if (!grid) return WX_OK;
        cudaSetDevice(grid->device);
        cudaError_t e = cudaFree(grid->dev);
        if (grid->values) {
            const cudaError_t e2 = cudaFree(grid->values);
            if (e == cudaSuccess) e = e2;
        }
        delete grid;
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFree(node pools)");
        return WX_OK;
    });
}

int wx_grid_set_values(wx_ctx *ctx, wx_grid *grid, const float *values, float band) {
    return wx::guard("wx_grid_set_values", [&]() -> int {
        if (!ctx || !grid || !values) return fail(ctx, WX_ERR_INVALID, "wx_grid_set_values: null argument");
        if (!(band > 0.0f) || !(band < 3.0e38f))
            return fail(ctx, WX_ERR_INVALID, "wx_grid_set_values: band must be positive and finite");
        WX_CUDA(ctx, cudaSetDevice(grid->device));
        const size_t bytes = (size_t)grid->info.n3 * wx::kN3Slots * sizeof(float);
        if (!grid->values && bytes) WX_CUDA(ctx, wx::dev_alloc(&grid->values, bytes));
        if (bytes) WX_CUDA(ctx, cudaMemcpy(grid->values, values, bytes, cudaMemcpyHostToDevice));
        grid->g.values = grid->values;
        grid->g.band = band;
        return WX_OK;
    });
}

int wx_grid_get_info(const wx_grid *grid, wx_grid_info *out) {
    return wx::guard("wx_grid_get_info", [&]() -> int {
        if (!grid || !out) return WX_ERR_INVALID;
        *out = grid->info;
        return WX_OK;
    });
}

int wx_render(wx_ctx *ctx, const wx_grid *grid, const wx_state_uniform *state, uint32_t width, uint32_t height,
              uint8_t *rgba8, wx_hit *hits, void *stream) {
    return wx::guard("wx_render", [&]() -> int {
        if (!ctx || !grid || !state || !rgba8) return fail(ctx, WX_ERR_INVALID, "wx_render: null argument");
        if (grid->device != ctx->device) return fail(ctx, WX_ERR_INVALID, "wx_render: grid is on another device");
        if (((uintptr_t)rgba8 & 3) || ((uintptr_t)hits & 15))
            return fail(ctx, WX_ERR_INVALID, "wx_render: rgba8 must be 4-byte and hits 16-byte aligned");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        const uint32_t tiles_x = width / 8, tiles_y = height / 4;
        const uint64_t ntiles = (uint64_t)tiles_x * tiles_y;
        if (ntiles == 0) return WX_OK;
        if ((uint64_t)width * height >= (1ull << 32)) return fail(ctx, WX_ERR_UNSUPPORTED, "wx_render: frame too large");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // Device memory and page-locked host memory are written by the kernel itself
        // (page-locked memory through its device alias, over the host link while the
        // march runs); pageable host memory goes through the context's staging buffer.
        uint32_t *out_rgba = reinterpret_cast<uint32_t *>(rgba8);
        wx_hit *out_hits = hits;
        bool dev_rgba = device_accessible(rgba8);
        bool dev_hits = hits ? device_accessible(hits) : true;
        if (!dev_rgba) {
            if (void *d = pinned_device_alias(rgba8)) {
                out_rgba = static_cast<uint32_t *>(d);
                dev_rgba = true;
            }
        }
        if (!dev_hits) {
            if (void *d = pinned_device_alias(hits)) {
                out_hits = static_cast<wx_hit *>(d);
                dev_hits = true;
            }
        }
        const size_t npix = (size_t)width * height;
        if (!dev_rgba || !dev_hits) {
            const size_t need = npix * 4 + (hits ? npix * sizeof(wx_hit) + 256 : 0);
            if (need > ctx->stage_bytes) {
                if (ctx->stage) {
                    WX_CUDA(ctx, cudaStreamSynchronize(st));
                    cudaFree(ctx->stage);
                }
                ctx->stage = nullptr;
                ctx->stage_bytes = 0;
                WX_CUDA(ctx, wx::dev_alloc(&ctx->stage, need));
                ctx->stage_bytes = need;
            }
            char *b = static_cast<char *>(ctx->stage);
            if (!dev_rgba) out_rgba = reinterpret_cast<uint32_t *>(b);
            if (hits && !dev_hits) out_hits = reinterpret_cast<wx_hit *>(b + ((npix * 4 + 255) & ~(size_t)255));
        }
        const wxk::Job job = make_job(grid, *state, width, height, out_rgba, out_hits, 0, ctx->tuning);
        if (ctx->tuning.kernel == 1) {
            PixelOutputs cur{ctx->device, st, {0, 0}, {0, 0}};
            cur.lo[0] = reinterpret_cast<uintptr_t>(out_rgba);
            cur.hi[0] = cur.lo[0] + npix * 4;
            if (hits) {
                cur.lo[1] = reinterpret_cast<uintptr_t>(out_hits);
                cur.hi[1] = cur.lo[1] + npix * sizeof(wx_hit);
            }
            const cudaError_t e = launch_pixel_tracked(job, ctx->tuning, cur);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "wxk::launch_pixel");
        } else {
            WX_CUDA(ctx, wxk::launch_persistent(job, ctx->take_counter(), ctx->tuning, ctx->num_sms, st));
        }
        // Copy back only the dispatched region; the rest of a host buffer is untouched.
        if (!dev_rgba)
            WX_CUDA(ctx, cudaMemcpy2DAsync(rgba8, (size_t)width * 4, out_rgba, (size_t)width * 4, (size_t)tiles_x * 32,
                                           (size_t)tiles_y * 4, cudaMemcpyDeviceToHost, st));
        if (hits && !dev_hits)
            WX_CUDA(ctx, cudaMemcpy2DAsync(hits, (size_t)width * sizeof(wx_hit), out_hits, (size_t)width * sizeof(wx_hit),
                                           (size_t)tiles_x * 8 * sizeof(wx_hit), (size_t)tiles_y * 4,
                                           cudaMemcpyDeviceToHost, st));
        return WX_OK;
    });
}

// ---- batched rendering: many frames of several grids in one persistent launch ----
static int build_jobs(wx_ctx *ctx, const wx_frame *frames, uint32_t n, std::vector<wxk::Job> &jobs,
                      uint32_t *total_tiles, uint64_t *rays) {
    jobs.clear();
    uint64_t tiles = 0, r = 0;
    for (uint32_t i = 0; i < n; i++) {
        const wx_frame &f = frames[i];
        if (!f.grid || !f.rgba8) return fail(ctx, WX_ERR_INVALID, "wx_frame: null grid or rgba8");
        if (((uintptr_t)f.rgba8 & 3) || ((uintptr_t)f.hits & 15))
            return fail(ctx, WX_ERR_INVALID, "wx_frame: rgba8 must be 4-byte and hits 16-byte aligned");
        if (f.grid->device != ctx->device) return fail(ctx, WX_ERR_INVALID, "wx_frame: grid is on another device");
        if (!device_accessible(f.rgba8) || (f.hits && !device_accessible(f.hits)))
            return fail(ctx, WX_ERR_INVALID, "wx_frame: batched outputs must be device memory");
        if ((uint64_t)f.width * f.height >= (1ull << 32)) return fail(ctx, WX_ERR_UNSUPPORTED, "wx_frame: too large");
        const wxk::Job j = make_job(f.grid, f.state, f.width, f.height, reinterpret_cast<uint32_t *>(f.rgba8), f.hits,
                                    (uint32_t)tiles, ctx->tuning);
        if (j.tiles == 0) continue;
        jobs.push_back(j);
        tiles += j.tiles;
        r += (uint64_t)(f.width & ~7u) * (f.height & ~3u);
        if (tiles >= (1ull << 31)) return fail(ctx, WX_ERR_UNSUPPORTED, "wx_render_batch: more than 2^31 tiles");
    }
    *total_tiles = (uint32_t)tiles;
    *rays = r;
    return WX_OK;
}

int wx_render_batch(wx_ctx *ctx, const wx_frame *frames, uint32_t n, void *stream) {
    return wx::guard("wx_render_batch", [&]() -> int {
        if (!ctx || (n && !frames)) return fail(ctx, WX_ERR_INVALID, "wx_render_batch: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        std::vector<wxk::Job> jobs;
        uint32_t total = 0;
        uint64_t rays = 0;
        int rc = build_jobs(ctx, frames, n, jobs, &total, &rays);
        if (rc != WX_OK) return rc;
        if (jobs.empty()) return WX_OK;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // The pinned staging table is reused: wait for the previous batch's copy.
        WX_CUDA(ctx, cudaEventSynchronize(ctx->jobs_done));
        if (jobs.size() > ctx->jobs_cap) {
            if (ctx->jobs_dev) {
                WX_CUDA(ctx, cudaDeviceSynchronize());
                cudaFree(ctx->jobs_dev);
                cudaFreeHost(ctx->jobs_host);
            }
            ctx->jobs_dev = nullptr;
            ctx->jobs_host = nullptr;
            ctx->jobs_cap = 0;
            const size_t cap = std::max<size_t>(jobs.size(), 256);
            WX_CUDA(ctx, wx::dev_alloc(&ctx->jobs_dev, cap * sizeof(wxk::Job)));
            WX_CUDA(ctx, wx::pinned_alloc(&ctx->jobs_host, cap * sizeof(wxk::Job)));
            ctx->jobs_cap = cap;
        }
        memcpy(ctx->jobs_host, jobs.data(), jobs.size() * sizeof(wxk::Job));
        WX_CUDA(ctx, cudaMemcpyAsync(ctx->jobs_dev, ctx->jobs_host, jobs.size() * sizeof(wxk::Job),
                                     cudaMemcpyHostToDevice, st));
        WX_CUDA(ctx, cudaEventRecord(ctx->jobs_done, st));
        WX_CUDA(ctx, wxk::launch_batched(ctx->jobs_dev, (uint32_t)jobs.size(), total, ctx->take_counter(), ctx->tuning,
                                         ctx->num_sms, wxk::all_modes(jobs.data(), jobs.size()), st));
        return WX_OK;
    });
}

int wx_batch_create(wx_ctx *ctx, const wx_frame *frames, uint32_t n, wx_batch **out) {
    return wx::guard("wx_batch_create", [&]() -> int {
        if (!ctx || !out || (n && !frames)) return fail(ctx, WX_ERR_INVALID, "wx_batch_create: null argument");
        WX_CUDA(ctx, cudaSetDevice(ctx->device));
        std::vector<wxk::Job> jobs;
        uint32_t total = 0;
        uint64_t rays = 0;
        int rc = build_jobs(ctx, frames, n, jobs, &total, &rays);
        if (rc != WX_OK) return rc;
        auto *b = new (std::nothrow) wx_batch();
        if (!b) return fail(ctx, WX_ERR_OOM, "host allocation failed");
        b->ctx = ctx;
        b->njobs = (uint32_t)jobs.size();
        b->total_tiles = total;
        b->rays = rays;
        auto bail = [&](cudaError_t e, const char *what) {
            wx_batch_destroy(b);
            return cuda_fail(ctx, e, what);
        };
        cudaError_t e;
        if ((e = wx::dev_alloc(&b->jobs_dev, std::max<size_t>(jobs.size(), 1) * sizeof(wxk::Job))) != cudaSuccess)
            return bail(e, "cudaMalloc(job table)");
        if (!jobs.empty() &&
            (e = cudaMemcpy(b->jobs_dev, jobs.data(), jobs.size() * sizeof(wxk::Job), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e, "cudaMemcpy(job table)");
        if ((e = wx::dev_alloc(&b->counter, sizeof(uint32_t))) != cudaSuccess) return bail(e, "cudaMalloc(counter)");
        // Capture counter reset + persistent launch into a graph, replayed by wx_batch_launch.
        cudaStream_t cs;
        if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
        if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
            cudaStreamDestroy(cs);
            return bail(e, "cudaStreamBeginCapture");
        }
        cudaError_t le = b->njobs ? wxk::launch_batched(b->jobs_dev, b->njobs, total, b->counter, ctx->tuning,
                                                        ctx->num_sms, wxk::all_modes(jobs.data(), jobs.size()), cs)
                                  : cudaMemsetAsync(b->counter, 0, sizeof(uint32_t), cs);
        e = cudaStreamEndCapture(cs, &b->graph);
        cudaStreamDestroy(cs);
        if (le != cudaSuccess) return bail(le, "capture launch_batched");
        if (e != cudaSuccess) return bail(e, "cudaStreamEndCapture");
        if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) return bail(e, "cudaGraphInstantiate");
        *out = b;
        return WX_OK;
    });
}

int wx_batch_launch(wx_batch *b, void *stream) {
    return wx::guard("wx_batch_launch", [&]() -> int {
        if (!b) return WX_ERR_INVALID;
        WX_CUDA(b->ctx, cudaSetDevice(b->ctx->device));
        WX_CUDA(b->ctx, cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
        return WX_OK;
    });
}

int wx_batch_info(const wx_batch *b, uint32_t *frames, uint32_t *tiles, uint64_t *rays) {
    return wx::guard("wx_batch_info", [&]() -> int {
        if (!b) return WX_ERR_INVALID;
        if (frames) *frames = b->njobs;
        if (tiles) *tiles = b->total_tiles;
        if (rays) *rays = b->rays;
        return WX_OK;
    });
}

int wx_batch_destroy(wx_batch *b) {
    return wx::guard("wx_batch_destroy", [&]() -> int {
        if (!b) return WX_OK;
        cudaSetDevice(b->ctx->device);
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        if (b->jobs_dev) cudaFree(b->jobs_dev);
        if (b->counter) cudaFree(b->counter);
        delete b;
        return WX_OK;
    });
}

}  // extern "C"
