// kernels.cu — sm_103a kernels of the raycast pass.
//
// k_pixel       one thread per pixel, one warp per pixel tile (8x4 by default:
//               the reference's workgroup, raycast.comp.wgsl:60), tiles in
//               launch order.
// k_persistent  persistent warps drawing tiles from a global queue (an atomic
//               counter in device scratch memory); kBatched = many frames
//               (jobs) of several grids in one launch.
// k_check_div   exhaustive check of the fast division against IEEE division.

#include <cuda_runtime.h>

#include <cstdint>

#include "wx_device.cuh"
#include "wx_kernels.h"

namespace {

using namespace wxd;
using wxk::Job;

// cp_main for one pixel of job J: colour, optional hit record, shadow ray (mode 3)
// or the glossy chain (mode 4). Tile tl of the job covers tile_w x tile_h
// pixels; lanes outside the dispatched region 8*floor(w/8) x 4*floor(h/4)
// (wgpu_context.rs:281) do nothing.
__device__ __forceinline__ void render_pixel(const Job &J, uint32_t tl, uint32_t lane) {
    const uint32_t gx = (tl % J.tiles_x) * J.tile_w + lane % J.tile_w;
    const uint32_t gy = (tl / J.tiles_x) * J.tile_h + lane / J.tile_w;
    if (gx >= (J.width & ~7u) || gy >= (J.height & ~3u)) return;
    const wx_state_uniform &s = J.s;
    const F3 dir = primary_dir(s, gx, gy);
    const F3 eye = f3(s.eye[0], s.eye[1], s.eye[2]);
    const March hit = hdda(J.g, eye, dir);
    F3 c;
    uint32_t shadow = 0;
    if (s.render_mode[0] == 4u) {
        c = glossy_colour(J.g, s, hit, dir);
    } else {
        bool need;
        F3 shadowed, src;
        c = primary_colour(s, hit, dir, &need, &shadowed, &src);
        if (need) {
            const March sh = hdda(J.g, src, -f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]));
            shadow = 1u | (sh.state << 1) | (sh.i << 8);
            if (sh.state == 0u) c = shadowed;
        }
    }
    const uint32_t pix = gy * J.width + gx;
    J.rgba[pix] = pack_rgba(c);
    if (J.hits)
        store_hit(J.hits + pix, hit.p, dot3(hit.p - eye, dir), hit.node,
                  hit.state | (hit.np << 2) | (hit.mask << 4) | (hit.i << 8), shadow);
}

// One warp per tile, tiles in launch order.
// Blocks of at most 256 threads with 64 registers a thread: 32 resident warps per SM.
#define WX_RAY_BOUNDS __launch_bounds__(256, 4)

__global__ void WX_RAY_BOUNDS k_pixel(const __grid_constant__ Job job, uint32_t ntiles) {
    const uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (tile >= ntiles) return;
    render_pixel(job, tile, threadIdx.x & 31u);
}

// First job whose tile range contains tile t (jobs sorted by tile_begin, no empty jobs).
__device__ __forceinline__ uint32_t find_job(const Job *__restrict__ jobs, uint32_t njobs, uint32_t t,
                                             uint32_t lo) {
    uint32_t hi = njobs;  // invariant: jobs[lo].tile_begin <= t < jobs[hi].tile_begin
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&jobs[mid].tile_begin) <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Persistent warps drawing whole tiles from a global queue (one atomic per
// 32 rays). Tiles are numbered job by job; a warp's successive tiles increase,
// so its job search starts at the previous job.
template <bool kBatched>
__global__ void WX_RAY_BOUNDS k_persistent(const Job *__restrict__ jobs, uint32_t njobs, const __grid_constant__ Job job0,
                             uint32_t total_tiles, uint32_t *__restrict__ ctr) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t cur_job = 0;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(ctr, 1u);
        t = __shfl_sync(~0u, t, 0);
        if (t >= total_tiles) break;
        if (kBatched) {
            cur_job = find_job(jobs, njobs, t, cur_job);
            const Job &J = jobs[cur_job];
            render_pixel(J, t - J.tile_begin, lane);
        } else {
            render_pixel(job0, t, lane);
        }
    }
}

__global__ void k_check_div(uint32_t max_m, unsigned long long *out) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;  // significand index and sign
    if (idx >= (2u << 23)) return;
    const uint32_t sig = idx & ((1u << 23) - 1u);
    const float x = __uint_as_float((idx >> 23 ? 0x80000000u : 0u) | (127u << 23) | sig);
    for (uint32_t m = 1; m < max_m; m += 2) {
        const float mf = __uint2float_rn(m);
        const float a = div_fast(x, mf, g_rcp_odd[m >> 1]);
        const float b = __fdiv_rn(x, mf);
        if (__float_as_uint(a) != __float_as_uint(b)) {
            if (atomicAdd(&out[0], 1ull) == 0ull) {
                out[1] = m;
                out[2] = __float_as_uint(x);
            }
        }
    }
}

template <class K>
int blocks_for(K kernel, int threads) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

}  // namespace

namespace wxk {

cudaError_t init_device_tables() {
    static_assert(sizeof(Job) % 8 == 0, "Job layout");
    float h[wxd::kRcpOdd];
    for (uint32_t j = 0; j < wxd::kRcpOdd; j++) {
        volatile float m = (float)(2 * j + 1);
        h[j] = 1.0f / m;  // host IEEE division, round to nearest
    }
    return cudaMemcpyToSymbol(wxd::g_rcp_odd, h, sizeof h);
}

int max_blocks_per_sm(int kernel, bool batched, int warps_per_block) {
    const int threads = 32 * warps_per_block;
    if (kernel == 1) return blocks_for(k_pixel, threads);
    return batched ? blocks_for(k_persistent<true>, threads) : blocks_for(k_persistent<false>, threads);
}

cudaError_t launch_pixel(const Job &job, const Tuning &t, cudaStream_t st) {
    const uint32_t wpb = (uint32_t)t.warps_per_block;
    k_pixel<<<(job.tiles + wpb - 1) / wpb, 32 * wpb, 0, st>>>(job, job.tiles);
    return cudaGetLastError();
}

static int grid_blocks(const Tuning &t, bool batched, int num_sms, uint32_t total_tiles) {
    const int per_sm = t.blocks_per_sm > 0 ? t.blocks_per_sm : max_blocks_per_sm(0, batched, t.warps_per_block);
    long blocks = (long)per_sm * num_sms;
    const long need = ((long)total_tiles + t.warps_per_block - 1) / t.warps_per_block;
    if (blocks > need) blocks = need;
    return (int)(blocks > 0 ? blocks : 1);
}

cudaError_t launch_persistent(const Job &job, uint32_t *ctr, const Tuning &t, int num_sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_persistent<false><<<grid_blocks(t, false, num_sms, job.tiles), 32 * t.warps_per_block, 0, st>>>(
        nullptr, 1, job, job.tiles, ctr);
    return cudaGetLastError();
}

cudaError_t launch_batched(const Job *jobs_dev, uint32_t njobs, uint32_t total_tiles, uint32_t *ctr,
                           const Tuning &t, int num_sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    Job dummy{};
    k_persistent<true><<<grid_blocks(t, true, num_sms, total_tiles), 32 * t.warps_per_block, 0, st>>>(
        jobs_dev, njobs, dummy, total_tiles, ctr);
    return cudaGetLastError();
}

cudaError_t check_division(uint32_t max_m, unsigned long long *out_dev, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out_dev, 0, 3 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (max_m > 2 * wxd::kRcpOdd) max_m = 2 * wxd::kRcpOdd;
    k_check_div<<<(2u << 23) / 256, 256, 0, st>>>(max_m, out_dev);
    return cudaGetLastError();
}

}  // namespace wxk
