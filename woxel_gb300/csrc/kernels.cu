// kernels.cu — sm_103a kernels of the raycast pass.
//
// k_pixel       one thread per pixel, one warp per pixel tile (8x4 by default:
//               the reference's workgroup, raycast.comp.wgsl:60), one launch per
//               frame; consecutive frames on a stream overlap (programmatic
//               dependent launch).
// k_persistent  persistent warps drawing tiles from a global queue (an atomic
//               counter in device scratch memory); kBatched = many frames
//               (jobs) of several grids in one launch.
// k_check_div   exhaustive check of the fast division against IEEE division.

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "wx_common.h"
#include "wx_device.cuh"
#include "wx_kernels.h"

namespace {

using namespace wxd;
using wxk::Job;

// cp_main for one pixel of job J: colour, optional hit record, shadow ray (mode 3)
// or the glossy chain (mode 4). Tile tl of the job covers tile_w x tile_h
// pixels; lanes outside the dispatched region 8*floor(w/8) x 4*floor(h/4)
// (wgpu_context.rs:281) do nothing. kAll = false compiles modes 0-3 only (the
// host sends frames of modes 4 and 5 to the kAll = true kernels): the glossy
// chain and the zero-crossing search would otherwise cost the march registers.
// Pixel (gx, gy) of lane `lane` of tile tl; false outside the dispatched region.
// Tile row: with order 1, the i-th row handed out is the middle row, then
// alternately the rows above and below it (a permutation of the rows).
__device__ __forceinline__ bool tile_pixel(const Job &J, uint32_t tl, uint32_t lane, uint32_t &gx, uint32_t &gy) {
    uint32_t row = tl / J.tiles_x;
    if (J.order) {
        const uint32_t mid = (J.tiles / J.tiles_x) >> 1;
        row = (row & 1u) ? mid - ((row + 1u) >> 1) : mid + (row >> 1);
    }
    gx = (tl % J.tiles_x) * J.tile_w + lane % J.tile_w;
    gy = row * J.tile_h + lane / J.tile_w;
    return gx < (J.width & ~7u) && gy < (J.height & ~3u);
}

template <bool kAll, bool kFmaStep01 = true>
__device__ __forceinline__ void render_pixel(const Job &J, uint32_t tl, uint32_t lane, bool wait_prev) {
    uint32_t gx, gy;
    // The warp's lanes leave each march at different iterations. Without the
    // explicit reconvergence points below they go on in small groups, each
    // running the shading once and starting its own shadow march.
    const bool valid = tile_pixel(J, tl, lane, gx, gy);
    const uint32_t act = __ballot_sync(~0u, valid);
    if (!valid) return;
    const wx_state_uniform &s = J.s;
    const F3 dir = primary_dir(s, gx, gy);
    const F3 eye = f3(s.eye[0], s.eye[1], s.eye[2]);
    const March hit = hdda<kFmaStep01>(J.g, eye, dir);
    __syncwarp(act);
    F3 c;
    uint32_t shadow = 0, reserved = 0;
    if (kAll && s.render_mode[0] == 4u) {
        c = glossy_colour(J.g, s, hit, dir);
    } else if (kAll && s.render_mode[0] == 5u) {  // zero crossing (extension); the mode is warp-uniform
        reserved = 0x7FC00000u;           // NaN: no crossing
        if (hit.state == 0u) {
            float ts;
            uint32_t ks;
            F3 N;
            if (surf_search(J.g, eye, dir, dot3(hit.p - eye, dir), &ts, &ks, &N)) {
                c = surface_colour(s, N);
                shadow = 1u | (ks << 8);
                reserved = __float_as_uint(ts);
            } else {
                const F3 a = maskf(hit.mask) * f3(0.2f, 0.2f, 0.3f);
                c = splat((a.x + a.y) + a.z);
            }
        } else {
            bool need;
            F3 shadowed, src;
            c = primary_colour(s, hit, dir, &need, &shadowed, &src);  // states 1, 2: mode 3's colours
        }
    } else if (!kFmaStep01) {  // modes 0-3 in the persistent kernels
        // Everything the stores need is reduced to a few words before the shadow
        // march (the packed colour, t, the info word), so that the direction and
        // both candidate colours are not live across it: the persistent kernels
        // then spill 32 bytes instead of 92 and the mixed batch runs at 4.80
        // instead of 4.58 Grays/s (k_pixel, with fewer registers, gains nothing).
        bool need;
        F3 shadowed, src;
        const F3 cc = primary_colour(s, hit, dir, &need, &shadowed, &src);
        uint32_t cpk = pack_rgba(cc);
        const float t = dot3(hit.p - eye, dir);
        const uint32_t info = hit.state | (hit.np << 2) | (hit.mask << 4) | (hit.i << 8);
        const F3 hp = hit.p;
        const uint32_t node = hit.node;
        __syncwarp(act);  // shadow rays of the warp start together
        if (need) {
            const March sh = hdda<kFmaStep01>(J.g, src, -f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]));
            shadow = 1u | (sh.state << 1) | (sh.i << 8);
            if (sh.state == 0u) cpk = pack_rgba(ambient_colour());  // shadowed is I_a
        }
        __syncwarp(act);
        const uint32_t pix = gy * J.width + gx;
        if (wait_prev) asm volatile("griddepcontrol.wait;" ::: "memory");
        if (!wx_in_range(pix, (uint64_t)J.width * J.height)) return;
        J.rgba[pix] = cpk;
        if (J.hits) store_hit(J.hits + pix, hp, t, node, info, shadow, 0u);
        return;
    } else {  // modes 0-3: every valid lane of the warp comes here (the __syncwarp below needs them all)
        bool need;
        F3 shadowed, src;
        c = primary_colour(s, hit, dir, &need, &shadowed, &src);
        __syncwarp(act);  // shadow rays of the warp start together
        if (need) {
            const March sh = hdda<kFmaStep01>(J.g, src, -f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]));
            shadow = 1u | (sh.state << 1) | (sh.i << 8);
            if (sh.state == 0u) c = shadowed;
        }
    }
    __syncwarp(act);
    const uint32_t pix = gy * J.width + gx;
    // A programmatically dependent launch (k_pixel) may run its march while the
    // previous kernel of the stream finishes; unless that kernel's outputs are
    // disjoint from this frame's, the stores wait for it to complete. A no-op
    // in a launch that is not programmatically dependent.
    if (wait_prev) asm volatile("griddepcontrol.wait;" ::: "memory");
    if (!wx_in_range(pix, (uint64_t)J.width * J.height)) return;
    J.rgba[pix] = pack_rgba(c);
    if (J.hits)
        store_hit(J.hits + pix, hit.p, dot3(hit.p - eye, dir), hit.node,
                  hit.state | (hit.np << 2) | (hit.mask << 4) | (hit.i << 8), shadow, reserved);
}

// Blocks of at most 256 threads. The persistent kernels: at least 5 resident,
// 48 registers a thread and 40 resident warps per SM. k_pixel: at least 6, 40
// registers and 48 warps (modes 0-3; the kernel of every mode keeps 48 registers,
// which its glossy and zero-crossing code needs). Measured on GB300 (16 frames of 2000 spheres at
// 1080p): k_pixel 3.34 Grays/s at 40 registers against 3.17 at 48 and 3.30 at 32
// (its finished blocks retire while the previous frame ends, so more resident warps
// pay); the persistent kernels are slower at 40 registers (the mixed batch 4.38
// against 4.80 Grays/s at 48; spills in the march loop) and beat 64 (32 warps) by 2%
// and 80 (24 warps) by 17% at 48.
#define WX_RAY_BOUNDS __launch_bounds__(256, 5)
#define WX_PIXEL_BOUNDS __launch_bounds__(256, kAll ? 5 : 6)

// One warp per tile of one frame, tiles in block order (rows in the job's order).
// Frames on one stream overlap in time: the next k_pixel starts once every block
// of this one has signalled launch_dependents. Block 0 signals only after the
// previous kernel has completed, so (1) a frame completes after its predecessor,
// and (2) a frame starts only after the frame two back has completed: while it
// runs, at most the frame just before it is still writing. disjoint (set by the
// host when this frame's outputs do not overlap that frame's) lets every block
// write without waiting and retire as soon as its tiles are done, so the
// previous frame's last blocks do not hold finished blocks on the SMs.
template <bool kAll>
__global__ void WX_PIXEL_BOUNDS k_pixel(const __grid_constant__ Job job, uint32_t ntiles, uint32_t disjoint) {
    if (blockIdx.x == 0) asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (tile >= ntiles) return;
    render_pixel<kAll>(job, tile, threadIdx.x & 31u, disjoint == 0u);
}

// ---------------------------------------------------------------------------
// k_wave: lanes that refill (modes 0-3). One warp per work unit of kR
// consecutive tiles (kR * 32 pixels, kR rays per lane on average). A lane whose
// ray has ended takes the unit's next pixel as soon as kRefill lanes of the
// warp are idle, so the march runs with most lanes busy; the ray's result goes
// to the warp's shared-memory slots and the unit's pixels are shaded 32 at a
// time once every ray has ended. The unit's shadow rays (mode 3) are queued in
// the same slots and marched the same way. Every ray performs exactly the
// ray_step sequence it performs in k_pixel, so pixels and hit records are
// identical. Launched like k_pixel (programmatic dependent launch).
// ---------------------------------------------------------------------------
constexpr uint32_t kWaveWords = 5;               // slot: p.xyz, info, node | queued shadow ray: src.xyz, pixel, colour
constexpr uint32_t kSlotInvalid = 0xFFFFFFFFu;   // info of a pixel outside the dispatched region
constexpr uint32_t kSlotDeferred = 0xFFFFFFFEu;  // info of a ray for the careful step, marched after the others
constexpr uint32_t kRefill = 8;                  // idle lanes that trigger a refill

__device__ __forceinline__ void wave_put(uint32_t *q, const Ray &r, uint32_t st) {
    q[0] = __float_as_uint(r.px);
    q[1] = __float_as_uint(r.py);
    q[2] = __float_as_uint(r.pz);
    q[3] = st | (r.np << 2) | (ray_mask(r) << 4) | (r.i << 8);
    q[4] = ray_node(r);
}

// The shadow record of a traced shadow ray and the pixel's colour: I_a when the
// shadow ray hit, else the queued I_a + I_d (raycast.comp.wgsl:188-193).
__device__ __forceinline__ void wave_shadow_done(const Job &J, const uint32_t *e, uint32_t ambient, uint32_t st,
                                                 uint32_t steps) {
    const uint32_t pixel = e[3];
    if (!wx_in_range(pixel, (uint64_t)J.width * J.height)) return;
    J.rgba[pixel] = st == 0u ? ambient : e[4] | 0xFF000000u;
    if (J.hits) reinterpret_cast<uint32_t *>(J.hits + pixel)[6] = 1u | (st << 1) | (steps << 8);
}

#define WX_WAVE_BOUNDS __launch_bounds__(256, 5)

template <uint32_t kR>
__global__ void WX_WAVE_BOUNDS k_wave(const __grid_constant__ Job J, uint32_t ntiles, uint32_t disjoint) {
    extern __shared__ uint32_t wave_smem[];
    if (blockIdx.x == 0) asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t tile0 = (blockIdx.x * (blockDim.x >> 5) + warp) * kR;
    if (tile0 >= ntiles) return;
    const uint32_t P = min(kR, ntiles - tile0) * 32u;  // the unit's pixels
    uint32_t *slot = wave_smem + warp * (kR * 32u * kWaveWords);
    const wx_state_uniform &s = J.s;
    const F3 eye = f3(s.eye[0], s.eye[1], s.eye[2]);
    const uint32_t below = (1u << lane) - 1u;

    // Phase 1: primary rays, lanes refilled from the unit's pixels.
    {
        Ray r;
        bool active = false;
        uint32_t mine = 0, next = 0;
        for (;;) {
            const uint32_t idle = __ballot_sync(~0u, !active);
            if (next < P && (idle == ~0u || __popc(idle) >= kRefill)) {
                if (!active) {
                    const uint32_t pix = next + __popc(idle & below);
                    if (pix < P) {
                        uint32_t gx, gy;
                        if (!tile_pixel(J, tile0 + pix / 32u, pix % 32u, gx, gy)) {
                            slot[pix * kWaveWords + 3] = kSlotInvalid;
                        } else {
                            const F3 dir = primary_dir(s, gx, gy);
                            if (ray_needs_careful_step(eye, dir)) {
                                slot[pix * kWaveWords + 3] = kSlotDeferred;
                            } else {
                                ray_init(r, eye, dir);
                                active = true;
                                mine = pix;
                            }
                        }
                    }
                }
                next += __popc(idle);
                continue;
            }
            if (idle == ~0u) break;
            if (active) {
                const uint32_t st = ray_step<false>(J.g, r);
                if (st != 0xFFu) {
                    wave_put(slot + mine * kWaveWords, r, st);
                    active = false;
                }
            }
        }
    }
    __syncwarp();
    // Rays that need the careful step (a direction component below 2^-126 in
    // magnitude, or a -0 eye coordinate): rare, marched 32 at a time.
    for (uint32_t base = 0; base < P; base += 32u) {
        const uint32_t pix = base + lane;
        const bool mine = slot[pix * kWaveWords + 3] == kSlotDeferred;
        if (!__any_sync(~0u, mine)) continue;
        if (mine) {
            uint32_t gx, gy;
            tile_pixel(J, tile0 + pix / 32u, lane, gx, gy);
            Ray r;
            ray_init(r, eye, primary_dir(s, gx, gy));
            uint32_t st;
            while ((st = ray_step<true>(J.g, r)) == 0xFFu) {
            }
            wave_put(slot + pix * kWaveWords, r, st);
        }
        __syncwarp();
    }

    // Phase 2: shading, 32 pixels at a time; lit pixels of mode 3 queue their
    // shadow ray in the slots already read.
    const bool wait_prev = disjoint == 0u;
    uint32_t nq = 0;
    for (uint32_t base = 0; base < P; base += 32u) {
        const uint32_t pix = base + lane;
        const uint32_t *q = slot + pix * kWaveWords;
        March hit;
        hit.p = f3(__uint_as_float(q[0]), __uint_as_float(q[1]), __uint_as_float(q[2]));
        const uint32_t info = q[3];
        hit.node = q[4];
        const bool valid = info != kSlotInvalid;
        hit.state = info & 3u;
        hit.np = (info >> 2) & 3u;
        hit.mask = (info >> 4) & 7u;
        hit.i = info >> 8;
        uint32_t gx, gy;
        tile_pixel(J, tile0 + pix / 32u, lane, gx, gy);
        const F3 dir = primary_dir(s, gx, gy);
        bool need = false;
        F3 shadowed, src;
        const F3 c = primary_colour(s, hit, dir, &need, &shadowed, &src);
        need = need && valid;
        __syncwarp();  // every slot of these 32 pixels is read before the queue reuses them
        const uint32_t qm = __ballot_sync(~0u, need);
        const uint32_t pixel = gy * J.width + gx;
        if (need) {
            uint32_t *e = slot + (nq + __popc(qm & below)) * kWaveWords;
            e[0] = __float_as_uint(src.x);
            e[1] = __float_as_uint(src.y);
            e[2] = __float_as_uint(src.z);
            e[3] = pixel;
            e[4] = pack_rgba(c);
        }
        nq += __popc(qm);
        if (valid) {
            if (wait_prev) asm volatile("griddepcontrol.wait;" ::: "memory");
            if (wx_in_range(pixel, (uint64_t)J.width * J.height)) {
                if (!need) J.rgba[pixel] = pack_rgba(c);
                if (J.hits) store_hit(J.hits + pixel, hit.p, dot3(hit.p - eye, dir), hit.node, info, 0u);
            }
        }
    }
    if (nq == 0u) return;
    __syncwarp();

    // Phase 3: the queued shadow rays toward the sun, lanes refilled from the queue.
    const F3 sdir = -f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
    const uint32_t ambient = pack_rgba(ambient_colour());
    const bool dir_careful = !(fabsf(sdir.x) >= 0x1p-126f && fabsf(sdir.y) >= 0x1p-126f && fabsf(sdir.z) >= 0x1p-126f);
    {
        Ray r;
        bool active = false;
        uint32_t mine = 0, next = 0;
        for (;;) {
            const uint32_t idle = __ballot_sync(~0u, !active);
            if (next < nq && (idle == ~0u || __popc(idle) >= kRefill)) {
                if (!active) {
                    const uint32_t k = next + __popc(idle & below);
                    if (k < nq) {
                        uint32_t *e = slot + k * kWaveWords;
                        const F3 src = f3(__uint_as_float(e[0]), __uint_as_float(e[1]), __uint_as_float(e[2]));
                        if (dir_careful || ray_needs_careful_step(src, sdir)) {
                            e[4] &= 0x00FFFFFFu;  // alpha 0 marks the entry for the careful pass
                        } else {
                            ray_init(r, src, sdir);
                            active = true;
                            mine = k;
                        }
                    }
                }
                next += __popc(idle);
                continue;
            }
            if (idle == ~0u) break;
            if (active) {
                const uint32_t st = ray_step<false>(J.g, r);
                if (st != 0xFFu) {
                    wave_shadow_done(J, slot + mine * kWaveWords, ambient, st, r.i);
                    active = false;
                }
            }
        }
    }
    __syncwarp();
    for (uint32_t base = 0; base < nq; base += 32u) {
        const uint32_t k = base + lane;
        const bool mine = k < nq && (slot[k * kWaveWords + 4] >> 24) == 0u;
        if (!__any_sync(~0u, mine)) continue;
        if (mine) {
            const uint32_t *e = slot + k * kWaveWords;
            const March sh = hdda(J.g, f3(__uint_as_float(e[0]), __uint_as_float(e[1]), __uint_as_float(e[2])), sdir);
            wave_shadow_done(J, e, ambient, sh.state, sh.i);
        }
    }
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
// Batched launches may carry a cancel table (the server's): a job whose
// cancel_id has been written to cancel[cancel_slot] (by the host, while the
// launch runs) has its remaining tiles skipped, which `skipped` counts.
template <bool kBatched, bool kAll>
__global__ void WX_RAY_BOUNDS k_persistent(const Job *__restrict__ jobs, uint32_t njobs, const __grid_constant__ Job job0,
                             uint32_t total_tiles, uint32_t *__restrict__ ctr, const uint32_t *cancel,
                             uint32_t *skipped) {
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
            if (cancel) {
                uint32_t id = 0, c = 0;
                if (lane == 0) {
                    id = __ldg(&J.cancel_id);
                    if (id) asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(cancel + __ldg(&J.cancel_slot)));
                }
                if (__shfl_sync(~0u, id != 0u && c == id, 0)) {
                    if (lane == 0 && skipped) atomicAdd(skipped, 1u);
                    continue;
                }
            }
            render_pixel<kAll, false>(J, t - J.tile_begin + J.tile_off, lane, true);
        } else {
            render_pixel<kAll, false>(job0, t, lane, true);
        }
    }
}

__global__ void k_check_div(uint32_t max_m, unsigned long long *out) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;  // significand index and sign
    if (idx >= (2u << 23)) return;
    const uint32_t sig = idx & ((1u << 23) - 1u);
    const float x = __uint_as_float((idx >> 23 ? 0x80000000u : 0u) | (127u << 23) | sig);
    for (uint32_t m = 1; m < max_m; m++) {
        const float mf = __uint2float_rn(m);
        const float a = div_fast(x, mf, g_rcp[m]);
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
    float h[wxd::kRcp];
    h[0] = 0.0f;
    for (uint32_t d = 1; d < wxd::kRcp; d++) {
        volatile float m = (float)d;
        h[d] = 1.0f / m;  // host IEEE division, round to nearest
    }
    cudaError_t e = cudaMemcpyToSymbol(wxd::g_rcp, h, sizeof h);
    // k_wave's slots: up to 8 warps x 8 tiles x 32 pixels x 5 words (40 KB).
    const int wave_max = 8 * 8 * 32 * (int)(kWaveWords * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wave<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, wave_max);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wave<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, wave_max);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_wave<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, wave_max);
    return e;
}

int max_blocks_per_sm(int kernel, bool batched, int warps_per_block) {
    const int threads = 32 * warps_per_block;
    if (kernel == 1) return blocks_for(k_pixel<false>, threads);
    return batched ? blocks_for(k_persistent<true, false>, threads) : blocks_for(k_persistent<false, false>, threads);
}

cudaError_t launch_pixel(const Job &job, const Tuning &t, bool disjoint, cudaStream_t st) {
    const uint32_t wpb = (uint32_t)t.warps_per_block;
    // Programmatic dependent launch: back-to-back frames on one stream overlap
    // the previous frame's last blocks with this frame's march (the kernel's
    // stores wait for the previous kernel; see render_pixel).
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((job.tiles + wpb - 1) / wpb);
    cfg.blockDim = dim3(32 * wpb);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const uint32_t dj = disjoint ? 1u : 0u;
    if (all_modes(job.s)) return cudaLaunchKernelEx(&cfg, k_pixel<true>, job, job.tiles, dj);
    if (t.rays > 1) {  // k_wave: t.rays tiles per warp, lanes refill
        const uint32_t per_block = wpb * (uint32_t)t.rays;
        cfg.gridDim = dim3((job.tiles + per_block - 1) / per_block);
        cfg.dynamicSmemBytes = (size_t)per_block * 32u * kWaveWords * sizeof(uint32_t);
        if (t.rays == 2) return cudaLaunchKernelEx(&cfg, k_wave<2>, job, job.tiles, dj);
        if (t.rays == 4) return cudaLaunchKernelEx(&cfg, k_wave<4>, job, job.tiles, dj);
        return cudaLaunchKernelEx(&cfg, k_wave<8>, job, job.tiles, dj);
    }
    return cudaLaunchKernelEx(&cfg, k_pixel<false>, job, job.tiles, dj);
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
    const int blocks = grid_blocks(t, false, num_sms, job.tiles);
    if (all_modes(job.s))
        k_persistent<false, true><<<blocks, 32 * t.warps_per_block, 0, st>>>(nullptr, 1, job, job.tiles, ctr, nullptr,
                                                                            nullptr);
    else
        k_persistent<false, false><<<blocks, 32 * t.warps_per_block, 0, st>>>(nullptr, 1, job, job.tiles, ctr, nullptr,
                                                                             nullptr);
    return cudaGetLastError();
}

cudaError_t launch_batched(const Job *jobs_dev, uint32_t njobs, uint32_t total_tiles, uint32_t *ctr,
                           const Tuning &t, int num_sms, bool all, cudaStream_t st, const uint32_t *cancel,
                           uint32_t *skipped) {
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    Job dummy{};
    const int blocks = grid_blocks(t, true, num_sms, total_tiles);
    if (all)
        k_persistent<true, true><<<blocks, 32 * t.warps_per_block, 0, st>>>(jobs_dev, njobs, dummy, total_tiles, ctr,
                                                                           cancel, skipped);
    else
        k_persistent<true, false><<<blocks, 32 * t.warps_per_block, 0, st>>>(jobs_dev, njobs, dummy, total_tiles, ctr,
                                                                            cancel, skipped);
    return cudaGetLastError();
}

bool all_modes(const wx_state_uniform &s) { return s.render_mode[0] == 4u || s.render_mode[0] == 5u; }

bool all_modes(const Job *jobs, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (all_modes(jobs[i].s)) return true;
    return false;
}

cudaError_t take_bounds_violations(unsigned long long *count) {
#ifdef WX_BOUNDS_CHECK
    cudaError_t e = cudaMemcpyFromSymbol(count, wxd::g_bounds_violations, sizeof *count);
    if (e != cudaSuccess) return e;
    const unsigned long long zero = 0;
    return cudaMemcpyToSymbol(wxd::g_bounds_violations, &zero, sizeof zero);
#else
    *count = 0;
    return cudaSuccess;
#endif
}

cudaError_t check_division(uint32_t max_m, unsigned long long *out_dev, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out_dev, 0, 3 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (max_m > wxd::kRcp) max_m = wxd::kRcp;
    k_check_div<<<(2u << 23) / 256, 256, 0, st>>>(max_m, out_dev);
    return cudaGetLastError();
}

}  // namespace wxk

// ---------------------------------------------------------------------------
// Batched rendering for callers that must not allocate (wx_render_batch_noalloc).
//
// Some callers cannot allocate device memory at render time: engines that
// reserve all GPU memory at start-up and forbid cudaMalloc afterwards, or code
// running where an allocation could stall or fail (a frame callback with a
// deadline). wx_render_batch needs a context whose scratch (queue counters,
// frame table) comes from cudaMalloc. This entry point instead keeps its
// scratch in the fixed device array below, which the library declares
// statically: every GPU that loads the library holds these 98,560 bytes until
// the process exits. Layout: the tile-queue counter at byte 0, the frame
// (job) table from byte 256, room for WX_NOALLOC_MAX_FRAMES frames.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocJobsOffset = 256;
constexpr size_t kNoallocBytes = kNoallocJobsOffset + (size_t)WX_NOALLOC_MAX_FRAMES * sizeof(Job);
static_assert(kNoallocBytes == WX_NOALLOC_SCRATCH_BYTES, "scratch size stated in woxel_gb300.h");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// The frame table travels to the array as the by-value parameter of a small
// table-writing kernel (up to kTableChunk frames per launch; launch parameters may
// take up to 32,764 bytes): the runtime copies a launch's parameters when the
// launch is enqueued, so a call's table is fixed when the call returns and later
// calls cannot change what an earlier one reads.
constexpr uint32_t kTableChunk = (32000 - 8) / sizeof(Job);
struct TableChunk {
    uint32_t first, count;  // first table entry written, entries in this chunk
    Job jobs[kTableChunk];
};
static_assert(sizeof(TableChunk) <= 32764, "kernel parameter limit");
static_assert(sizeof(Job) % 4 == 0, "the table is copied in 4-byte words");

__global__ void k_noalloc_table(const __grid_constant__ TableChunk c) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(c.jobs);
    uint32_t *dst = reinterpret_cast<uint32_t *>(g_noalloc_scratch + kNoallocJobsOffset + (size_t)c.first * sizeof(Job));
    const uint32_t words = c.count * (uint32_t)(sizeof(Job) / 4);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

// Per-device state of the one-time set-up (host side).
struct NoallocDevice {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch on this device
    int num_sms = 0;
};
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;  // guards the one-time set-up
NoallocDevice g_noalloc_dev[kNoallocMaxDevices];

int noalloc_fail(int code, const char *msg) {
    wx::set_thread_error(msg);
    return code;
}

// Once per device, with that device current: find the array's device address
// (host code cannot use the symbol itself) and load the division table.
int noalloc_setup(int device, NoallocDevice **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocDevice &d = g_noalloc_dev[device];
    if (!d.ready) {
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&d.scratch), g_noalloc_scratch);
        if (e != cudaSuccess) return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: cudaGetSymbolAddress failed");
        if ((e = wxk::init_device_tables()) != cudaSuccess)
            return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: loading the division table failed");
        if ((e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
            return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: cudaDeviceGetAttribute failed");
        d.ready = true;
    }
    *out = &d;
    return WX_OK;
}

bool noalloc_device_memory(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The table entry of one frame with the default launch shape (8x4 tiles), as
// wx_render_batch builds it; tiles = queue tiles of the frames before it.
int noalloc_job(const wx_frame &f, int device, uint64_t tiles, Job &j) {
    const wxk::Tuning tuning;
    memset(&j, 0, sizeof j);
    int gdev = -1;
    if (!f.rgba8 || !wxk::grid_device_view(f.grid, &j.g, &gdev))
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: frame with a NULL grid or rgba8");
    if (gdev != device) return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: grids on different devices");
    if (((uintptr_t)f.rgba8 & 3) || ((uintptr_t)f.hits & 15))
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: rgba8 must be 4-byte and hits 16-byte aligned");
    if (!noalloc_device_memory(f.rgba8) || (f.hits && !noalloc_device_memory(f.hits)))
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: outputs must be device memory");
    if ((uint64_t)f.width * f.height >= (1ull << 32))
        return noalloc_fail(WX_ERR_UNSUPPORTED, "wx_render_batch_noalloc: frame too large");
    j.width = f.width;
    j.height = f.height;
    j.tile_w = (uint16_t)tuning.tile_w;
    j.tile_h = (uint16_t)(32 / tuning.tile_w);
    j.order = (uint32_t)tuning.order;
    j.tiles_x = ((f.width & ~7u) + j.tile_w - 1) / j.tile_w;
    j.tiles = j.tiles_x * (((f.height & ~3u) + j.tile_h - 1) / j.tile_h);
    j.tile_begin = (uint32_t)tiles;
    j.rgba = reinterpret_cast<uint32_t *>(f.rgba8);
    j.hits = f.hits;
    j.s = f.state;
    return WX_OK;
}

int noalloc_render(int device, const wx_frame *frames, uint32_t n, cudaStream_t st) {
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
        cudaGetLastError();
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: stream is not a valid stream");
    }
    if (sdev != device)
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: stream belongs to another device than the grids");
    NoallocDevice *d = nullptr;
    int rc = noalloc_setup(device, &d);
    if (rc != WX_OK) return rc;
    // Pass 1 checks every frame before anything is enqueued; pass 2 writes the table
    // one chunk (one table-writing launch) at a time. Frames without dispatched
    // pixels get no entry, which keeps every entry's tile range non-empty.
    TableChunk chunk;
    uint32_t njobs = 0;
    uint64_t tiles = 0;
    bool all = false;
    for (uint32_t i = 0; i < n; i++) {
        Job &j = chunk.jobs[0];
        if ((rc = noalloc_job(frames[i], device, tiles, j)) != WX_OK) return rc;
        if (j.tiles == 0) continue;
        tiles += j.tiles;
        all = all || wxk::all_modes(j.s);
        njobs++;
        if (tiles >= (1ull << 31)) return noalloc_fail(WX_ERR_UNSUPPORTED, "wx_render_batch_noalloc: too many tiles");
    }
    if (njobs == 0) return WX_OK;
    chunk.first = 0;
    chunk.count = 0;
    tiles = 0;
    for (uint32_t i = 0; i < n; i++) {
        Job &j = chunk.jobs[chunk.count];
        noalloc_job(frames[i], device, tiles, j);
        if (j.tiles == 0) continue;
        tiles += j.tiles;
        if (++chunk.count == kTableChunk || chunk.first + chunk.count == njobs) {
            k_noalloc_table<<<1, 256, 0, st>>>(chunk);
            if (cudaGetLastError() != cudaSuccess)
                return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: frame table launch failed");
            chunk.first += chunk.count;
            chunk.count = 0;
        }
    }
    Job *jobs_dev = reinterpret_cast<Job *>(d->scratch + kNoallocJobsOffset);
    uint32_t *counter = reinterpret_cast<uint32_t *>(d->scratch);
    wxk::Tuning t;  // defaults; launch_batched clears the counter (it keeps the last call's value otherwise)
    const cudaError_t e = wxk::launch_batched(jobs_dev, njobs, (uint32_t)tiles, counter, t, d->num_sms, all, st);
    if (e != cudaSuccess) return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: launch failed");
    return WX_OK;
}

}  // namespace

extern "C" int wx_render_batch_noalloc(const wx_frame *frames, uint32_t n, void *stream) {
    if (n == 0) return WX_OK;
    if (!frames) return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: frames is NULL");
    if (n > WX_NOALLOC_MAX_FRAMES)
        return noalloc_fail(WX_ERR_INVALID,
                            "wx_render_batch_noalloc: more than WX_NOALLOC_MAX_FRAMES (256) frames in one call");
    wxk::DevGrid g;
    int device = -1;
    if (!wxk::grid_device_view(frames[0].grid, &g, &device))
        return noalloc_fail(WX_ERR_INVALID, "wx_render_batch_noalloc: frame 0 has a NULL grid");
    if (device < 0 || device >= kNoallocMaxDevices)
        return noalloc_fail(WX_ERR_UNSUPPORTED, "wx_render_batch_noalloc: device index above 63");
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: cudaGetDevice failed");
    if (prev != device && cudaSetDevice(device) != cudaSuccess)
        return noalloc_fail(WX_ERR_CUDA, "wx_render_batch_noalloc: cudaSetDevice failed");
    const int rc = noalloc_render(device, frames, n, static_cast<cudaStream_t>(stream));
    if (prev != device) cudaSetDevice(prev);
    return rc;
}
