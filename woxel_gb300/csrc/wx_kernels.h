// wx_kernels.h — host-side view of the kernels in kernels.cu (internal).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "woxel_gb300.h"

namespace wxk {

// Device node pools of one grid (see api.cpp for the layout).
struct DevGrid {
    const int4 *root;        // root block: header, N5 origins, dense root-key table (api.cpp)
    const uint32_t *slot5;   // N5 slot words
    const uint32_t *slot4;   // N4 slot words
    const uint8_t *leaf;     // N3: one byte per voxel, 0 hit, 1..254 distance, 255 = see ovf
    const uint2 *ovf;        // (voxel key = leaf << 9 | offset, distance), sorted by key
    const float *values;     // level-set value per leaf voxel (zero-crossing mode), or null
    uint32_t n5, n_ovf;
    float band;              // value of voxels outside leaves (+band; -band in active tiles)
    uint32_t inside;         // every N5 lies in [-4096, 4096)^3 (origins -4096 or 0 on each axis)
    uint32_t n4, n3;         // node counts of the N4 and N3 pools (checked in bounds-checked builds)
};

// One frame of one grid: the unit the persistent kernels draw ray tiles from.
struct Job {
    DevGrid g;
    uint32_t width, height;
    uint16_t tile_w, tile_h;       // pixel tile of one warp (tile_w * tile_h = 32)
    uint32_t order;                // tile rows: 0 top to bottom, 1 middle row first, then outwards
    uint32_t tiles_x, tiles;       // tiles per row / per frame over the dispatched region
    uint32_t tile_begin;           // first global (queue) tile id of this job
    uint32_t tile_off;             // first frame tile of this job (a job may cover part of a frame)
    uint32_t *rgba;
    wx_hit *hits;
    wx_state_uniform s;
    // Cancellation (batched launches given a cancel table): the job's tiles are
    // skipped once cancel[cancel_slot] == cancel_id (nonzero). 0 = never.
    uint32_t cancel_slot, cancel_id;
};

struct Tuning {
    int kernel = 1;            // 1 one warp per tile (k_pixel), 0 persistent warps on a tile queue
    int warps_per_block = 4;   // 1..16
    int blocks_per_sm = 0;     // 0 = as many as fit
    int tile_w = 8;            // 4, 8, 16 or 32 pixels wide (x 32/tile_w high)
    int order = 1;             // Job::order
    int rays = 1;              // k_pixel: 1 pixel per lane; 2, 4 or 8 tiles per warp with lanes that refill (k_wave)
};

cudaError_t init_device_tables();
int max_blocks_per_sm(int kernel, bool batched, int warps_per_block);
// disjoint: the job's outputs do not overlap those of the previous kernel on st,
// a k_pixel launch (see k_pixel); false is always safe.
cudaError_t launch_pixel(const Job &job, const Tuning &t, bool disjoint, cudaStream_t st);
cudaError_t launch_persistent(const Job &job, uint32_t *ctr, const Tuning &t, int num_sms, cudaStream_t st);
// all: some job renders mode 4 or 5 (the kernels compiled for every mode).
// cancel (may be NULL): the table the jobs' cancel_slot index; skipped (may be
// NULL) counts the tiles skipped for a cancelled job (the caller clears it).
cudaError_t launch_batched(const Job *jobs_dev, uint32_t njobs, uint32_t total_tiles, uint32_t *ctr,
                           const Tuning &t, int num_sms, bool all, cudaStream_t st,
                           const uint32_t *cancel = nullptr, uint32_t *skipped = nullptr);
// Modes 4 (glossy) and 5 (zero crossing) need the kernels compiled for every mode.
bool all_modes(const wx_state_uniform &s);
bool all_modes(const Job *jobs, size_t n);
// Device pools and device of a grid handle (defined in api.cpp); false for NULL.
bool grid_device_view(const wx_grid *grid, DevGrid *out, int *device);
// Device index and SM count of a context (defined in api.cpp).
void ctx_device_info(const wx_ctx *ctx, int *device, int *num_sms);

// GPU SDF build (sdf.cu). The tree structure the sweeps look neighbours up in:
// the root block of the grid layout (header, origins, root-key table) and the
// child-index tables (slot -> child DFS index or 0xFFFFFFFF).
struct SdfTree {
    const int4 *root;
    uint32_t n5;
    const uint32_t *c5, *c4;
};
cudaError_t sdf_child_table(const uint64_t *kid, const uint32_t *pre, const uint32_t *first, uint64_t nodes,
                            int slots_log2, uint32_t *cidx, cudaStream_t st);
cudaError_t sdf_child_origins(const uint32_t *cidx, const int4 *org, uint64_t nodes, int log2d, int child_span_log2,
                              int4 *org_child, cudaStream_t st);
cudaError_t sdf_init(const uint64_t *solid, uint64_t ncells, uint32_t *d, cudaStream_t st);
cudaError_t sdf_neighbours(int level, const int4 *org, uint32_t nc, const SdfTree &t, uint32_t *nb, cudaStream_t st);
// Both passes of one level; ctr[2] (not reset here) is set when a wait hit its bound.
// spin_limit: polls (256 ns apart) a CTA makes for its container before it sets
// the error flag ctr[2] and every CTA of the sweep returns.
constexpr uint32_t kSdfSpinLimit = 1u << 23;  // about 2 s
cudaError_t sdf_sweep(int level, uint32_t *d, const uint32_t *nb, uint32_t nc, uint32_t *indeg, uint32_t *queue,
                      uint32_t *ctr, int num_sms, uint32_t spin_limit, cudaStream_t st);
cudaError_t sdf_pack_internal(const uint64_t *kid, const uint64_t *val, const uint32_t *cidx, const uint32_t *d,
                              uint64_t nslots, uint32_t *slot, uint32_t *err, cudaStream_t st);
cudaError_t sdf_pack_leaves(const uint32_t *d, uint64_t ncells, uint8_t *leaf, uint2 *ovf, uint32_t cap,
                            uint32_t *n_ovf, cudaStream_t st);

// Exhaustive check of the fast floor-division path against IEEE division:
// every divisor m < max_m and every significand of [1,2) and [-2,-1).
// out[0] = mismatch count, out[1] = first mismatching m, out[2] = its x bits.
cudaError_t check_division(uint32_t max_m, unsigned long long *out_dev, cudaStream_t st);
// Bounds-checked builds: reads and zeroes the device's count of out-of-range indices.
cudaError_t take_bounds_violations(unsigned long long *count);

}  // namespace wxk
