/*
 * woxel_oracle.h — CPU oracle for woxel's primary-ray pass.
 *
 * TEST INFRASTRUCTURE ONLY. The CUDA path is compared against this oracle;
 * nothing in the product links, loads or calls it. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use it.
 *
 * It restates, in plain C with IEEE binary32 arithmetic and no contraction
 * (-ffp-contract=off), the reference's algorithm for this path:
 *   src/vdb/data_structure.rs:43-91   coordinate maths (global_to_node, offsets)
 *   src/vdb/vdb345.rs:26-66           set_voxel
 *   src/vdb/vdb345.rs:69-106          get_voxel
 *   src/vdb/vdb345.rs:108-287         origins / masks / atlas / count_nodes
 *   src/vdb/vdb345.rs:290-670         compute_sdf (two-pass chamfer, literal loops)
 *   src/vdb/vdb345.rs:673-694         arr32_from_arr64 / closest_power_of_3 / origin_from_idx
 *   src/shaders/raycast.comp.wgsl:60-519   cp_main, hdda_ray, ray_trace, reflect_ray2/1,
 *                                          get_vdb_leaf_from_{leaf,nothing,node5,node4,node3}
 *   src/render/gpu_types/compute_state.rs:87-131 + src/render/camera.rs:31-35  uniform build
 *
 * Parity status: the reference (Rust + wgpu 0.17 / naga 0.13 WGSL) cannot run in
 * this environment, so the march and SDF are pinned by the reference's own unit
 * tests only where those exist (coordinate KATs, set/get round trip); the raycast
 * output itself is "parity unpinned" against a reference execution. The
 * arithmetic choices WGSL leaves open are pinned here:
 *   - no FMA contraction; '/' and sqrt are IEEE correctly rounded;
 *   - normalize(v) = v / sqrt((x*x + y*y) + z*z);
 *   - min/max with one NaN operand return the other operand; on equal values
 *     (including +0/-0) min returns its first operand, max its first operand;
 *   - dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z;  mix(a,b,t) = a*(1-t) + b*t;
 *   - f32 -> i32 conversion saturates, NaN -> 0;
 *   - f32 -> unorm8: NaN or x <= 0 -> 0, x >= 1 -> 255, else floor(x*255 + 0.5).
 */
#ifndef WOXEL_ORACLE_H
#define WOXEL_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 256-byte uniform, field order of ComputeState (compute_state.rs:9-29). */
typedef struct orc_state {
    float view_projection[16];
    float camera_to_world[16];
    float eye[4];
    float u[4];
    float mv[4];
    float wp[4];
    uint32_t render_mode[4];
    uint32_t show_345[4];
    float sun_dir[4];
    float sun_color[4];
} orc_state;

/* Per-pixel record; byte layout identical to the product's wx_hit. */
typedef struct orc_hit {
    float p[3];
    float t;
    uint32_t node;
    uint32_t info;     /* state | level<<2 | mask<<4 | steps<<8 */
    uint32_t shadow;   /* traced | state<<1 | steps<<8 */
    uint32_t reserved;
} orc_hit;

/* Per-pixel instrumentation of the primary ray (plus its shadow ray). */
typedef struct orc_stats {
    uint32_t steps;          /* loop iterations of the primary hdda_ray */
    uint32_t bytes;          /* node-visit bytes of the primary ray */
    uint32_t shadow_steps;
    uint32_t shadow_bytes;
    uint32_t grazing;        /* 1 if any step was within 1 ulp of a tie or a cell boundary */
    uint32_t reserved[3];
} orc_stats;

/* The flattened grid as the Rust side holds it (masks(), origins(), atlas()). */
typedef struct orc_view {
    const uint32_t *kids5, *vals5;   /* n5 * 1024 words */
    const uint32_t *kids4, *vals4;   /* n4 * 128 words */
    const uint32_t *vals3;           /* n3 * 16 words */
    const int32_t *origins;          /* n5 * 4 (x, y, z, pad) */
    uint64_t n5, n4, n3;
    const uint32_t *atlas[3];        /* N5, N4, N3 atlases, texel (x,y,z) at (z*H + y)*W + x */
    uint32_t dims[3][3];             /* W, H, D of each atlas */
    /* Zero-crossing mode (render_mode 5, no reference counterpart): level-set value of
       every leaf voxel (n3 * 512, DFS leaf order, voxel x<<6 | y<<3 | z) and the band
       that voxels outside leaves read (+band, or -band inside an active tile). NULL:
       mode 5 finds no crossing. */
    const float *values;
    float band;
} orc_view;

typedef struct orc_tree orc_tree;

/* ---- coordinate maths (data_structure.rs:43-91) ---- */
void orc_global_to_node(const int32_t g[3], int total_log2, int32_t out[3]);
uint64_t orc_global_to_offset(const int32_t g[3], int log2d, int total_log2);
void orc_offset_to_child(uint64_t offset, int log2d, uint32_t out[3]);
uint64_t orc_child_to_offset(const uint32_t c[3], int log2d);

/* ---- tree (vdb345.rs) ---- */
orc_tree *orc_tree_new(void);
void orc_tree_free(orc_tree *t);
void orc_set_voxel(orc_tree *t, const int32_t p[3], uint32_t value);
/* get_voxel: returns kind (0 Offs, 1 Leaf, 2 Innr, 3 Root, 4 Bkgr); *value, *level filled. */
int orc_get_voxel(const orc_tree *t, const int32_t p[3], uint64_t *value, int *level);
/* Build a tree from masks()/origins() in DFS order (leaf values := 1). */
orc_tree *orc_tree_from_masks(const uint32_t *kids5, const uint32_t *vals5, uint64_t n5,
                              const uint32_t *kids4, const uint32_t *vals4, uint64_t n4,
                              const uint32_t *vals3, uint64_t n3, const int32_t *origins);
void orc_count_nodes(const orc_tree *t, uint64_t out[3]);
void orc_compute_sdf(orc_tree *t);
/* masks(): buffers sized by orc_count_nodes; origins as x,y,z,pad. */
void orc_masks(const orc_tree *t, uint32_t *kids5, uint32_t *vals5, uint32_t *kids4,
               uint32_t *vals4, uint32_t *vals3, int32_t *origins);
/* atlas(): side lengths (32*d5, 16*d4, 8*d3) written to side[3]; atlases may be NULL
 * to query sizes; otherwise each must hold side^3 words, texture layout. */
void orc_atlas(const orc_tree *t, uint32_t side[3], uint32_t *a5, uint32_t *a4, uint32_t *a3);

/* ---- uniform (compute_state.rs:87-131, camera.rs:31-35, egui_dev.rs:355-368) ---- */
void orc_state_build(const float eye[3], const float target[3], const float up[3],
                     float aspect, float fovy_deg, float resolution_width,
                     uint32_t render_mode, const uint32_t show_345[3],
                     const float sun_dir[3], const float sun_color[3], float sun_intensity,
                     orc_state *out);

/* ---- synthetic workloads (no reference counterpart: the benchmark's seeded grids,
 * cameras and sun, stated independently of the product so that a CPU run can build
 * them alone). splitmix64 is the seeded stream. ---- */
/* Sun defaults of the reference app (egui_dev.rs:355-368). */
void orc_sun_default(float dir[3], float color[3], float *intensity);
/* count spheres drawn as cx, cy, cz in lo + (hi - lo) * U and r in rmin + (rmax - rmin) * U;
 * out holds count * 4 doubles (cx, cy, cz, r). */
void orc_sphere_list(uint32_t count, float rmin, float rmax, float lo, float hi, uint64_t seed,
                     double *out);
/* set_voxel(ijk, 1) for every voxel with |min_s(|ijk - c_s| - r_s)| < band. 0 or 1 (no memory). */
int orc_gen_spheres(orc_tree *t, const double *spheres, uint32_t count, double band);
/* Level-set values (n3 * 512 floats, DFS leaf order, voxel x<<6 | y<<3 | z) of the sphere
 * union: min_s(|ijk - c_s| - r_s) clamped to [-band, band]. 0 or 1 (no memory). */
int orc_gen_spheres_values(const orc_tree *t, const double *spheres, uint32_t count, double band, float *out);
/* set_voxel(origin + (v >> 6, v >> 3 & 7, v & 7), 1) for every set bit v of mask. */
void orc_set_leaf(orc_tree *t, const int32_t origin[3], const uint64_t mask[8]);
/* 3-octave value-noise leaves of [lo, lo + extent)^3 at the given occupancy, voxels
 * active with probability p_voxel; only leaves with every origin coordinate in
 * [box_lo, box_hi) are set (all when box_lo >= box_hi). Returns the leaves kept in the
 * whole domain, -1 on bad arguments or no memory. */
int64_t orc_gen_noise_leaves(orc_tree *t, int32_t lo, uint32_t extent, double occupancy, double p_voxel,
                             uint64_t seed, int32_t box_lo, int32_t box_hi);
/* count eyes uniform on the sphere of the given radius, |y| <= 0.9 radius (float x, y, z). */
void orc_orbit_eyes(uint32_t count, float radius, uint64_t seed, float *eyes);

/* ---- the raycast pass (raycast.comp.wgsl:60-519) ---- */
/* Renders the (8*floor(W/8)) x (4*floor(H/4)) pixels the dispatch covers.
 * rgba: W*H*4 bytes (row-major, y*W + x); hits/stats may be NULL.
 * nthreads <= 1 runs on the calling thread. Returns 0 on success. */
int orc_render(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
               uint8_t *rgba, orc_hit *hits, orc_stats *stats, int nthreads);
/* Same, restricted to the pixel tiles [tile_begin, tile_end) of the 8x4 tile grid. */
int orc_render_tiles(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
                     uint64_t tile_begin, uint64_t tile_end, uint8_t *rgba, orc_hit *hits,
                     orc_stats *stats, int nthreads);
/* Same, for an explicit list of tile indices (row-major over the 8x4 tile grid). */
int orc_render_tile_list(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
                         const uint64_t *tiles, uint64_t ntiles, uint8_t *rgba, orc_hit *hits,
                         orc_stats *stats, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
