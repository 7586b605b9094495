/*
 * woxel_gb300.h — C ABI of the GB300 (sm_103a) primary-ray pass for woxel's
 * VDB345 grids: an HDDA march with grid-SDF empty-space skipping.
 *
 * The entry points replace woxel's wgpu compute pass (`cp_main`,
 * src/shaders/raycast.comp.wgsl:60-68, dispatched at
 * src/render/wgpu_context.rs:270-282) and the grid upload that feeds it
 * (src/render/wgpu_context.rs:101-159). Inputs keep the reference's own data:
 * the 256-byte ComputeState uniform (src/render/gpu_types/compute_state.rs:9-29)
 * and the flattened VDB345 view (masks()/origins()/atlas(),
 * src/vdb/vdb345.rs:108-264). Outputs are RGBA8 (the rgba8unorm storage texture
 * of src/render/gpu_types/texture.rs:25-75) plus an optional per-pixel hit record.
 *
 * Conventions: every function returns an int status (WX_OK == 0); nothing
 * aborts or throws across this boundary. A context is used from one host
 * thread at a time; grids are immutable after upload and may be used from any
 * stream of the context's device. Pointers named *_dev are device pointers;
 * output pointers of wx_render may be device or host memory (host memory is
 * staged through the context and copied back on the given stream).
 */
#ifndef WOXEL_GB300_H
#define WOXEL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define WX_OK 0
#define WX_ERR_INVALID 1      /* bad argument or malformed grid */
#define WX_ERR_CUDA 2         /* a CUDA runtime call failed */
#define WX_ERR_OOM 3          /* device or host allocation failed */
#define WX_ERR_UNSUPPORTED 4  /* valid input outside what this library handles */
#define WX_ERR_BUDGET 5       /* request does not fit the memory budget */
#define WX_ERR_TIMEOUT 6      /* a bounded wait expired */
#define WX_ERR_CANCELLED 7    /* work was cancelled */

/* ---- render modes (src/render/egui_dev.rs:11-18) ---- */
#define WX_MODE_GRAY 0u
#define WX_MODE_RGB 1u
#define WX_MODE_RAY 2u
#define WX_MODE_DIFFUSE 3u
#define WX_MODE_GLOSSY 4u
/* Extension, no reference counterpart: after the primary HDDA hit, search the
 * zero crossing of the grid's level-set values (wx_grid_set_values) along the
 * ray: samples every 0.25 voxel from 1 voxel before the hit, 64 at most,
 * trilinear values, secant between the last positive and the first
 * non-positive sample; Lambert colour of mode 3 with the trilinear gradient as
 * normal and no shadow ray. wx_hit: p, t, node and info of the HDDA hit;
 * shadow = found | sample index << 8; reserved = the crossing's t as float
 * bits (NaN when none was found, and the colour is then mode 0's). */
#define WX_MODE_SURFACE 5u

/* 256-byte uniform; field order and padding of ComputeState
 * (src/render/gpu_types/compute_state.rs:9-29). Matrices are column-major. */
typedef struct wx_state_uniform {
    float view_projection[16];
    float camera_to_world[16];
    float eye[4];
    float u[4];
    float mv[4];
    float wp[4];
    uint32_t render_mode[4];
    uint32_t show_345[4];
    float sun_dir[4];
    float sun_color[4]; /* alpha = intensity */
} wx_state_uniform;

/* Per-pixel result of the primary ray (no counterpart in the reference,
 * which only writes colour). 32 bytes. */
typedef struct wx_hit {
    float p[3];        /* march position when hdda_ray returned; floor(p) is the voxel ijk */
    float t;           /* dot(p - eye, dir) = ((dx*dir.x + dy*dir.y) + dz*dir.z), FP32 */
    uint32_t node;     /* DFS pool index of the deepest cached node (the leaf when
                          level == 3); 0xFFFFFFFF when level == 0 */
    uint32_t info;     /* bits 0-1 state (0 hit, 1 out of bounds, 2 step cap),
                          bits 2-3 level (cached parents, 0..3), bits 4-6 last step
                          mask x,y,z, bits 8-18 loop iteration i */
    uint32_t shadow;   /* mode 3: bit 0 shadow ray traced, bits 1-2 its state,
                          bits 8-18 its iteration count; 0 otherwise */
    uint32_t reserved;
} wx_hit;

/* The flattened grid exactly as woxel's Rust side holds it:
 *   masks()   src/vdb/vdb345.rs:119-161 (u64 words split lo/hi, DFS order)
 *   origins() src/vdb/vdb345.rs:108-117 (sorted root keys; x,y,z + stride pad)
 *   atlas()   src/vdb/vdb345.rs:163-264 as uploaded by src/render/wgpu_context.rs:119-151:
 *             an R32Uint 3-D texture whose texel (x,y,z) sits at (z*H + y)*W + x. */
typedef struct wx_vdb345_view {
    const uint32_t *kids5, *vals5; /* n5 * 1024 words each */
    const uint32_t *kids4, *vals4; /* n4 * 128 words each */
    const uint32_t *vals3;         /* n3 * 16 words */
    const int32_t *origins;        /* n5 entries of origin_stride int32 (x, y, z, ...) */
    uint64_t n5, n4, n3;
    uint32_t origin_stride;        /* 3 or 4 (the reference's storage buffer uses 4) */
    const uint32_t *atlas[3];      /* N5, N4, N3 atlases */
    uint32_t dims[3][3];           /* W, H, D of each atlas */
} wx_vdb345_view;

typedef struct wx_grid_info {
    uint64_t n5, n4, n3;           /* node counts per level */
    uint64_t device_bytes;         /* bytes of device node pools */
    uint64_t active_voxels;        /* popcount of the leaf value masks */
} wx_grid_info;

typedef struct wx_ctx wx_ctx;
typedef struct wx_grid wx_grid;
typedef struct wx_topology wx_topology;
typedef struct wx_batch wx_batch;

/* Launch shape of the raycast kernels (set per context; see wx_ctx_set_tuning). */
typedef struct wx_tuning {
    int32_t kernel;          /* 1 (default): one warp per pixel tile, one launch per frame,
                                consecutive frames overlapping (see wx_render);
                                0: persistent warps drawing pixel tiles from a queue */
    int32_t warps_per_block; /* 1..8 (default 4) */
    int32_t blocks_per_sm;   /* persistent kernel: 0 = as many as fit */
    int32_t tile_width;      /* pixel tile of one warp: 4, 8 (default: the reference's 8x4
                                workgroup), 16 or 32 wide, 32/tile_width high */
    int32_t tile_order;      /* order in which tile rows are handed out: 0 top to bottom;
                                1 (default) the middle row first, then alternately the rows
                                above and below it, so that the costly centre of a centred
                                view starts first and a frame's last tiles are its cheap
                                edges. The pixels written are the same either way. */
    int32_t rays_per_lane;   /* kernel 1 only, modes 0-3: 1 (default) one pixel per lane;
                                2, 4 or 8: each warp takes that many consecutive tiles and a
                                lane whose ray has ended takes the warp's next pixel, so the
                                march runs with most lanes busy (results are shaded, and
                                shadow rays marched, in the same way afterwards). The pixels
                                written are the same either way. */
} wx_tuning;

/* One frame of a batched launch: a camera uniform over one resident grid. */
typedef struct wx_frame {
    const wx_grid *grid;
    wx_state_uniform state;
    uint32_t width, height;
    uint8_t *rgba8;  /* device memory, width*height*4 bytes */
    wx_hit *hits;    /* device memory or NULL */
} wx_frame;

/* ---- library ---- */
const char *wx_status_string(int status);
/* Last error message of the calling thread (for calls without a context). */
const char *wx_thread_last_error(void);
const char *wx_version(void);

/* ---- context: replaces WgpuContext's device/queue (wgpu_context.rs:38-99) ---- */
int wx_ctx_create(int device, wx_ctx **out);
int wx_ctx_destroy(wx_ctx *ctx);
const char *wx_last_error(const wx_ctx *ctx);

/* ---- grids: replace the atlas/mask upload (wgpu_context.rs:101-159, 506-573) ---- */
/* Drop-in: repack the Rust side's flattened view into device node pools. */
int wx_grid_upload(wx_ctx *ctx, const wx_vdb345_view *view, wx_grid **out);
/* Native: compute the per-level SDF (vdb345.rs:290-670) on the host and pack
 * the pools directly from a topology, without the padded atlas. */
int wx_grid_build(wx_ctx *ctx, wx_topology *topo, wx_grid **out);
/* wx_grid_build with the SDF and the packing on the GPU (compute_sdf,
 * vdb345.rs:290-670): the same device pools word for word. Needs N5 origins
 * that are multiples of 4096 (else WX_ERR_UNSUPPORTED). Temporary device
 * memory: about 4 bytes per leaf voxel plus 200 bytes per node.
 * The sweeps hand containers to CTAs through a ready queue; a CTA whose
 * container is not ready polls for it, at most the context's SDF wait limit
 * (wx_ctx_set_sdf_wait_limit) times, then sets an error flag on which every
 * CTA returns: the call then returns WX_ERR_TIMEOUT, builds no grid and leaves
 * the context usable. */
int wx_grid_build_gpu(wx_ctx *ctx, const wx_topology *topo, wx_grid **out);
/* Bound of wx_grid_build_gpu's waits, in polls 256 ns apart (0 restores the
 * default, 2^23, about 2 s). No counterpart in the reference, whose failures
 * panic (wgpu_context.rs:44-101). */
int wx_ctx_set_sdf_wait_limit(wx_ctx *ctx, uint32_t polls);
/* Fault injection for tests of callers' error paths: the library's next
 * `count` device or page-locked host allocations (grid pools, staging, job
 * tables, server arena and slots, GPU SDF temporaries) fail as an exhausted
 * device would, without calling CUDA: the call reports WX_ERR_OOM, frees what
 * it had allocated and leaves the context usable. 0 stops injecting. */
int wx_inject_alloc_failures(uint32_t count);
int wx_grid_release(wx_ctx *ctx, wx_grid *grid);
/* Attaches level-set values for WX_MODE_SURFACE: one float per leaf voxel
 * (n3 * 512, DFS leaf order, voxel order x<<6 | y<<3 | z), the signed distance
 * in voxel units, negative inside; voxels outside leaves read +band, or -band
 * inside an active tile. Replaces earlier values; freed with the grid. Servers
 * (wx_server_add_grid) and batch plans (wx_batch_create) keep the device view a
 * grid had when they took it: attach values first. Not while a render of the
 * grid is in flight. No reference counterpart (the reference's raycast reads no
 * values). */
int wx_grid_set_values(wx_ctx *ctx, wx_grid *grid, const float *values, float band);
int wx_grid_get_info(const wx_grid *grid, wx_grid_info *out);
/* Copies a grid's device pools to host memory; any pointer may be NULL.
 * slot5: n5*32768 u32, slot4: n4*4096 u32 (bit 31 = child index, else the skip
 * distance, 0 = hit), leaf: n3*512 bytes (0 hit, 1..254 distance, 255 = see
 * ovf), ovf: *n_ovf pairs (leaf << 9 | voxel, distance) sorted by key.
 * No reference counterpart. */
int wx_grid_read_pools(wx_ctx *ctx, const wx_grid *grid, uint32_t *slot5, uint32_t *slot4, uint8_t *leaf,
                       uint32_t *ovf, uint64_t *n_ovf);

/* ---- the raycast pass: replaces cp_main (raycast.comp.wgsl:60-68) ---- */
/* Renders the (8*floor(w/8)) x (4*floor(h/4)) pixels the reference dispatch
 * covers (wgpu_context.rs:281); other pixels are not written. rgba8 holds
 * w*h*4 bytes row-major; hits (w*h records) may be NULL. stream is a
 * cudaStream_t (NULL = legacy default stream). Outputs in device memory or in
 * page-locked host memory are written by the kernel (complete when the stream
 * is synchronised); pageable host outputs are staged on the device and copied
 * back (complete on return).
 * With tuning kernel 1 the frame is a programmatic dependent launch: it may start
 * while the previous kernel on the stream finishes. When that kernel is the
 * previous frame of this library and the outputs of the two frames do not
 * overlap, the new frame writes without waiting for it; otherwise its writes
 * wait for that kernel to complete. Stream order holds either way for the work
 * after the frame. A kernel of the caller's own that lets its dependents start
 * early (programmatic dependent launch) and immediately precedes the frame must
 * not access the frame's outputs. */
int wx_render(wx_ctx *ctx, const wx_grid *grid, const wx_state_uniform *state, uint32_t width,
              uint32_t height, uint8_t *rgba8, wx_hit *hits, void *stream);

/* ---- launch tuning (no counterpart in the reference: wgpu_context.rs:280
 * notes the workgroup choice as a TODO) ---- */
int wx_ctx_set_tuning(wx_ctx *ctx, const wx_tuning *tuning);
int wx_ctx_get_tuning(const wx_ctx *ctx, wx_tuning *tuning);
/* Autotuner: renders `frames` (device outputs, as for wx_render_batch) once per
 * frame with each candidate tuning, reps times after one warm-up pass, timing
 * with CUDA events, and installs the fastest on the context. candidates NULL
 * (ncand ignored) uses the built-in set of WX_AUTOTUNE_BUILTIN candidates: for
 * tile orders 1 then 0, both kernels x tile widths {4, 8, 16} x {2, 4, 8} warps
 * per block at one ray per lane, the persistent kernel at 4 blocks of 4 warps per
 * SM (tile widths 4, 8), and kernel 1 with {2, 4, 8} rays per lane x tile widths
 * {4, 8} x {2, 4} warps per block. times_ms (ncand or WX_AUTOTUNE_BUILTIN
 * entries, may be NULL) receives each candidate's mean time for all frames. */
#define WX_AUTOTUNE_BUILTIN 64
int wx_autotune(wx_ctx *ctx, const wx_frame *frames, uint32_t n, const wx_tuning *candidates, uint32_t ncand,
                uint32_t reps, wx_tuning *best, double *times_ms);

/* ---- batched rendering: many cameras over several resident grids in one
 * persistent launch drawing 8x4 ray tiles from a global queue. Per frame the
 * result equals wx_render's. No counterpart in the reference, which renders
 * one frame per dispatch (wgpu_context.rs:270-282). ---- */
/* One-shot: uploads the frame table and launches on `stream`. */
int wx_render_batch(wx_ctx *ctx, const wx_frame *frames, uint32_t n, void *stream);
/* Plan: the frame table is uploaded once and the launch (queue reset +
 * persistent kernel) is captured in a CUDA graph; wx_batch_launch replays it.
 * Outputs of the frames are rewritten on every launch. */
int wx_batch_create(wx_ctx *ctx, const wx_frame *frames, uint32_t n, wx_batch **out);
int wx_batch_launch(wx_batch *batch, void *stream);
int wx_batch_info(const wx_batch *batch, uint32_t *frames, uint32_t *tiles, uint64_t *rays);
int wx_batch_destroy(wx_batch *batch);

/* ---- batched rendering that allocates nothing (no counterpart in the
 * reference) ----
 * For callers that must not allocate device memory while rendering: engines
 * that reserve all GPU memory at start-up and forbid cudaMalloc afterwards, or
 * code on a deadline (a frame callback) where an allocation could stall or
 * fail. It renders like wx_render_batch (same results per frame) but needs no
 * context and calls no allocating routine: its work-queue counter and frame
 * table live in one fixed device array of WX_NOALLOC_SCRATCH_BYTES that the
 * library declares statically, so every GPU that loads the library holds that
 * memory until the process exits. The caller passes the grids and the device
 * output buffers.
 * Limits: at most WX_NOALLOC_MAX_FRAMES frames per call (more is rejected with
 * WX_ERR_INVALID); all grids on one device, and `stream` a stream of that
 * device (else WX_ERR_INVALID); outputs in device memory; default launch shape
 * (8x4 tiles).
 * The first call on a device does a one-time set-up on that device (it looks
 * up the array's device address and loads the kernels' division table). The
 * frame table reaches the array
 * through the parameters of small table-writing kernels, which the runtime
 * copies when they are enqueued, so the call does not wait for the GPU and a
 * later call cannot change the table of an earlier one. Every call reuses the
 * same array and clears its counter, so calls that overlap on the GPU (on
 * different streams, or from other host threads before earlier work finished)
 * race; the caller must serialise them (calls on one stream are ordered). */
#define WX_NOALLOC_MAX_FRAMES 256
#define WX_NOALLOC_SCRATCH_BYTES 98560 /* 256 + 256 frames x 384-byte table entries */
int wx_render_batch_noalloc(const wx_frame *frames, uint32_t n, void *stream);

/* ---- serving: continuous batching of render requests (no counterpart in the
 * reference, whose render loop draws one frame per window event,
 * src/runtime.rs:97-109). Requests are admitted in arrival order while their
 * output buffers fit the HBM budget, then rendered in time-sliced batches
 * (at most slice_tiles 8x4 tiles per launch, a large request spanning several
 * slices) with up to max_inflight launches in flight, so requests that arrive
 * while others are on the GPU join the next slice. Grids stay resident. ---- */
typedef struct wx_server wx_server;

#define WX_SERVE_FIFO 1u /* baseline: one whole request per launch, one launch in flight */

typedef struct wx_server_config {
    uint64_t budget_bytes;  /* HBM budget: resident grids + the output arena */
    uint32_t max_inflight;  /* launches in flight, 1..8 (default 2) */
    uint32_t slice_tiles;   /* tiles per launch; 0 = 262144 (four 1080p frames) */
    uint32_t max_frames;    /* request pieces per launch, 1..1024 (default 256) */
    uint32_t flags;         /* WX_SERVE_FIFO */
} wx_server_config;

typedef struct wx_request {
    uint32_t grid_id;       /* from wx_server_add_grid */
    uint32_t want_hits;     /* nonzero: also produce wx_hit records */
    uint32_t width, height;
    wx_state_uniform state;
    uint64_t user;          /* returned unchanged in the result */
} wx_request;

typedef struct wx_result {
    uint64_t ticket, user;
    int32_t status;         /* WX_OK, or WX_ERR_CANCELLED */
    uint32_t width, height;
    const uint8_t *rgba8;   /* device memory in the server's arena, valid until wx_server_release */
    const wx_hit *hits;     /* NULL unless requested */
    double t_submit, t_admit, t_done; /* seconds on the server's steady clock */
} wx_result;

typedef struct wx_server_stats {
    uint64_t submitted, completed, cancelled, launches;
    uint64_t rays_done;        /* dispatched pixels of completed requests */
    uint64_t arena_bytes, arena_in_use, arena_peak;
    uint64_t pending, active;
    uint64_t tiles_cancelled_queued;   /* tiles of cancelled requests never launched */
    uint64_t tiles_cancelled_launched; /* tiles skipped by launches already on the GPU */
} wx_server_stats;

/* Creates the scheduler and allocates the output arena (budget minus the
 * grids added later is checked at admission). */
int wx_server_create(wx_ctx *ctx, const wx_server_config *cfg, wx_server **out);
/* Registers a resident grid; its device bytes count against the budget. The
 * server keeps the grid's device view as it is now (level-set values included). */
int wx_server_add_grid(wx_server *srv, const wx_grid *grid, uint32_t *grid_id);
/* Queues a request (never blocks on the GPU). WX_ERR_BUDGET if it could never fit. */
int wx_server_submit(wx_server *srv, const wx_request *req, uint64_t *ticket);
/* Cancels a request (its result reports WX_ERR_CANCELLED and has no buffers).
 * Pending: it is never admitted. Admitted: its tiles not yet launched are
 * dropped, and launches already on the GPU skip its remaining tiles as soon as
 * the cancellation reaches the device (a cancel table the batched kernel reads
 * before each tile, written concurrently with the launches); the result arrives
 * once no launch refers to the request. The other requests are not affected.
 * WX_ERR_INVALID for an unknown or already finished request. The reference has
 * no counterpart (its render loop cannot stop a dispatch). */
int wx_server_cancel(wx_server *srv, uint64_t ticket);
/* Moves up to max finished results into out; waits up to wait_ms for the first. */
int wx_server_poll(wx_server *srv, wx_result *out, uint32_t max, uint32_t *n, int wait_ms);
/* Copies a polled result's rgba8 (width*height*4 bytes) and, if requested,
 * hits (width*height records) into host memory; either pointer may be NULL. */
int wx_server_copy_result(wx_server *srv, uint64_t ticket, uint8_t *rgba8_host, wx_hit *hits_host);
/* Returns a finished request's buffers to the arena. */
int wx_server_release(wx_server *srv, uint64_t ticket);
int wx_server_get_stats(wx_server *srv, wx_server_stats *out);
/* Open-loop replay: submits reqs[i] at arrival_s[i] seconds after the call,
 * collects every result into results[i] (in request order), releasing buffers
 * as results arrive when release != 0. Returns when all have finished or
 * timeout_s elapses (WX_ERR_TIMEOUT). */
int wx_server_replay(wx_server *srv, const wx_request *reqs, const double *arrival_s, uint32_t n,
                     wx_result *results, int release, double timeout_s);
/* Stops the scheduler (waits for in-flight launches) and frees the arena. */
int wx_server_destroy(wx_server *srv);

/* Exhaustive GPU check of the kernels' fast floor(p / size) path against IEEE
 * division: every divisor m < max_m (<= 4096) and every significand of
 * [1,2) and [-2,-1). out = {mismatches, first bad m, its x bits}. */
int wx_check_division(wx_ctx *ctx, uint32_t max_m, uint64_t out[3]);

/* Bounds-checked build (libwoxel_gb300_checked.so, compiled with
 * WX_BOUNDS_CHECK): every node-pool index the raycast kernels use and every
 * pixel they write is compared with its pool or frame size; an index out of
 * range is counted, never accessed (the ray ends), and no kernel traps. Returns
 * in *count the number counted on the context's device since the last call and
 * resets it, after waiting for the device. The normal build returns
 * WX_ERR_UNSUPPORTED. */
int wx_bounds_violations(wx_ctx *ctx, uint64_t *count);

/* ---- host-side helpers (no GPU needed) ---- */
/* ComputeState::build (compute_state.rs:87-131) for a look_at_rh camera
 * (camera.rs:31-35). show_345 may be NULL. */
int wx_state_build(const float eye[3], const float target[3], const float up[3], float aspect,
                   float fovy_deg, float resolution_width, uint32_t render_mode,
                   const uint32_t show_345[3], const float sun_dir[3], const float sun_color[3],
                   float sun_intensity, wx_state_uniform *out);
/* SunSettings::default (egui_dev.rs:355-368). */
void wx_sun_default(float dir[3], float color[3], float *intensity);

/* Topology: the node structure of a VDB345 grid (child/value masks, DFS order). */
int wx_topology_from_masks(const uint32_t *kids5, const uint32_t *vals5, uint64_t n5,
                           const uint32_t *kids4, const uint32_t *vals4, uint64_t n4,
                           const uint32_t *vals3, uint64_t n3, const int32_t *origins,
                           uint32_t origin_stride, wx_topology **out);
/* As set_voxel (vdb345.rs:26-66) on each ijk. */
int wx_topology_from_voxels(const int32_t *ijk, uint64_t n, wx_topology **out);
/* Leaves given as 8-aligned origins (x,y,z) and 8 u64 value-mask words each. */
int wx_topology_from_leaves(const int32_t *origins, const uint64_t *masks, uint64_t n,
                            wx_topology **out);
void wx_topology_free(wx_topology *topo);
int wx_topology_counts(const wx_topology *topo, uint64_t counts[3]);
uint64_t wx_topology_active_voxels(const wx_topology *topo);
/* masks()/origins() export; origins written with stride 4 (x,y,z,0). */
int wx_topology_masks(const wx_topology *topo, uint32_t *kids5, uint32_t *vals5,
                      uint32_t *kids4, uint32_t *vals4, uint32_t *vals3, int32_t *origins);
/* compute_sdf (vdb345.rs:290-670); nthreads <= 0 picks the hardware count. */
int wx_topology_sdf(wx_topology *topo, int nthreads);
/* atlas() export in the uploaded texture layout; side[3] = 32*d5, 16*d4, 8*d3.
 * Pass NULL atlases to query sides. Leaf value texels are written as value_texel. */
int wx_topology_atlas(const wx_topology *topo, uint32_t side[3], uint32_t *a5, uint32_t *a4,
                      uint32_t *a3, uint32_t value_texel);

/* ---- OpenVDB files: VdbReader::new + read_vdb345_grid (src/vdb/read.rs:62-349) ----
 * Reads the tree topology of one grid (grid_name NULL = the first) of an
 * uncompressed, active-mask-compressed or zip (zlib) compressed file (the
 * reference's assets use flag 2: active mask, half-float values; zip buffers are
 * decoded as read.rs:546-563 decodes them). Leaf values are not read: the march
 * only uses the value masks. Blosc-compressed grids give WX_ERR_UNSUPPORTED. */
typedef struct wx_vdb_info {
    uint32_t file_version, compression, half_float, reserved;
    int64_t file_voxel_count; /* grid metadata "file_voxel_count", -1 if absent */
    char grid_name[64];
} wx_vdb_info;
int wx_vdb_read_topology(const char *path, const char *grid_name, wx_topology **out, wx_vdb_info *info);
/* The grid's leaf values (the tree-data section, read.rs:571-629) in the layout
 * of wx_grid_set_values: n3 * 512 floats in DFS leaf order (half-float files
 * converted). Inactive voxels the file leaves implicit read +background, or
 * -background where the node's metadata says so (the OpenVDB format's rule; the
 * reference reader leaves them zero). values NULL: only *count (n3 * 512) and
 * *background are returned. */
int wx_vdb_read_leaf_values(const char *path, const char *grid_name, float *values, uint64_t capacity,
                            uint64_t *count, float *background);

/* ---- synthetic grids (seeded; f32 narrow-band level sets use value = signed distance) ---- */
/* Voxels with |(|ijk - c| - r)| < band are active. */
int wx_gen_sphere(float cx, float cy, float cz, float radius, float band, wx_topology **out);
/* Union of `count` spheres, radii U[rmin, rmax], centres U[lo, hi)^3. */
int wx_gen_spheres(uint32_t count, float rmin, float rmax, float lo, float hi, float band,
                   uint64_t seed, wx_topology **out);
/* Level-set values of those generators for every leaf voxel of `topo` (the
 * layout of wx_grid_set_values): min over the spheres of |ijk - c| - r,
 * clamped to [-band, band]. Same arguments as the generator that built topo. */
int wx_gen_sphere_values(const wx_topology *topo, float cx, float cy, float cz, float radius, float band,
                         float *values);
int wx_gen_spheres_values(const wx_topology *topo, uint32_t count, float rmin, float rmax, float lo, float hi,
                          float band, uint64_t seed, float *values);
/* Leaves on the 8^3 lattice of [lo, lo + extent)^3 kept where 3-octave value
 * noise exceeds the quantile giving `occupancy`; voxels active with p_voxel. */
int wx_gen_noise_leaves(int32_t lo, uint32_t extent, double occupancy, double p_voxel,
                        uint64_t seed, int nthreads, wx_topology **out);
/* Orbit eyes at `radius` around the origin, directions uniform on the sphere
 * with |y| <= 0.9 * radius (keeps look_at_rh's +y up well conditioned). */
int wx_orbit_eyes(uint32_t count, float radius, uint64_t seed, float *eyes_xyz);

#ifdef __cplusplus
}
#endif
#endif
