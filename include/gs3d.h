/*
 * gs3d.h - C ABI of the GB300 (sm_103a) Gaussian-splat rebin library.
 *
 * The library replaces the per-frame rebin path of the webgpu-3dgs renderer
 * (src/renderers/GaussianSplatRenderer.ts:1104-1266):
 *
 *   preprocess -> exclusive prefix scan -> (tile|depth) key emit
 *   -> 64-bit LSD radix sort -> tile-range identify -> tiled alpha-blend raster
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (GS3D_OK = 0).  Work is stream ordered and asynchronous: a call returns once
 * its kernels are enqueued.  Device-side failures (key capacity overflow, a
 * bounded spin that ran out) are latched in a device word and reported by the
 * next gs3d_synchronize() or copy-out.  A context is single-threaded, like the
 * JavaScript thread that drives the reference renderer; separate contexts may
 * be driven from separate threads.
 *
 * Buffer layouts are the reference's: the four splat arrays of SceneSyncer
 * (vec4 f32 each), the 64-byte ProjectedSplat, interleaved u32 [hi, lo] sort
 * keys, u32 sort values, u32 tile_offsets[T+1] and an rgba16float image.
 */
#ifndef GS3D_H
#define GS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS3D_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define GS3D_OK                0
#define GS3D_ERR_INVALID_ARG   1  /* null pointer, bad size, bad enum        */
#define GS3D_ERR_OOM           2  /* cudaMalloc / pinned allocation failed   */
#define GS3D_ERR_CAPACITY      3  /* live ref count exceeded the key buffers;
                                     capacity has been grown, re-run rebin   */
#define GS3D_ERR_CUDA          4  /* any other CUDA runtime error            */
#define GS3D_ERR_TIMEOUT       5  /* a bounded device spin gave up           */
#define GS3D_ERR_STATE         6  /* call order: e.g. raster before rebin    */
#define GS3D_ERR_NO_DEVICE     7  /* no CUDA device / wrong architecture     */

/* ---- plain-old-data types mirrored from the reference ------------------ */

/* CameraUniforms (src/shaders/compute/preprocess_splats.wgsl:1-8), filled by
 * Camera.getUniformData (src/Camera.ts:172-191): column-major f32 mat4s. */
typedef struct gs3d_camera {
    float view[16];
    float projection[16];
    float inverse_view[16];
    float inverse_projection[16];
    float position[4];   /* x, y, z, 1                       */
    float viewport[4];   /* width, height, width/height, 0   */
} gs3d_camera;

/* ProjectedSplat (preprocess_splats.wgsl:18-31), stride 64 bytes
 * (src/types/config.ts:2). */
typedef struct gs3d_projected_splat {
    float mean_px[2];
    float depth;         /* view-space z (negative in front)  */
    float radius_px;
    float conic[3];
    float opacity;
    float color[3];
    uint32_t valid;
    uint32_t tile_min[2];
    uint32_t tile_max[2];
} gs3d_projected_splat;

typedef struct gs3d_config {
    int      device;              /* CUDA ordinal                                  */
    uint32_t tile_w, tile_h;      /* tile pixel size; 0 -> 16x16 (Scene.ts:6)      */
    uint32_t max_tiles_per_splat; /* initial key capacity = N * this; 0 -> 16
                                     (config.ts:4).  Grown on overflow, never
                                     truncated.                                    */
    void*    stream;              /* cudaStream_t to enqueue on; NULL -> the
                                     library creates a non-blocking stream         */
    uint32_t flags;               /* GS3D_FLAG_* bits                              */
} gs3d_config;

/* gs3d_rebin runs the fused path by default: the four depth-digit passes of
 * the LSD sort are applied to the N splats before their refs are expanded
 * (every ref of a splat shares its depth), refs are emitted in depth order
 * and only the tile-id digits are sorted over the R refs.  The result (sorted
 * keys, values, tile_offsets, image) is identical to the stage-wise path; the
 * stage-wise path additionally leaves splat_ref_offsets in splat order.  This
 * flag selects the stage-wise path (the six reference stages in order). */
#define GS3D_FLAG_STAGEWISE_REBIN 1u
/* Records a CUDA event pair around every stage on the context's stream;
 * gs3d_read_stage_times returns the accumulated device time per stage. */
#define GS3D_FLAG_STAGE_TIMING    2u
/* Fused rebins (gs3d_rebin, gs3d_rebin_batch) run as a CUDA graph: the
 * first rebin of a batch layout (views, scenes, sizes, tile size, schedule,
 * buffer allocations) runs once eagerly and is captured; later rebins of the
 * same layout only rewrite the view table and replay the graph.  Stage
 * timing events are not recorded in graph mode. */
#define GS3D_FLAG_CUDA_GRAPH      4u
/* Shades every tile of the two-pixel raster as half-strip work items (the
 * split the key-count and learned schedules give their heaviest tiles), for
 * tests and measurements.  The image is unchanged. */
#define GS3D_FLAG_SPLIT_ALL_TILES 8u

/* Stage indices of gs3d_read_stage_times (the reference's profiler labels,
 * GaussianSplatRenderer.ts:1144-1260, plus the fused path's depth sort). */
#define GS3D_STAGE_PREPROCESS 0  /* preprocess-splats                         */
#define GS3D_STAGE_DEPTH_SORT 1  /* fused path: per-splat depth digits        */
#define GS3D_STAGE_SCAN       2  /* prefix-scan-*                             */
#define GS3D_STAGE_EMIT       3  /* emit-tile-refs                            */
#define GS3D_STAGE_SORT       4  /* radix-* (fused path: tile digits only)    */
#define GS3D_STAGE_IDENTIFY   5  /* identify-tile-ranges                      */
#define GS3D_STAGE_RASTER     6  /* rasterize-tiles                           */
#define GS3D_STAGE_COUNT      7

/* One view of a batched rebin (extension: the reference renders one view per
 * frame).  scene 0 is the gs3d_set_splats scene; others come from
 * gs3d_add_scene. */
typedef struct gs3d_view {
    gs3d_camera camera;
    uint32_t scene;
    uint32_t width, height;
    uint32_t reserved;
} gs3d_view;

/* Where a view of the last rebin lives in the batch-wide buffers: its image
 * starts at pixel pixel_offset of the splat target, its tiles are global
 * tiles [tile_base, tile_base + tiles_x*tiles_y) of tile_offsets, its
 * splat-views are [splat_base, splat_base + splat_count) of projected_splats,
 * and its sorted values hold splat_base + splat id. */
typedef struct gs3d_view_info {
    uint64_t pixel_offset;
    uint32_t width, height;
    uint32_t tiles_x, tiles_y, tile_base;
    uint32_t splat_base, splat_count;
    uint32_t scene;
} gs3d_view_info;

/* Raster work order (the persistent raster CTAs pull tiles from a queue).
 * The key-count and learned orders also split: tiles whose expected cost
 * per strip exceeds half of one raster CTA's fair share of the frame (the
 * head of the order) are shaded as two half-strip work items per strip.
 * The learned order falls back to the key count on its own while the
 * measured prediction error exceeds its bound (gs3d_set_schedule_gate). */
#define GS3D_SCHEDULE_ROW_MAJOR 0u  /* the reference's dispatch order          */
#define GS3D_SCHEDULE_KEY_COUNT 1u  /* decreasing key count (longest first)    */
#define GS3D_SCHEDULE_LEARNED   2u  /* decreasing cost predicted by the cost
                                       MLP (gs3d_set_cost_model)               */

/* State of the raster schedule after the last rebin (extension). */
typedef struct gs3d_schedule_status {
    uint32_t schedule;     /* requested GS3D_SCHEDULE_*                             */
    uint32_t active;       /* order the last raster ran in: GS3D_SCHEDULE_KEY_COUNT
                              when the learned schedule's gate fell back           */
    float mae_log;         /* running mean |predicted - measured log(1 + cost)| over
                              all tiles (each frame weighted 1/4, the first as is)  */
    float last_mae_log;    /* the last learned frame's                              */
    float bound;           /* the gate's bound on mae_log                           */
    uint32_t frames;       /* learned frames measured since gs3d_set_cost_model     */
    uint32_t fallbacks;    /* of those, frames rendered in key-count order          */
    uint32_t split_tiles;  /* tiles of the last raster shaded as half strips        */
} gs3d_schedule_status;

/* Cost MLP (extension): 16 tile features -> 64 -> 64 -> 1, ReLU, predicting
 * log(1 + raster cost), the cost being the splats a tile's CTA iterates
 * before its last pixel terminates.  Parameters are f32, in this order:
 * W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3. */
#define GS3D_MLP_FEATURES 16
#define GS3D_MLP_HIDDEN   64
#define GS3D_MLP_PARAMS   (64 * 16 + 64 + 64 * 64 + 64 + 64 + 1)

/* Named device buffers (BufferManager names, GaussianSplatRenderer.ts:338-465). */
typedef enum gs3d_buffer {
    GS3D_BUF_SPLAT_POSITIONS   = 0,  /* vec4 f32 x N                               */
    GS3D_BUF_SPLAT_SCALES      = 1,
    GS3D_BUF_SPLAT_ROTATIONS   = 2,  /* (w, x, y, z)                               */
    GS3D_BUF_SPLAT_COLORS      = 3,  /* rgba                                       */
    GS3D_BUF_SPLAT_SH_REST     = 4,  /* f32 x N x 3*((deg+1)^2-1), f_rest order    */
    GS3D_BUF_PROJECTED_SPLATS  = 5,  /* gs3d_projected_splat x N                   */
    GS3D_BUF_SPLAT_REF_COUNTS  = 6,  /* u32 x N                                    */
    GS3D_BUF_SPLAT_REF_OFFSETS = 7,  /* u32 x (N+1), [N] = total                   */
    GS3D_BUF_REF_COUNTER       = 8,  /* u32 x 1 (live ref count R)                 */
    GS3D_BUF_SORT_KEYS_A       = 9,  /* u32 [hi=tile, lo=bits(-depth)] x capacity;
                                        holds the sorted keys after a rebin        */
    GS3D_BUF_SORT_VALUES_A     = 10, /* u32 splat id x capacity (sorted)           */
    GS3D_BUF_SORT_KEYS_B       = 11, /* ping-pong partner                          */
    GS3D_BUF_SORT_VALUES_B     = 12,
    GS3D_BUF_TILE_OFFSETS      = 13, /* u32 x (T+1)                                */
    GS3D_BUF_SPLAT_TARGET      = 14, /* rgba16float x W x H (premultiplied)        */
    GS3D_BUF_TILE_COSTS        = 15, /* u32 x T: splats iterated before the tile's
                                        last pixel terminated (extension)          */
    GS3D_BUF_COUNT_            = 16
} gs3d_buffer;

/* ---- lifetime ----------------------------------------------------------- */

/* GaussianSplatRenderer constructor + init (GaussianSplatRenderer.ts:331-471). */
int gs3d_create(struct gs3d_ctx** out_ctx, const gs3d_config* cfg);
int gs3d_destroy(struct gs3d_ctx* ctx);
/* Human-readable text of the last failing call on this context (never NULL);
 * with ctx == NULL, of the calling thread's last failing context-free call. */
const char* gs3d_last_error(const struct gs3d_ctx* ctx);
int gs3d_abi_version(void);

/* ---- scene ---------------------------------------------------------------- */

/* SceneSyncer.setSplatData (src/SceneSyncer.ts:25-38): copies the splat SoA
 * (vec4 f32 per splat) into library-owned device buffers.  sh_rest may be NULL
 * (degree 0, the reference's only colour path); otherwise it holds
 * 3*((sh_degree+1)^2-1) floats per splat in PLY f_rest order
 * (src/workers/SceneWorker.ts:457-463).  memory: 0 = host pointers,
 * 1 = device pointers.  Binning buffers are resized as in
 * GaussianSplatRenderer.resizeBinningBuffers (:209-227). */
int gs3d_set_splats(struct gs3d_ctx* ctx, uint32_t n,
                    const float* positions, const float* scales,
                    const float* rotations, const float* colors,
                    const float* sh_rest, uint32_t sh_degree, int memory);

/* Adds another resident scene for batched rendering (extension; the
 * reference holds one scene).  Arguments as gs3d_set_splats; the first scene
 * added to an empty context becomes scene 0. */
int gs3d_add_scene(struct gs3d_ctx* ctx, uint32_t n,
                   const float* positions, const float* scales,
                   const float* rotations, const float* colors,
                   const float* sh_rest, uint32_t sh_degree, int memory,
                   uint32_t* out_scene);

/* setTileSize (GaussianSplatRenderer.ts:301-317): clamps to the device limit
 * (tile_w * tile_h <= 1024) and reports the size in use. */
int gs3d_set_tile_size(struct gs3d_ctx* ctx, uint32_t tile_w, uint32_t tile_h,
                       uint32_t* out_tile_w, uint32_t* out_tile_h);

/* The uniform writes at the top of rebin (GaussianSplatRenderer.ts:1112-1131)
 * plus Viewport's camera upload (src/Viewport.ts:183): sets the camera and the
 * viewport; resizes tile_offsets and the splat target on a viewport change
 * (resizeViewportTargets, :231-295). */
int gs3d_set_camera(struct gs3d_ctx* ctx, const gs3d_camera* cam,
                    uint32_t width, uint32_t height);

/* ---- stages (rebin, GaussianSplatRenderer.ts:1143-1265) ------------------- */
int gs3d_preprocess(struct gs3d_ctx* ctx);          /* preprocess_splats.wgsl      */
int gs3d_prefix_scan(struct gs3d_ctx* ctx);         /* prefix_scan_{local,blocks,add} */
int gs3d_emit_tile_refs(struct gs3d_ctx* ctx);      /* emit_tile_refs.wgsl         */
int gs3d_radix_sort(struct gs3d_ctx* ctx);          /* radix_{histogram,scatter}, scan_{local,add} */
int gs3d_identify_tile_ranges(struct gs3d_ctx* ctx);/* identify_tile_ranges.wgsl   */
int gs3d_rasterize_tiles(struct gs3d_ctx* ctx);     /* rasterize_tiles.wgsl        */

/* rebin (GaussianSplatRenderer.ts:1104-1266): set_camera + all six stages. */
int gs3d_rebin(struct gs3d_ctx* ctx, const gs3d_camera* cam,
               uint32_t width, uint32_t height);

/* Replaces the context's GS3D_FLAG_* bits. */
int gs3d_set_flags(struct gs3d_ctx* ctx, uint32_t flags);

/* With GS3D_FLAG_STAGE_TIMING: waits for the recorded stages, writes the
 * device milliseconds and stage executions accumulated since the last call
 * (GS3D_STAGE_COUNT entries each; either pointer may be NULL) and resets. */
int gs3d_read_stage_times(struct gs3d_ctx* ctx, double* ms, uint32_t* executions);

/* Batched rebin (extension): renders n_views views, of any resident scenes
 * and sizes, in one launch sequence.  Per view the sorted keys (hi = the
 * view's tile_base + local tile id), values (splat_base + splat id),
 * tile_offsets and image equal a single-view rebin of that view. */
int gs3d_rebin_batch(struct gs3d_ctx* ctx, const gs3d_view* views, uint32_t n_views);
int gs3d_get_view_info(struct gs3d_ctx* ctx, uint32_t view, gs3d_view_info* out);

/* Selects the raster work order (GS3D_SCHEDULE_*); the image is the same
 * under every schedule.  GS3D_SCHEDULE_LEARNED needs a cost model. */
int gs3d_set_schedule(struct gs3d_ctx* ctx, uint32_t schedule);

/* ---- tuning (extension) -----------------------------------------------------
 * Knobs that change the speed of a rebin but never its image: for the same
 * cameras every tuning renders bit-identical pixels (a pixel blends the
 * splats whose radius circle covers it in (depth, splat id) order, whatever
 * the tile grid), while the tile grid, key layout and tile_offsets follow
 * tile_w x tile_h. */
typedef struct gs3d_tuning {
    uint32_t tile_w, tile_h;  /* tile pixel size: up to 1024 pixels, or up to 2048
                                 with tile_w a multiple of 8 and tile_h of 16 (such
                                 tiles are shaded by the culled two-pixel raster
                                 only: the stage-wise rebin rejects them)             */
    uint32_t digit_bits;      /* widest radix digit of the tile-id passes: 4, 6, 8 or
                                 11 (fused rebin; the stage-wise sort uses at most 8);
                                 8 when narrower digits would need over 4 passes     */
    uint32_t raster_batch;    /* splats staged per raster batch: a multiple of 32 in
                                 [32, 1024]; 0 = one per tile pixel (at most 1024)    */
} gs3d_tuning;

typedef struct gs3d_tune_result {
    gs3d_tuning tuning;
    float ms_per_view;        /* device time of one batched rebin / views             */
    uint32_t tile_passes;     /* radix passes over the refs under this tuning         */
    uint64_t refs;            /* live ref count of the measured batch                 */
} gs3d_tune_result;

int gs3d_set_tuning(struct gs3d_ctx* ctx, const gs3d_tuning* tuning);
int gs3d_get_tuning(struct gs3d_ctx* ctx, gs3d_tuning* out);

/* Autotuner: times the batched rebin of `views` (warm-up, then `reps` timed
 * repetitions, CUDA events on the context's stream) under every candidate
 * of tile size {8x8, 16x16, 32x32, 32x64, 64x32} x digit width {4, 8, 11} x
 * raster batch {128, 256, 512}, applies the fastest and writes up to max_results
 * measurements (n_results = candidates measured; candidates whose refs
 * exceed the 2^30 limit of one rebin are skipped).  Blocking. */
int gs3d_autotune(struct gs3d_ctx* ctx, const gs3d_view* views, uint32_t n_views,
                  uint32_t reps, gs3d_tune_result* results, uint32_t max_results,
                  uint32_t* n_results);

/* Installs the cost MLP: GS3D_MLP_PARAMS f32 parameters and the per-feature
 * mean and standard deviation the features are normalized with (host
 * pointers). */
int gs3d_set_cost_model(struct gs3d_ctx* ctx, const float* params,
                        const float* feature_mean, const float* feature_std);

/* The learned schedule's fallback gate (extension).  After every learned
 * raster the library compares the model's predictions with the costs the
 * raster recorded (tile_costs) on the device; while the running error
 * exceeds `bound` (mean |log error| over tiles, default 0.5) the next frames
 * are ordered by key count, and the learned order returns once the error is
 * back within the bound.  Installing a model resets the running error. */
int gs3d_set_schedule_gate(struct gs3d_ctx* ctx, float bound);
/* Schedule state after the last rebin (blocking: waits for the stream). */
int gs3d_get_schedule_status(struct gs3d_ctx* ctx, gs3d_schedule_status* out);

/* Raw features (n_tiles x 16 f32) of every tile of the last rebin and, in
 * targets (n_tiles f32, may be NULL), log(1 + measured raster cost).
 * memory: 0 = host pointers (blocking), 1 = device pointers (stream ordered). */
int gs3d_tile_features(struct gs3d_ctx* ctx, float* features, float* targets,
                       uint32_t n_tiles, int memory);

/* Cost-MLP kernels on caller device buffers, enqueued on `stream` (no
 * context): f32 training forward (acts: n x 129 = h1 | h2 | y), backward
 * (grads += d mean((y - target)^2) / d params; zero grads first), Adam step
 * (step >= 1), and bf16 tensor-core inference (mma.sync). */
int gs3d_mlp_forward(const float* params, const float* x, uint32_t n, float* acts, float* y,
                     void* stream);
int gs3d_mlp_backward(const float* params, const float* x, const float* acts,
                      const float* target, uint32_t n, float* grads, void* stream);
int gs3d_mlp_adam(float* params, float* m, float* v, const float* grads, uint32_t count,
                  float lr, float beta1, float beta2, float eps, uint32_t step, void* stream);
int gs3d_mlp_infer(const float* params, const float* x, uint32_t n, float* y, void* stream);

/* Waits for the context's stream and reports latched device errors.  After
 * GS3D_ERR_CAPACITY the key buffers have already been grown to the observed
 * ref count; re-issue the rebin. */
int gs3d_synchronize(struct gs3d_ctx* ctx);

/* ---- PLY ingest (SceneWorker.ts:146-550) ------------------------------------- */

#define GS3D_PLY_ASCII      0u
#define GS3D_PLY_BINARY_LE  1u
#define GS3D_PLY_BINARY_BE  2u
#define GS3D_PLY_NEW_SCENE  0xffffffffu  /* gs3d_load_ply target: add a scene */

typedef struct gs3d_ply_info {
    uint64_t splat_count;     /* vertex rows                                          */
    uint64_t header_bytes;    /* through the newline after end_header                 */
    uint32_t format;          /* GS3D_PLY_*                                           */
    uint32_t f_rest_count;    /* f_rest_* properties of the vertex element            */
    uint32_t sh_degree;       /* inferred from f_rest_count (SceneWorker.ts:501-506)  */
    uint32_t vertex_stride;   /* bytes per binary vertex row (0 for ASCII)            */
    float bounds_min[3];      /* position bounds (gs3d_load_ply only)                 */
    float bounds_max[3];
} gs3d_ply_info;

/* Parses and validates the header of a Gaussian-splat PLY held in host
 * memory (no device, no context): formats ascii / binary_little_endian /
 * binary_big_endian, the 14 required vertex properties, no list properties.
 * Errors: GS3D_ERR_INVALID_ARG with the reference's message in
 * gs3d_last_error(NULL). */
int gs3d_ply_inspect(const void* data, size_t size, gs3d_ply_info* out);

/* Loads a Gaussian-splat PLY (host memory) into the context: the vertex rows
 * are copied to the device and decoded and activated there (positions, colors
 * = clamp01(0.5 + C0 f_dc) and clamp01(sigmoid(opacity)), scales = exp,
 * rotations normalised, computed in f64 and rounded to f32; f_rest kept in
 * file order).  target 0 replaces the gs3d_set_splats scene;
 * GS3D_PLY_NEW_SCENE adds a scene (its id in *out_scene).  SH is used for
 * colour when the f_rest count is 3 * ((d+1)^2 - 1) for the inferred degree
 * d, or a larger multiple of 3 (the first coefficients of each channel). */
int gs3d_load_ply(struct gs3d_ctx* ctx, const void* data, size_t size, uint32_t target,
                  uint32_t* out_scene, gs3d_ply_info* info);

/* ---- headless composite (render passes after the rasterizer) ------------------ */

#define GS3D_COMPOSITE_SPLATS       0u  /* composite_splats.wgsl                       */
#define GS3D_COMPOSITE_TILE_HEATMAP 1u  /* debug_tile_overlay.wgsl, then the composite */

/* Composites view `view` of the last rebin over `background` (premultiplied
 * rgba; the reference's framebuffer holds the grid pass there) with the
 * premultiplied "over" blend of the composite pass, into width x height RGBA8
 * pixels (round(clamp01(x) * 255), row-major, top row first).  Mode
 * GS3D_COMPOSITE_TILE_HEATMAP first tints each tile green -> red by its key
 * count / debug_ref (0 -> 256, GaussianSplatRenderer.ts:75) at 40% opacity,
 * through an rgba16float target as the overlay pass does.  memory: 0 = host
 * destination (blocking), 1 = device destination (stream ordered).  `bytes`
 * must be at least width * height * 4. */
int gs3d_composite(struct gs3d_ctx* ctx, uint32_t view, uint32_t mode, uint32_t debug_ref,
                   const float background[4], void* rgba8, size_t bytes, int memory);

/* ---- buffer access ---------------------------------------------------------- */

/* Device pointer and size in bytes of a named buffer (for zero-copy callers). */
int gs3d_buffer_info(struct gs3d_ctx* ctx, gs3d_buffer which,
                     void** device_ptr, size_t* bytes);
/* Blocking copy-out of the first `bytes` bytes of a named buffer. */
int gs3d_read_buffer(struct gs3d_ctx* ctx, gs3d_buffer which,
                     void* host_dst, size_t bytes);
/* Blocking copy-out of bytes [offset, offset + bytes) of a named buffer. */
int gs3d_read_buffer_range(struct gs3d_ctx* ctx, gs3d_buffer which, size_t offset,
                           void* host_dst, size_t bytes);
/* Blocking copy-in (stage-wise parity: feed another implementation's
 * intermediate buffer into the next stage). */
int gs3d_write_buffer(struct gs3d_ctx* ctx, gs3d_buffer which,
                      const void* host_src, size_t bytes);
/* Stream-ordered copy-out of the first `bytes` bytes of a named buffer into
 * host memory (asynchronous when host_dst is page-locked).  The copy lands
 * once gs3d_synchronize returns.  Replaces the reference's staging-buffer
 * readback (mapAsync, GaussianSplatRenderer.ts:1287-1295). */
int gs3d_copy_buffer_async(struct gs3d_ctx* ctx, gs3d_buffer which,
                           void* host_dst, size_t bytes);
/* Live ref count of the last rebin (blocking read of ref_counter). */
int gs3d_ref_count(struct gs3d_ctx* ctx, uint32_t* out_count);
/* readTileCounts (GaussianSplatRenderer.ts:1278-1310): per-tile key counts
 * max(0, off[t+1]-off[t]); `n` must be >= tile count. */
int gs3d_read_tile_counts(struct gs3d_ctx* ctx, uint32_t* counts, size_t n);

/* ---- context-free, allocation-free scan ----------------------------------- */

/* No counterpart in the reference.  Exclusive prefix scan of n u32 counts
 * into offsets[0..n] (offsets[n] = total), the same single-pass scan as
 * gs3d_prefix_scan, for callers that cannot let a library allocate device
 * memory: applications whose GPU memory belongs to their own pool or caching
 * allocator, and frame loops that must not hit the implicit device
 * synchronisation of cudaMalloc/cudaFree.  It allocates nothing and needs no
 * context: the look-back scratch is a fixed 256 KB device array inside the
 * library, held by every GPU that loads it until the process exits.
 *   - counts and offsets are device pointers owned by the caller; the call
 *     enqueues on `stream` (a cudaStream_t, NULL = legacy default stream) on
 *     the current device and returns without waiting;
 *   - n may be at most 67,108,864 (2^26); larger n is rejected with
 *     GS3D_ERR_INVALID_ARG and a message in gs3d_last_error(NULL);
 *   - the first call on each device loads the library's kernels and scratch
 *     array on it, so make it before any stream capture (later calls only
 *     look the scratch address up again, which stays valid across a reset
 *     of the device);
 *   - every call on a device shares the one scratch array: calls whose
 *     kernels overlap on the GPU (different streams, no ordering between
 *     them) race and give wrong offsets; order them on one stream;
 *   - GS3D_OK means the scan was enqueued, not that it succeeded: the device
 *     errors it can meet (a total of 2^32 or more, a look-back wait that gave
 *     up) are latched in the scratch array and reported by
 *     gs3d_prefix_scan_noalloc_status. */
int gs3d_prefix_scan_noalloc(const uint32_t* counts, uint32_t* offsets, uint32_t n,
                             void* stream);
/* No counterpart in the reference.  Device errors of the last
 * gs3d_prefix_scan_noalloc call on the current device, read behind the work
 * already enqueued on `stream` (the call waits for that stream):
 *   GS3D_OK            the offsets are complete and exact;
 *   GS3D_ERR_CAPACITY  the counts sum to 2^32 or more: offsets[n] holds
 *                      0xffffffff and the offsets past the overflow are not
 *                      valid;
 *   GS3D_ERR_TIMEOUT   a bounded look-back wait gave up: the offsets are
 *                      incomplete.
 * Like the scan itself it allocates nothing.  With calls on several streams
 * of one device it reports whichever call wrote the scratch array last. */
int gs3d_prefix_scan_noalloc_status(void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GS3D_H */
