/*
 * gs_oracle.h - CPU restatement of the webgpu-3dgs rebin path.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests compare the CUDA library with this code,
 * and it is the timed CPU baseline; it is never linked into, loaded by, or called from
 * the library's product path.
 *
 * Parity status: UNPINNED against executable reference output.  The reference
 * is WGSL run through WebGPU, which cannot execute in this environment, and it
 * ships no tests, fixtures or golden vectors.  Each function below restates
 * one WGSL/TypeScript source (cited file:line) with an explicit f32 operation
 * order; hand-derived known-answer tests pin the restatement to the WGSL text.
 */
#ifndef GS_ORACLE_H
#define GS_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Camera uniform: 72 floats = view, projection, inverse view, inverse
 * projection (column-major), position.xyz1, viewport (W, H, W/H, 0). */
void orc_camera_uniform(const float eye[3], const float target[3],
                        const float up[3], double fovy, double aspect,
                        double znear, double zfar, double width, double height,
                        float out72[72]);

/* SceneWorker.writeGaussianSplat activations (SceneWorker.ts:407-464). */
void orc_activate(uint32_t n, const double* xyz, const double* f_dc,
                  const double* opacity, const double* scale_log,
                  const double* rot, float* positions, float* colors,
                  float* scales, float* rotations);

/* preprocess_splats.wgsl:76-184 (+ optional SH extension). */
void orc_preprocess(uint32_t n, const float cam[72], const uint32_t tile_count[2],
                    const float inv_tile[2], const float* positions,
                    const float* scales, const float* rotations,
                    const float* colors, const float* sh_rest,
                    uint32_t sh_degree, void* projected, uint32_t* ref_counts,
                    int threads);

/* prefix_scan_{local,blocks,add}.wgsl: exclusive scan, offsets[n] = total. */
uint32_t orc_prefix_scan(uint32_t n, const uint32_t* counts, uint32_t* offsets);

/* emit_tile_refs.wgsl:57-79.  keys: u32 pairs [hi, lo]. */
void orc_emit(uint32_t n, uint32_t tiles_x, const void* projected,
              const uint32_t* offsets, uint32_t* keys, uint32_t* values);

/* radix_histogram.wgsl + scan + radix_scatter.wgsl: 8 stable 8-bit LSD
 * passes over the 64-bit (hi, lo) key.  Result in keys/values. */
void orc_radix_sort(uint32_t r, uint32_t* keys, uint32_t* values,
                    uint32_t* tmp_keys, uint32_t* tmp_values, int threads);

/* identify_tile_ranges.wgsl:31-52 (tile_offsets must be pre-zeroed, as the
 * renderer's clearBuffer does at GaussianSplatRenderer.ts:1137). */
void orc_identify(uint32_t r, const uint32_t* keys, uint32_t* tile_offsets);

/* rasterize_tiles.wgsl:44-110.  image: float rgba x W x H.  tile_costs
 * (optional): per tile, the number of splats iterated before the last pixel
 * of the tile terminated (the whole range when some pixel never does). */
void orc_rasterize(uint32_t width, uint32_t height, uint32_t tile_w,
                   uint32_t tile_h, uint32_t tiles_x, uint32_t tiles_y,
                   const void* projected, const uint32_t* tile_offsets,
                   const uint32_t* values, float* image, uint32_t* tile_costs,
                   int threads);

/* Work counts of the same loop: out = {pairs iterated, pairs whose exp is
 * evaluated (inside the radius, power <= 0), pairs blended}. */
void orc_raster_pairs(uint32_t width, uint32_t height, uint32_t tile_w, uint32_t tile_h,
                      uint32_t tiles_x, uint32_t tiles_y, const void* projected,
                      const uint32_t* tile_offsets, const uint32_t* values, uint64_t out[3],
                      int threads);

/* Whole rebin in one call with caller-provided buffers; returns R, or
 * 0xFFFFFFFF when R exceeds key_capacity (nothing past the scan is run). */
uint32_t orc_rebin(uint32_t n, const float cam[72], uint32_t width,
                   uint32_t height, uint32_t tile_w, uint32_t tile_h,
                   const float* positions, const float* scales,
                   const float* rotations, const float* colors,
                   const float* sh_rest, uint32_t sh_degree, void* projected,
                   uint32_t* ref_counts, uint32_t* offsets,
                   uint32_t key_capacity, uint32_t* keys, uint32_t* values,
                   uint32_t* tmp_keys, uint32_t* tmp_values,
                   uint32_t* tile_offsets, float* image, uint32_t* tile_costs,
                   int threads);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
