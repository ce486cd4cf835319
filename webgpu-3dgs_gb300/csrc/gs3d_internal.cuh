// gs3d_internal.cuh - device-side structures and helpers shared by the
// sm_103a kernels of the rebin library.  Not part of the public ABI.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gs3d.h"

namespace gs3d {

// ---------------------------------------------------------------------------
// Device-resident per-frame uniforms: CameraUniforms + SplatBinningUniforms +
// TileUniforms of the reference (preprocess_splats.wgsl:1-16,
// rasterize_tiles.wgsl:12-15), written once per rebin by one H2D copy.
struct FrameUniforms {
  gs3d_camera cam;          // 288 B
  uint32_t tile_count[2];   // tiles_x, tiles_y
  uint32_t splat_count;
  uint32_t num_tiles;
  float inv_tile[2];        // f32(1.0 / tile size), GaussianSplatRenderer.ts:1127-1128
  uint32_t viewport[2];     // width, height
  uint32_t tile_size[2];
  uint32_t tile_base;       // first global tile id of this view (batched path)
  uint32_t pad;
};
static_assert(sizeof(FrameUniforms) % 16 == 0, "FrameUniforms is copied as 16-byte words");

// One view of a batched rebin.  A single-view rebin is a batch of one.
// Splat-views of all views are concatenated (view v owns global indices
// [splat_base, splat_base + f.splat_count)), and so are tiles (global tile
// id = f.tile_base + ty * tiles_x + tx) and images (pixel_base).
struct ViewDesc {
  FrameUniforms f;
  const float4* pos;
  const float4* scale;
  const float4* rot;
  const float4* color;
  const float* sh;
  uint32_t sh_degree;
  uint32_t splat_base;
  uint32_t block_base;  // preprocess blocks of the scene groups' leaders before this view
  uint32_t batch_splats;  // splat-views in the whole batch (same in every view)
  uint64_t pixel_base;  // first pixel of this view's image in the batch target
  uint32_t batch_tiles;   // tiles in the whole batch (same in every view)
  uint32_t group_next;    // next view of the same scene in the batch, or kNoView
  uint64_t pad2;
};
constexpr uint32_t kNoView = 0xffffffffu;
static_assert(sizeof(ViewDesc) % 16 == 0, "ViewDesc is copied as 16-byte words");

// Largest v with key(v) <= x over a non-decreasing per-view field.
template <typename F>
__device__ __forceinline__ uint32_t find_view(uint32_t n_views, uint32_t x, F key) {
  uint32_t lo = 0, hi = n_views;  // key(lo) <= x < key(hi) (key(n_views) = inf)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (key(mid) <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// Device error latch bits (read and cleared by gs3d_synchronize).
enum : uint32_t {
  DEVERR_CAPACITY = 1u,  // live ref count exceeded key capacity: nothing written
  DEVERR_TIMEOUT = 2u,   // a bounded look-back spin gave up
  DEVERR_RANGE = 4u,     // a key's tile id was outside tile_offsets
  DEVERR_BUCKET = 8u,    // a radix digit held 2^30 keys or more (30-bit look-back counts)
};

constexpr int kMaxSortPasses = 8;
constexpr int kRadixBins = 256;
// Histograms of the fused rebin's tile-id passes: 2048 bins a pass (11-bit
// digits use them all, narrower digits the first 2^bits).
constexpr int kTileHistStride = 2048;
constexpr int kMaxTilePasses = kMaxSortPasses - 4;

// Per-frame control block, zeroed at the start of every rebin.
struct Ctrl {
  uint32_t error;
  uint32_t scan_tile_counter;
  uint32_t sort_part_counter[kMaxSortPasses];
  uint32_t raster_queue;
  uint32_t sched_counter[2];
  uint32_t raster_heavy;  // tiles at the head of the raster order shaded as half strips
  uint32_t emit_chunk;    // next 256-splat chunk of the depth-ordered emit
  uint32_t pad;
  uint32_t sort_hist[kMaxSortPasses][kRadixBins];  // global digit histograms
  uint32_t sched_hist[2][kRadixBins];
  uint32_t tile_hist[kMaxTilePasses][kTileHistStride];  // fused rebin's tile passes
};

// Fallback gate of the learned raster schedule, kept on the device across
// frames (set by gs3d_set_cost_model, updated after every learned raster).
struct SchedGate {
  float bound;            // largest running error at which the learned order is used
  float mae;              // running mean |predicted - measured log(1 + cost)|
  float last_mae;         // the last frame's
  uint32_t frames;        // frames measured
  uint32_t use_learned;   // order of the next frame: 1 learned, 0 key count
  uint32_t used_learned;  // order of the last frame
  uint32_t fallbacks;     // frames rendered in key-count order by the gate
  uint32_t pad;
};

// Bounded spins: a device wait gives up after this many polls (with
// __nanosleep back-off this is on the order of a second), latches
// DEVERR_TIMEOUT and returns instead of hanging the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

// ---------------------------------------------------------------------------
// PTX helpers
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// 16-byte global->shared asynchronous copy (L2 only).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem_dst)),
               "l"(gmem_src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// mbarrier + bulk (TMA, non-tensor) copy helpers.
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// Plain arrive (release at CTA scope): completes the phase of a count-1
// barrier without a transaction.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Bulk copy global -> shared, completion signalled on `bar` (bytes % 16 == 0,
// both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Device waits on an mbarrier give up after this much wall time (and the
// caller latches DEVERR_TIMEOUT).
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Bounded parity wait; returns false if the limit ran out.  Each try_wait
// may suspend the thread until the phase completes (up to the hint, 1 ms),
// so waiting threads issue almost nothing; the wait is bounded by
// kWaitLimitNs of wall time.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint64_t t0 = 0;
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(1000000u)
        : "memory");
    if (ok) return true;
    const uint64_t t = global_ns();
    if (t0 == 0) t0 = t;
    else if (t - t0 > kWaitLimitNs) return false;
  }
}

__device__ __forceinline__ void latch_error(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

// Per-device launch set-up (shared-memory attributes, occupancy) is cached
// in arrays of this many devices.
constexpr int kMaxDevices = 64;
// The calling thread's current device, checked against kMaxDevices.
inline cudaError_t current_device(int* dev) {
  const cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess) return e;
  return (*dev < 0 || *dev >= kMaxDevices) ? cudaErrorInvalidDevice : cudaSuccess;
}

// Shared-memory histogram add with a warp-uniform fast path: coherent digits
// (the high byte of neighbouring tile ids, a depth exponent byte) would
// otherwise serialise the lanes of a warp on one address.  Every lane of the
// warp must call it.
__device__ __forceinline__ void hist_add_256(uint32_t* h, uint32_t d, bool active) {
  const uint32_t act = __ballot_sync(0xffffffffu, active);
  const uint32_t d0 = __shfl_sync(0xffffffffu, d, act ? __ffs(act) - 1 : 0);
  const bool same = __all_sync(0xffffffffu, !active || d == d0);
  if (same) {
    if (act && (threadIdx.x & 31) == (uint32_t)(__ffs(act) - 1)) atomicAdd(h + d0, __popc(act));
  } else if (active) {
    atomicAdd(h + d, 1u);
  }
}

// Live ref count guarded by capacity: a count above capacity was latched as
// DEVERR_CAPACITY by emit and every later stage treats it as zero.
__device__ __forceinline__ uint32_t live_refs(const uint32_t* ref_counter, uint32_t capacity) {
  const uint32_t r = *ref_counter;
  return r > capacity ? 0u : r;
}

// ---------------------------------------------------------------------------
// Host-side launchers (one translation unit per stage).
struct SortPlan {
  int passes;                    // number of digit passes (digits of up to 8 bits)
  int word[kMaxSortPasses];      // 0 = hi (tile id), 1 = lo (depth bits)
  int shift[kMaxSortPasses];
  int nbits[kMaxSortPasses];     // digit width of the pass: 2, 4, 6, 8 or 11
};
// 4 depth-bit passes, then the tile-id bits below the highest set bit of
// num_tiles - 1 in digits of at most tile_digit_bits (4, 6, 8 or 11) bits.  A digit
// is (word >> shift) & ((1 << nbits) - 1); digits of neighbouring passes may
// overlap by a bit, which a stable LSD sequence tolerates.
SortPlan make_sort_plan(uint32_t num_tiles, int tile_digit_bits = 8);
__host__ __device__ inline uint32_t digit_mask(int nbits) { return (1u << nbits) - 1u; }

// Projects every splat-view of the batch (total_blocks = sum of
// ceil(splat_count / 256) over views; max_sh_degree bounds the views' SH
// degrees and sizes the shared-memory staging).
cudaError_t launch_preprocess(const ViewDesc* views, uint32_t n_views, uint32_t total_blocks,
                              uint32_t max_sh_degree, gs3d_projected_splat* out, uint32_t* counts,
                              uint32_t* depth_keys, uint32_t* depth_ids, uint32_t* rect8,
                              uint32_t* err, cudaStream_t s);
// Exclusive scan of counts[gather[i]] (counts[i] when gather is null).
cudaError_t launch_scan(const uint32_t* counts, const uint32_t* gather, uint32_t* offsets,
                        uint32_t n, unsigned long long* status, uint32_t* tile_counter,
                        uint32_t epoch, uint32_t* total_out, uint32_t* err, cudaStream_t s);
size_t scan_status_words(uint32_t n);
// Message of the calling thread's last failing context-free call.
const char* noalloc_last_error();
// Sets the message gs3d_last_error(NULL) returns on the calling thread.
void set_context_free_error(const char* msg);
// Emit in splat order (the reference's emit_tile_refs, one view).
cudaError_t launch_emit(const FrameUniforms* d_frame, uint32_t n,
                        const gs3d_projected_splat* proj, const uint32_t* offsets,
                        const uint32_t* ref_counter, uint32_t capacity, uint2* keys,
                        uint32_t* values, uint32_t* err, cudaStream_t s);
cudaError_t launch_sort(const SortPlan& plan, const uint32_t* ref_counter, uint32_t capacity,
                        uint2* keys_a, uint32_t* vals_a, uint2* keys_b, uint32_t* vals_b,
                        uint32_t* status, Ctrl* ctrl, int sm_count, cudaStream_t s);
size_t sort_status_words(uint32_t capacity, int passes);
// Status words any sort plan of a capacity needs (11-bit tile passes included).
size_t sort_status_words_max(uint32_t capacity);
// Key/value buffers handed to the sort must hold this many entries: passes
// always fetch whole partitions, 4096 keys of 8 bytes or 6144 of 4 bytes
// (entries past the live count are read and ignored).
uint32_t sort_capacity_round(uint32_t capacity);
// Tile-id passes of the fused rebin: histograms already in
// g_hist[p * kTileHistStride + digit].
cudaError_t launch_sort_tile_passes(const SortPlan& plan, const uint32_t* ref_counter,
                                    uint32_t capacity, uint2* keys_a, uint32_t* vals_a,
                                    uint2* keys_b, uint32_t* vals_b, uint32_t* status,
                                    uint32_t* g_hist, uint32_t* part_counters, uint32_t* err,
                                    int sm_count, cudaStream_t s);
// Stable LSD passes of `plan` (word ignored) over 32-bit keys; the histograms
// are computed here.  count is read on the device.
cudaError_t launch_sort_u32(const SortPlan& plan, const uint32_t* count, uint32_t capacity,
                            uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b,
                            uint32_t* vals_b, uint32_t* status, uint32_t* g_hist,
                            uint32_t* part_counters, uint32_t* err, int sm_count, cudaStream_t s);
// Four 8-bit passes over 32-bit per-splat depth keys (count read on device).
cudaError_t launch_sort_depth_keys(const uint32_t* count, uint32_t capacity, uint32_t* keys_a,
                                   uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b,
                                   uint32_t* status, uint32_t* g_hist, uint32_t* part_counters,
                                   uint32_t* err, int sm_count, cudaStream_t s);
// Raster work order: tile indices sorted by decreasing expected cost
// (schedule = GS3D_SCHEDULE_KEY_COUNT: the tile's key count), so the
// persistent raster CTAs start the longest tiles first.
// keys_a/order_a and est (the expected cost of every tile) must already be
// written for GS3D_SCHEDULE_LEARNED (launch_learned_keys); for the key-count
// schedule they are computed here.  Also sets ctrl->raster_heavy
// (launch_heavy_count).
cudaError_t launch_schedule(uint32_t schedule, const uint32_t* tile_offsets, uint32_t num_tiles,
                            const uint32_t* num_tiles_dev, uint32_t* keys_a, uint32_t* order_a,
                            uint32_t* keys_b, uint32_t* order_b, float* est, uint32_t* status,
                            Ctrl* ctrl, uint32_t raster_ctas, uint32_t strips, bool split_all,
                            int sm_count, cudaStream_t s);
// The per-tile split: *heavy = the number of tiles (the head of an order by
// decreasing est) whose expected cost per strip exceeds half of one raster
// CTA's fair share of the frame, sum(est) * strips / raster_ctas; those tiles
// are shaded as two half-strip work items per strip.  all: every tile (est
// may be null).
cudaError_t launch_heavy_count(const float* est, uint32_t n, uint32_t raster_ctas,
                               uint32_t strips, bool all, uint32_t* heavy, cudaStream_t s);

// ---- learned schedule (learned.cu) ----
constexpr int kFeatures = 16;
constexpr int kHidden = 64;
constexpr int kMlpParams = kHidden * kFeatures + kHidden + kHidden * kHidden + kHidden + kHidden + 1;
cudaError_t launch_tile_features(const ViewDesc* views, uint32_t n_views, uint32_t num_tiles,
                                 uint32_t tile_w, uint32_t tile_h, const uint32_t* tile_offsets,
                                 const uint32_t* values, const gs3d_projected_splat* proj,
                                 const float* mean, const float* inv_std, float* out,
                                 cudaStream_t s);
cudaError_t launch_mlp_infer(const float* params, const float* x, uint32_t n, float* y,
                             cudaStream_t s);
cudaError_t launch_mlp_forward(const float* params, const float* x, uint32_t n, float* acts,
                               float* y, cudaStream_t s);
cudaError_t launch_mlp_backward(const float* params, const float* x, const float* acts,
                                const float* target, uint32_t n, float* grads, cudaStream_t s);
cudaError_t launch_adam(float* p, float* m, float* v, const float* g, uint32_t count, float lr,
                        float beta1, float beta2, float eps, uint32_t step, cudaStream_t s);
// Schedule keys (decreasing expected cost first) and expected costs: from the
// cost MLP's predictions while gate->use_learned, else from the key counts.
cudaError_t launch_learned_keys(const float* pred, uint32_t n, const SchedGate* gate,
                                const uint32_t* tile_offsets, uint32_t* keys, uint32_t* ids,
                                float* est, cudaStream_t s);
// After a learned raster: the frame's mean |pred - log(1 + cost)| over tiles
// updates the gate's running error and its choice for the next frame.
cudaError_t launch_gate_update(const float* pred, const uint32_t* costs, uint32_t n,
                               SchedGate* gate, cudaStream_t s);
cudaError_t launch_log_costs(const uint32_t* costs, uint32_t n, float* out, cudaStream_t s);

// Emit in depth-sorted order over all splat-views of a batch (global tile
// ids, global splat-view values) + histograms of the tile-id digit places.
// rect8: the preprocess's one-word tile rectangles (null: read the
// rectangles from the projected records).
cudaError_t launch_emit_sorted(const ViewDesc* views, uint32_t n_views, uint32_t total,
                               const gs3d_projected_splat* proj, const uint32_t* rect8,
                               const uint32_t* sorted_keys,
                               const uint32_t* sorted_ids,
                               const uint32_t* sorted_offsets, const uint32_t* ref_counter,
                               uint32_t capacity, uint2* keys, uint32_t* values,
                               const SortPlan& tile_plan, uint32_t* g_hist,
                               uint32_t* chunk_ticket, uint32_t* err, int sm_count,
                               cudaStream_t s);
cudaError_t launch_identify(const uint2* keys, const uint32_t* ref_counter, uint32_t capacity,
                            uint32_t num_tiles, uint32_t* tile_offsets, uint32_t* err,
                            int sm_count, cudaStream_t s);
// Rasterizes every tile of the batch.  Persistent CTAs pull tile indices
// from a device work queue (order[k] = k-th tile to render, identity when
// order is null) through *queue_counter, which must be zero at launch.
struct RasterArgs {
  const ViewDesc* views;
  uint32_t n_views;
  uint32_t num_tiles;     // total over views
  uint32_t tile_w, tile_h;
  const gs3d_projected_splat* proj;
  const uint32_t* tile_offsets;
  const uint32_t* values;
  uint2* image;
  uint32_t* tile_costs;   // may be null
  const uint32_t* order;  // may be null
  uint32_t* queue_counter;
  uint32_t batch;         // splats staged per batch (0 = tile_w * tile_h)
  bool culled;
  uint32_t split;         // CTAs per tile (row strips), set by launch_raster
  // tiles at the head of the order shaded as two half-strip items per strip
  // (device count, two-pixel culled variant only; may be null: none)
  const uint32_t* heavy;
};
cudaError_t launch_raster(const RasterArgs& a, int sm_count, cudaStream_t s);
// Row strips per tile and resident CTAs of the raster launch for these args.
cudaError_t raster_shape(const RasterArgs& a, int sm_count, uint32_t* strips,
                         uint32_t* resident_ctas);

// Headless composite of one view's splat target over a background colour,
// optionally through the tile heat-map overlay; out = W*H RGBA8 words.
cudaError_t launch_composite(const uint2* image, uint32_t W, uint32_t H,
                             const uint32_t* tile_offsets, uint32_t tile_w, uint32_t tile_h,
                             uint32_t tiles_x, uint32_t tiles_y, uint32_t heatmap,
                             uint32_t debug_ref, const float bg[4], uint32_t* out,
                             cudaStream_t s);

// ---- PLY ingest (ply.cu) ----------------------------------------------------
enum PlyScalar : uint32_t { PLY_I8, PLY_U8, PLY_I16, PLY_U16, PLY_I32, PLY_U32, PLY_F32, PLY_F64 };
struct PlyField {
  uint32_t offset;  // byte offset within a vertex row
  uint32_t type;    // PlyScalar
};
constexpr int kPlyRequired = 14;  // x y z opacity scale_0..2 rot_0..3 f_dc_0..2
constexpr int kPlyMaxRest = 45;
// Where the vertex rows of a parsed PLY are and how to read them.  ASCII
// bodies are converted on the host into little-endian f64 rows first.
struct PlyLayout {
  uint64_t count = 0;          // vertex rows
  uint64_t rows_offset = 0;    // byte offset of the first vertex row (binary)
  uint64_t header_bytes = 0;
  uint32_t stride = 0;         // bytes per vertex row
  uint32_t format = 0;         // GS3D_PLY_*
  uint32_t f_rest_count = 0;   // f_rest_* properties
  uint32_t sh_degree = 0;      // inferred from f_rest_count
  PlyField req[kPlyRequired];
  uint32_t sh_k = 0;           // SH coefficients per channel used for colour (0: none)
  PlyField rest[kPlyMaxRest];  // the used f_rest fields, [channel][coefficient]
  uint32_t vertex_props = 0;   // properties per vertex row
};
const char* ply_required_name(int k);
// Parses the header and lays out the vertex element (host only).  On error
// returns false with the message in *err.
bool ply_parse_layout(const uint8_t* data, size_t size, PlyLayout* out, std::string* err);
// Tokenizes an ASCII body into count x vertex_props f64 values (host only).
bool ply_ascii_rows(const uint8_t* data, size_t size, const PlyLayout& lay,
                    std::vector<double>* rows, std::string* err);
// Decodes n vertex rows on the device into the four vec4 SoA arrays and the
// SH block (lay.sh_k coefficients per channel, channel-major), activating as
// the reference's loader does; the first non-finite required value latches
// 1 + its field index in *bad; bounds = 6 ordered-u32 words (min xyz, max xyz).
cudaError_t launch_ply_decode(const uint8_t* rows, uint64_t n, const PlyLayout& lay,
                              bool big_endian, float4* pos, float4* scale,
                              float4* rot, float4* color, float* sh, uint32_t* bad,
                              uint32_t* bounds, cudaStream_t s);

}  // namespace gs3d
