// ctx.cu - context, buffer ownership and the C ABI of include/gs3d.h.
//
// Mirrors the host side of the reference renderer:
//   - gs3d_create / gs3d_destroy: GaussianSplatRenderer constructor + init
//     (src/renderers/GaussianSplatRenderer.ts:331-471) and the BufferManager
//     buffers it creates (:338-465);
//   - gs3d_set_splats: SceneSyncer.setSplatData (src/SceneSyncer.ts:25-38)
//     followed by resizeBinningBuffers (:209-227);
//   - gs3d_set_camera: the uniform uploads of rebin (:1112-1131) and, on a
//     viewport change, resizeViewportTargets (:231-295);
//   - gs3d_rebin: the stage sequence of rebin (:1104-1266).
//
// Differences by design: no dispatch or buffer clamping (the reference clamps
// dispatch counts to maxComputeWorkgroupsPerDimension and buffers to
// maxStorageBufferBindingSize, silently truncating large scenes); the key
// buffers start at N * max_tiles_per_splat entries like the reference but
// overflow is detected on the device and reported, after which the buffers
// are grown and the caller re-issues the rebin.
//
// Every rebin runs over a device-side view table (ViewDesc); a single-view
// rebin is a batch of one, gs3d_rebin_batch renders many views, of several
// scenes and uneven sizes, in one launch sequence.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gs3d_internal.cuh"

using namespace gs3d;

namespace {

// Refs are indexed by u32 and key buffers hold whole 12288-key blocks (the
// 4096- and 6144-key partitions of the sort passes).
constexpr uint32_t kMaxCapacity = 0xFFFFE000u;
constexpr int kUploadSlots = 8;
constexpr uint32_t kPreBlock = 256;  // preprocess threads per block

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct SceneBufs {
  uint32_t n = 0, sh_degree = 0;
  DevBuf pos, scale, rot, color, sh;
};

__global__ void probe_kernel(int* out) {
  if (out) *out = 1;
}

}  // namespace

struct gs3d_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // splat-target copy-outs run on their own stream; the next raster (the only
  // writer of the target) waits for the last one (copy_done)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t frame_done = nullptr, copy_done = nullptr;
  int sm_count = 0;
  std::string err = "no error";

  uint32_t tile_w = 16, tile_h = 16, max_tiles_per_splat = 16;
  uint32_t digit_bits = 8;    // widest tile-id radix digit (gs3d_tuning)
  uint32_t raster_batch = 0;  // splats per raster batch, 0 = tile area (gs3d_tuning)
  uint32_t flags = 0;
  uint32_t schedule = GS3D_SCHEDULE_ROW_MAJOR;

  std::vector<SceneBufs> scenes;  // scene 0 = the gs3d_set_splats scene
  bool have_scene = false;

  // binning buffers, sized for the largest batch seen
  DevBuf proj, counts, offsets, ref_counter;
  DevBuf keys_a, vals_a, keys_b, vals_b;
  uint32_t capacity = 0;
  DevBuf scan_status, sort_status;
  uint32_t scan_epoch = 0;
  DevBuf depth_keys_a, depth_ids_a, depth_keys_b, depth_ids_b, sorted_offsets, depth_status;
  DevBuf rect8;  // one-word tile rectangles per splat-view (fused rebin, small grids)
  DevBuf tile_offsets, image, tile_costs, composite_out;
  DevBuf sched_keys_a, sched_keys_b, sched_order_a, sched_order_b, sched_status;
  // cost model (learned schedule)
  bool have_model = false;
  DevBuf model_params, model_mean, model_inv_std, tile_feats, tile_preds;
  DevBuf tile_est;    // expected cost per tile of the last ordered raster
  DevBuf gate;        // SchedGate: the learned schedule's fallback gate
  float gate_bound = 0.5f;

  // the current batch (a single-view frame is a batch of one)
  bool have_camera = false;
  std::vector<ViewDesc> views;       // host copy
  std::vector<gs3d_view_info> info;  // per-view layout
  uint32_t total_splats = 0, total_tiles = 0, total_blocks = 0, max_sh = 0;
  uint64_t total_pixels = 0;
  DevBuf d_views;
  ViewDesc* h_upload = nullptr;  // pinned ring of view tables
  size_t upload_cap = 0;         // views per slot
  cudaEvent_t upload_ev[kUploadSlots] = {};
  int upload_slot = 0;

  DevBuf ctrl;
  uint32_t* h_word = nullptr;  // pinned scratch for small reads
  uint64_t alloc_gen = 0;      // bumped by every device (re)allocation

  // CUDA-graph replay of the fused rebin (GS3D_FLAG_CUDA_GRAPH)
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> sig;     // batch signature the graph was captured for
    ViewDesc* h_views = nullptr;   // pinned view table read by the graph's copy node
    size_t cap = 0;
    cudaEvent_t copied = nullptr;  // recorded after each replay (pinned slot reuse)
    void* result_keys = nullptr;   // buffer holding the sorted keys after a replay
  } graph;

  // optional stage timing (GS3D_FLAG_STAGE_TIMING)
  struct Pending {
    int stage;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_next = 0;
  std::vector<Pending> pending;
  double stage_ms[GS3D_STAGE_COUNT] = {};
  uint32_t stage_n[GS3D_STAGE_COUNT] = {};
};

namespace {

int fail(gs3d_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(gs3d_ctx* c, cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? GS3D_ERR_OOM
                   : (e == cudaErrorNoKernelImageForDevice || e == cudaErrorNoDevice ||
                      e == cudaErrorInsufficientDriver)
                       ? GS3D_ERR_NO_DEVICE
                       : GS3D_ERR_CUDA;
  return fail(c, code, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define CK(expr, what)                                    \
  do {                                                    \
    cudaError_t e_ = (expr);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

#define TRY(expr)                 \
  do {                            \
    const int r_ = (expr);        \
    if (r_ != GS3D_OK) return r_; \
  } while (0)

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

// Grow-only allocation; contents are not preserved.
int ensure(gs3d_ctx* c, DevBuf& b, size_t bytes, const char* name) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return GS3D_OK;
  if (b.p) {
    CK(cudaStreamSynchronize(c->stream), "synchronize before resize");
    if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream), "copy-outs before resize");
    release(b);
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, GS3D_ERR_OOM, "cudaMalloc of %zu bytes for %s failed: %s", bytes, name,
                cudaGetErrorString(e));
  }
  b.p = p;
  b.bytes = bytes;
  ++c->alloc_gen;
  return GS3D_OK;
}

uint32_t* u32(DevBuf& b) { return static_cast<uint32_t*>(b.p); }
Ctrl* ctrl_of(gs3d_ctx* c) { return static_cast<Ctrl*>(c->ctrl.p); }
ViewDesc* dviews(gs3d_ctx* c) { return static_cast<ViewDesc*>(c->d_views.p); }

int ensure_key_capacity(gs3d_ctx* c, uint64_t want) {
  if (want > kMaxCapacity)
    return fail(c, GS3D_ERR_CAPACITY, "%llu tile refs exceed the %u-ref limit of one rebin",
                (unsigned long long)want, kMaxCapacity);
  if (want <= c->capacity && c->keys_a.p) return GS3D_OK;
  const uint32_t cap = (uint32_t)std::max<uint64_t>(want, 1);
  const size_t alloc = sort_capacity_round(cap);  // sort passes fetch whole partitions
  TRY(ensure(c, c->keys_a, alloc * sizeof(uint2), "sort_keys_a"));
  TRY(ensure(c, c->keys_b, alloc * sizeof(uint2), "sort_keys_b"));
  TRY(ensure(c, c->vals_a, alloc * sizeof(uint32_t), "sort_values_a"));
  TRY(ensure(c, c->vals_b, alloc * sizeof(uint32_t), "sort_values_b"));
  TRY(ensure(c, c->sort_status, sort_status_words_max(cap) * sizeof(uint32_t),
             "sort look-back status"));
  c->capacity = cap;
  return GS3D_OK;
}

// Per-splat-view buffers for a batch of `m` splat-views.
int ensure_splat_buffers(gs3d_ctx* c, uint32_t m) {
  TRY(ensure(c, c->proj, (size_t)m * sizeof(gs3d_projected_splat), "projected_splats"));
  TRY(ensure(c, c->counts, (size_t)m * 4, "splat_ref_counts"));
  TRY(ensure(c, c->offsets, ((size_t)m + 1) * 4, "splat_ref_offsets"));
  TRY(ensure(c, c->scan_status, scan_status_words(m) * 8, "scan look-back status"));
  const size_t md = sort_capacity_round(std::max<uint32_t>(m, 1));
  TRY(ensure(c, c->depth_keys_a, md * 4, "depth keys"));
  TRY(ensure(c, c->depth_keys_b, md * 4, "depth keys"));
  TRY(ensure(c, c->depth_ids_a, md * 4, "depth ids"));
  TRY(ensure(c, c->depth_ids_b, md * 4, "depth ids"));
  TRY(ensure(c, c->sorted_offsets, ((size_t)m + 1) * 4, "depth-ordered offsets"));
  TRY(ensure(c, c->depth_status, sort_status_words(m, 4) * 4, "depth sort status"));
  TRY(ensure(c, c->rect8, (size_t)m * 4, "tile rectangles"));
  return GS3D_OK;
}

int set_device(gs3d_ctx* c) {
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  return GS3D_OK;
}

// Reads the latched device error word (stream must be idle) and clears it.
int check_device_errors(gs3d_ctx* c) {
  CK(cudaMemcpy(c->h_word, &ctrl_of(c)->error, sizeof(uint32_t), cudaMemcpyDeviceToHost),
     "read error word");
  const uint32_t e = c->h_word[0];
  if (e == 0) return GS3D_OK;
  CK(cudaMemset(&ctrl_of(c)->error, 0, sizeof(uint32_t)), "clear error word");
  if (e & DEVERR_CAPACITY) {
    CK(cudaMemcpy(c->h_word, c->ref_counter.p, sizeof(uint32_t), cudaMemcpyDeviceToHost),
       "read ref_counter");
    const uint64_t r = c->h_word[0];
    if (r > kMaxCapacity)
      return fail(c, GS3D_ERR_CAPACITY, "%llu tile refs exceed the %u-ref limit of one rebin",
                  (unsigned long long)r, kMaxCapacity);
    TRY(ensure_key_capacity(c, std::min<uint64_t>(r + r / 8 + 1024, kMaxCapacity)));
    return fail(c, GS3D_ERR_CAPACITY,
                "live ref count %llu exceeded the key capacity; capacity is now %u, re-run "
                "the rebin",
                (unsigned long long)r, c->capacity);
  }
  if (e & DEVERR_TIMEOUT)
    return fail(c, GS3D_ERR_TIMEOUT, "a bounded device wait gave up (look-back or bulk copy)");
  if (e & DEVERR_BUCKET)
    return fail(c, GS3D_ERR_CAPACITY,
                "one radix digit of this frame holds 2^30 keys or more; split the batch");
  return fail(c, GS3D_ERR_INVALID_ARG,
              "a sort key's tile id or a splat offset was out of range for this frame");
}

constexpr size_t kEventPool = 4096;

int drain_timing(gs3d_ctx* c) {
  for (const auto& p : c->pending) {
    CK(cudaEventSynchronize(p.b), "stage timing");
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, p.a, p.b), "stage timing");
    c->stage_ms[p.stage] += ms;
    c->stage_n[p.stage] += 1;
  }
  c->pending.clear();
  c->ev_next = 0;
  return GS3D_OK;
}

// A pair of events around one stage when timing is on.
struct StageScope {
  gs3d_ctx* c;
  int stage;
  cudaEvent_t a = nullptr;
  StageScope(gs3d_ctx* ctx, int st) : c(ctx), stage(st) {
    if (!(c->flags & GS3D_FLAG_STAGE_TIMING)) return;
    if (c->ev_pool.empty()) {
      c->ev_pool.resize(kEventPool);
      for (auto& e : c->ev_pool) cudaEventCreate(&e);
    }
    if (c->ev_next + 2 > c->ev_pool.size()) drain_timing(c);
    a = c->ev_pool[c->ev_next++];
    cudaEventRecord(a, c->stream);
  }
  ~StageScope() {
    if (!a) return;
    cudaEvent_t b = c->ev_pool[c->ev_next++];
    cudaEventRecord(b, c->stream);
    c->pending.push_back({stage, a, b});
  }
};

int sync_and_check(gs3d_ctx* c) {
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream), "copy-out stream");
  return check_device_errors(c);
}

int upload_scene(gs3d_ctx* c, SceneBufs& sc, uint32_t n, const float* positions,
                 const float* scales, const float* rotations, const float* colors,
                 const float* sh_rest, uint32_t sh_degree, int memory) {
  if (memory != 0 && memory != 1) return fail(c, GS3D_ERR_INVALID_ARG, "memory must be 0 or 1");
  if (sh_degree > 3) return fail(c, GS3D_ERR_INVALID_ARG, "sh_degree %u > 3", sh_degree);
  if (n > 0 && (!positions || !scales || !rotations || !colors))
    return fail(c, GS3D_ERR_INVALID_ARG, "null splat array");
  if (n > 0 && sh_degree > 0 && !sh_rest)
    return fail(c, GS3D_ERR_INVALID_ARG, "sh_degree %u needs sh_rest", sh_degree);
  if (n > (1u << 30)) return fail(c, GS3D_ERR_INVALID_ARG, "too many splats (%u)", n);
  TRY(set_device(c));
  const size_t v4 = (size_t)n * 16;
  const uint32_t kc = 3u * ((sh_degree + 1) * (sh_degree + 1) - 1);
  TRY(ensure(c, sc.pos, v4, "splat_positions"));
  TRY(ensure(c, sc.scale, v4, "splat_scales"));
  TRY(ensure(c, sc.rot, v4, "splat_rotations"));
  TRY(ensure(c, sc.color, v4, "splat_colors"));
  if (kc) TRY(ensure(c, sc.sh, (size_t)n * kc * sizeof(float), "splat_sh_rest"));
  const cudaMemcpyKind kind = memory ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (n) {
    CK(cudaMemcpyAsync(sc.pos.p, positions, v4, kind, c->stream), "upload positions");
    CK(cudaMemcpyAsync(sc.scale.p, scales, v4, kind, c->stream), "upload scales");
    CK(cudaMemcpyAsync(sc.rot.p, rotations, v4, kind, c->stream), "upload rotations");
    CK(cudaMemcpyAsync(sc.color.p, colors, v4, kind, c->stream), "upload colors");
    if (kc)
      CK(cudaMemcpyAsync(sc.sh.p, sh_rest, (size_t)n * kc * sizeof(float), kind, c->stream),
         "upload sh_rest");
  }
  CK(cudaStreamSynchronize(c->stream), "splat upload");
  sc.n = n;
  sc.sh_degree = sh_degree;
  return GS3D_OK;
}

// Builds the batch layout on the host, sizes every buffer for it and uploads
// the view table through a pinned ring slot (stream ordered).
int set_views(gs3d_ctx* c, const gs3d_view* views, uint32_t n_views, bool upload = true) {
  if (n_views == 0 || !views) return fail(c, GS3D_ERR_INVALID_ARG, "empty view list");
  std::vector<ViewDesc> vds(n_views, ViewDesc{});
  std::vector<gs3d_view_info> infos(n_views, gs3d_view_info{});
  uint64_t splats = 0, tiles = 0, pixels = 0, blocks = 0;
  uint32_t max_sh = 0;
  for (uint32_t v = 0; v < n_views; ++v) {
    const gs3d_view& in = views[v];
    if (in.scene >= c->scenes.size())
      return fail(c, GS3D_ERR_INVALID_ARG, "view %u names unknown scene %u", v, in.scene);
    const SceneBufs& sc = c->scenes[in.scene];
    const uint32_t w = std::max<uint32_t>(1, in.width);   // GaussianSplatRenderer.ts:1040
    const uint32_t h = std::max<uint32_t>(1, in.height);
    const uint32_t tx = (w + c->tile_w - 1) / c->tile_w;  // :1042-1043
    const uint32_t ty = (h + c->tile_h - 1) / c->tile_h;
    ViewDesc& d = vds[v];
    FrameUniforms& f = d.f;
    f.cam = in.camera;
    f.tile_count[0] = tx;
    f.tile_count[1] = ty;
    f.splat_count = sc.n;
    f.num_tiles = tx * ty;
    f.inv_tile[0] = (float)(1.0 / c->tile_w);  // :1127-1128, f64 division stored as f32
    f.inv_tile[1] = (float)(1.0 / c->tile_h);
    f.viewport[0] = w;
    f.viewport[1] = h;
    f.tile_size[0] = c->tile_w;
    f.tile_size[1] = c->tile_h;
    f.tile_base = (uint32_t)tiles;
    d.pos = static_cast<const float4*>(sc.pos.p);
    d.scale = static_cast<const float4*>(sc.scale.p);
    d.rot = static_cast<const float4*>(sc.rot.p);
    d.color = static_cast<const float4*>(sc.color.p);
    d.sh = sc.sh_degree ? static_cast<const float*>(sc.sh.p) : nullptr;
    d.sh_degree = sc.sh_degree;
    d.splat_base = (uint32_t)splats;
    d.pixel_base = pixels;
    gs3d_view_info& vi = infos[v];
    vi.pixel_offset = pixels;
    vi.width = w;
    vi.height = h;
    vi.tiles_x = tx;
    vi.tiles_y = ty;
    vi.tile_base = (uint32_t)tiles;
    vi.splat_base = (uint32_t)splats;
    vi.splat_count = sc.n;
    vi.scene = in.scene;
    max_sh = std::max(max_sh, d.sh ? sc.sh_degree : 0u);
    d.group_next = kNoView;
    splats += sc.n;
    tiles += (uint64_t)tx * ty;
    pixels += (uint64_t)w * h;
  }
  // scene groups: views of one scene are projected by one preprocess block
  // per 256 splats (the first view of the scene leads, the others chain)
  {
    std::vector<int64_t> last(c->scenes.size(), -1);
    for (uint32_t v = 0; v < n_views; ++v) {
      const uint32_t sid = views[v].scene;
      vds[v].block_base = (uint32_t)blocks;
      if (last[sid] < 0) {
        blocks += (c->scenes[sid].n + kPreBlock - 1) / kPreBlock;
      } else {
        vds[(size_t)last[sid]].group_next = v;
      }
      last[sid] = v;
    }
  }
  if (splats >= (1ull << 30))  // depth-sort look-back counts are 30-bit
    return fail(c, GS3D_ERR_INVALID_ARG, "batch holds 2^30 splat-views or more");
  if (tiles >= (1ull << 31)) return fail(c, GS3D_ERR_INVALID_ARG, "batch holds too many tiles");
  for (ViewDesc& d : vds) {
    d.batch_splats = (uint32_t)splats;
    d.batch_tiles = (uint32_t)tiles;
  }

  TRY(ensure_splat_buffers(c, (uint32_t)splats));
  TRY(ensure(c, c->tile_offsets, (tiles + 1) * 4, "tile_offsets"));
  TRY(ensure(c, c->tile_costs, std::max<uint64_t>(tiles, 1) * 4, "tile_costs"));
  TRY(ensure(c, c->image, std::max<uint64_t>(pixels, 1) * 8, "splat_target"));
  const size_t td = sort_capacity_round((uint32_t)std::max<uint64_t>(tiles, 1));
  TRY(ensure(c, c->sched_keys_a, td * 4, "schedule keys"));
  TRY(ensure(c, c->sched_keys_b, td * 4, "schedule keys"));
  TRY(ensure(c, c->sched_order_a, td * 4, "schedule order"));
  TRY(ensure(c, c->sched_order_b, td * 4, "schedule order"));
  TRY(ensure(c, c->sched_status, sort_status_words((uint32_t)tiles, 4) * 4, "schedule status"));
  TRY(ensure(c, c->tile_feats, std::max<uint64_t>(tiles, 1) * kFeatures * 4, "tile features"));
  TRY(ensure(c, c->tile_preds, std::max<uint64_t>(tiles, 1) * 4, "tile cost predictions"));
  TRY(ensure(c, c->tile_est, std::max<uint64_t>(tiles, 1) * 4, "tile expected costs"));
  TRY(ensure(c, c->d_views, (size_t)n_views * sizeof(ViewDesc), "view table"));
  if (c->capacity < 1) TRY(ensure_key_capacity(c, 1));

  if (!upload) {  // the caller uploads the table (CUDA-graph replay)
    c->views.swap(vds);
    c->info.swap(infos);
    c->total_splats = (uint32_t)splats;
    c->total_tiles = (uint32_t)tiles;
    c->total_pixels = pixels;
    c->total_blocks = (uint32_t)blocks;
    c->max_sh = max_sh;
    c->have_camera = true;
    return GS3D_OK;
  }
  if (n_views > c->upload_cap) {  // grow the pinned ring (idle stream first)
    CK(cudaStreamSynchronize(c->stream), "upload ring resize");
    if (c->h_upload) cudaFreeHost(c->h_upload);
    c->h_upload = nullptr;
    c->upload_cap = 0;
    const size_t cap = std::max<size_t>(n_views, 64);
    CK(cudaMallocHost(&c->h_upload, cap * kUploadSlots * sizeof(ViewDesc)), "pinned view ring");
    c->upload_cap = cap;
  }
  const int slot = c->upload_slot;
  c->upload_slot = (slot + 1) % kUploadSlots;
  CK(cudaEventSynchronize(c->upload_ev[slot]), "view ring slot reuse");
  ViewDesc* h = c->h_upload + (size_t)slot * c->upload_cap;
  std::memcpy(h, vds.data(), n_views * sizeof(ViewDesc));
  CK(cudaMemcpyAsync(c->d_views.p, h, n_views * sizeof(ViewDesc), cudaMemcpyHostToDevice,
                     c->stream),
     "upload view table");
  CK(cudaEventRecord(c->upload_ev[slot], c->stream), "view ring event");

  c->views.swap(vds);
  c->info.swap(infos);
  c->total_splats = (uint32_t)splats;
  c->total_tiles = (uint32_t)tiles;
  c->total_pixels = pixels;
  c->total_blocks = (uint32_t)blocks;
  c->max_sh = max_sh;
  c->have_camera = true;
  return GS3D_OK;
}

int require_frame(gs3d_ctx* c, const char* stage) {
  if (!c->have_scene) return fail(c, GS3D_ERR_STATE, "%s: no splats set", stage);
  if (!c->have_camera) return fail(c, GS3D_ERR_STATE, "%s: no camera set", stage);
  return GS3D_OK;
}

int require_single(gs3d_ctx* c, const char* stage) {
  TRY(require_frame(c, stage));
  if (c->views.size() != 1)
    return fail(c, GS3D_ERR_STATE, "%s: the stage entry points run one view (set_camera)", stage);
  return GS3D_OK;
}

SortPlan tile_digit_plan(uint32_t num_tiles, uint32_t digit_bits) {
  const SortPlan full = make_sort_plan(num_tiles, (int)digit_bits);
  SortPlan tp{};
  for (int p = 4; p < full.passes; ++p) {  // the tile-id digit places only
    tp.word[tp.passes] = full.word[p];
    tp.shift[tp.passes] = full.shift[p];
    tp.nbits[tp.passes] = full.nbits[p];
    ++tp.passes;
  }
  return tp;
}

int raster_stage(gs3d_ctx* c, bool culled) {
  if ((uint64_t)c->tile_w * c->tile_h > 1024 && !culled)
    return fail(c, GS3D_ERR_INVALID_ARG,
                "tiles of %ux%u pixels are shaded by the culled two-pixel raster only; the "
                "stage-wise rebin's one-pixel raster takes at most 1024",
                c->tile_w, c->tile_h);
  StageScope t(c, GS3D_STAGE_RASTER);
  RasterArgs a{};
  a.views = dviews(c);
  a.n_views = (uint32_t)c->views.size();
  a.num_tiles = c->total_tiles;
  a.tile_w = c->tile_w;
  a.tile_h = c->tile_h;
  // raster_batch 0 stages one splat per tile pixel, at most 1024 (the staged
  // batches of a 2048-pixel tile would not fit shared memory)
  a.batch = c->raster_batch ? c->raster_batch
                            : ((uint64_t)c->tile_w * c->tile_h > 1024 ? 1024u : 0u);
  a.culled = culled;
  uint32_t strips = 1, raster_ctas = 1;
  CK(raster_shape(a, c->sm_count, &strips, &raster_ctas), "raster shape");
  const bool split_all = (c->flags & GS3D_FLAG_SPLIT_ALL_TILES) != 0;
  const bool learned = c->schedule == GS3D_SCHEDULE_LEARNED && c->total_tiles > 1;
  const uint32_t* order = nullptr;
  const uint32_t* heavy = nullptr;
  if (c->schedule != GS3D_SCHEDULE_ROW_MAJOR && c->total_tiles > 1) {
    if (learned) {
      const uint32_t nv = (uint32_t)c->views.size();
      CK(launch_tile_features(dviews(c), nv, c->total_tiles, c->tile_w, c->tile_h,
                              u32(c->tile_offsets), u32(c->vals_a),
                              static_cast<gs3d_projected_splat*>(c->proj.p),
                              static_cast<float*>(c->model_mean.p),
                              static_cast<float*>(c->model_inv_std.p),
                              static_cast<float*>(c->tile_feats.p), c->stream),
         "tile features");
      CK(launch_mlp_infer(static_cast<float*>(c->model_params.p),
                          static_cast<float*>(c->tile_feats.p), c->total_tiles,
                          static_cast<float*>(c->tile_preds.p), c->stream),
         "cost MLP inference");
      CK(launch_learned_keys(static_cast<float*>(c->tile_preds.p), c->total_tiles,
                             static_cast<SchedGate*>(c->gate.p), u32(c->tile_offsets),
                             u32(c->sched_keys_a), u32(c->sched_order_a),
                             static_cast<float*>(c->tile_est.p), c->stream),
         "learned schedule keys");
    }
    CK(launch_schedule(c->schedule, u32(c->tile_offsets), c->total_tiles,
                       &dviews(c)->batch_tiles, u32(c->sched_keys_a), u32(c->sched_order_a),
                       u32(c->sched_keys_b), u32(c->sched_order_b),
                       static_cast<float*>(c->tile_est.p), u32(c->sched_status), ctrl_of(c),
                       raster_ctas, strips, split_all, c->sm_count, c->stream),
       "raster schedule");
    order = u32(c->sched_order_a);
    heavy = &ctrl_of(c)->raster_heavy;
  } else if (split_all) {  // row-major order, every tile split
    CK(launch_heavy_count(nullptr, c->total_tiles, raster_ctas, strips, true,
                          &ctrl_of(c)->raster_heavy, c->stream),
       "split all tiles");
    heavy = &ctrl_of(c)->raster_heavy;
  }
  a.heavy = heavy;
  a.proj = static_cast<gs3d_projected_splat*>(c->proj.p);
  a.tile_offsets = u32(c->tile_offsets);
  a.values = u32(c->vals_a);
  a.image = static_cast<uint2*>(c->image.p);
  a.tile_costs = u32(c->tile_costs);
  a.order = order;
  a.queue_counter = &ctrl_of(c)->raster_queue;
  CK(cudaMemsetAsync(a.queue_counter, 0, sizeof(uint32_t), c->stream), "reset raster queue");
  // the previous frame's splat target may still be copying out (captured as
  // an external event wait in graph mode; a never-recorded event is no wait)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(c->stream, &cap), "capture status");
  CK(cudaStreamWaitEvent(c->stream, c->copy_done,
                         cap == cudaStreamCaptureStatusActive ? cudaEventWaitExternal : 0),
     "wait for the previous copy-out");
  CK(launch_raster(a, c->sm_count, c->stream), "rasterize_tiles");
  if (learned)  // the gate measures this frame's prediction error
    CK(launch_gate_update(static_cast<float*>(c->tile_preds.p), u32(c->tile_costs),
                          c->total_tiles, static_cast<SchedGate*>(c->gate.p), c->stream),
       "schedule gate");
  return GS3D_OK;
}

// Fused rebin over the current batch: depth digits sorted over splat-views,
// refs emitted in depth order, tile digits sorted over refs.  For every view
// the sorted keys, values, tile_offsets and image equal the stage-wise
// sequence's.
int fused_rebin(gs3d_ctx* c) {
  TRY(require_frame(c, "rebin"));
  Ctrl* k = ctrl_of(c);
  const uint32_t nv = (uint32_t)c->views.size();
  CK(cudaMemsetAsync(c->ctrl.p, 0, sizeof(Ctrl), c->stream), "reset control block");
  // tile rectangles fit one word when every view has at most 256 tiles per axis
  bool small_grids = true;
  for (const ViewDesc& v : c->views)
    small_grids = small_grids && v.f.tile_count[0] <= 256 && v.f.tile_count[1] <= 256;
  uint32_t* rect8 = small_grids ? u32(c->rect8) : nullptr;
  {
    StageScope t(c, GS3D_STAGE_PREPROCESS);
    CK(launch_preprocess(dviews(c), nv, c->total_blocks, c->max_sh,
                         static_cast<gs3d_projected_splat*>(c->proj.p), u32(c->counts),
                         u32(c->depth_keys_a), u32(c->depth_ids_a), rect8, &k->error, c->stream),
       "preprocess");
  }
  {
    StageScope t(c, GS3D_STAGE_DEPTH_SORT);
    CK(launch_sort_depth_keys(&dviews(c)->batch_splats, c->total_splats, u32(c->depth_keys_a),
                              u32(c->depth_ids_a), u32(c->depth_keys_b), u32(c->depth_ids_b),
                              u32(c->depth_status), &k->sort_hist[0][0],
                              &k->sort_part_counter[0], &k->error, c->sm_count, c->stream),
       "depth sort");
  }
  c->scan_epoch = (c->scan_epoch % ((1u << 30) - 1)) + 1;
  {
    StageScope t(c, GS3D_STAGE_SCAN);
    // cleared every rebin: a graph replay reuses the captured epoch
    CK(cudaMemsetAsync(c->scan_status.p, 0, scan_status_words(c->total_splats) * 8, c->stream),
       "clear scan status");
    CK(launch_scan(u32(c->counts), u32(c->depth_ids_a), u32(c->sorted_offsets), c->total_splats,
                   static_cast<unsigned long long*>(c->scan_status.p), &k->scan_tile_counter,
                   c->scan_epoch, u32(c->ref_counter), &k->error, c->stream),
       "prefix scan (depth order)");
  }
  const SortPlan tp = tile_digit_plan(c->total_tiles, c->digit_bits);
  {
    StageScope t(c, GS3D_STAGE_EMIT);
    CK(launch_emit_sorted(dviews(c), nv, c->total_splats,
                          static_cast<gs3d_projected_splat*>(c->proj.p), rect8, u32(c->depth_keys_a),
                          u32(c->depth_ids_a),
                          u32(c->sorted_offsets), u32(c->ref_counter), c->capacity,
                          static_cast<uint2*>(c->keys_a.p), u32(c->vals_a), tp,
                          &k->tile_hist[0][0], &k->emit_chunk, &k->error, c->sm_count,
                          c->stream),
       "emit (depth order)");
  }
  {
    StageScope t(c, GS3D_STAGE_SORT);
    CK(launch_sort_tile_passes(tp, u32(c->ref_counter), c->capacity,
                               static_cast<uint2*>(c->keys_a.p), u32(c->vals_a),
                               static_cast<uint2*>(c->keys_b.p), u32(c->vals_b),
                               u32(c->sort_status), &k->tile_hist[0][0], &k->sort_part_counter[4],
                               &k->error, c->sm_count, c->stream),
       "tile-digit sort");
  }
  if (tp.passes % 2) {
    std::swap(c->keys_a, c->keys_b);
    std::swap(c->vals_a, c->vals_b);
  }
  {
    StageScope t(c, GS3D_STAGE_IDENTIFY);
    CK(launch_identify(static_cast<uint2*>(c->keys_a.p), u32(c->ref_counter), c->capacity,
                       c->total_tiles, u32(c->tile_offsets), &k->error, c->sm_count, c->stream),
       "identify_tile_ranges");
  }
  return raster_stage(c, true);
}

void destroy_graph(gs3d_ctx* c) {
  if (c->graph.exec) cudaGraphExecDestroy(c->graph.exec);
  c->graph.exec = nullptr;
  c->graph.sig.clear();
}

std::vector<uint64_t> graph_signature(gs3d_ctx* c) {
  std::vector<uint64_t> sig = {c->views.size(), c->tile_w,     c->tile_h,
                               c->schedule,     c->capacity,   c->alloc_gen,
                               c->max_sh,       c->digit_bits, c->raster_batch,
                               c->flags & ~GS3D_FLAG_STAGE_TIMING};
  for (const ViewDesc& v : c->views) {
    sig.push_back((uint64_t)(uintptr_t)v.pos);
    sig.push_back(((uint64_t)v.f.viewport[0] << 32) | v.f.viewport[1]);
    sig.push_back(v.f.splat_count);
  }
  return sig;
}

// Fused rebin through a CUDA graph: captured once per batch signature (the
// view-table upload from a fixed pinned slot, the counter resets and every
// kernel of the rebin), then replayed with only the pinned view table
// rewritten.  Any reallocation or layout change re-captures.
int graph_rebin(gs3d_ctx* c) {
  TRY(require_frame(c, "rebin"));
  const size_t nv = c->views.size();
  std::vector<uint64_t> sig = graph_signature(c);
  if (!c->graph.exec || sig != c->graph.sig) {
    destroy_graph(c);
    if (nv > c->graph.cap) {
      CK(cudaStreamSynchronize(c->stream), "graph view slot");
      if (c->graph.h_views) cudaFreeHost(c->graph.h_views);
      c->graph.h_views = nullptr;
      c->graph.cap = 0;
      CK(cudaMallocHost(&c->graph.h_views, nv * sizeof(ViewDesc)), "graph view slot");
      c->graph.cap = nv;
    }
    if (!c->graph.copied)
      CK(cudaEventCreateWithFlags(&c->graph.copied, cudaEventDisableTiming), "graph event");
    // one eager rebin first: launch configurations are cached and the key
    // buffers sized before anything is captured
    std::memcpy(c->graph.h_views, c->views.data(), nv * sizeof(ViewDesc));
    CK(cudaMemcpyAsync(c->d_views.p, c->graph.h_views, nv * sizeof(ViewDesc),
                       cudaMemcpyHostToDevice, c->stream),
       "upload view table");
    TRY(fused_rebin(c));
    CK(cudaStreamSynchronize(c->stream), "graph warm-up");
    sig = graph_signature(c);
    const uint32_t saved_flags = c->flags;
    c->flags &= ~GS3D_FLAG_STAGE_TIMING;  // no timing events inside the graph
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const cudaError_t ce = cudaMemcpyAsync(c->d_views.p, c->graph.h_views, nv * sizeof(ViewDesc),
                                           cudaMemcpyHostToDevice, c->stream);
    const int rc = ce == cudaSuccess ? fused_rebin(c) : GS3D_ERR_CUDA;
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
    c->flags = saved_flags;
    if (rc != GS3D_OK || ce != cudaSuccess || ee != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return rc != GS3D_OK ? rc : fail(c, GS3D_ERR_CUDA, "rebin graph capture failed");
    }
    const cudaError_t ie = cudaGraphInstantiate(&c->graph.exec, g, 0);
    cudaGraphDestroy(g);
    CK(ie, "graph instantiate");
    c->graph.sig = sig;
    c->graph.result_keys = c->keys_a.p;  // where a replay leaves the sorted keys
  }
  // the previous replay read the pinned table at its start; wait for it
  CK(cudaEventSynchronize(c->graph.copied), "graph view slot reuse");
  std::memcpy(c->graph.h_views, c->views.data(), nv * sizeof(ViewDesc));
  CK(cudaGraphLaunch(c->graph.exec, c->stream), "graph launch");
  CK(cudaEventRecord(c->graph.copied, c->stream), "graph event");
  if (c->keys_a.p != c->graph.result_keys) {  // an eager rebin renamed the ping-pong pair
    std::swap(c->keys_a, c->keys_b);
    std::swap(c->vals_a, c->vals_b);
  }
  return GS3D_OK;
}

}  // namespace

extern "C" {

int gs3d_abi_version(void) { return GS3D_ABI_VERSION; }

const char* gs3d_last_error(const gs3d_ctx* c) { return c ? c->err.c_str() : noalloc_last_error(); }

int gs3d_create(gs3d_ctx** out, const gs3d_config* cfg) {
  if (!out) return GS3D_ERR_INVALID_ARG;
  *out = nullptr;
  gs3d_ctx* c = new (std::nothrow) gs3d_ctx();
  if (!c) return GS3D_ERR_OOM;
  gs3d_config def{};
  if (!cfg) cfg = &def;
  c->device = cfg->device;
  if (cfg->tile_w) c->tile_w = cfg->tile_w;
  if (cfg->tile_h) c->tile_h = cfg->tile_h;
  if (cfg->max_tiles_per_splat) c->max_tiles_per_splat = cfg->max_tiles_per_splat;
  c->flags = cfg->flags;
  auto bail = [&](int rc) {
    gs3d_destroy(c);
    return rc;
  };
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count <= c->device || c->device < 0) {
    cudaGetLastError();
    return bail(GS3D_ERR_NO_DEVICE);
  }
  if (set_device(c) != GS3D_OK) return bail(GS3D_ERR_NO_DEVICE);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) return bail(GS3D_ERR_NO_DEVICE);
  if (prop.major != 10 || prop.minor != 3) {
    fprintf(stderr, "gs3d: device %d is sm_%d%d; this library is built for sm_103a only\n",
            c->device, prop.major, prop.minor);
    return bail(GS3D_ERR_NO_DEVICE);
  }
  c->sm_count = prop.multiProcessorCount;
  if (cfg->stream) {
    c->stream = static_cast<cudaStream_t>(cfg->stream);
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
      return bail(GS3D_ERR_CUDA);
    c->own_stream = true;
  }
  probe_kernel<<<1, 1, 0, c->stream>>>(nullptr);
  if (cudaGetLastError() != cudaSuccess) return bail(GS3D_ERR_NO_DEVICE);
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->frame_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming) != cudaSuccess)
    return bail(GS3D_ERR_CUDA);
  c->scenes.resize(1);
  if (ensure(c, c->ctrl, sizeof(Ctrl), "control block") != GS3D_OK ||
      ensure(c, c->ref_counter, 16, "ref_counter") != GS3D_OK)
    return bail(GS3D_ERR_OOM);
  if (cudaMallocHost(&c->h_word, 64) != cudaSuccess) return bail(GS3D_ERR_OOM);
  for (int i = 0; i < kUploadSlots; ++i)
    if (cudaEventCreateWithFlags(&c->upload_ev[i], cudaEventDisableTiming) != cudaSuccess)
      return bail(GS3D_ERR_CUDA);
  if (cudaMemsetAsync(c->ctrl.p, 0, sizeof(Ctrl), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->ref_counter.p, 0, 16, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return bail(GS3D_ERR_CUDA);
  *out = c;
  return GS3D_OK;
}

int gs3d_destroy(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (SceneBufs& s : c->scenes) {
    release(s.pos);
    release(s.scale);
    release(s.rot);
    release(s.color);
    release(s.sh);
  }
  DevBuf* bufs[] = {&c->proj,          &c->counts,        &c->offsets,       &c->ref_counter,
                    &c->keys_a,        &c->vals_a,        &c->keys_b,        &c->vals_b,
                    &c->scan_status,   &c->sort_status,   &c->depth_keys_a,  &c->depth_ids_a,
                    &c->depth_keys_b,  &c->depth_ids_b,   &c->sorted_offsets, &c->depth_status,
                    &c->rect8,
                    &c->tile_offsets,  &c->image,         &c->tile_costs,    &c->sched_keys_a,
                    &c->sched_keys_b,  &c->sched_order_a, &c->sched_order_b, &c->sched_status,
                    &c->d_views,       &c->ctrl,          &c->model_params,  &c->model_mean,
                    &c->model_inv_std, &c->tile_feats,    &c->tile_preds,    &c->composite_out,
                    &c->tile_est,      &c->gate};
  for (DevBuf* b : bufs) release(*b);
  for (int i = 0; i < kUploadSlots; ++i)
    if (c->upload_ev[i]) cudaEventDestroy(c->upload_ev[i]);
  for (auto& e : c->ev_pool) cudaEventDestroy(e);
  destroy_graph(c);
  if (c->graph.copied) cudaEventDestroy(c->graph.copied);
  if (c->graph.h_views) cudaFreeHost(c->graph.h_views);
  if (c->h_upload) cudaFreeHost(c->h_upload);
  if (c->h_word) cudaFreeHost(c->h_word);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->frame_done) cudaEventDestroy(c->frame_done);
  if (c->copy_done) cudaEventDestroy(c->copy_done);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return GS3D_OK;
}

int gs3d_set_splats(gs3d_ctx* c, uint32_t n, const float* positions, const float* scales,
                    const float* rotations, const float* colors, const float* sh_rest,
                    uint32_t sh_degree, int memory) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(upload_scene(c, c->scenes[0], n, positions, scales, rotations, colors, sh_rest, sh_degree,
                   memory));
  // resizeBinningBuffers (GaussianSplatRenderer.ts:209-227)
  TRY(ensure_splat_buffers(c, n));
  TRY(ensure_key_capacity(
      c, std::min<uint64_t>((uint64_t)std::max<uint32_t>(n, 1) * c->max_tiles_per_splat,
                            kMaxCapacity)));
  c->have_scene = true;
  c->have_camera = false;  // the view table refers to the scene's size
  return GS3D_OK;
}

int gs3d_add_scene(gs3d_ctx* c, uint32_t n, const float* positions, const float* scales,
                   const float* rotations, const float* colors, const float* sh_rest,
                   uint32_t sh_degree, int memory, uint32_t* out_scene) {
  if (!c || !out_scene) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  SceneBufs sc;
  const int rc = upload_scene(c, sc, n, positions, scales, rotations, colors, sh_rest, sh_degree,
                              memory);
  if (rc != GS3D_OK) {
    release(sc.pos);
    release(sc.scale);
    release(sc.rot);
    release(sc.color);
    release(sc.sh);
    return rc;
  }
  if (!c->have_scene) {  // the first scene also fills slot 0
    c->scenes[0] = sc;
    *out_scene = 0;
  } else {
    c->scenes.push_back(sc);
    *out_scene = (uint32_t)c->scenes.size() - 1;
  }
  c->have_scene = true;
  return GS3D_OK;
}

int gs3d_composite(gs3d_ctx* c, uint32_t view, uint32_t mode, uint32_t debug_ref,
                   const float background[4], void* rgba8, size_t bytes, int memory) {
  if (!c || !rgba8) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  if (mode > GS3D_COMPOSITE_TILE_HEATMAP)
    return fail(c, GS3D_ERR_INVALID_ARG, "unknown composite mode %u", mode);
  if (memory != 0 && memory != 1) return fail(c, GS3D_ERR_INVALID_ARG, "memory must be 0 or 1");
  if (view >= c->info.size())
    return fail(c, GS3D_ERR_STATE, "composite: view %u of %zu rendered", view, c->info.size());
  TRY(set_device(c));
  const gs3d_view_info& v = c->info[view];
  const size_t need = (size_t)v.width * v.height * 4;
  if (bytes < need)
    return fail(c, GS3D_ERR_INVALID_ARG, "composite needs %zu bytes, got %zu", need, bytes);
  const float zero[4] = {0.f, 0.f, 0.f, 0.f};
  uint32_t* dst = static_cast<uint32_t*>(rgba8);
  if (memory == 0) {
    TRY(ensure(c, c->composite_out, std::max<size_t>(need, 4), "composite target"));
    dst = static_cast<uint32_t*>(c->composite_out.p);
  }
  CK(launch_composite(static_cast<const uint2*>(c->image.p) + v.pixel_offset, v.width, v.height,
                      u32(c->tile_offsets) + v.tile_base, c->tile_w, c->tile_h, v.tiles_x,
                      v.tiles_y, mode, debug_ref ? debug_ref : 256u,
                      background ? background : zero, dst, c->stream),
     "composite");
  if (memory == 0) {
    CK(cudaMemcpyAsync(rgba8, dst, need, cudaMemcpyDeviceToHost, c->stream), "composite copy");
    CK(cudaStreamSynchronize(c->stream), "composite copy");
  }
  return GS3D_OK;
}

int gs3d_load_ply(gs3d_ctx* c, const void* data, size_t size, uint32_t target,
                  uint32_t* out_scene, gs3d_ply_info* info) {
  if (!c || !data) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  if (target != 0 && target != GS3D_PLY_NEW_SCENE)
    return fail(c, GS3D_ERR_INVALID_ARG, "target must be 0 or GS3D_PLY_NEW_SCENE");
  TRY(set_device(c));
  const uint8_t* bytes = static_cast<const uint8_t*>(data);
  PlyLayout lay;
  std::string err;
  if (!ply_parse_layout(bytes, size, &lay, &err))
    return fail(c, GS3D_ERR_INVALID_ARG, "%s", err.c_str());
  const uint8_t* rows = bytes + lay.rows_offset;
  std::vector<double> ascii;
  if (lay.format == GS3D_PLY_ASCII) {
    if (!ply_ascii_rows(bytes, size, lay, &ascii, &err))
      return fail(c, GS3D_ERR_INVALID_ARG, "%s", err.c_str());
    rows = reinterpret_cast<const uint8_t*>(ascii.data());
  }
  const uint32_t n = (uint32_t)lay.count;
  const uint32_t deg = lay.sh_k ? lay.sh_degree : 0u;
  SceneBufs fresh;
  SceneBufs& sc = target == 0 ? c->scenes[0] : fresh;
  const size_t v4 = (size_t)n * 16;
  DevBuf d_rows, d_words;
  auto cleanup = [&](int rc) {
    release(d_rows);
    release(d_words);
    if (&sc == &fresh) {
      release(fresh.pos);
      release(fresh.scale);
      release(fresh.rot);
      release(fresh.color);
      release(fresh.sh);
    }
    return rc;
  };
  int rc = GS3D_OK;
  if ((rc = ensure(c, sc.pos, v4, "splat_positions")) || (rc = ensure(c, sc.scale, v4, "splat_scales")) ||
      (rc = ensure(c, sc.rot, v4, "splat_rotations")) || (rc = ensure(c, sc.color, v4, "splat_colors")) ||
      (lay.sh_k && (rc = ensure(c, sc.sh, (size_t)n * 3 * lay.sh_k * sizeof(float), "splat_sh_rest"))) ||
      (rc = ensure(c, d_rows, std::max<size_t>((size_t)n * lay.stride, 16), "ply rows")) ||
      (rc = ensure(c, d_words, 64, "ply status")))
    return cleanup(rc);
  uint32_t words[7] = {0u, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  cudaError_t e = cudaMemcpyAsync(d_words.p, words, sizeof(words), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && n)
    e = cudaMemcpyAsync(d_rows.p, rows, (size_t)n * lay.stride, cudaMemcpyHostToDevice, c->stream);
  uint32_t* dw = static_cast<uint32_t*>(d_words.p);
  if (e == cudaSuccess)
    e = launch_ply_decode(static_cast<const uint8_t*>(d_rows.p), n, lay,
                          lay.format == GS3D_PLY_BINARY_BE, static_cast<float4*>(sc.pos.p),
                          static_cast<float4*>(sc.scale.p), static_cast<float4*>(sc.rot.p),
                          static_cast<float4*>(sc.color.p), static_cast<float*>(sc.sh.p), dw,
                          dw + 1, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(words, d_words.p, sizeof(words), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cleanup(cuda_fail(c, e, "ply decode"));
  if (words[0] != 0)
    return cleanup(fail(c, GS3D_ERR_INVALID_ARG, "Invalid Gaussian Splat PLY row: missing '%s'",
                        ply_required_name((int)words[0] - 1)));
  release(d_rows);
  release(d_words);
  sc.n = n;
  sc.sh_degree = deg;
  if (&sc == &fresh) {
    if (!c->have_scene) {
      c->scenes[0] = fresh;
      if (out_scene) *out_scene = 0;
    } else {
      c->scenes.push_back(fresh);
      if (out_scene) *out_scene = (uint32_t)c->scenes.size() - 1;
    }
  } else {
    if (out_scene) *out_scene = 0;
    TRY(ensure_splat_buffers(c, n));
    TRY(ensure_key_capacity(
        c, std::min<uint64_t>((uint64_t)std::max<uint32_t>(n, 1) * c->max_tiles_per_splat,
                              kMaxCapacity)));
    c->have_camera = false;
  }
  c->have_scene = true;
  if (info) {
    *info = gs3d_ply_info{};
    info->splat_count = lay.count;
    info->header_bytes = lay.header_bytes;
    info->format = lay.format;
    info->f_rest_count = lay.f_rest_count;
    info->sh_degree = lay.sh_degree;
    info->vertex_stride = lay.format == GS3D_PLY_ASCII ? 0u : lay.stride;
    auto unord = [](uint32_t o) {
      const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
      float f;
      std::memcpy(&f, &u, 4);
      return f;
    };
    for (int k = 0; k < 3; ++k) {
      info->bounds_min[k] = n ? unord(words[1 + k]) : 0.0f;
      info->bounds_max[k] = n ? unord(words[4 + k]) : 0.0f;
    }
  }
  return GS3D_OK;
}

namespace {
void apply_tile_size(gs3d_ctx* c, uint32_t tx, uint32_t ty) {
  if (tx != c->tile_w || ty != c->tile_h) {
    c->tile_w = tx;
    c->tile_h = ty;
    c->have_camera = false;  // tile grid recomputed at the next set_camera
  }
}
}  // namespace

int gs3d_set_tile_size(gs3d_ctx* c, uint32_t tx, uint32_t ty, uint32_t* out_x, uint32_t* out_y) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  // clampTileSize (GaussianSplatRenderer.ts:162-167) with CUDA's 1024-thread block limit
  tx = std::max<uint32_t>(1, std::min<uint32_t>(tx ? tx : 1, 1024));
  ty = std::max<uint32_t>(1, std::min<uint32_t>(ty ? ty : 1, 1024 / tx));
  apply_tile_size(c, tx, ty);
  if (out_x) *out_x = tx;
  if (out_y) *out_y = ty;
  return GS3D_OK;
}

int gs3d_set_camera(gs3d_ctx* c, const gs3d_camera* cam, uint32_t width, uint32_t height) {
  if (!c || !cam) return fail(c, GS3D_ERR_INVALID_ARG, "null camera");
  if (!c->have_scene) return fail(c, GS3D_ERR_STATE, "set_camera: no splats set");
  TRY(set_device(c));
  gs3d_view v{};
  v.camera = *cam;
  v.scene = 0;
  v.width = width;
  v.height = height;
  return set_views(c, &v, 1);
}

int gs3d_preprocess(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_single(c, "preprocess"));
  TRY(set_device(c));
  // start of a frame: counters, histograms and the error latch
  CK(cudaMemsetAsync(c->ctrl.p, 0, sizeof(Ctrl), c->stream), "reset control block");
  StageScope t(c, GS3D_STAGE_PREPROCESS);
  CK(launch_preprocess(dviews(c), 1, c->total_blocks, c->max_sh,
                       static_cast<gs3d_projected_splat*>(c->proj.p), u32(c->counts), nullptr,
                       nullptr, nullptr, &ctrl_of(c)->error, c->stream),
     "preprocess");
  return GS3D_OK;
}

int gs3d_prefix_scan(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_single(c, "prefix_scan"));
  TRY(set_device(c));
  CK(cudaMemsetAsync(&ctrl_of(c)->scan_tile_counter, 0, sizeof(uint32_t), c->stream),
     "reset scan ticket");
  c->scan_epoch = (c->scan_epoch % ((1u << 30) - 1)) + 1;  // 1 .. 2^30-1, never 0
  StageScope t(c, GS3D_STAGE_SCAN);
  CK(cudaMemsetAsync(c->scan_status.p, 0, scan_status_words(c->total_splats) * 8, c->stream),
     "clear scan status");
  CK(launch_scan(u32(c->counts), nullptr, u32(c->offsets), c->total_splats,
                 static_cast<unsigned long long*>(c->scan_status.p),
                 &ctrl_of(c)->scan_tile_counter, c->scan_epoch, u32(c->ref_counter),
                 &ctrl_of(c)->error, c->stream),
     "prefix scan");
  return GS3D_OK;
}

int gs3d_emit_tile_refs(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_single(c, "emit_tile_refs"));
  TRY(set_device(c));
  StageScope t(c, GS3D_STAGE_EMIT);
  CK(launch_emit(&dviews(c)->f, c->total_splats, static_cast<gs3d_projected_splat*>(c->proj.p),
                 u32(c->offsets), u32(c->ref_counter), c->capacity,
                 static_cast<uint2*>(c->keys_a.p), u32(c->vals_a), &ctrl_of(c)->error,
                 c->stream),
     "emit_tile_refs");
  return GS3D_OK;
}

int gs3d_radix_sort(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_single(c, "radix_sort"));
  TRY(set_device(c));
  // the stage-wise sort builds 256-bin histograms: digits of at most 8 bits
  const SortPlan plan = make_sort_plan(c->total_tiles, (int)std::min<uint32_t>(c->digit_bits, 8));
  {
    StageScope t(c, GS3D_STAGE_SORT);
    CK(launch_sort(plan, u32(c->ref_counter), c->capacity, static_cast<uint2*>(c->keys_a.p),
                   u32(c->vals_a), static_cast<uint2*>(c->keys_b.p), u32(c->vals_b),
                   u32(c->sort_status), ctrl_of(c), c->sm_count, c->stream),
       "radix sort");
  }
  if (plan.passes % 2) {  // sorted data ended in the B buffers: rename
    std::swap(c->keys_a, c->keys_b);
    std::swap(c->vals_a, c->vals_b);
  }
  return GS3D_OK;
}

int gs3d_identify_tile_ranges(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_frame(c, "identify_tile_ranges"));
  TRY(set_device(c));
  StageScope t(c, GS3D_STAGE_IDENTIFY);
  CK(launch_identify(static_cast<uint2*>(c->keys_a.p), u32(c->ref_counter), c->capacity,
                     c->total_tiles, u32(c->tile_offsets), &ctrl_of(c)->error, c->sm_count,
                     c->stream),
     "identify_tile_ranges");
  return GS3D_OK;
}

int gs3d_rasterize_tiles(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(require_frame(c, "rasterize_tiles"));
  TRY(set_device(c));
  return raster_stage(c, /*culled=*/!(c->flags & GS3D_FLAG_STAGEWISE_REBIN));
}

int gs3d_rebin(gs3d_ctx* c, const gs3d_camera* cam, uint32_t width, uint32_t height) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(set_device(c));
  if ((c->flags & GS3D_FLAG_CUDA_GRAPH) && !(c->flags & GS3D_FLAG_STAGEWISE_REBIN)) {
    if (!cam) return fail(c, GS3D_ERR_INVALID_ARG, "null camera");
    if (!c->have_scene) return fail(c, GS3D_ERR_STATE, "rebin: no splats set");
    gs3d_view v{};
    v.camera = *cam;
    v.width = width;
    v.height = height;
    TRY(set_views(c, &v, 1, false));
    return graph_rebin(c);
  }
  TRY(gs3d_set_camera(c, cam, width, height));
  if (!(c->flags & GS3D_FLAG_STAGEWISE_REBIN)) return fused_rebin(c);
  TRY(gs3d_preprocess(c));
  TRY(gs3d_prefix_scan(c));
  TRY(gs3d_emit_tile_refs(c));
  TRY(gs3d_radix_sort(c));
  TRY(gs3d_identify_tile_ranges(c));
  TRY(gs3d_rasterize_tiles(c));
  return GS3D_OK;
}

int gs3d_rebin_batch(gs3d_ctx* c, const gs3d_view* views, uint32_t n_views) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  if (!c->have_scene) return fail(c, GS3D_ERR_STATE, "rebin_batch: no scene");
  TRY(set_device(c));
  if (c->flags & GS3D_FLAG_CUDA_GRAPH) {
    TRY(set_views(c, views, n_views, false));
    return graph_rebin(c);
  }
  TRY(set_views(c, views, n_views));
  return fused_rebin(c);
}

int gs3d_get_view_info(gs3d_ctx* c, uint32_t view, gs3d_view_info* out) {
  if (!c || !out) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  if (view >= c->info.size())
    return fail(c, GS3D_ERR_INVALID_ARG, "view %u out of range (%zu views)", view,
                c->info.size());
  *out = c->info[view];
  return GS3D_OK;
}

int gs3d_set_tuning(gs3d_ctx* c, const gs3d_tuning* t) {
  if (!c || !t) return fail(c, GS3D_ERR_INVALID_ARG, "null tuning");
  if (t->digit_bits != 4 && t->digit_bits != 6 && t->digit_bits != 8 && t->digit_bits != 11)
    return fail(c, GS3D_ERR_INVALID_ARG, "digit_bits must be 4, 6, 8 or 11 (got %u)",
                t->digit_bits);
  if (t->raster_batch % 32 != 0 || t->raster_batch > 1024)
    return fail(c, GS3D_ERR_INVALID_ARG,
                "raster_batch must be 0 or a multiple of 32 up to 1024 (got %u)",
                t->raster_batch);
  // up to 1024 pixels; up to 2048 where the two-pixel raster shades the tile
  // as row strips of at most 512 threads (sides multiples of 8 and 16)
  const uint64_t area = (uint64_t)t->tile_w * t->tile_h;
  const bool wide = area > 1024 && area <= 2048 && t->tile_w % 8 == 0 && t->tile_h % 16 == 0;
  if (t->tile_w == 0 || t->tile_h == 0 || (area > 1024 && !wide))
    return fail(c, GS3D_ERR_INVALID_ARG,
                "tile %ux%u: 1..1024 pixels, or up to 2048 with a width that divides by 8 "
                "and a height by 16",
                t->tile_w, t->tile_h);
  apply_tile_size(c, t->tile_w, t->tile_h);
  c->digit_bits = t->digit_bits;
  c->raster_batch = t->raster_batch;
  return GS3D_OK;
}

int gs3d_get_tuning(gs3d_ctx* c, gs3d_tuning* out) {
  if (!c || !out) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  out->tile_w = c->tile_w;
  out->tile_h = c->tile_h;
  out->digit_bits = c->digit_bits;
  out->raster_batch = c->raster_batch;
  return GS3D_OK;
}

int gs3d_autotune(gs3d_ctx* c, const gs3d_view* views, uint32_t n_views, uint32_t reps,
                  gs3d_tune_result* results, uint32_t max_results, uint32_t* n_results) {
  if (!c || !views || n_views == 0)
    return fail(c, GS3D_ERR_INVALID_ARG, "autotune needs at least one view");
  if (!c->have_scene) return fail(c, GS3D_ERR_STATE, "autotune: no scene");
  TRY(set_device(c));
  if (n_results) *n_results = 0;
  if (reps == 0) reps = 3;
  gs3d_tuning saved{};
  TRY(gs3d_get_tuning(c, &saved));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0), "autotune event");
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(c, GS3D_ERR_CUDA, "autotune event");
  }
  std::vector<gs3d_tune_result> res;
  int rc = GS3D_OK;
  // square tiles of 8, 16 and 32, and the 2048-pixel 32x64 and 64x32
  const uint32_t shapes[][2] = {{8, 8}, {16, 16}, {32, 32}, {32, 64}, {64, 32}};
  const uint32_t digits[] = {4, 8, 11}, batches[] = {128, 256, 512};
  for (const auto& shape : shapes) {
    for (uint32_t digit : digits) {
      for (uint32_t batch : batches) {
        const gs3d_tuning t{shape[0], shape[1], digit, batch};
        rc = gs3d_set_tuning(c, &t);
        if (rc != GS3D_OK) break;
        // warm-up: sizes the key buffers (capacity retries), captures the graph
        int wr = GS3D_ERR_CAPACITY;
        for (int attempt = 0; attempt < 3 && wr == GS3D_ERR_CAPACITY; ++attempt) {
          wr = gs3d_rebin_batch(c, views, n_views);
          if (wr == GS3D_OK) wr = gs3d_synchronize(c);
        }
        if (wr == GS3D_ERR_CAPACITY) continue;  // beyond the ref limit under this tile size
        if (wr != GS3D_OK) {
          rc = wr;
          break;
        }
        cudaEventRecord(e0, c->stream);
        for (uint32_t r = 0; r < reps && rc == GS3D_OK; ++r) rc = gs3d_rebin_batch(c, views, n_views);
        cudaEventRecord(e1, c->stream);
        if (rc == GS3D_OK) rc = gs3d_synchronize(c);
        if (rc != GS3D_OK) break;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
          rc = fail(c, GS3D_ERR_CUDA, "autotune timing");
          break;
        }
        uint32_t refs = 0;
        rc = gs3d_ref_count(c, &refs);
        if (rc != GS3D_OK) break;
        gs3d_tune_result r{};
        r.tuning = t;
        r.ms_per_view = ms / (float)reps / (float)n_views;
        r.tile_passes = (uint32_t)tile_digit_plan(c->total_tiles, digit).passes;
        r.refs = refs;
        res.push_back(r);
      }
      if (rc != GS3D_OK) break;
    }
    if (rc != GS3D_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != GS3D_OK || res.empty()) {
    const std::string why = rc != GS3D_OK ? c->err : std::string("no candidate fitted");
    gs3d_set_tuning(c, &saved);
    return fail(c, rc != GS3D_OK ? rc : GS3D_ERR_CAPACITY, "autotune: %s", why.c_str());
  }
  size_t best = 0;
  for (size_t i = 1; i < res.size(); ++i)
    if (res[i].ms_per_view < res[best].ms_per_view) best = i;
  TRY(gs3d_set_tuning(c, &res[best].tuning));
  if (results)
    for (size_t i = 0; i < res.size() && i < max_results; ++i) results[i] = res[i];
  if (n_results) *n_results = (uint32_t)res.size();
  return GS3D_OK;
}

int gs3d_set_schedule(gs3d_ctx* c, uint32_t schedule) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  if (schedule > GS3D_SCHEDULE_LEARNED)
    return fail(c, GS3D_ERR_INVALID_ARG, "unknown schedule %u", schedule);
  if (schedule == GS3D_SCHEDULE_LEARNED && !c->have_model)
    return fail(c, GS3D_ERR_STATE, "the learned schedule needs gs3d_set_cost_model first");
  c->schedule = schedule;
  return GS3D_OK;
}

int gs3d_set_cost_model(gs3d_ctx* c, const float* params, const float* mean, const float* std_) {
  if (!c || !params || !mean || !std_) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  TRY(set_device(c));
  float inv[kFeatures];
  for (int k = 0; k < kFeatures; ++k) {
    if (!(std_[k] > 0.0f)) return fail(c, GS3D_ERR_INVALID_ARG, "feature std %d is not > 0", k);
    inv[k] = 1.0f / std_[k];
  }
  TRY(ensure(c, c->model_params, kMlpParams * 4, "cost model"));
  TRY(ensure(c, c->model_mean, kFeatures * 4, "cost model"));
  TRY(ensure(c, c->model_inv_std, kFeatures * 4, "cost model"));
  CK(cudaStreamSynchronize(c->stream), "install cost model");
  CK(cudaMemcpy(c->model_params.p, params, kMlpParams * 4, cudaMemcpyHostToDevice), "cost model");
  CK(cudaMemcpy(c->model_mean.p, mean, kFeatures * 4, cudaMemcpyHostToDevice), "cost model");
  CK(cudaMemcpy(c->model_inv_std.p, inv, kFeatures * 4, cudaMemcpyHostToDevice), "cost model");
  // a new model starts trusted, its running error unmeasured
  TRY(ensure(c, c->gate, sizeof(SchedGate), "schedule gate"));
  SchedGate g{};
  g.bound = c->gate_bound;
  g.use_learned = 1;
  CK(cudaMemcpy(c->gate.p, &g, sizeof(g), cudaMemcpyHostToDevice), "schedule gate");
  c->have_model = true;
  return GS3D_OK;
}

int gs3d_set_schedule_gate(gs3d_ctx* c, float bound) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  if (!(bound >= 0.0f)) return fail(c, GS3D_ERR_INVALID_ARG, "gate bound must be >= 0");
  TRY(set_device(c));
  c->gate_bound = bound;
  if (c->gate.p) {  // stream ordered with the rebins that read it
    CK(cudaMemcpyAsync(&static_cast<SchedGate*>(c->gate.p)->bound, &c->gate_bound,
                       sizeof(float), cudaMemcpyHostToDevice, c->stream),
       "schedule gate");
    CK(cudaStreamSynchronize(c->stream), "schedule gate");
  }
  return GS3D_OK;
}

int gs3d_get_schedule_status(gs3d_ctx* c, gs3d_schedule_status* out) {
  if (!c || !out) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  TRY(set_device(c));
  TRY(sync_and_check(c));
  *out = gs3d_schedule_status{};
  out->schedule = c->schedule;
  out->active = c->schedule;
  out->bound = c->gate_bound;
  if (c->gate.p) {
    SchedGate g{};
    CK(cudaMemcpy(&g, c->gate.p, sizeof(g), cudaMemcpyDeviceToHost), "schedule gate");
    out->mae_log = g.mae;
    out->last_mae_log = g.last_mae;
    out->frames = g.frames;
    out->fallbacks = g.fallbacks;
    if (c->schedule == GS3D_SCHEDULE_LEARNED && g.frames > 0 && !g.used_learned)
      out->active = GS3D_SCHEDULE_KEY_COUNT;
  }
  if (c->ctrl.p) {
    CK(cudaMemcpy(&out->split_tiles, &ctrl_of(c)->raster_heavy, sizeof(uint32_t),
                  cudaMemcpyDeviceToHost),
       "split tiles");
  }
  return GS3D_OK;
}

int gs3d_tile_features(gs3d_ctx* c, float* features, float* targets, uint32_t n_tiles,
                       int memory) {
  if (!c || !features) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  if (memory != 0 && memory != 1) return fail(c, GS3D_ERR_INVALID_ARG, "memory must be 0 or 1");
  TRY(require_frame(c, "tile_features"));
  if (n_tiles < c->total_tiles)
    return fail(c, GS3D_ERR_INVALID_ARG, "room for %u tiles, the frame has %u", n_tiles,
                c->total_tiles);
  TRY(set_device(c));
  float* fdst = memory ? features : static_cast<float*>(c->tile_feats.p);
  CK(launch_tile_features(dviews(c), (uint32_t)c->views.size(), c->total_tiles, c->tile_w,
                          c->tile_h, u32(c->tile_offsets), u32(c->vals_a),
                          static_cast<gs3d_projected_splat*>(c->proj.p), nullptr, nullptr, fdst,
                          c->stream),
     "tile features");
  float* tdst = nullptr;
  if (targets) {
    tdst = memory ? targets : static_cast<float*>(c->tile_preds.p);
    CK(launch_log_costs(u32(c->tile_costs), c->total_tiles, tdst, c->stream), "tile targets");
  }
  if (!memory) {
    TRY(sync_and_check(c));
    CK(cudaMemcpy(features, fdst, (size_t)c->total_tiles * kFeatures * 4, cudaMemcpyDeviceToHost),
       "features copy-out");
    if (targets)
      CK(cudaMemcpy(targets, tdst, (size_t)c->total_tiles * 4, cudaMemcpyDeviceToHost),
         "targets copy-out");
  }
  return GS3D_OK;
}

int gs3d_mlp_forward(const float* params, const float* x, uint32_t n, float* acts, float* y,
                     void* stream) {
  if (!params || !x || !acts || !y) return GS3D_ERR_INVALID_ARG;
  return launch_mlp_forward(params, x, n, acts, y, static_cast<cudaStream_t>(stream)) ==
                 cudaSuccess
             ? GS3D_OK
             : GS3D_ERR_CUDA;
}

int gs3d_mlp_backward(const float* params, const float* x, const float* acts,
                      const float* target, uint32_t n, float* grads, void* stream) {
  if (!params || !x || !acts || !target || !grads) return GS3D_ERR_INVALID_ARG;
  return launch_mlp_backward(params, x, acts, target, n, grads,
                             static_cast<cudaStream_t>(stream)) == cudaSuccess
             ? GS3D_OK
             : GS3D_ERR_CUDA;
}

int gs3d_mlp_adam(float* p, float* m, float* v, const float* g, uint32_t count, float lr,
                  float beta1, float beta2, float eps, uint32_t step, void* stream) {
  if (!p || !m || !v || !g || step == 0) return GS3D_ERR_INVALID_ARG;
  return launch_adam(p, m, v, g, count, lr, beta1, beta2, eps, step,
                     static_cast<cudaStream_t>(stream)) == cudaSuccess
             ? GS3D_OK
             : GS3D_ERR_CUDA;
}

int gs3d_mlp_infer(const float* params, const float* x, uint32_t n, float* y, void* stream) {
  if (!params || !x || !y) return GS3D_ERR_INVALID_ARG;
  return launch_mlp_infer(params, x, n, y, static_cast<cudaStream_t>(stream)) == cudaSuccess
             ? GS3D_OK
             : GS3D_ERR_CUDA;
}

int gs3d_read_stage_times(gs3d_ctx* c, double* ms, uint32_t* n) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(set_device(c));
  TRY(drain_timing(c));
  for (int i = 0; i < GS3D_STAGE_COUNT; ++i) {
    if (ms) ms[i] = c->stage_ms[i];
    if (n) n[i] = c->stage_n[i];
    c->stage_ms[i] = 0.0;
    c->stage_n[i] = 0;
  }
  return GS3D_OK;
}

int gs3d_set_flags(gs3d_ctx* c, uint32_t flags) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  if (flags & ~(GS3D_FLAG_STAGEWISE_REBIN | GS3D_FLAG_STAGE_TIMING | GS3D_FLAG_CUDA_GRAPH |
                GS3D_FLAG_SPLIT_ALL_TILES))
    return fail(c, GS3D_ERR_INVALID_ARG, "unknown flag bits 0x%x", flags);
  c->flags = flags;
  return GS3D_OK;
}

int gs3d_synchronize(gs3d_ctx* c) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  TRY(set_device(c));
  return sync_and_check(c);
}

static DevBuf* named(gs3d_ctx* c, gs3d_buffer which) {
  SceneBufs& s0 = c->scenes[0];
  switch (which) {
    case GS3D_BUF_SPLAT_POSITIONS: return &s0.pos;
    case GS3D_BUF_SPLAT_SCALES: return &s0.scale;
    case GS3D_BUF_SPLAT_ROTATIONS: return &s0.rot;
    case GS3D_BUF_SPLAT_COLORS: return &s0.color;
    case GS3D_BUF_SPLAT_SH_REST: return &s0.sh;
    case GS3D_BUF_PROJECTED_SPLATS: return &c->proj;
    case GS3D_BUF_SPLAT_REF_COUNTS: return &c->counts;
    case GS3D_BUF_SPLAT_REF_OFFSETS: return &c->offsets;
    case GS3D_BUF_REF_COUNTER: return &c->ref_counter;
    case GS3D_BUF_SORT_KEYS_A: return &c->keys_a;
    case GS3D_BUF_SORT_VALUES_A: return &c->vals_a;
    case GS3D_BUF_SORT_KEYS_B: return &c->keys_b;
    case GS3D_BUF_SORT_VALUES_B: return &c->vals_b;
    case GS3D_BUF_TILE_OFFSETS: return &c->tile_offsets;
    case GS3D_BUF_SPLAT_TARGET: return &c->image;
    case GS3D_BUF_TILE_COSTS: return &c->tile_costs;
    default: return nullptr;
  }
}

int gs3d_buffer_info(gs3d_ctx* c, gs3d_buffer which, void** ptr, size_t* bytes) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  DevBuf* b = named(c, which);
  if (!b) return fail(c, GS3D_ERR_INVALID_ARG, "unknown buffer %d", (int)which);
  if (ptr) *ptr = b->p;
  if (bytes) *bytes = b->bytes;
  return GS3D_OK;
}

int gs3d_read_buffer(gs3d_ctx* c, gs3d_buffer which, void* dst, size_t bytes) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  DevBuf* b = named(c, which);
  if (!b) return fail(c, GS3D_ERR_INVALID_ARG, "unknown buffer %d", (int)which);
  if (bytes > b->bytes)
    return fail(c, GS3D_ERR_INVALID_ARG, "read of %zu bytes from a %zu-byte buffer", bytes,
                b->bytes);
  if (bytes && !dst) return fail(c, GS3D_ERR_INVALID_ARG, "null destination");
  TRY(set_device(c));
  TRY(sync_and_check(c));
  if (bytes) CK(cudaMemcpy(dst, b->p, bytes, cudaMemcpyDeviceToHost), "copy-out");
  return GS3D_OK;
}

int gs3d_read_buffer_range(gs3d_ctx* c, gs3d_buffer which, size_t offset, void* dst,
                           size_t bytes) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  DevBuf* b = named(c, which);
  if (!b) return fail(c, GS3D_ERR_INVALID_ARG, "unknown buffer %d", (int)which);
  if (offset > b->bytes || bytes > b->bytes - offset)
    return fail(c, GS3D_ERR_INVALID_ARG, "read of [%zu, +%zu) from a %zu-byte buffer", offset,
                bytes, b->bytes);
  if (bytes && !dst) return fail(c, GS3D_ERR_INVALID_ARG, "null destination");
  TRY(set_device(c));
  TRY(sync_and_check(c));
  if (bytes)
    CK(cudaMemcpy(dst, static_cast<const char*>(b->p) + offset, bytes, cudaMemcpyDeviceToHost),
       "copy-out");
  return GS3D_OK;
}

int gs3d_write_buffer(gs3d_ctx* c, gs3d_buffer which, const void* src, size_t bytes) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  DevBuf* b = named(c, which);
  if (!b) return fail(c, GS3D_ERR_INVALID_ARG, "unknown buffer %d", (int)which);
  if (bytes > b->bytes)
    return fail(c, GS3D_ERR_INVALID_ARG, "write of %zu bytes into a %zu-byte buffer", bytes,
                b->bytes);
  if (bytes && !src) return fail(c, GS3D_ERR_INVALID_ARG, "null source");
  TRY(set_device(c));
  CK(cudaStreamSynchronize(c->stream), "synchronize before copy-in");
  CK(cudaStreamSynchronize(c->copy_stream), "copy-outs before copy-in");
  if (bytes) CK(cudaMemcpy(b->p, src, bytes, cudaMemcpyHostToDevice), "copy-in");
  return GS3D_OK;
}

int gs3d_copy_buffer_async(gs3d_ctx* c, gs3d_buffer which, void* dst, size_t bytes) {
  if (!c) return GS3D_ERR_INVALID_ARG;
  DevBuf* b = named(c, which);
  if (!b) return fail(c, GS3D_ERR_INVALID_ARG, "unknown buffer %d", (int)which);
  if (bytes > b->bytes)
    return fail(c, GS3D_ERR_INVALID_ARG, "copy of %zu bytes from a %zu-byte buffer", bytes,
                b->bytes);
  if (bytes && !dst) return fail(c, GS3D_ERR_INVALID_ARG, "null destination");
  TRY(set_device(c));
  if (!bytes) return GS3D_OK;
  if (which == GS3D_BUF_SPLAT_TARGET) {
    // off the rebin stream: the next rebin runs while this frame copies out
    CK(cudaEventRecord(c->frame_done, c->stream), "frame event");
    CK(cudaStreamWaitEvent(c->copy_stream, c->frame_done, 0), "copy waits for the frame");
    CK(cudaMemcpyAsync(dst, b->p, bytes, cudaMemcpyDeviceToHost, c->copy_stream),
       "async copy-out");
    CK(cudaEventRecord(c->copy_done, c->copy_stream), "copy event");
    return GS3D_OK;
  }
  CK(cudaMemcpyAsync(dst, b->p, bytes, cudaMemcpyDeviceToHost, c->stream), "async copy-out");
  return GS3D_OK;
}

int gs3d_ref_count(gs3d_ctx* c, uint32_t* out) {
  if (!c || !out) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  return gs3d_read_buffer(c, GS3D_BUF_REF_COUNTER, out, sizeof(uint32_t));
}

int gs3d_read_tile_counts(gs3d_ctx* c, uint32_t* counts, size_t n) {
  if (!c || !counts) return fail(c, GS3D_ERR_INVALID_ARG, "null argument");
  if (!c->have_camera) return fail(c, GS3D_ERR_STATE, "no frame");
  const size_t tiles = c->total_tiles;
  if (n < tiles) return fail(c, GS3D_ERR_INVALID_ARG, "need room for %zu tiles", tiles);
  uint32_t* off = new (std::nothrow) uint32_t[tiles + 1];
  if (!off) return fail(c, GS3D_ERR_OOM, "host allocation");
  const int rc = gs3d_read_buffer(c, GS3D_BUF_TILE_OFFSETS, off, (tiles + 1) * 4);
  if (rc == GS3D_OK)
    for (size_t t = 0; t < tiles; ++t) counts[t] = off[t + 1] >= off[t] ? off[t + 1] - off[t] : 0;
  delete[] off;
  return rc;
}

}  // extern "C"
