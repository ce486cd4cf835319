// emit.cu - stage 3 of the rebin: one (key, value) pair per (splat, tile).
//
// Same output as src/shaders/compute/emit_tile_refs.wgsl:57-79: for each
// valid splat, keys[off + k] = {hi: ty * tiles_x + tx, lo: bits(-depth)} and
// values[off + k] = splat id, tiles in row-major order of the splat's tile
// rectangle.  The reference loops per splat (one thread writes a whole
// footprint, divergent for large splats); here a block owns 256 consecutive
// splats, whose refs form one contiguous range of the output, and its threads
// walk that range with unit stride, each ref finding its splat by a binary
// search over the block's offsets in shared memory.  Stores are therefore
// fully coalesced whatever the footprint distribution.
//
// Capacity: the reference writes past maxRefs relying on robust buffer
// access (emit_tile_refs.wgsl:68-77).  Here the live count is compared with
// the key capacity first; on overflow nothing is written and
// DEVERR_CAPACITY is latched.
#include <algorithm>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
    emit_kernel(const FrameUniforms* __restrict__ fu, uint32_t n,
                const gs3d_projected_splat* __restrict__ proj, const uint32_t* __restrict__ offsets,
                const uint32_t* __restrict__ ref_counter, uint32_t capacity,
                uint2* __restrict__ keys, uint32_t* __restrict__ values,
                uint32_t* __restrict__ err) {
  __shared__ uint32_t s_off[kThreads + 1];
  __shared__ uint32_t s_tminx[kThreads], s_tminy[kThreads], s_w[kThreads], s_cnt[kThreads];
  __shared__ uint32_t s_lo[kThreads];

  const uint32_t total = *ref_counter;
  if (total > capacity) {
    if (blockIdx.x == 0 && threadIdx.x == 0) latch_error(err, DEVERR_CAPACITY);
    return;
  }
  const uint32_t first = blockIdx.x * kThreads;
  const uint32_t i = first + threadIdx.x;
  const uint32_t tiles_x = __ldg(&fu->tile_count[0]);

  if (i < n) {
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(proj + i));
    const uint32_t valid = __ldg(&proj[i].valid);
    const uint4 r3 = __ldg(reinterpret_cast<const uint4*>(proj + i) + 3);
    const uint32_t w = r3.z - r3.x + 1u, h = r3.w - r3.y + 1u;
    s_off[threadIdx.x] = __ldg(offsets + i);
    s_tminx[threadIdx.x] = r3.x;
    s_tminy[threadIdx.x] = r3.y;
    s_w[threadIdx.x] = w;
    s_cnt[threadIdx.x] = valid ? w * h : 0u;
    s_lo[threadIdx.x] = __float_as_uint(-r0.z);
  }
  const uint32_t last = min(n, first + kThreads);  // one past the block's last splat
  if (threadIdx.x == 0) s_off[last - first] = __ldg(offsets + last);
  __syncthreads();

  const uint32_t nloc = last - first;
  const uint32_t begin = s_off[0], end = s_off[nloc];
  if (end < begin || end > total) {  // inconsistent offsets: write nothing
    if (threadIdx.x == 0) latch_error(err, DEVERR_RANGE);
    return;
  }
  for (uint32_t j = begin + threadIdx.x; j < end; j += kThreads) {
    // largest s with s_off[s] <= j (ties: the last splat with that offset)
    uint32_t lo = 0, hi = nloc;  // invariant: s_off[lo] <= j < s_off[hi]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (s_off[mid] <= j) lo = mid; else hi = mid;
    }
    const uint32_t k = j - s_off[lo];
    if (k >= s_cnt[lo]) continue;  // not covered by the splat's rectangle
    const uint32_t w = s_w[lo];
    const uint32_t ty = s_tminy[lo] + k / w;
    const uint32_t tx = s_tminx[lo] + k % w;
    keys[j] = make_uint2(ty * tiles_x + tx, s_lo[lo]);
    values[j] = first + lo;
  }
}

// Fused-rebin emit over a batch: chunk c holds the depth-sorted positions
// [256c, 256c+256); the splat-view at position i is g = sorted_ids[i], it
// belongs to the view v whose range holds g, and its refs start at
// sorted_offsets[i].  Keys carry global tile ids (view tile base + local
// tile) so the later tile-digit passes also separate the views; values carry
// g.  Besides the keys/values the kernel accumulates the 256-bin histograms
// of the tile-id digit places those passes sort, so they need no separate
// histogram read.
//
// The grid is the resident blocks of every SM and each block takes chunks
// from a ticket counter until none are left, keeping its histograms in
// shared memory across its chunks: the global histogram then takes one atomic
// per (block, nonzero bin) rather than one per (chunk, nonzero bin).  All
// blocks add to the same few hundred words, so per-chunk flushes (tens of
// millions of atomics per batch on a few L2 slices) cost more than the emit's
// own stores.  Tickets rather than a fixed stride, because the refs of a chunk
// range from 256 to millions (near splats covering a whole view).
template <int TP, int BINS>
__global__ void __launch_bounds__(kThreads)
    emit_sorted_kernel(const ViewDesc* __restrict__ views, uint32_t n_views, uint32_t n,
                       const gs3d_projected_splat* __restrict__ proj,
                       const uint32_t* __restrict__ rect8,
                       const uint32_t* __restrict__ sorted_keys,
                       const uint32_t* __restrict__ sorted_ids,
                       const uint32_t* __restrict__ sorted_offsets,
                       const uint32_t* __restrict__ ref_counter, uint32_t capacity,
                       uint2* __restrict__ keys, uint32_t* __restrict__ values, int4 shifts,
                       uint4 masks, uint32_t* __restrict__ g_hist,
                       uint32_t* __restrict__ chunk_ticket, uint32_t* __restrict__ err) {
  __shared__ uint32_t s_off[kThreads + 1];
  // per splat, read as two 16-byte words by every ref it owns:
  // [count, rectangle width, bits(1/width), tiles_x - width] and
  // [global tile of the rectangle's first tile, depth bits, splat-view id, -]
  __shared__ uint4 s_ra[kThreads], s_rb[kThreads];
  __shared__ uint32_t s_hist[TP > 0 ? TP : 1][BINS];
  __shared__ uint32_t s_first, s_next;  // tickets: the block's first chunk, its next one

  const uint32_t total = *ref_counter;
  if (total > capacity) {
    if (blockIdx.x == 0 && threadIdx.x == 0) latch_error(err, DEVERR_CAPACITY);
    return;
  }
  for (int k = threadIdx.x; k < TP * BINS; k += kThreads) (&s_hist[0][0])[k] = 0u;
  const int sh[4] = {shifts.x, shifts.y, shifts.z, shifts.w};
  const uint32_t mk[4] = {masks.x, masks.y, masks.z, masks.w};
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t chunks = (n + kThreads - 1) / kThreads;
  // The next chunk's ticket and its sorted ids, depth keys and offsets are
  // fetched while the current chunk expands, and its rectangles gathered
  // before the barrier that ends the chunk (while the warps that finished
  // wait there), so a chunk starts with its fields in registers.
  uint32_t p_id = 0, p_key = 0, p_off = 0, p_end = 0;
  uint4 p_rect = make_uint4(0u, 0u, 0u, 0u);  // [x0, y0, x1, y1]
  auto fetch = [&](uint32_t c) {
    const uint32_t i = c * kThreads + threadIdx.x;
    if (c < chunks && i < n) {
      p_id = __ldg(sorted_ids + i);
      p_key = __ldg(sorted_keys + i);
      p_off = __ldg(sorted_offsets + i);
    }
    if (threadIdx.x == 0 && c < chunks) p_end = __ldg(sorted_offsets + min(n, (c + 1) * kThreads));
  };
  // only the tile rectangle is gathered (one 32-byte sector of the record):
  // the depth bits come in order from the depth sort, the ref count from the
  // scan's offsets (0 for culled splats, whose rectangle is zeroed) (or,
  // where every view's tile grid fits 8 bits, the 4-byte word of the
  // preprocess's compact rectangle array, which stays in L2)
  auto gather = [&](uint32_t c) {
    if (c >= chunks || c * kThreads + threadIdx.x >= n) return;
    if (rect8 != nullptr) {
      const uint32_t rr = __ldg(rect8 + p_id);
      const uint32_t x0 = rr & 0xffu, y0 = (rr >> 8) & 0xffu;
      p_rect = make_uint4(x0, y0, x0 + ((rr >> 16) & 0xffu), y0 + (rr >> 24));
    } else {
      p_rect = __ldg(reinterpret_cast<const uint4*>(proj + p_id) + 3);
    }
  };
  if (threadIdx.x == 0) s_first = atomicAdd(chunk_ticket, 1u);
  __syncthreads();
  uint32_t chunk = s_first;
  fetch(chunk);
  gather(chunk);
  while (chunk < chunks) {
    if (threadIdx.x == 0) s_next = atomicAdd(chunk_ticket, 1u);
    const uint32_t first = chunk * kThreads;
    const uint32_t i = first + threadIdx.x;
    if (i < n) {
      const uint32_t id = p_id;
      const uint32_t x0 = p_rect.x, y0 = p_rect.y;
      const uint32_t w = p_rect.z - p_rect.x + 1u, h = p_rect.w - p_rect.y + 1u;
      const uint32_t v =
          find_view(n_views, id, [&](uint32_t k) { return __ldg(&views[k].splat_base); });
      s_off[threadIdx.x] = p_off;
      const uint32_t tx = __ldg(&views[v].f.tile_count[0]);
      // ref k of the splat: row = k / w, tile = first + row * tx + (k - row * w)
      //                                      = first + row * (tx - w) + k
      s_ra[threadIdx.x] = make_uint4(w * h, w, __float_as_uint(1.0f / (float)w), tx - w);
      s_rb[threadIdx.x] = make_uint4(__ldg(&views[v].f.tile_base) + y0 * tx + x0, p_key, id, 0u);
    }
    const uint32_t last = min(n, first + kThreads);
    if (threadIdx.x == 0) s_off[last - first] = p_end;
    __syncthreads();  // the chunk's fields and the next ticket are in shared memory
    const uint32_t next = s_next;
    fetch(next);

    const uint32_t nloc = last - first;
    const uint32_t begin = s_off[0], end = s_off[nloc];
    // block-uniform (shared values): an inconsistent chunk is skipped
    if (end < begin || end > total) {
      if (threadIdx.x == 0) latch_error(err, DEVERR_RANGE);
    } else {
      // Each warp expands a contiguous share of the block's refs, 32 at a time.
      // The owner of a ref is the last splat starting at or before it.  The
      // owners of a 32-ref chunk are the owner c0 of its first ref and the
      // splats c0+1 .. c0+32 starting inside it; while those starts are
      // distinct (every valid splat has a ref, and culled splats, which have
      // none, sort after all valid ones) one OR-reduction of their start bits
      // gives every lane its owner.  A chunk with equal starts (zero-count
      // splats) searches per ref instead.
      const uint32_t share = ((end - begin + kThreads - 1) / kThreads) * 32u;
      const uint32_t wbeg = min(end, begin + warp * share), wend = min(end, wbeg + share);
      uint32_t c0 = 0;  // owner of ref wbeg: the last splat starting at or before it
      {
        uint32_t lo = 0, hi = nloc;  // invariant: s_off[lo] <= wbeg < s_off[hi]
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (s_off[mid] <= wbeg) lo = mid; else hi = mid;
        }
        c0 = lo;
      }
      for (uint32_t cb = wbeg; cb < wend; cb += 32) {  // warp-uniform trip count
        const uint32_t j = cb + lane;
        const uint32_t cand = c0 + 1 + lane;
        const uint32_t st = cand <= nloc ? s_off[cand] : 0xffffffffu;
        const uint32_t rel = st - cb;
        const uint32_t down = __shfl_down_sync(0xffffffffu, st, 1);
        const uint32_t next_st = lane < 31 ? down : (cand < nloc ? s_off[cand + 1] : 0xffffffffu);
        uint32_t o;
        if (!__any_sync(0xffffffffu, rel < 32 && next_st == st)) {
          const uint32_t starts = __reduce_or_sync(0xffffffffu, rel < 32 ? 1u << rel : 0u);
          o = c0 + __popc(starts & (0xffffffffu >> (31 - lane)));
        } else {
          uint32_t lo = c0, hi = nloc;  // s_off[c0] <= cb <= j
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_off[mid] <= j) lo = mid; else hi = mid;
          }
          o = lo;
        }
        c0 = __shfl_sync(0xffffffffu, o, 31);  // owner of the chunk's last ref
        bool live = j < wend;
        uint32_t tile = 0;
        if (live) {
          const uint32_t k = j - s_off[o];
          const uint4 ra = s_ra[o];
          if (k < ra.x) {
            // row = floor(k / w) by a float reciprocal: exact while k + w < 2^22
            // (k < w * h <= tiles of one view)
            const uint32_t row = (uint32_t)(((float)k + 0.5f) * __uint_as_float(ra.z));
            const uint4 rb = s_rb[o];
            tile = rb.x + row * ra.w + k;
            keys[j] = make_uint2(tile, rb.y);
            values[j] = rb.z;
          } else {
            live = false;
          }
        }
#pragma unroll
        for (int p = 0; p < TP; ++p) hist_add_256(s_hist[p], (tile >> sh[p]) & mk[p], live);
      }
    }
    gather(next);
    __syncthreads();  // the chunk's readers are done with its fields and with s_next
    chunk = next;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < TP * BINS; k += kThreads) {
    const uint32_t v = (&s_hist[0][0])[k];
    if (v) atomicAdd(g_hist + (k / BINS) * kTileHistStride + k % BINS, v);
  }
}

// Resident blocks per SM of one emit instance (its registers and shared
// memory decide), asked once per instance.
template <int TP, int BINS>
uint32_t emit_blocks_per_sm() {
  static int per_sm = 0;
  if (per_sm == 0) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, emit_sorted_kernel<TP, BINS>, kThreads,
                                                      0) != cudaSuccess) {
      (void)cudaGetLastError();
      b = 1;
    }
    per_sm = b < 1 ? 1 : b;
  }
  return (uint32_t)per_sm;
}

}  // namespace

cudaError_t launch_emit_sorted(const ViewDesc* views, uint32_t n_views, uint32_t n,
                               const gs3d_projected_splat* proj, const uint32_t* rect8,
                               const uint32_t* sorted_keys,
                               const uint32_t* sorted_ids,
                               const uint32_t* sorted_offsets, const uint32_t* ref_counter,
                               uint32_t capacity, uint2* keys, uint32_t* values,
                               const SortPlan& tile_plan, uint32_t* g_hist,
                               uint32_t* chunk_ticket, uint32_t* err, int sm_count,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const uint32_t chunks = (n + kThreads - 1) / kThreads;
  const uint32_t sms = sm_count > 0 ? (uint32_t)sm_count : 1u;
  int4 sh = make_int4(0, 0, 0, 0);
  uint4 mk = make_uint4(0, 0, 0, 0);
  int* shp = &sh.x;
  uint32_t* mkp = &mk.x;
  for (int p = 0; p < tile_plan.passes && p < 4; ++p) {
    shp[p] = tile_plan.shift[p];
    mkp[p] = digit_mask(tile_plan.nbits[p]);
  }
  bool wide = false;  // an 11-bit digit needs 2048-bin histograms
  for (int p = 0; p < tile_plan.passes; ++p) wide = wide || tile_plan.nbits[p] > 8;
#define GS3D_EMIT_CASE(TP, BINS)                                                              \
  case TP:                                                                                    \
    emit_sorted_kernel<TP, BINS><<<std::min(chunks, sms * emit_blocks_per_sm<TP, BINS>()),    \
                                   kThreads, 0, s>>>(                                         \
        views, n_views, n, proj, rect8, sorted_keys, sorted_ids, sorted_offsets, ref_counter, \
        capacity, keys, values, sh, mk, g_hist, chunk_ticket, err);                           \
    break;
  if (wide) {
    switch (tile_plan.passes) {
      GS3D_EMIT_CASE(1, 2048)
      GS3D_EMIT_CASE(2, 2048)
      GS3D_EMIT_CASE(3, 2048)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (tile_plan.passes) {
      GS3D_EMIT_CASE(0, kRadixBins)
      GS3D_EMIT_CASE(1, kRadixBins)
      GS3D_EMIT_CASE(2, kRadixBins)
      GS3D_EMIT_CASE(3, kRadixBins)
      GS3D_EMIT_CASE(4, kRadixBins)
      default:
        return cudaErrorInvalidValue;
    }
  }
#undef GS3D_EMIT_CASE
  return cudaGetLastError();
}

cudaError_t launch_emit(const FrameUniforms* d_frame, uint32_t n,
                        const gs3d_projected_splat* proj, const uint32_t* offsets,
                        const uint32_t* ref_counter, uint32_t capacity, uint2* keys,
                        uint32_t* values, uint32_t* err, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const uint32_t blocks = (n + kThreads - 1) / kThreads;
  emit_kernel<<<blocks, kThreads, 0, s>>>(d_frame, n, proj, offsets, ref_counter, capacity, keys,
                                          values, err);
  return cudaGetLastError();
}

}  // namespace gs3d
