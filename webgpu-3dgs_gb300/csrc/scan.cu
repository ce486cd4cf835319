// scan.cu - stage 2 of the rebin: exclusive prefix scan of splat_ref_counts.
//
// Replaces the reference's three dispatches prefix_scan_local / _blocks / _add
// (src/shaders/compute/prefix_scan_*.wgsl, scan_core.wgsl), whose middle phase
// is a single thread walking every block sum, with one single-pass kernel:
// tiles of 2048 counts are claimed in order through an atomic ticket, scanned
// with warp shuffles, and chained by decoupled look-back on a per-tile status
// word.  Output contract of prefix_scan_blocks.wgsl:41-42 is kept:
// offsets[n] = ref_counter[0] = total.
//
// Status words are 64-bit: [63:34] launch epoch, [33:32] flag, [31:0] value.
// The epoch changes every launch, so the status array never needs clearing;
// entries carrying another epoch read as "not ready".  Prefixes are summed in
// 64 bits; a total that does not fit 32 bits saturates at 0xffffffff and
// latches DEVERR_CAPACITY (no rebin can hold that many refs).
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr uint32_t kTile = kThreads * kItems;  // 2048 counts per tile
constexpr uint32_t kFlagAgg = 1u, kFlagInc = 2u;

__device__ __forceinline__ unsigned long long pack(uint32_t epoch, uint32_t flag, uint32_t v) {
  return ((unsigned long long)epoch << 34) | ((unsigned long long)flag << 32) | v;
}

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__global__ void __launch_bounds__(kThreads)
    scan_kernel(const uint32_t* __restrict__ in, const uint32_t* __restrict__ gather,
                uint32_t* __restrict__ out, uint32_t n,
                unsigned long long* __restrict__ status, uint32_t* __restrict__ ticket,
                uint32_t epoch, uint32_t* __restrict__ total_out, uint32_t* __restrict__ err) {
  __shared__ uint32_t s_tile, s_prefix;
  __shared__ uint32_t s_warp[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t num_tiles = (n + kTile - 1) / kTile;
  const size_t base = (size_t)tile * kTile + (size_t)threadIdx.x * kItems;

  // 128-bit accesses need 16-byte aligned buffers (caller-provided pointers
  // may be offset); otherwise the scalar path is taken
  const bool vec_in = (reinterpret_cast<uintptr_t>(in) & 15u) == 0;
  const bool vec_out = (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
  uint32_t v[kItems];
  if (gather != nullptr) {  // counts read through a permutation (fused rebin)
#pragma unroll
    for (int k = 0; k < kItems; ++k) v[k] = (base + k < n) ? __ldg(in + __ldg(gather + base + k)) : 0u;
  } else if (vec_in && base + kItems <= n) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(in + base));
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(in + base) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int k = 0; k < kItems; ++k) v[k] = (base + k < n) ? __ldg(in + base + k) : 0u;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) sum += v[k];

  const uint32_t winc = warp_inclusive(sum, lane);
  if (lane == 31) s_warp[warp] = winc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < kThreads / 32 ? s_warp[lane] : 0u;
    const uint32_t wi = warp_inclusive(w, lane);
    if (lane < kThreads / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
    const uint32_t tile_total = __shfl_sync(0xffffffffu, wi, kThreads / 32 - 1);

    // ---- decoupled look-back (warp 0) ----
    unsigned long long excl = 0;
    if (tile == 0) {
      if (lane == 0) st_relaxed_u64(status, pack(epoch, kFlagInc, tile_total));
    } else {
      if (lane == 0) st_relaxed_u64(status + tile, pack(epoch, kFlagAgg, tile_total));
      int pred = (int)tile - 1;
      bool timed_out = false;
      while (true) {
        const int idx = pred - lane;
        uint32_t flag = kFlagInc, val = 0;
        uint32_t spins = 0;
        while (true) {
          if (idx >= 0) {
            const unsigned long long w64 = ld_relaxed_u64(status + idx);
            flag = ((uint32_t)(w64 >> 34) == epoch) ? (uint32_t)(w64 >> 32) & 3u : 0u;
            val = (uint32_t)w64;
          } else {
            flag = kFlagInc;
            val = 0;
          }
          if (__all_sync(0xffffffffu, flag != 0u)) break;
          if (++spins > kSpinLimit) {
            timed_out = true;
            break;
          }
          if (spins > 32) __nanosleep(64);
        }
        if (__any_sync(0xffffffffu, timed_out)) {
          if (lane == 0) latch_error(err, DEVERR_TIMEOUT);
          break;
        }
        const uint32_t inc_mask = __ballot_sync(0xffffffffu, flag == kFlagInc);
        if (inc_mask) {
          const int first = __ffs(inc_mask) - 1;  // nearest inclusive predecessor
          unsigned long long x = lane <= first ? val : 0u;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          excl += x;
          break;
        }
        unsigned long long x = val;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        excl += x;
        pred -= 32;
      }
    }
    const unsigned long long inc = excl + tile_total;
    const bool overflow = inc > 0xffffffffull;
    const uint32_t inc32 = overflow ? 0xffffffffu : (uint32_t)inc;
    if (lane == 0) {
      if (tile > 0) st_relaxed_u64(status + tile, pack(epoch, kFlagInc, inc32));
      if (overflow) latch_error(err, DEVERR_CAPACITY);
      s_prefix = overflow ? 0xffffffffu : (uint32_t)excl;
      if (tile == num_tiles - 1) {
        *total_out = inc32;
        out[n] = inc32;
      }
    }
  }
  __syncthreads();

  uint32_t run = s_prefix + s_warp[warp] + (winc - sum);
  uint32_t o[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    o[k] = run;
    run += v[k];
  }
  if (vec_out && base + kItems <= n) {
    reinterpret_cast<uint4*>(out + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<uint4*>(out + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
  } else {
#pragma unroll
    for (int k = 0; k < kItems; ++k)
      if (base + k < n) out[base + k] = o[k];
  }
}

__global__ void scan_empty_kernel(uint32_t* out, uint32_t* total_out) {
  out[0] = 0u;
  *total_out = 0u;
}

}  // namespace

size_t scan_status_words(uint32_t n) { return (n + kTile - 1) / kTile + 1; }

cudaError_t launch_scan(const uint32_t* counts, const uint32_t* gather, uint32_t* offsets,
                        uint32_t n, unsigned long long* status, uint32_t* tile_counter,
                        uint32_t epoch, uint32_t* total_out, uint32_t* err, cudaStream_t s) {
  if (n == 0) {
    scan_empty_kernel<<<1, 1, 0, s>>>(offsets, total_out);
    return cudaGetLastError();
  }
  const uint32_t tiles = (n + kTile - 1) / kTile;
  scan_kernel<<<tiles, kThreads, 0, s>>>(counts, gather, offsets, n, status, tile_counter, epoch,
                                         total_out, err);
  return cudaGetLastError();
}

}  // namespace gs3d
