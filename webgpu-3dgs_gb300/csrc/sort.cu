// sort.cu - stage 4 of the rebin: stable LSD radix sort of the 64-bit
// (tile | depth) keys with their splat-id values.
//
// The reference runs eight 8-bit passes, each as three dispatch groups
// (radix_histogram.wgsl, a recursive Blelloch scan, radix_scatter.wgsl with a
// serial lane-0 rank).  This file implements the onesweep scheme instead:
//
//   1. one histogram kernel reads every key once and builds the 256-bin
//      histogram of every digit place that is sorted (and clears the
//      look-back status of the passes);
//   2. one kernel per pass: a persistent CTA claims partitions (4096 8-byte
//      or 6144 4-byte keys) in
//      order, ranks its keys stably with warp ballots (8 ballots give each
//      lane the mask of lanes holding the same 8-bit digit) and per-warp
//      shared-memory histograms, publishes its per-digit counts, resolves
//      each digit's global offset by decoupled look-back over earlier
//      partitions, reorders the partition in shared memory and writes each
//      digit run out contiguously.
//
// Digit places above the highest set bit of (tile count - 1) are always zero
// and are skipped: 4 depth passes + ceil(tile bits / 8) tile passes instead of
// 8.  Passes alternate A->B->A; with an odd pass count the sorted result ends
// in the B buffers and the host swaps the buffer names.
//
// The same pass kernel, instantiated for 32-bit keys, sorts the per-splat
// depth keys of the fused rebin (fused_rebin in ctx.cu).
//
// The order produced is identical to the reference's: lexicographic
// (tile id, depth bits, emit position), since every pass is a stable
// counting sort on one digit.
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;   // histogram kernel
constexpr int kHistItems = 16;  // keys a histogram thread loads per round
constexpr int kPassThreads = 512;                  // onesweep pass (8-bit and narrower digits)
constexpr int kWarps = kPassThreads / 32;          // 16
constexpr int kItems = 8;
constexpr uint32_t kPart = kPassThreads * kItems;  // 4096 keys per partition (uint2 keys)
// key buffers are padded to whole partitions of every pass kernel (4096 and
// 6144 keys)
constexpr uint32_t kRoundPart = 12288;
constexpr uint32_t kFlagAgg = 1u, kFlagInc = 2u;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr int kLookback = 16;  // predecessor status words fetched per look-back step

template <typename K>
struct KeyOps;
template <>
struct KeyOps<uint2> {  // [hi = tile id, lo = depth bits]
  static __device__ __forceinline__ uint2 sentinel() { return make_uint2(0xffffffffu, 0xffffffffu); }
  static __device__ __forceinline__ uint32_t digit(uint2 k, int word, int shift) {
    return ((word ? k.y : k.x) >> shift) & 0xffu;
  }
};
template <>
struct KeyOps<uint32_t> {
  static __device__ __forceinline__ uint32_t sentinel() { return 0xffffffffu; }
  static __device__ __forceinline__ uint32_t digit(uint32_t k, int, int shift) {
    return (k >> shift) & 0xffu;
  }
};

// Keys a pass thread ranks per partition.  A partition costs about the same
// time whatever its keys' width (ranking, barriers and the look-back's L2
// round trips dominate), so 4-byte keys take 12 a thread: their 6144-key
// partitions fill the 48 KB buffer of a 4096-key partition of 8-byte keys,
// and two CTAs still fit an SM.
template <typename K>
struct PassItems {
  static constexpr int value = 8;
};
template <>
struct PassItems<uint32_t> {
  static constexpr int value = 12;
};
template <typename K>
constexpr uint32_t pass_part() {
  return kPassThreads * (uint32_t)PassItems<K>::value;
}

template <typename K>
constexpr size_t pass_smem() {  // two partition buffers + per-warp u16 histograms
  return 2 * (size_t)pass_part<K>() * (sizeof(K) + sizeof(uint32_t)) +
         (size_t)kWarps * kRadixBins * sizeof(uint16_t);
}

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Exclusive scan over the first 256 threads' values (one per digit); every
// thread of the block must call it, threads >= 256 pass 0 and get garbage.
__device__ __forceinline__ uint32_t block_exclusive_256(uint32_t x, uint32_t* s_wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t inc = warp_inclusive(x, lane);
  __syncthreads();  // s_wsum may still be read from a previous call
  if (lane == 31 && warp < 8) s_wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < 8 ? s_wsum[lane] : 0u;
    const uint32_t wi = warp_inclusive(w, lane);
    if (lane < 8) s_wsum[lane] = wi - w;
  }
  __syncthreads();
  return warp < 8 ? s_wsum[warp] + inc - x : 0u;
}

// Mask of lanes whose digit equals this lane's (digits below 2^NBITS).
template <int NBITS>
__device__ __forceinline__ uint32_t match_digit(uint32_t d) {
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < NBITS; ++b) {
    const uint32_t bit = (d >> b) & 1u;
    const uint32_t bal = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bal : ~bal;
  }
  return peers;
}

struct PassDev {
  int word[kMaxSortPasses];
  int shift[kMaxSortPasses];
  uint32_t mask[kMaxSortPasses];
};

// Histogram of every sorted digit place + clear of the look-back status.
// The top place (the depth keys' exponent byte: a handful of values) is
// counted in per-lane sub-histograms 257 words apart, so lanes adding the
// same digit hit different banks instead of serialising on one word; they
// are summed at the block's flush.
constexpr uint32_t kLaneStride = kRadixBins + 1;
template <typename K, int P>
__global__ void __launch_bounds__(kThreads)
    sort_histogram_kernel(const K* __restrict__ keys, const uint32_t* __restrict__ ref_counter,
                          uint32_t capacity, PassDev pd, uint32_t* __restrict__ g_hist,
                          uint32_t* __restrict__ status, size_t status_stride) {
  __shared__ uint32_t s_hist[P][kRadixBins];
  __shared__ uint32_t s_top[32 * kLaneStride];
  for (int k = threadIdx.x; k < P * kRadixBins; k += kThreads) (&s_hist[0][0])[k] = 0u;
  for (int k = threadIdx.x; k < 32 * (int)kLaneStride; k += kThreads) s_top[k] = 0u;
  __syncthreads();
  const uint32_t lane_base = (threadIdx.x & 31u) * kLaneStride;

  const uint32_t R = live_refs(ref_counter, capacity);
  const size_t parts = (R + kPart - 1) / kPart;
  const size_t gtid = (size_t)blockIdx.x * kThreads + threadIdx.x;
  const size_t gstride = (size_t)gridDim.x * kThreads;

  // clear the status words of the partitions this sort will use
  const size_t words = parts * kRadixBins;
  for (size_t k = gtid; k < words * P; k += gstride) {
    const size_t p = k / words, o = k - p * words;
    status[p * status_stride + o] = 0u;
  }

  int word[P], shift[P];
  uint32_t mask[P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    word[p] = pd.word[p];
    shift[p] = pd.shift[p];
    mask[p] = pd.mask[p];
  }
  // kHistItems keys a thread per round, all loads issued before the first
  // histogram add: one load in flight per thread would leave the kernel at a
  // fraction of HBM bandwidth behind its shared-memory atomics
  const size_t rstride = gstride * kHistItems;
  for (size_t base = (size_t)blockIdx.x * kThreads * kHistItems; base < R; base += rstride) {
    K k[kHistItems];
#pragma unroll
    for (int i = 0; i < kHistItems; ++i) {
      const size_t idx = base + (size_t)i * kThreads + threadIdx.x;
      k[i] = idx < R ? keys[idx] : KeyOps<K>::sentinel();
    }
#pragma unroll
    for (int i = 0; i < kHistItems; ++i) {
      const bool in = base + (size_t)i * kThreads + threadIdx.x < R;
#pragma unroll
      for (int p = 0; p < P - 1; ++p)
        hist_add_256(s_hist[p], KeyOps<K>::digit(k[i], word[p], shift[p]) & mask[p], in);
      if (in)
        atomicAdd(s_top + lane_base +
                      (KeyOps<K>::digit(k[i], word[P - 1], shift[P - 1]) & mask[P - 1]),
                  1u);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < (int)kRadixBins; d += kThreads) {
    uint32_t sum = 0;
    for (int l = 0; l < 32; ++l) sum += s_top[l * kLaneStride + d];
    s_hist[P - 1][d] += sum;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P * kRadixBins; k += kThreads) {
    const uint32_t v = (&s_hist[0][0])[k];
    if (v) atomicAdd(g_hist + k, v);
  }
}

template <typename K>
constexpr size_t part_buf_bytes() {
  return (size_t)pass_part<K>() * (sizeof(K) + sizeof(uint32_t));
}

// Inclusive scan over lanes 0..7 (the eight digit warps' totals).
__device__ __forceinline__ uint32_t scan8_inclusive(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// One LSD pass.  Persistent CTAs claim partitions in order (pass_part).  A
// partition is claimed when the CTA has resolved its current one (barrier C
// below), and fetched by two bulk (TMA) copies into the other shared-memory
// buffer while the current partition is written out; the claimed partition's
// id travels with the buffer's mbarrier arrive.  Claiming late keeps the
// window between a claim and the publication of the partition's digit counts
// short, so successors' look-backs rarely find an unpublished predecessor.
// Claiming cannot deadlock: the smallest unfinished partition is always some
// CTA's current one, and it waits only on smaller, finished partitions.
//
// Four block barriers per partition:
//   A  every warp has ranked its items (per-warp digit counts complete, the
//      input buffer fully read into registers, the fetch landed everywhere);
//   B  per-digit warp offsets and digit-warp prefix sums are in shared memory;
//   B' every (warp, digit) entry holds the digit's start in the partition plus
//      the warp's offset within the digit;
//   C  the partition is reordered by digit and each digit's global
//      destination is resolved.
// Threads waiting for a fetch sleep in mbarrier.try_wait (suspend hint)
// rather than spinning, so they take no issue slots from the other CTA.
template <typename K, int NBITS>
__global__ void __launch_bounds__(kPassThreads, 1024 / kPassThreads)
    onesweep_kernel(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                    K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                    const uint32_t* __restrict__ ref_counter, uint32_t capacity, int word,
                    int shift, const uint32_t* __restrict__ hist, uint32_t* __restrict__ status,
                    uint32_t* __restrict__ part_counter, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr size_t kBuf = part_buf_bytes<K>();
  constexpr int kI = PassItems<K>::value;   // keys a thread ranks
  constexpr uint32_t kP = pass_part<K>();   // keys a partition holds
  // [kWarps][256] per-warp digit counts, then per-warp exclusive offsets
  uint16_t* s_whist = reinterpret_cast<uint16_t*>(smem + 2 * kBuf);
  __shared__ uint32_t s_bucket[kRadixBins], s_dloc[kRadixBins], s_dest[kRadixBins];
  __shared__ uint32_t s_wsum[kWarps];
  __shared__ uint32_t s_part[2];  // partition id of each buffer
  __shared__ uint64_t s_bar[2];

  if (blockDim.x != kPassThreads) {  // the indexing below is written for this block size
    if (threadIdx.x == 0) latch_error(err, DEVERR_RANGE);
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t R = live_refs(ref_counter, capacity);
  const uint32_t num_parts = (R + kP - 1) / kP;
  // digits are NBITS wide; the all-ones sentinel of the tail items maps to
  // the largest digit and ranks after every real item of it
  constexpr uint32_t kDigitMask = NBITS >= 8 ? 0xffu : ((1u << NBITS) - 1u);

  // one thread only: claim the next partition and start its fetch into buffer
  // b (whose previous readers are past a block barrier), or, with no
  // partition left, complete the buffer's phase empty
  auto claim_into = [&](int b) {
    const uint32_t part = atomicAdd(part_counter, 1u);
    s_part[b] = part;  // published by the arrive below (release)
    if (part < num_parts) {
      unsigned char* buf = smem + b * kBuf;
      const uint32_t kb = kP * sizeof(K), vb = kP * sizeof(uint32_t);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&s_bar[b], kb + vb);
      bulk_g2s(buf, keys_in + (size_t)part * kP, kb, &s_bar[b]);
      bulk_g2s(buf + kb, vals_in + (size_t)part * kP, vb, &s_bar[b]);
    } else {
      mbar_arrive(&s_bar[b]);
    }
  };

  const bool digit_thread = tid < kRadixBins;  // threads 0..255 own one digit each
  if (tid == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
  }
  // global bucket bases of this digit place (the scan's barriers also order
  // the mbarrier initialisation before any wait).  Look-back counts are kept
  // modulo 2^30, exact while every bucket holds fewer keys.
  {
    const uint32_t h = digit_thread ? __ldg(hist + tid) : 0u;
    if (blockIdx.x == 0 && h >= (1u << 30)) latch_error(err, DEVERR_BUCKET);
    const uint32_t bb = block_exclusive_256(h, s_wsum);
    if (digit_thread) s_bucket[tid] = bb;
  }
  __syncthreads();
  if (tid == 0) claim_into(0);
  int b = 0;
  uint32_t phase0 = 0, phase1 = 0;

  for (;;) {
    uint16_t* wh = s_whist + warp * kRadixBins;
    // this warp's count row; its previous readers finished before barrier C
    reinterpret_cast<uint4*>(wh)[lane] = make_uint4(0u, 0u, 0u, 0u);
    __syncwarp();
    K* s_keys = reinterpret_cast<K*>(smem + b * kBuf);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + b * kBuf + kP * sizeof(K));
    const bool landed = mbar_wait(&s_bar[b], b ? phase1 : phase0);
    if (b) phase1 ^= 1u; else phase0 ^= 1u;
    const uint32_t part = landed ? s_part[b] : num_parts;
    const uint32_t count = part < num_parts ? min(kP, R - part * kP) : 0u;

    // ---- registers <- shared (warp-striped: lane-contiguous) ----
    K key[kI];
    uint32_t val[kI];
    uint32_t dr[kI];  // digit | rank-in-warp << 8
    const uint32_t wloc = warp * (32u * kI);
#pragma unroll
    for (int i = 0; i < kI; ++i) {
      const uint32_t loc = wloc + i * 32u + lane;
      if (loc < count) {
        key[i] = s_keys[loc];
        val[i] = s_vals[loc];
      } else {
        key[i] = KeyOps<K>::sentinel();  // largest digit, ranked last
        val[i] = 0u;
      }
    }
    // ---- stable rank within the warp ----
#pragma unroll
    for (int i = 0; i < kI; ++i) {
      const uint32_t d = KeyOps<K>::digit(key[i], word, shift) & kDigitMask;
      const uint32_t peers = match_digit<NBITS>(d);
      const uint32_t prior = wh[d];
      __syncwarp();
      if ((__ffs(peers) - 1) == lane) wh[d] = (uint16_t)(prior + __popc(peers));
      __syncwarp();
      dr[i] = d | ((prior + __popc(peers & lanemask_lt())) << 8);
    }
    // A: counts complete, input buffer read, the fetch had landed for everyone
    if (!__syncthreads_and(landed)) {  // bounded wait gave up: stop this CTA
      if (tid == 0) {
        latch_error(err, DEVERR_TIMEOUT);
        mbar_wait(&s_bar[b], b ? phase1 ^ 1u : phase0 ^ 1u);  // one more bounded wait
      }
      break;
    }
    if (part >= num_parts) break;  // every thread read the same id

    // ---- per digit (thread = digit): warp offsets, partition totals ----
    uint32_t run = 0, pub = 0;
    uint32_t* st = status + (size_t)part * kRadixBins + tid;
    if (digit_thread) {
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        const uint32_t t = s_whist[w * kRadixBins + tid];
        s_whist[w * kRadixBins + tid] = (uint16_t)run;
        run += t;
      }
      pub = ((uint32_t)tid == kDigitMask) ? run - (kP - count) : run;
      st_relaxed_u32(st, ((part == 0 ? kFlagInc : kFlagAgg) << 30) | pub);
      const uint32_t inc = warp_inclusive(run, lane);
      s_dloc[tid] = inc - run;  // exclusive within the digit warp
      if (lane == 31) s_wsum[warp] = inc;
    }
    __syncthreads();  // B

    // each digit's start in the partition (exclusive prefix of the eight digit
    // warps' totals + the start within its warp), folded into every warp's
    // per-digit offset: a partition position is then one table entry plus
    // the item's rank (positions < 2^16)
    uint32_t dstart = 0;
    if (digit_thread) {
      const uint32_t wv = lane < 8 ? s_wsum[lane] : 0u;
      const uint32_t wex = scan8_inclusive(wv, lane) - wv;
      dstart = s_dloc[tid] + __shfl_sync(0xffffffffu, wex, warp);
#pragma unroll
      for (int w = 0; w < kWarps; ++w)
        s_whist[w * kRadixBins + tid] = (uint16_t)(s_whist[w * kRadixBins + tid] + dstart);
    }
    __syncthreads();  // B'

    // ---- reorder the partition in place ----
#pragma unroll
    for (int i = 0; i < kI; ++i) {
      const uint32_t pos = wh[dr[i] & 0xffu] + (dr[i] >> 8);
      s_keys[pos] = key[i];
      s_vals[pos] = val[i];
    }

    // ---- decoupled look-back, one thread per digit ----
    uint32_t excl = 0;
    bool ok = true;
    if (digit_thread && part > 0) {
      // windows of kLookback predecessors: their status words are fetched
      // together, so one L2 round trip covers the window
      int pp = (int)part - 1;
      bool found = false;
      while (!found && ok && pp >= 0) {
        uint32_t lw[kLookback];
#pragma unroll
        for (int k = 0; k < kLookback; ++k)
          lw[k] = (pp - k >= 0) ? ld_relaxed_u32(status + (size_t)(pp - k) * kRadixBins + tid)
                                : (kFlagInc << 30);
#pragma unroll
        for (int k = 0; k < kLookback; ++k) {
          if (found || !ok) break;
          uint32_t spins = 0;
          while ((lw[k] >> 30) == 0u) {  // not published yet: poll this one
            if (++spins > kSpinLimit) {
              ok = false;
              break;
            }
            if (spins > 16) __nanosleep(32);
            lw[k] = ld_relaxed_u32(status + (size_t)(pp - k) * kRadixBins + tid);
          }
          if (!ok) break;
          excl += lw[k] & kValueMask;
          if ((lw[k] >> 30) == kFlagInc) found = true;
        }
        pp -= kLookback;
      }
      st_relaxed_u32(st, (kFlagInc << 30) | ((excl + pub) & kValueMask));
    }
    if (digit_thread) s_dest[tid] = s_bucket[tid] + excl - dstart;
    // C: partition reordered, destinations resolved
    if (!__syncthreads_and(ok)) {  // nothing written for this partition
      if (tid == 0) latch_error(err, DEVERR_TIMEOUT);
      break;  // no fetch is in flight: the next claim comes after this barrier
    }
    // the other buffer's last readers (previous write-out) passed barrier A;
    // the last thread claims (with more than 256 threads it owns no digit)
    if (tid == kPassThreads - 1) claim_into(b ^ 1);
    // ---- write each digit run contiguously ----
    for (uint32_t j = tid; j < count; j += kPassThreads) {
      const K k = s_keys[j];
      const uint32_t dst = s_dest[KeyOps<K>::digit(k, word, shift) & kDigitMask] + j;
      if (dst < R) {
        keys_out[dst] = k;
        vals_out[dst] = s_vals[j];
      } else {
        latch_error(err, DEVERR_RANGE);
      }
    }
    b ^= 1;
  }
}

// ---- 11-bit digits -----------------------------------------------------------
// The same pass for 2048-bin digits (tile-id passes of the fused rebin): the
// per-warp counts take 64 KB, so one CTA runs per SM; every thread owns four
// consecutive digits for the per-digit work and the look-back.
constexpr int kWideBits = 11;
constexpr int kWideThreads = 512;
constexpr int kWideWarps = kWideThreads / 32;         // 16
constexpr uint32_t kWidePart = kWideThreads * kItems;  // 4096 keys per partition
constexpr size_t wide_buf_bytes() { return (size_t)kWidePart * (sizeof(uint2) + sizeof(uint32_t)); }
constexpr uint32_t kWideBins = 1u << kWideBits;
constexpr uint32_t kWideDigitsPerThread = kWideBins / kWideThreads;  // 4
constexpr int kWideLookback = 8;

template <typename K>
constexpr size_t wide_pass_smem() {
  return 2 * wide_buf_bytes() + (size_t)kWideWarps * kWideBins * sizeof(uint16_t) +
         3 * (size_t)kWideBins * sizeof(uint32_t);
}

__device__ __forceinline__ uint32_t wide_digit(uint2 k, int word, int shift) {
  return ((word ? k.y : k.x) >> shift) & (kWideBins - 1u);
}

// Inclusive scan over lanes 0..15 (the sixteen digit warps' totals).
__device__ __forceinline__ uint32_t scan16_inclusive(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__global__ void __launch_bounds__(kWideThreads, 1)
    onesweep_wide_kernel(const uint2* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                         uint2* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                         const uint32_t* __restrict__ ref_counter, uint32_t capacity, int word,
                         int shift, const uint32_t* __restrict__ hist,
                         uint32_t* __restrict__ status, uint32_t* __restrict__ part_counter,
                         uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr size_t kBuf = wide_buf_bytes();
  uint16_t* s_whist = reinterpret_cast<uint16_t*>(smem + 2 * kBuf);  // [kWideWarps][2048]
  uint32_t* s_bucket = reinterpret_cast<uint32_t*>(smem + 2 * kBuf + kWideWarps * kWideBins * 2);
  uint32_t* s_dloc = s_bucket + kWideBins;  // exclusive start within the digit warp
  uint32_t* s_dest = s_dloc + kWideBins;
  __shared__ uint32_t s_wsum[kWideWarps];
  __shared__ uint32_t s_part[2];
  __shared__ uint64_t s_bar[2];

  if (blockDim.x != kWideThreads) {  // the indexing below is written for this block size
    if (threadIdx.x == 0) latch_error(err, DEVERR_RANGE);
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t R = live_refs(ref_counter, capacity);
  const uint32_t num_parts = (R + kWidePart - 1) / kWidePart;
  constexpr uint32_t kDigitMask = kWideBins - 1u;
  const uint32_t d0 = tid * kWideDigitsPerThread;  // this thread's digits d0 .. d0+3

  auto claim_into = [&](int b) {
    const uint32_t part = atomicAdd(part_counter, 1u);
    s_part[b] = part;
    if (part < num_parts) {
      unsigned char* buf = smem + b * kBuf;
      const uint32_t kb = kWidePart * sizeof(uint2), vb = kWidePart * sizeof(uint32_t);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&s_bar[b], kb + vb);
      bulk_g2s(buf, keys_in + (size_t)part * kWidePart, kb, &s_bar[b]);
      bulk_g2s(buf + kb, vals_in + (size_t)part * kWidePart, vb, &s_bar[b]);
    } else {
      mbar_arrive(&s_bar[b]);
    }
  };

  if (tid == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
  }
  // global bucket bases: exclusive scan of the 2048-bin histogram
  {
    uint32_t h[kWideDigitsPerThread], t = 0;
#pragma unroll
    for (uint32_t k = 0; k < kWideDigitsPerThread; ++k) {
      h[k] = __ldg(hist + d0 + k);
      if (blockIdx.x == 0 && h[k] >= (1u << 30)) latch_error(err, DEVERR_BUCKET);
      t += h[k];
    }
    const uint32_t inc = warp_inclusive(t, lane);
    if (lane == 31) s_wsum[warp] = inc;
    __syncthreads();
    const uint32_t wv = lane < kWideWarps ? s_wsum[lane] : 0u;
    const uint32_t wex = scan16_inclusive(wv, lane) - wv;
    uint32_t run = __shfl_sync(0xffffffffu, wex, warp) + inc - t;
#pragma unroll
    for (uint32_t k = 0; k < kWideDigitsPerThread; ++k) {
      s_bucket[d0 + k] = run;
      run += h[k];
    }
  }
  __syncthreads();
  if (tid == 0) claim_into(0);
  int b = 0;
  uint32_t phase0 = 0, phase1 = 0;

  for (;;) {
    uint16_t* wh = s_whist + warp * kWideBins;
#pragma unroll
    for (int k = 0; k < (int)(kWideBins * 2 / 16 / 32); ++k)  // 4 KB row: 8 x 16 B per lane
      reinterpret_cast<uint4*>(wh)[lane + 32 * k] = make_uint4(0u, 0u, 0u, 0u);
    __syncwarp();
    uint2* s_keys = reinterpret_cast<uint2*>(smem + b * kBuf);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + b * kBuf + kWidePart * sizeof(uint2));
    const bool landed = mbar_wait(&s_bar[b], b ? phase1 : phase0);
    if (b) phase1 ^= 1u; else phase0 ^= 1u;
    const uint32_t part = landed ? s_part[b] : num_parts;
    const uint32_t count = part < num_parts ? min(kWidePart, R - part * kWidePart) : 0u;

    uint2 key[kItems];
    uint32_t val[kItems];
    uint32_t dr[kItems];  // digit | rank-in-warp << 11
    const uint32_t wloc = warp * (32u * kItems);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const uint32_t loc = wloc + i * 32u + lane;
      if (loc < count) {
        key[i] = s_keys[loc];
        val[i] = s_vals[loc];
      } else {
        key[i] = make_uint2(0xffffffffu, 0xffffffffu);
        val[i] = 0u;
      }
    }
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const uint32_t d = wide_digit(key[i], word, shift);
      const uint32_t peers = match_digit<kWideBits>(d);
      const uint32_t prior = wh[d];
      __syncwarp();
      if ((__ffs(peers) - 1) == lane) wh[d] = (uint16_t)(prior + __popc(peers));
      __syncwarp();
      dr[i] = d | ((prior + __popc(peers & lanemask_lt())) << kWideBits);
    }
    // A: counts complete, input buffer read, the fetch had landed for everyone
    if (!__syncthreads_and(landed)) {
      if (tid == 0) {
        latch_error(err, DEVERR_TIMEOUT);
        mbar_wait(&s_bar[b], b ? phase1 ^ 1u : phase0 ^ 1u);
      }
      break;
    }
    if (part >= num_parts) break;

    // ---- per digit: warp offsets, partition totals (four digits a thread) ----
    uint32_t run[kWideDigitsPerThread], pub[kWideDigitsPerThread];
    uint32_t t = 0;
#pragma unroll
    for (uint32_t k = 0; k < kWideDigitsPerThread; ++k) {
      const uint32_t d = d0 + k;
      uint32_t r = 0;
#pragma unroll
      for (int w = 0; w < kWideWarps; ++w) {
        const uint32_t c = s_whist[w * kWideBins + d];
        s_whist[w * kWideBins + d] = (uint16_t)r;
        r += c;
      }
      run[k] = r;
      pub[k] = (d == kDigitMask) ? r - (kWidePart - count) : r;
      st_relaxed_u32(status + (size_t)part * kWideBins + d,
                     ((part == 0 ? kFlagInc : kFlagAgg) << 30) | pub[k]);
      t += r;
    }
    {
      const uint32_t inc = warp_inclusive(t, lane);
      uint32_t x = inc - t;
#pragma unroll
      for (uint32_t k = 0; k < kWideDigitsPerThread; ++k) {
        s_dloc[d0 + k] = x;  // exclusive within the digit warp (128 digits)
        x += run[k];
      }
      if (lane == 31) s_wsum[warp] = inc;
    }
    __syncthreads();  // B

    const uint32_t wv = lane < kWideWarps ? s_wsum[lane] : 0u;
    const uint32_t wex = scan16_inclusive(wv, lane) - wv;

    // ---- reorder the partition in place ----
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const uint32_t d = dr[i] & kDigitMask;
      const uint32_t pos = s_dloc[d] + __shfl_sync(0xffffffffu, wex, d >> 7) + wh[d] +
                           (dr[i] >> kWideBits);
      s_keys[pos] = key[i];
      s_vals[pos] = val[i];
    }

    // ---- decoupled look-back, four digits a thread ----
    const uint32_t wbase = __shfl_sync(0xffffffffu, wex, warp);  // digits d0.. are in `warp`
    uint32_t excl[kWideDigitsPerThread] = {0u, 0u, 0u, 0u};
    bool ok = true;
    if (part > 0) {
      uint32_t found = 0;  // bit k: digit d0 + k reached an inclusive prefix
      int pp = (int)part - 1;
      while (found != 0xfu && ok && pp >= 0) {
        uint32_t lw[kWideLookback][kWideDigitsPerThread];
#pragma unroll
        for (int i = 0; i < kWideLookback; ++i)
#pragma unroll
          for (uint32_t k = 0; k < kWideDigitsPerThread; ++k)
            lw[i][k] = (pp - i >= 0 && !((found >> k) & 1u))
                           ? ld_relaxed_u32(status + (size_t)(pp - i) * kWideBins + d0 + k)
                           : (kFlagInc << 30);
#pragma unroll
        for (uint32_t k = 0; k < kWideDigitsPerThread; ++k) {
#pragma unroll
          for (int i = 0; i < kWideLookback; ++i) {
            if (((found >> k) & 1u) || !ok) break;
            uint32_t spins = 0;
            while ((lw[i][k] >> 30) == 0u) {  // not published yet: poll this one
              if (++spins > kSpinLimit) {
                ok = false;
                break;
              }
              if (spins > 16) __nanosleep(32);
              lw[i][k] = ld_relaxed_u32(status + (size_t)(pp - i) * kWideBins + d0 + k);
            }
            if (!ok) break;
            if (pp - i >= 0) excl[k] += lw[i][k] & kValueMask;
            if ((lw[i][k] >> 30) == kFlagInc) found |= 1u << k;
          }
        }
        pp -= kWideLookback;
      }
#pragma unroll
      for (uint32_t k = 0; k < kWideDigitsPerThread; ++k)
        st_relaxed_u32(status + (size_t)part * kWideBins + d0 + k,
                       (kFlagInc << 30) | ((excl[k] + pub[k]) & kValueMask));
    }
#pragma unroll
    for (uint32_t k = 0; k < kWideDigitsPerThread; ++k)
      s_dest[d0 + k] = s_bucket[d0 + k] + excl[k] - (s_dloc[d0 + k] + wbase);
    // C: partition reordered, destinations resolved
    if (!__syncthreads_and(ok)) {
      if (tid == 0) latch_error(err, DEVERR_TIMEOUT);
      break;
    }
    if (tid == kWideThreads - 1) claim_into(b ^ 1);
    for (uint32_t j = tid; j < count; j += kWideThreads) {
      const uint2 k = s_keys[j];
      const uint32_t dst = s_dest[wide_digit(k, word, shift)] + j;
      if (dst < R) {
        keys_out[dst] = k;
        vals_out[dst] = s_vals[j];
      } else {
        latch_error(err, DEVERR_RANGE);
      }
    }
    b ^= 1;
  }
}

cudaError_t onesweep_wide_setup() {
  // once per device (the attribute is a per-device setting); contexts on
  // other host threads may launch concurrently
  static std::mutex mu;
  static bool done[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = current_device(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (!done[dev]) {
    e = cudaFuncSetAttribute(onesweep_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)wide_pass_smem<uint2>());
    if (e != cudaSuccess) return e;
    done[dev] = true;
  }
  return cudaSuccess;
}

template <typename K, int NBITS>
cudaError_t onesweep_setup(int* per_sm) {
  // once per device and instantiation (the attribute is a per-device
  // setting); contexts on other host threads may launch concurrently
  static std::mutex mu;
  static int v[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = current_device(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (v[dev] == 0) {
    e = cudaFuncSetAttribute(onesweep_kernel<K, NBITS>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pass_smem<K>());
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, onesweep_kernel<K, NBITS>,
                                                      kPassThreads, pass_smem<K>());
    if (e != cudaSuccess) return e;
    v[dev] = n > 0 ? n : 1;
  }
  *per_sm = v[dev];
  return cudaSuccess;
}

// One pass, with the ballot count fitted to the digit's width.
template <typename K>
cudaError_t launch_pass(int nbits, const K* kin, const uint32_t* vin, K* kout, uint32_t* vout,
                        const uint32_t* ref_counter, uint32_t capacity, int word, int shift,
                        const uint32_t* hist, uint32_t* status, uint32_t* part_counter,
                        uint32_t* err, int sm_count, size_t parts_cap, cudaStream_t s) {
  int per_sm = 0;
  cudaError_t e;
#define GS3D_PASS(NB)                                                                        \
  e = onesweep_setup<K, NB>(&per_sm);                                                       \
  if (e != cudaSuccess) return e;                                                           \
  onesweep_kernel<K, NB><<<(int)std::min<size_t>((size_t)sm_count * per_sm, parts_cap),      \
                           kPassThreads, pass_smem<K>(), s>>>(kin, vin, kout, vout,          \
                                                              ref_counter, capacity, word,   \
                                                              shift, hist, status,           \
                                                              part_counter, err);            \
  break;
  if (nbits == kWideBits) {  // 2048-bin digits: (tile | depth) keys only
    if constexpr (std::is_same<K, uint2>::value) {
      e = onesweep_wide_setup();
      if (e != cudaSuccess) return e;
      onesweep_wide_kernel<<<(int)std::min<size_t>((size_t)sm_count, parts_cap), kWideThreads,
                             wide_pass_smem<uint2>(), s>>>(kin, vin, kout, vout, ref_counter,
                                                           capacity, word, shift, hist, status,
                                                           part_counter, err);
      return cudaGetLastError();
    } else {
      return cudaErrorInvalidValue;
    }
  }
  switch (nbits) {  // 2, 4, 6 or 8 (make_sort_plan)
    case 2: GS3D_PASS(2)
    case 4: GS3D_PASS(4)
    case 6: GS3D_PASS(6)
    default: GS3D_PASS(8)
  }
#undef GS3D_PASS
  return cudaGetLastError();
}

template <typename K>
cudaError_t launch_histogram(int passes, const PassDev& pd, const K* keys,
                             const uint32_t* ref_counter, uint32_t capacity, uint32_t* g_hist,
                             uint32_t* status, size_t stride, int grid, cudaStream_t s) {
#define GS3D_HIST_CASE(P)                                                                    \
  case P:                                                                                    \
    sort_histogram_kernel<K, P><<<grid, kThreads, 0, s>>>(keys, ref_counter, capacity, pd,   \
                                                          g_hist, status, stride);           \
    break;
  switch (passes) {
    GS3D_HIST_CASE(1)
    GS3D_HIST_CASE(2)
    GS3D_HIST_CASE(3)
    GS3D_HIST_CASE(4)
    GS3D_HIST_CASE(5)
    GS3D_HIST_CASE(6)
    GS3D_HIST_CASE(7)
    GS3D_HIST_CASE(8)
    default:
      return cudaErrorInvalidValue;
  }
#undef GS3D_HIST_CASE
  return cudaGetLastError();
}

// Runs `plan` over keys/vals A<->B; the histogram of every pass must be in
// g_hist[p][256] (computed here unless hist_ready) and status must hold
// sort_status_words(capacity, passes) words.
template <typename K>
cudaError_t run_passes(const SortPlan& plan, const uint32_t* ref_counter, uint32_t capacity,
                       K* keys_a, uint32_t* vals_a, K* keys_b, uint32_t* vals_b,
                       uint32_t* status, uint32_t* g_hist, size_t hist_stride,
                       uint32_t* part_counters, uint32_t* err, bool hist_ready, int sm_count,
                       cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  const size_t parts_cap = ((size_t)capacity + kPart - 1) / kPart + 1;
  const size_t stride = parts_cap * kRadixBins;
  // look-back status of pass p: parts_cap words per bin, passes back to back
  size_t status_off[kMaxSortPasses + 1] = {0};
  for (int p = 0; p < plan.passes; ++p)
    status_off[p + 1] =
        status_off[p] + parts_cap * (plan.nbits[p] == kWideBits ? kWideBins : kRadixBins);
  if (!hist_ready)  // the histogram kernel builds 256-bin histograms only
    for (int p = 0; p < plan.passes; ++p)
      if (plan.nbits[p] > 8 || hist_stride != kRadixBins) return cudaErrorInvalidValue;
  PassDev pd{};
  for (int p = 0; p < plan.passes; ++p) {
    pd.word[p] = plan.word[p];
    pd.shift[p] = plan.shift[p];
    pd.mask[p] = digit_mask(plan.nbits[p]);
  }
  if (!hist_ready) {
    e = launch_histogram<K>(plan.passes, pd, keys_a, ref_counter, capacity, g_hist, status,
                            stride, sm_count * 4, s);
  } else {
    e = cudaMemsetAsync(status, 0, status_off[plan.passes] * sizeof(uint32_t), s);
  }
  if (e != cudaSuccess) return e;
  for (int p = 0; p < plan.passes; ++p) {
    const bool even = (p % 2) == 0;
    e = launch_pass<K>(plan.nbits[p], even ? keys_a : keys_b, even ? vals_a : vals_b,
                       even ? keys_b : keys_a, even ? vals_b : vals_a, ref_counter, capacity,
                       plan.word[p], plan.shift[p], g_hist + (size_t)p * hist_stride,
                       status + status_off[p], part_counters + p, err, sm_count, parts_cap, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

SortPlan make_sort_plan(uint32_t num_tiles, int tile_digit_bits) {
  SortPlan p{};
  int n = 0;
  for (int s = 0; s < 32; s += 8) {  // depth bits (lo word)
    p.word[n] = 1;
    p.shift[n] = s;
    p.nbits[n] = 8;
    ++n;
  }
  const uint32_t max_tile = num_tiles > 0 ? num_tiles - 1 : 0;
  const int bits = max_tile ? 32 - __builtin_clz(max_tile) : 0;
  // at most kMaxSortPasses - 4 tile passes: wider digits when narrow ones
  // would need more
  int w = (tile_digit_bits == 4 || tile_digit_bits == 6 || tile_digit_bits == 11)
              ? tile_digit_bits : 8;
  if ((bits + w - 1) / w > kMaxSortPasses - 4) w = 8;
  for (int s = 0; s < bits; s += w) {  // tile-id bits (hi word)
    const int left = bits - s < w ? bits - s : w;  // the top digit may be narrower
    p.word[n] = 0;
    p.shift[n] = s;
    // kernels exist for 2, 4, 6, 8 and 11 bits
    p.nbits[n] = left > 8 ? kWideBits : (left + 1) & ~1;
    ++n;
  }
  p.passes = n;
  return p;
}

uint32_t sort_capacity_round(uint32_t capacity) {
  return (uint32_t)(((uint64_t)capacity + kRoundPart - 1) / kRoundPart * kRoundPart);
}

size_t sort_status_words(uint32_t capacity, int passes) {
  const size_t parts = ((size_t)capacity + kPart - 1) / kPart + 1;
  return parts * kRadixBins * (size_t)passes;
}

size_t sort_status_words_max(uint32_t capacity) {
  // the larger of 8 passes of 256 bins and 4 tile passes, 3 of them 2048-bin
  const size_t parts = ((size_t)capacity + kPart - 1) / kPart + 1;
  return parts * std::max<size_t>(kMaxSortPasses * kRadixBins, 3 * kWideBins + kRadixBins);
}

cudaError_t launch_sort(const SortPlan& plan, const uint32_t* ref_counter, uint32_t capacity,
                        uint2* keys_a, uint32_t* vals_a, uint2* keys_b, uint32_t* vals_b,
                        uint32_t* status, Ctrl* ctrl, int sm_count, cudaStream_t s) {
  // the sort may run more than once per frame: its tickets and histograms
  cudaError_t e = cudaMemsetAsync(ctrl->sort_part_counter, 0, sizeof(ctrl->sort_part_counter), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctrl->sort_hist, 0, sizeof(ctrl->sort_hist), s);
  if (e != cudaSuccess) return e;
  return run_passes<uint2>(plan, ref_counter, capacity, keys_a, vals_a, keys_b, vals_b, status,
                           &ctrl->sort_hist[0][0], kRadixBins, ctrl->sort_part_counter,
                           &ctrl->error, false, sm_count, s);
}

cudaError_t launch_sort_tile_passes(const SortPlan& plan, const uint32_t* ref_counter,
                                    uint32_t capacity, uint2* keys_a, uint32_t* vals_a,
                                    uint2* keys_b, uint32_t* vals_b, uint32_t* status,
                                    uint32_t* g_hist, uint32_t* part_counters, uint32_t* err,
                                    int sm_count, cudaStream_t s) {
  return run_passes<uint2>(plan, ref_counter, capacity, keys_a, vals_a, keys_b, vals_b, status,
                           g_hist, kTileHistStride, part_counters, err, true, sm_count, s);
}

cudaError_t launch_sort_u32(const SortPlan& plan, const uint32_t* count, uint32_t capacity,
                            uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b,
                            uint32_t* vals_b, uint32_t* status, uint32_t* g_hist,
                            uint32_t* part_counters, uint32_t* err, int sm_count, cudaStream_t s) {
  return run_passes<uint32_t>(plan, count, capacity, keys_a, vals_a, keys_b, vals_b, status,
                              g_hist, kRadixBins, part_counters, err, false, sm_count, s);
}

cudaError_t launch_sort_depth_keys(const uint32_t* count, uint32_t capacity, uint32_t* keys_a,
                                   uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b,
                                   uint32_t* status, uint32_t* g_hist, uint32_t* part_counters,
                                   uint32_t* err, int sm_count, cudaStream_t s) {
  SortPlan plan{};
  plan.passes = 4;
  for (int p = 0; p < 4; ++p) {
    plan.word[p] = 1;
    plan.shift[p] = 8 * p;
    plan.nbits[p] = 8;
  }
  return run_passes<uint32_t>(plan, count, capacity, keys_a, vals_a, keys_b, vals_b, status,
                              g_hist, kRadixBins, part_counters, err, false, sm_count, s);
}

}  // namespace gs3d
