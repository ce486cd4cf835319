// schedule.cu - work order of the persistent raster CTAs.
//
// The reference dispatches one workgroup per tile in row-major order
// (GaussianSplatRenderer.ts:1259-1265).  Per-tile raster cost spans orders of
// magnitude, and a long tile that starts late stretches the whole pass, so
// the persistent raster pulls tiles from a queue ordered by decreasing
// expected cost (longest-processing-time first).  The order only changes
// which CTA renders a tile and when; every pixel's arithmetic is unchanged.
//
// Key-count schedule: expected cost = the tile's key count (the plain
// schedule the learned one falls back to).  Learned schedule: expected cost
// = the cost MLP's prediction (learned.cu); both sort 16-bit keys.
//
// Both also split: the tiles whose expected cost per strip exceeds half of a
// raster CTA's fair share of the frame (the head of the order) are shaded as
// two half-strip work items per strip, so a tile far heavier than the rest
// does not leave one CTA running alone at the end of the raster.
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;

// key = 0xffff - min(count, 0xffff): ascending key order = descending count;
// two 8-bit passes sort it.  The expected cost is the key count.
__global__ void __launch_bounds__(kThreads)
    keycount_keys_kernel(const uint32_t* __restrict__ tile_offsets, uint32_t num_tiles,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ ids,
                         float* __restrict__ est) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= num_tiles) return;
  const uint32_t lo = __ldg(tile_offsets + t), hi = __ldg(tile_offsets + t + 1);
  const uint32_t n = hi > lo ? hi - lo : 0u;
  keys[t] = 0xffffu - min(n, 0xffffu);
  ids[t] = t;
  est[t] = (float)n;
}

// One block: the sum of the expected costs, then the count of tiles above
// half of a raster CTA's fair share (deterministic: fixed per-thread order,
// fixed tree reduction).
constexpr int kHeavyThreads = 1024;
__global__ void __launch_bounds__(kHeavyThreads)
    heavy_count_kernel(const float* __restrict__ est, uint32_t n, uint32_t raster_ctas,
                       uint32_t strips, uint32_t all, uint32_t* __restrict__ heavy) {
  __shared__ float s_sum[kHeavyThreads / 32];
  __shared__ uint32_t s_cnt[kHeavyThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (all) {
    if (threadIdx.x == 0) *heavy = n;
    return;
  }
  float sum = 0.0f;
  for (uint32_t t = threadIdx.x; t < n; t += kHeavyThreads) sum += __ldg(est + t);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) s_sum[warp] = sum;
  __syncthreads();
  float total = 0.0f;
  for (int w = 0; w < kHeavyThreads / 32; ++w) total += s_sum[w];
  // a strip costs about est; the frame about sum(est) * strips
  const float thr = 0.5f * total * (float)strips / (float)max(raster_ctas, 1u);
  uint32_t cnt = 0;
  for (uint32_t t = threadIdx.x; t < n; t += kHeavyThreads) cnt += __ldg(est + t) > thr ? 1u : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) s_cnt[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t c = 0;
    for (int w = 0; w < kHeavyThreads / 32; ++w) c += s_cnt[w];
    *heavy = c;
  }
}

}  // namespace

cudaError_t launch_heavy_count(const float* est, uint32_t n, uint32_t raster_ctas,
                               uint32_t strips, bool all, uint32_t* heavy, cudaStream_t s) {
  heavy_count_kernel<<<1, kHeavyThreads, 0, s>>>(est, n, raster_ctas, strips, all ? 1u : 0u,
                                                 heavy);
  return cudaGetLastError();
}

cudaError_t launch_schedule(uint32_t schedule, const uint32_t* tile_offsets, uint32_t num_tiles,
                            const uint32_t* num_tiles_dev, uint32_t* keys_a, uint32_t* order_a,
                            uint32_t* keys_b, uint32_t* order_b, float* est, uint32_t* status,
                            Ctrl* ctrl, uint32_t raster_ctas, uint32_t strips, bool split_all,
                            int sm_count, cudaStream_t s) {
  if (num_tiles == 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (schedule == GS3D_SCHEDULE_KEY_COUNT) {
    keycount_keys_kernel<<<(num_tiles + kThreads - 1) / kThreads, kThreads, 0, s>>>(
        tile_offsets, num_tiles, keys_a, order_a, est);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  e = launch_heavy_count(est, num_tiles, raster_ctas, strips, split_all, &ctrl->raster_heavy, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ctrl->sched_counter, 0, sizeof(ctrl->sched_counter), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ctrl->sched_hist, 0, sizeof(ctrl->sched_hist), s);
  if (e != cudaSuccess) return e;
  SortPlan plan{};
  plan.passes = 2;
  plan.word[0] = plan.word[1] = 1;
  plan.shift[0] = 0;
  plan.shift[1] = 8;
  plan.nbits[0] = plan.nbits[1] = 8;
  // two passes: the result is back in keys_a / order_a
  return launch_sort_u32(plan, num_tiles_dev, num_tiles, keys_a, order_a, keys_b, order_b,
                         status, &ctrl->sched_hist[0][0], ctrl->sched_counter, &ctrl->error,
                         sm_count, s);
}

}  // namespace gs3d
