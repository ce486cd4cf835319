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
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;

// key = 0xffff - min(count, 0xffff): ascending key order = descending count;
// two 8-bit passes sort it.
__global__ void __launch_bounds__(kThreads)
    keycount_keys_kernel(const uint32_t* __restrict__ tile_offsets, uint32_t num_tiles,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ ids) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= num_tiles) return;
  const uint32_t lo = __ldg(tile_offsets + t), hi = __ldg(tile_offsets + t + 1);
  const uint32_t n = hi > lo ? hi - lo : 0u;
  keys[t] = 0xffffu - min(n, 0xffffu);
  ids[t] = t;
}

}  // namespace

cudaError_t launch_schedule(uint32_t schedule, const uint32_t* tile_offsets, uint32_t num_tiles,
                            const uint32_t* num_tiles_dev, uint32_t* keys_a, uint32_t* order_a,
                            uint32_t* keys_b, uint32_t* order_b, uint32_t* status, Ctrl* ctrl,
                            int sm_count, cudaStream_t s) {
  if (num_tiles == 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (schedule == GS3D_SCHEDULE_KEY_COUNT) {
    keycount_keys_kernel<<<(num_tiles + kThreads - 1) / kThreads, kThreads, 0, s>>>(
        tile_offsets, num_tiles, keys_a, order_a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
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
