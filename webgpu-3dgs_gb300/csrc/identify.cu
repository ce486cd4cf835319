// identify.cu - stage 5 of the rebin: per-tile ranges of the sorted keys.
//
// Same write pattern as src/shaders/compute/identify_tile_ranges.wgsl:31-52,
// including its conventions: a start boundary at i fills
// tile_offsets[prev + 1 ..= curr] = i (from 0 when i = 0), an end boundary
// writes tile_offsets[curr + 1] = i + 1, and tiles after the last populated
// one keep the 0 of the preceding clear, so tile_offsets is not a strict
// prefix array (readers guard with hi >= lo, GaussianSplatRenderer.ts:1301).
// Grid-stride over the live count, which is read on the device.
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
    identify_kernel(const uint2* __restrict__ keys, const uint32_t* __restrict__ ref_counter,
                    uint32_t capacity, uint32_t num_tiles, uint32_t* __restrict__ tile_offsets,
                    uint32_t* __restrict__ err) {
  const uint32_t n = live_refs(ref_counter, capacity);
  const uint32_t stride = gridDim.x * kThreads;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) {
    const uint32_t curr = __ldg(&keys[i].x);
    if (curr >= num_tiles) {  // tile id outside tile_offsets[0..num_tiles]
      latch_error(err, DEVERR_RANGE);
      continue;
    }
    const uint32_t prev = i > 0 ? __ldg(&keys[i - 1].x) : 0u;
    if (i == 0u || prev != curr) {
      const uint32_t from = i == 0u ? 0u : prev + 1u;
      for (uint32_t t = from; t <= curr; ++t) tile_offsets[t] = i;
    }
    if (i == n - 1u || __ldg(&keys[i + 1].x) != curr) tile_offsets[curr + 1u] = i + 1u;
  }
}

}  // namespace

cudaError_t launch_identify(const uint2* keys, const uint32_t* ref_counter, uint32_t capacity,
                            uint32_t num_tiles, uint32_t* tile_offsets, uint32_t* err,
                            int sm_count, cudaStream_t s) {
  cudaError_t e =
      cudaMemsetAsync(tile_offsets, 0, ((size_t)num_tiles + 1) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  identify_kernel<<<sm_count * 8, kThreads, 0, s>>>(keys, ref_counter, capacity, num_tiles,
                                                    tile_offsets, err);
  return cudaGetLastError();
}

}  // namespace gs3d
