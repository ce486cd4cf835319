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

// Boundary writes for sorted position i with tile curr, its predecessor's
// tile prev (ignored at i = 0) and its successor's tile next (ignored at the
// last position).
__device__ __forceinline__ void boundary(uint32_t i, uint32_t n, uint32_t prev, uint32_t curr,
                                         uint32_t next, uint32_t num_tiles,
                                         uint32_t* __restrict__ tile_offsets,
                                         uint32_t* __restrict__ err) {
  if (curr >= num_tiles) {  // tile id outside tile_offsets[0..num_tiles]
    latch_error(err, DEVERR_RANGE);
    return;
  }
  if (i == 0u || prev != curr) {
    const uint32_t from = i == 0u ? 0u : prev + 1u;
    for (uint32_t t = from; t <= curr; ++t) tile_offsets[t] = i;
  }
  if (i == n - 1u || next != curr) tile_offsets[curr + 1u] = i + 1u;
}

// Each thread owns two consecutive keys, read with one 16-byte load; the
// neighbouring tiles come from the adjacent lanes.
__global__ void __launch_bounds__(kThreads)
    identify_kernel(const uint2* __restrict__ keys, const uint32_t* __restrict__ ref_counter,
                    uint32_t capacity, uint32_t num_tiles, uint32_t* __restrict__ tile_offsets,
                    uint32_t* __restrict__ err) {
  const uint32_t n = live_refs(ref_counter, capacity);
  const uint32_t pairs = (n + 1) / 2;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * kThreads;
  const uint32_t first = blockIdx.x * kThreads + threadIdx.x;
  // warp-uniform trip count so the shuffles see every lane
  const uint32_t rounds = (pairs + stride - 1) / stride;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t g = first + r * stride;
    const uint32_t i0 = 2 * g;
    const bool live = g < pairs;
    uint32_t t0 = 0, t1 = 0;
    if (live) {
      if (i0 + 1 < n) {
        const uint4 kk = __ldg(reinterpret_cast<const uint4*>(keys + i0));
        t0 = kk.x;
        t1 = kk.z;
      } else {
        t0 = __ldg(&keys[i0].x);
      }
    }
    uint32_t prev = __shfl_up_sync(0xffffffffu, t1, 1);
    uint32_t next = __shfl_down_sync(0xffffffffu, t0, 1);
    if (!live) continue;
    if (lane == 0 && i0 > 0) prev = __ldg(&keys[i0 - 1].x);
    if ((lane == 31 || g + 1 >= pairs) && i0 + 2 < n) next = __ldg(&keys[i0 + 2].x);
    boundary(i0, n, prev, t0, i0 + 1 < n ? t1 : 0u, num_tiles, tile_offsets, err);
    if (i0 + 1 < n) boundary(i0 + 1, n, t0, t1, next, num_tiles, tile_offsets, err);
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
