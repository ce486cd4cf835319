// raster.cu - stage 6 of the rebin: tiled front-to-back alpha blending.
//
// Same per-pixel arithmetic and termination rules as
// src/shaders/compute/rasterize_tiles.wgsl:44-110: one CTA per tile, one
// thread per pixel, pixel centre = pixel + 0.5; per splat: circular cull at
// radius_px, power = -0.5 * d^T conic d, skip power > 0, alpha =
// min(0.99, opacity * exp(power)), skip alpha < 1/255, C += T * alpha * rgb,
// T *= 1 - alpha, stop the pixel once T < 1e-4 (checked after blending);
// the output is rgba16float (C, 1 - T), premultiplied, no background.
//
// GB300 specifics: each batch of sorted splats is staged into shared memory
// with 16-byte cp.async copies, double-buffered so the next batch streams in
// while the current one is blended, and the whole CTA leaves as soon as a
// block-wide vote finds every pixel terminated (the reference keeps looping
// over the tile's remaining batches).  Each CTA also records the tile's cost:
// the number of splats iterated before its last pixel terminated.
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

struct SplatStage {  // first 48 bytes of a ProjectedSplat
  float4 a;  // mean_px.xy, depth, radius_px
  float4 b;  // conic.xyz, opacity
  float4 c;  // color.xyz, valid
};

__global__ void raster_kernel(const FrameUniforms* __restrict__ fu, uint32_t tiles_x,
                              uint32_t tile_w, uint32_t tile_h,
                              const gs3d_projected_splat* __restrict__ proj,
                              const uint32_t* __restrict__ tile_offsets,
                              const uint32_t* __restrict__ values, uint2* __restrict__ image,
                              uint32_t* __restrict__ tile_costs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t nt = tile_w * tile_h;  // == blockDim.x == batch size
  SplatStage* buf0 = reinterpret_cast<SplatStage*>(smem);
  SplatStage* buf1 = buf0 + nt;
  __shared__ uint32_t s_cost;

  const uint32_t tid = threadIdx.x;
  const uint32_t tile = blockIdx.y * tiles_x + blockIdx.x;
  const uint32_t px = blockIdx.x * tile_w + tid % tile_w;
  const uint32_t py = blockIdx.y * tile_h + tid / tile_w;
  const uint32_t W = fu->viewport[0], H = fu->viewport[1];
  const bool in_bounds = px < W && py < H;
  const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;

  const uint32_t start = __ldg(tile_offsets + tile);
  const uint32_t end = __ldg(tile_offsets + tile + 1);
  const uint32_t len = end > start ? end - start : 0u;
  const uint32_t nbatches = (len + nt - 1) / nt;
  if (tid == 0) s_cost = 0u;

  float cr = 0.f, cg = 0.f, cb = 0.f, T = 1.0f;
  bool done = !in_bounds;
  uint32_t used = 0;  // splats iterated by this pixel

  auto stage = [&](uint32_t batch, SplatStage* dst) {
    const uint32_t idx = start + batch * nt + tid;
    if (idx < end) {
      const uint32_t id = __ldg(values + idx);
      const float4* src = reinterpret_cast<const float4*>(proj + id);
      cp_async16(&dst[tid].a, src + 0);
      cp_async16(&dst[tid].b, src + 1);
      cp_async16(&dst[tid].c, src + 2);
    }
    cp_async_commit();
  };

  if (nbatches > 0) stage(0, buf0);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage(bi + 1, (bi & 1) ? buf0 : buf1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const uint32_t cnt = min(nt, end - (start + bi * nt));
    if (!done) {
      for (uint32_t j = 0; j < cnt; ++j) {
        const float4 a = cur[j].a;
        const float dx = pfx - a.x, dy = pfy - a.y;
        if (dx * dx + dy * dy > a.w * a.w) continue;
        const float4 b = cur[j].b;
        const float power = -0.5f * (b.x * dx * dx + 2.0f * b.y * dx * dy + b.z * dy * dy);
        if (power > 0.0f) continue;
        const float alpha = fminf(0.99f, b.w * __expf(power));
        if (alpha < 1.0f / 255.0f) continue;
        const float4 c = cur[j].c;
        const float ta = T * alpha;
        cr += ta * c.x;
        cg += ta * c.y;
        cb += ta * c.z;
        T *= 1.0f - alpha;
        if (T < 1.0e-4f) {
          done = true;
          used = bi * nt + j + 1;
          break;
        }
      }
      if (!done) used = bi * nt + cnt;
    }
    if (__syncthreads_and(done)) {
      cp_async_wait<0>();  // drain the prefetch of the next batch before leaving
      break;
    }
  }
  if (in_bounds) {
    atomicMax(&s_cost, used);
    const __half2 rg = __floats2half2_rn(cr, cg);
    const __half2 ba = __floats2half2_rn(cb, 1.0f - T);
    image[(size_t)py * W + px] =
        make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&ba));
  }
  if (tile_costs != nullptr) {
    __syncthreads();
    if (tid == 0) tile_costs[tile] = s_cost;
  }
}

}  // namespace

cudaError_t launch_raster(const FrameUniforms* d_frame, uint32_t tiles_x, uint32_t tiles_y,
                          uint32_t tile_w, uint32_t tile_h, const gs3d_projected_splat* proj,
                          const uint32_t* tile_offsets, const uint32_t* values, uint2* image,
                          uint32_t* tile_costs, cudaStream_t s) {
  if (tiles_x == 0 || tiles_y == 0) return cudaSuccess;
  const uint32_t nt = tile_w * tile_h;
  const size_t smem = 2 * (size_t)nt * sizeof(SplatStage);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(raster_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  raster_kernel<<<dim3(tiles_x, tiles_y), nt, smem, s>>>(d_frame, tiles_x, tile_w, tile_h, proj,
                                                         tile_offsets, values, image, tile_costs);
  return cudaGetLastError();
}

}  // namespace gs3d
