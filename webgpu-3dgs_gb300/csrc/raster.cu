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
// GB300 specifics:
//  * each batch of sorted splats is staged into shared memory with 16-byte
//    cp.async copies, double-buffered so the next batch streams in while the
//    current one is blended;
//  * the CTA leaves as soon as a block-wide vote finds every pixel
//    terminated (the reference keeps looping over the remaining batches);
//  * (culled variant) each warp owns a compact pixel block (8x4 for tiles
//    whose sides divide by 8 and 4) and tests every staged splat once against
//    it; a splat is skipped for the whole warp only when every pixel of the
//    block is provably rejected by the per-pixel tests themselves: outside
//    the radius circle, or alpha < 1/255 by the bound
//    alpha <= opacity * exp(-0.5 * lambda_min(conic) * |d|^2), both with
//    margins that cover f32 rounding.  Pixels therefore blend exactly the
//    same splats in the same order, and the image is bit-identical to the
//    one-thread-per-pixel variant;
//  * each CTA records the tile's cost: the number of splats iterated before
//    its last pixel terminated.
//
// The per-pixel update is written with explicit round-to-nearest intrinsics so
// both variants compile to the same arithmetic.
#include <algorithm>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

struct SplatStage {  // first 48 bytes of a ProjectedSplat
  float4 a;  // mean_px.xy, depth, radius_px
  float4 b;  // conic.xyz, opacity
  float4 c;  // color.xyz, valid
};

struct Pixel {
  float cr, cg, cb, T;
};

// rasterize_tiles.wgsl:81-98 for one (pixel, splat) pair; true once the
// pixel's transmittance fell below 1e-4.
__device__ __forceinline__ bool blend_one(float pfx, float pfy, const SplatStage& s, Pixel& p) {
  const float4 a = s.a;
  const float dx = __fsub_rn(pfx, a.x);
  const float dy = __fsub_rn(pfy, a.y);
  if (__fmaf_rn(dx, dx, __fmul_rn(dy, dy)) > __fmul_rn(a.w, a.w)) return false;
  const float4 b = s.b;
  const float q = __fmaf_rn(__fmul_rn(b.x, dx), dx,
                            __fmaf_rn(__fmul_rn(__fmul_rn(2.0f, b.y), dx), dy,
                                      __fmul_rn(__fmul_rn(b.z, dy), dy)));
  const float power = __fmul_rn(-0.5f, q);
  if (power > 0.0f) return false;
  const float alpha = fminf(0.99f, __fmul_rn(b.w, __expf(power)));
  if (alpha < 1.0f / 255.0f) return false;
  const float4 c = s.c;
  const float ta = __fmul_rn(p.T, alpha);
  p.cr = __fmaf_rn(ta, c.x, p.cr);
  p.cg = __fmaf_rn(ta, c.y, p.cg);
  p.cb = __fmaf_rn(ta, c.z, p.cb);
  p.T = __fmul_rn(p.T, __fsub_rn(1.0f, alpha));
  return p.T < 1.0e-4f;
}

__device__ __forceinline__ void store_pixel(uint2* image, uint32_t W, uint32_t px, uint32_t py,
                                            const Pixel& p) {
  const __half2 rg = __floats2half2_rn(p.cr, p.cg);
  const __half2 ba = __floats2half2_rn(p.cb, 1.0f - p.T);
  image[(size_t)py * W + px] =
      make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&ba));
}

__device__ __forceinline__ void stage_batch(const gs3d_projected_splat* __restrict__ proj,
                                            const uint32_t* __restrict__ values, uint32_t idx,
                                            uint32_t end, SplatStage* dst) {
  if (idx < end) {
    const uint32_t id = __ldg(values + idx);
    const float4* src = reinterpret_cast<const float4*>(proj + id);
    cp_async16(&dst->a, src + 0);
    cp_async16(&dst->b, src + 1);
    cp_async16(&dst->c, src + 2);
  }
  cp_async_commit();
}

struct TileGeom {
  uint32_t tile;      // global tile id
  uint32_t ox, oy;    // pixel origin of the tile in its view
  uint32_t W, H;      // view size
  uint2* image;       // the view's image
};

__device__ __forceinline__ TileGeom tile_geom(const RasterArgs& a, uint32_t t) {
  const uint32_t v =
      find_view(a.n_views, t, [&](uint32_t k) { return __ldg(&a.views[k].f.tile_base); });
  const ViewDesc& vd = a.views[v];
  const uint32_t lt = t - __ldg(&vd.f.tile_base);
  const uint32_t tx_count = __ldg(&vd.f.tile_count[0]);
  TileGeom g;
  g.tile = t;
  g.ox = (lt % tx_count) * a.tile_w;
  g.oy = (lt / tx_count) * a.tile_h;
  g.W = __ldg(&vd.f.viewport[0]);
  g.H = __ldg(&vd.f.viewport[1]);
  g.image = a.image + __ldg(&vd.pixel_base);
  return g;
}

// One thread per pixel, linear pixel order (the reference's layout).
__device__ void raster_tile_plain(const RasterArgs& a, const TileGeom& g, SplatStage* buf0,
                                  SplatStage* buf1, uint32_t* s_cost) {
  const uint32_t nt = a.tile_w * a.tile_h;  // == blockDim.x == batch size
  const uint32_t tid = threadIdx.x;
  const uint32_t px = g.ox + tid % a.tile_w;
  const uint32_t py = g.oy + tid / a.tile_w;
  const bool in_bounds = px < g.W && py < g.H;
  const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;

  const uint32_t start = __ldg(a.tile_offsets + g.tile);
  const uint32_t end = __ldg(a.tile_offsets + g.tile + 1);
  const uint32_t len = end > start ? end - start : 0u;
  const uint32_t nbatches = (len + nt - 1) / nt;

  Pixel p{0.f, 0.f, 0.f, 1.0f};
  bool done = !in_bounds;
  uint32_t used = 0;

  if (nbatches > 0) stage_batch(a.proj, a.values, start + tid, end, buf0 + tid);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage_batch(a.proj, a.values, start + (bi + 1) * nt + tid, end,
                  ((bi & 1) ? buf0 : buf1) + tid);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const uint32_t cnt = min(nt, end - (start + bi * nt));
    if (!done) {
      for (uint32_t j = 0; j < cnt; ++j) {
        if (blend_one(pfx, pfy, cur[j], p)) {
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
    atomicMax(s_cost, used);
    store_pixel(g.image, g.W, px, py, p);
  }
}

// Squared distance below which a splat may still touch some pixel of a
// warp's block (conservative; see the file comment).
__device__ __forceinline__ float reach_d2(const SplatStage& s) {
  const float r = s.a.w;
  const float circle = r * r * 1.0001f + 1e-3f;
  const float A = s.b.x, B = s.b.y, Cc = s.b.z, op = s.b.w;
  // smallest eigenvalue of the conic, shrunk to cover its rounding
  const float h = 0.5f * (A - Cc);
  float lmin = 0.5f * (A + Cc) - sqrtf(h * h + B * B);
  lmin = lmin * 0.999f - 1e-7f * (fabsf(A) + fabsf(Cc));
  const float lim = op * (255.0f * 1.001f);  // alpha >= 1/255 needs exp(power) >= 1/lim
  if (!(lim > 1.0f)) return -1.0f;           // alpha < 1/255 at every pixel
  // very elongated conics: the rounding of d^T conic d could exceed the
  // bound's margin, so only the circle test is used
  if (!(lmin > 1e-4f * (fabsf(A) + fabsf(Cc)))) return circle;
  const float alpha_d2 = 2.0f * logf(lim) / lmin * 1.001f + 1e-3f;
  return fminf(circle, alpha_d2);
}

// Culled variant: warps own compact pixel blocks and skip splats that no
// pixel of their block can blend.  blockDim.x == tile_w * tile_h, a multiple
// of 32.
__device__ void raster_tile_culled(const RasterArgs& a, const TileGeom& g, SplatStage* buf0,
                                   SplatStage* buf1, float* s_reach, uint32_t* s_cost) {
  const uint32_t nt = a.tile_w * a.tile_h;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t lx, ly;
  if ((a.tile_w % 8 == 0) && (a.tile_h % 4 == 0)) {  // 8x4 pixel block per warp
    const uint32_t bw = a.tile_w / 8;
    lx = (warp % bw) * 8 + (lane & 7);
    ly = (warp / bw) * 4 + (lane >> 3);
  } else {
    lx = tid % a.tile_w;
    ly = tid / a.tile_w;
  }
  const uint32_t px = g.ox + lx;
  const uint32_t py = g.oy + ly;
  const bool in_bounds = px < g.W && py < g.H;
  const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;
  // the warp's pixel-centre bounding box
  float xlo = pfx, xhi = pfx, ylo = pfy, yhi = pfy;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    xlo = fminf(xlo, __shfl_xor_sync(0xffffffffu, xlo, o));
    xhi = fmaxf(xhi, __shfl_xor_sync(0xffffffffu, xhi, o));
    ylo = fminf(ylo, __shfl_xor_sync(0xffffffffu, ylo, o));
    yhi = fmaxf(yhi, __shfl_xor_sync(0xffffffffu, yhi, o));
  }

  const uint32_t start = __ldg(a.tile_offsets + g.tile);
  const uint32_t end = __ldg(a.tile_offsets + g.tile + 1);
  const uint32_t len = end > start ? end - start : 0u;
  const uint32_t nbatches = (len + nt - 1) / nt;

  Pixel p{0.f, 0.f, 0.f, 1.0f};
  bool done = !in_bounds;
  uint32_t used = 0;

  if (nbatches > 0) stage_batch(a.proj, a.values, start + tid, end, buf0 + tid);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage_batch(a.proj, a.values, start + (bi + 1) * nt + tid, end,
                  ((bi & 1) ? buf0 : buf1) + tid);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const uint32_t cnt = min(nt, end - (start + bi * nt));
    if (tid < cnt) s_reach[tid] = reach_d2(cur[tid]);  // own copy is complete
    __syncthreads();
    if (__any_sync(0xffffffffu, !done)) {
      for (uint32_t k0 = 0; k0 < cnt; k0 += 32) {
        const uint32_t j = k0 + lane;
        bool hit = false;
        if (j < cnt) {
          const float mx = cur[j].a.x, my = cur[j].a.y;
          const float ex = mx - fminf(fmaxf(mx, xlo), xhi);
          const float ey = my - fminf(fmaxf(my, ylo), yhi);
          hit = ex * ex + ey * ey <= s_reach[j];
        }
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const uint32_t b = __ffs(mask) - 1;
          mask &= mask - 1;
          if (!done && blend_one(pfx, pfy, cur[k0 + b], p)) {
            done = true;
            used = bi * nt + k0 + b + 1;
          }
        }
        if (__all_sync(0xffffffffu, done)) break;
      }
      if (!done) used = bi * nt + cnt;
    }
    if (__syncthreads_and(done)) {
      cp_async_wait<0>();
      break;
    }
  }
  if (in_bounds) {
    atomicMax(s_cost, used);
    store_pixel(g.image, g.W, px, py, p);
  }
}

// Persistent CTAs pull tile indices from the work queue.
template <bool CULLED>
__global__ void raster_kernel(RasterArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t nt = a.tile_w * a.tile_h;
  SplatStage* buf0 = reinterpret_cast<SplatStage*>(smem);
  SplatStage* buf1 = buf0 + nt;
  float* s_reach = reinterpret_cast<float*>(buf1 + nt);
  __shared__ uint32_t s_item, s_cost;
  while (true) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(a.queue_counter, 1u);
      s_cost = 0u;
    }
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= a.num_tiles) break;
    const uint32_t t = a.order != nullptr ? __ldg(a.order + item) : item;
    const TileGeom g = tile_geom(a, t);
    if (CULLED)
      raster_tile_culled(a, g, buf0, buf1, s_reach, &s_cost);
    else
      raster_tile_plain(a, g, buf0, buf1, &s_cost);
    __syncthreads();  // s_cost complete; shared buffers free for the next tile
    if (threadIdx.x == 0 && a.tile_costs != nullptr) a.tile_costs[t] = s_cost;
  }
}

}  // namespace

cudaError_t launch_raster(const RasterArgs& a, int sm_count, cudaStream_t s) {
  if (a.num_tiles == 0) return cudaSuccess;
  const uint32_t nt = a.tile_w * a.tile_h;
  const bool culled = a.culled && (nt % 32 == 0);
  const size_t smem = 2 * (size_t)nt * sizeof(SplatStage) + (culled ? nt * sizeof(float) : 0);
  auto kern = culled ? raster_kernel<true> : raster_kernel<false>;
  // launch configuration per (variant, tile area), computed once per process
  static int cache[2][1025] = {};
  int& per_sm = cache[culled ? 1 : 0][nt];
  if (per_sm == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(smem, 48 * 1024));
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, (int)nt, smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(n, 1);
  }
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      a.num_tiles, (uint64_t)sm_count * (uint64_t)std::max(per_sm, 1));
  kern<<<grid, nt, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gs3d
