// composite.cu - the render passes after the rasterizer, headless: the
// per-tile splat-count heat map overlay (src/shaders/render/
// debug_tile_overlay.wgsl) and the premultiplied "over" composite onto the
// framebuffer (composite_splats.wgsl with the blend state of
// GaussianSplatRenderer.ts:938-945), writing an RGBA8 buffer instead of a
// swapchain texture.
//
// One thread per pixel; f32 arithmetic without contraction so the result is
// reproducible bit for bit: overlay = tint * 0.4 + base * (1 - 0.4), stored
// to half (the reference's rgba16float debug target); out = src + dst *
// (1 - src.a); unorm8 = round-to-nearest-even(clamp01(x) * 255).
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

__device__ __forceinline__ float clamp01(float x) { return fminf(1.0f, fmaxf(0.0f, x)); }

__device__ __forceinline__ uint32_t unorm8(float x) {
  return __float2uint_rn(__fmul_rn(clamp01(x), 255.0f));
}

__global__ void composite_kernel(const uint2* __restrict__ image, uint32_t W, uint32_t H,
                                 const uint32_t* __restrict__ tile_offsets, uint32_t tile_w,
                                 uint32_t tile_h, uint32_t tiles_x, uint32_t tiles_y,
                                 uint32_t heatmap, uint32_t debug_ref, float4 bg,
                                 uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * H) return;
  const uint2 raw = __ldg(image + i);
  const __half2 rg = *reinterpret_cast<const __half2*>(&raw.x);
  const __half2 ba = *reinterpret_cast<const __half2*>(&raw.y);
  float r = __low2float(rg), g = __high2float(rg), b = __low2float(ba), a = __high2float(ba);
  if (heatmap) {
    const uint32_t px = i % W, py = i / W;
    const uint32_t tx = min(px / tile_w, tiles_x - 1), ty = min(py / tile_h, tiles_y - 1);
    const uint32_t t = ty * tiles_x + tx;
    // tile_offsets is not a strict prefix array (trailing zeros): guard hi >= lo
    const uint32_t lo = __ldg(tile_offsets + t), hi = __ldg(tile_offsets + t + 1);
    const uint32_t count = hi >= lo ? hi - lo : 0u;
    const float tt = clamp01(__fdiv_rn((float)count, fmaxf(1.0f, (float)debug_ref)));
    const float tr = clamp01(__fmul_rn(tt, 2.0f));
    const float tg = clamp01(__fsub_rn(2.0f, __fmul_rn(tt, 2.0f)));
    const float ao = 0.4f, keep = __fsub_rn(1.0f, ao);
    // the overlay target is rgba16float
    r = __half2float(__float2half_rn(__fadd_rn(__fmul_rn(tr, ao), __fmul_rn(r, keep))));
    g = __half2float(__float2half_rn(__fadd_rn(__fmul_rn(tg, ao), __fmul_rn(g, keep))));
    b = __half2float(__float2half_rn(__fadd_rn(__fmul_rn(0.0f, ao), __fmul_rn(b, keep))));
    a = __half2float(__float2half_rn(__fadd_rn(ao, __fmul_rn(a, keep))));
  }
  // blend one / one-minus-src-alpha, colour and alpha
  const float inv = __fsub_rn(1.0f, a);
  const uint32_t R = unorm8(__fadd_rn(r, __fmul_rn(bg.x, inv)));
  const uint32_t G = unorm8(__fadd_rn(g, __fmul_rn(bg.y, inv)));
  const uint32_t B = unorm8(__fadd_rn(b, __fmul_rn(bg.z, inv)));
  const uint32_t A = unorm8(__fadd_rn(a, __fmul_rn(bg.w, inv)));
  out[i] = R | (G << 8) | (B << 16) | (A << 24);
}

}  // namespace

cudaError_t launch_composite(const uint2* image, uint32_t W, uint32_t H,
                             const uint32_t* tile_offsets, uint32_t tile_w, uint32_t tile_h,
                             uint32_t tiles_x, uint32_t tiles_y, uint32_t heatmap,
                             uint32_t debug_ref, const float bg[4], uint32_t* out,
                             cudaStream_t s) {
  const uint64_t n = (uint64_t)W * H;
  if (n == 0) return cudaSuccess;
  const uint32_t threads = 256;
  composite_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(
      image, W, H, tile_offsets, tile_w, tile_h, tiles_x, tiles_y, heatmap, debug_ref,
      make_float4(bg[0], bg[1], bg[2], bg[3]), out);
  return cudaGetLastError();
}

}  // namespace gs3d
