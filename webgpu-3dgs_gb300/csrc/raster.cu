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
//  * each batch of sorted splats (RasterArgs::batch splats, by default one
//    per tile pixel) is staged into shared memory with 16-byte cp.async
//    copies, double-buffered so the next batch streams in while the current
//    one is blended;
//  * the CTA leaves as soon as a block-wide vote finds every pixel
//    terminated (the reference keeps looping over the remaining batches);
//  * each staged splat is converted once per tile into its raster form (r^2,
//    the quadratic form's coefficients, the visibility bound), so a (pixel,
//    splat) pair costs one ex2 and a branch-free handful of FP32 operations
//    (a skipped splat blends with alpha = 0, which leaves the pixel
//    bit-unchanged);
//  * (culled variant) each warp owns a compact pixel block (8x4 for tiles
//    whose sides divide by 8 and 4) and tests every staged splat once against
//    it; a splat is skipped for the whole warp only when no pixel centre of
//    the block can pass the per-pixel tests: the block lies outside the
//    radius circle, or the minimum of d^T conic d over the block keeps
//    alpha below 1/255, with margins that cover f32 rounding and the fast
//    division of the edge minimisers.  Pixels therefore blend exactly the
//    same splats in the same order, and the image is bit-identical to the
//    one-thread-per-pixel variant;
//  * (two-pixel variant, tiles whose sides divide by 8) each warp owns an 8x8
//    block, a lane shading rows y and y + 4 of one column with the paired
//    FP32 instructions of sm_100 (each half rounded like the scalar path);
//    tiles above 512 pixels are shaded by four (else two) CTAs, one row
//    strip each, whose tile costs combine by maximum;
//  * each CTA records the tile's cost: the number of splats iterated before
//    its last pixel terminated.
//
// The variants share the per-pixel arithmetic (the two-pixel one as paired
// instructions with the same per-half rounding), so their images are
// bit-identical.  For splats whose quadratic form can cancel badly the
// radius test and power = -0.5 d^T conic d follow the reference's f32
// expression order exactly (no contraction; SplatStage below); the others,
// the exponent (ex2 in the log2 domain) and the blend (fused multiply-adds)
// differ from the reference only in rounding, which the 2/255 image
// tolerance covers.
#include <algorithm>
#include <map>
#include <mutex>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

// A staged splat in one of two forms of the quadratic form q(d) = b.x dx^2 +
// b.y dx dy + b.z dy^2 (c.w says which):
//   fast  (c.w = 0): b = log2(e)/2 (conic.x, 2 conic.y, conic.z), q = Q =
//         -power log2(e), evaluated with FMAs;
//   exact (c.w = 1): b = (conic.x, 2 conic.y, conic.z), q = s = d^T conic d
//         = -2 power, evaluated in the reference's operation order without
//         contraction (every sum a scalar __fadd_rn: a paired FP32 multiply
//         feeding a paired add is contracted into a paired FMA).
// Splats take the exact form when the terms of q can reach 2^12 inside the
// radius, (|conic.x| + 2 |conic.y| + |conic.z|) r^2 > 2^12: there the terms
// cancel (elongated splats seen far from their mean), and the rounding order
// decides the result.  Below that bound the fast form's q differs from the
// reference's by about 2^-11 at most, so each alpha differs by a relative
// 1e-3 and a pixel, whose blend weights alpha_i T_i sum to at most 1, by
// about that much.  b.w = vis, in q's units.
struct SplatStage {  // first 48 bytes of a ProjectedSplat, prepared in place (prepare())
  float4 a;  // mean_px.x, mean_px.y, radius_px^2, opacity
  float4 b;  // q coefficients (see above), vis
  float4 c;  // color.xyz, form
};

constexpr float kHalfLog2e = 0.72134752044448170f;
constexpr float kExactFormBound = 4096.0f;

struct Pixel {
  float cr, cg, cb, T;
};

// ex2.approx: 2^x on the SFU.
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Converts the staged ProjectedSplat prefix (mean, depth, radius | conic,
// opacity | color, valid) into the raster form.  vis = the largest Q at which
// alpha can still reach 1/255, with a 1% margin, in the units of the splat's
// form (-1: never visible; +inf: conic too ill-conditioned for the alpha
// bound, or a non-finite opacity or conic: use the circle only).
__device__ __forceinline__ void prepare(SplatStage& s) {
  const float4 a = s.a, b = s.b;
  const float A = b.x, B = b.y, C = b.z, op = b.w;
  float vis;
  const float lim = op * 255.0f;
  if (lim < 0.999f) {
    vis = -1.0f;  // alpha = opacity * exp(power) <= opacity < 1/255 everywhere
  } else if (lim > 1.0f && A * C - B * B >= 1e-3f * (A + C) * (A + C) && A > 0.0f && C > 0.0f) {
    vis = __log2f(lim) * 1.01f + 1e-3f;
  } else {
    vis = __int_as_float(0x7f800000);
  }
  const float r2 = a.w * a.w;
  const float terms = (fabsf(A) + 2.0f * fabsf(B) + fabsf(C)) * r2;
  s.a = make_float4(a.x, a.y, r2, op);
  if (terms <= kExactFormBound) {
    s.b = make_float4(kHalfLog2e * A, 2.0f * kHalfLog2e * B, kHalfLog2e * C, vis);
    s.c.w = 0.0f;
  } else {  // also non-finite terms
    s.b = make_float4(A, 2.0f * B, C, vis / kHalfLog2e);
    s.c.w = 1.0f;
  }
}

// rasterize_tiles.wgsl:81-98 for one (pixel, splat) pair: the splat's alpha
// at the pixel centre and whether it passes the per-pixel tests (not outside
// the radius, power not > 0, alpha not < 1/255: a NaN passes, as in the
// reference).  A skipped splat blends with alpha = 0 (blend_alpha), which
// leaves C and T bit-unchanged.
__device__ __forceinline__ float splat_alpha(float pfx, float pfy, const SplatStage& s,
                                             bool& ok) {
  const float4 a = s.a, b = s.b;
  const float dx = pfx - a.x;
  const float dy = pfy - a.y;
  if (s.c.w == 0.0f) {
    // fast form: q < 0 cannot occur (no power > 0 test needed): these splats'
    // conics have condition numbers below 455 (their terms, at least 9 times
    // the condition number, stay within kExactFormBound), so q, computed to
    // a relative 1e-3, and the reference's s keep the sign of the positive
    // definite form at every pixel centre, which lies 6e-8 pixels or more
    // from the mean unless exactly on it
    const float d2 = fmaf(dx, dx, dy * dy);
    const float q = fmaf(b.x * dx, dx, fmaf(b.y * dx, dy, b.z * dy * dy));  // -power log2(e)
    const float alpha = fminf(0.99f, a.w * ex2_approx(-q));
    ok = !(d2 > a.z) && !(alpha < 1.0f / 255.0f);
    return alpha;
  }
  // the reference's order: d^2 = dx dx + dy dy, s = (c0 dx) dx + (2 c1 dx) dy + (c2 dy) dy
  const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  const float q = __fadd_rn(
      __fadd_rn(__fmul_rn(__fmul_rn(b.x, dx), dx), __fmul_rn(__fmul_rn(b.y, dx), dy)),
      __fmul_rn(__fmul_rn(b.z, dy), dy));
  const float alpha = fminf(0.99f, a.w * ex2_approx(__fmul_rn(q, -kHalfLog2e)));  // exp(-s/2)
  ok = !(d2 > a.z) && !(q < 0.0f) && !(alpha < 1.0f / 255.0f);
  return alpha;
}

// Blends alpha (0 when !ok, which leaves C and T bit-unchanged); returns
// true when the pixel terminates here.
__device__ __forceinline__ bool blend_alpha(Pixel& p, const float4 c, float alpha, bool ok) {
  const float al = ok ? alpha : 0.0f;
  const float ta = p.T * al;
  p.cr = fmaf(ta, c.x, p.cr);
  p.cg = fmaf(ta, c.y, p.cg);
  p.cb = fmaf(ta, c.z, p.cb);
  p.T = p.T * (1.0f - al);
  return ok && p.T < 1.0e-4f;
}

template <bool EARLY_OUT>
__device__ __forceinline__ bool blend_one(float pfx, float pfy, const SplatStage& s, Pixel& p,
                                          bool live) {
  if (EARLY_OUT) {  // outside the radius (d^2 as splat_alpha forms it): alpha would be 0
    const float dx = pfx - s.a.x, dy = pfy - s.a.y;
    const float d2 = s.c.w == 0.0f ? fmaf(dx, dx, dy * dy)
                                   : __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 > s.a.z) return false;
  }
  bool ok;
  const float alpha = splat_alpha(pfx, pfy, s, ok);
  return blend_alpha(p, s.c, alpha, ok && live);
}

// Two pixels of one column in the halves of a float2 (the two-pixel
// variant).  Every component is computed by the scalar operation of
// splat_alpha / blend_alpha, in the same order and rounding (the paired
// FP32 instructions of sm_100 round each half like their scalar forms), so
// each pixel is bit-identical to the one-pixel variants.
__device__ __forceinline__ float2 bcast(float x) { return make_float2(x, x); }

struct Pixel2 {
  float2 cr, cg, cb, T;
};

__device__ __forceinline__ float2 splat_alpha2(float pfx, float2 pfy, const SplatStage& s,
                                               bool& ok0, bool& ok1) {
  const float4 a = s.a, b = s.b;
  const float dx = pfx - a.x;
  const float2 dy = __fadd2_rn(pfy, bcast(-a.y));
  float2 d2, q, ev;
  if (s.c.w == 0.0f) {  // fast form (splat-uniform branch; no q < 0 test, see splat_alpha)
    d2 = __ffma2_rn(bcast(dx), bcast(dx), __fmul2_rn(dy, dy));
    q = __ffma2_rn(bcast(b.x * dx), bcast(dx),
                   __ffma2_rn(bcast(b.y * dx), dy, __fmul2_rn(__fmul2_rn(bcast(b.z), dy), dy)));
    const float2 e = make_float2(ex2_approx(-q.x), ex2_approx(-q.y));
    const float2 am = __fmul2_rn(bcast(a.w), e);
    const float2 alpha = make_float2(fminf(0.99f, am.x), fminf(0.99f, am.y));
    ok0 = !(d2.x > a.z) && !(alpha.x < 1.0f / 255.0f);
    ok1 = !(d2.y > a.z) && !(alpha.y < 1.0f / 255.0f);
    return alpha;
  } else {  // exact form in the reference's order, the column's dx terms shared; the
            // products are paired, every sum a scalar __fadd_rn (never merged into an FMA)
    const float dxx = __fmul_rn(dx, dx);
    const float t1 = __fmul_rn(__fmul_rn(b.x, dx), dx);
    const float2 dyy = __fmul2_rn(dy, dy);
    const float2 t2 = __fmul2_rn(bcast(__fmul_rn(b.y, dx)), dy);
    const float2 t3 = __fmul2_rn(__fmul2_rn(bcast(b.z), dy), dy);
    d2 = make_float2(__fadd_rn(dxx, dyy.x), __fadd_rn(dxx, dyy.y));
    q = make_float2(__fadd_rn(__fadd_rn(t1, t2.x), t3.x), __fadd_rn(__fadd_rn(t1, t2.y), t3.y));
    ev = __fmul2_rn(q, bcast(-kHalfLog2e));
  }
  const float2 e = make_float2(ex2_approx(ev.x), ex2_approx(ev.y));
  const float2 am = __fmul2_rn(bcast(a.w), e);
  const float2 alpha = make_float2(fminf(0.99f, am.x), fminf(0.99f, am.y));
  ok0 = !(d2.x > a.z) && !(q.x < 0.0f) && !(alpha.x < 1.0f / 255.0f);
  ok1 = !(d2.y > a.z) && !(q.y < 0.0f) && !(alpha.y < 1.0f / 255.0f);
  return alpha;
}

__device__ __forceinline__ void blend_alpha2(Pixel2& p, const float4 c, float2 alpha, bool ok0,
                                             bool ok1) {
  const float2 al = make_float2(ok0 ? alpha.x : 0.0f, ok1 ? alpha.y : 0.0f);
  const float2 ta = __fmul2_rn(p.T, al);
  p.cr = __ffma2_rn(ta, bcast(c.x), p.cr);
  p.cg = __ffma2_rn(ta, bcast(c.y), p.cg);
  p.cb = __ffma2_rn(ta, bcast(c.z), p.cb);
  p.T = __fmul2_rn(p.T, __fadd2_rn(bcast(1.0f), make_float2(-al.x, -al.y)));
}

__device__ __forceinline__ void store_pixel(uint2* image, uint32_t W, uint32_t px, uint32_t py,
                                            const Pixel& p) {
  const __half2 rg = __floats2half2_rn(p.cr, p.cg);
  const __half2 ba = __floats2half2_rn(p.cb, 1.0f - p.T);
  image[(size_t)py * W + px] =
      make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&ba));
}

// Stages sorted splats [first, min(first + batch, end)) into dst; thread t
// copies entries t, t + nt, ... (one commit group per thread and batch).
__device__ __forceinline__ void stage_batch(const gs3d_projected_splat* __restrict__ proj,
                                            const uint32_t* __restrict__ values, uint32_t first,
                                            uint32_t end, uint32_t batch, uint32_t nt,
                                            SplatStage* dst) {
  for (uint32_t k = threadIdx.x; k < batch; k += nt) {
    const uint32_t idx = first + k;
    if (idx >= end) break;
    const uint32_t id = __ldg(values + idx);
    const float4* src = reinterpret_cast<const float4*>(proj + id);
    cp_async16(&dst[k].a, src + 0);
    cp_async16(&dst[k].b, src + 1);
    cp_async16(&dst[k].c, src + 2);
  }
  cp_async_commit();
}

// Can the splat reach alpha >= 1/255 inside the rectangle of pixel centres
// [x0,x1] x [y0,y1]?  Exact minimum of the splat's q over the rectangle (the
// quadratic form's minimum over a box not holding the mean lies on an edge,
// at the clamped stationary point of that edge; scale-invariant, so either
// form works), compared with vis; plus the radius circle.  Conservative by
// the margins folded into vis and the circle: vis is finite only for conics
// of condition number below about 10^3, where the rounding of q in any
// operation order stays far inside the 1% margin.  NaN means, radii, conics
// or opacities are never culled (the per-pixel tests decide, as in the
// reference).
__device__ __forceinline__ bool rect_may_hit(const SplatStage& s, float2 xr, float2 yr) {
  const float4 a = s.a, b = s.b;
  // the box corners relative to the mean (x - m computed as x + (-m))
  const float2 xd = __fadd2_rn(xr, bcast(-a.x)), yd = __fadd2_rn(yr, bcast(-a.y));
  const float x0 = xd.x, x1 = xd.y, y0 = yd.x, y1 = yd.y;
  const float ex = fminf(fmaxf(0.0f, x0), x1), ey = fminf(fmaxf(0.0f, y0), y1);
  if (ex * ex + ey * ey > a.z * 1.0001f + 1e-3f) return false;
  const float vis = b.w;
  if (vis < 0.0f) return false;
  if (ex == 0.0f && ey == 0.0f) return true;  // the mean lies inside
  if (vis == __int_as_float(0x7f800000)) return true;
  const float qa = b.x, qb = b.y, qc = b.z;
  // edge stationary points, by the fast reciprocal division: an error d in
  // the point raises q there by qa d^2 (qc d^2) over the edge minimum, far
  // inside the margins folded into vis
  const float sy = __fdividef(-qb, 2.0f * qc), sx = __fdividef(-qb, 2.0f * qa);
  // q = qa x^2 + qb x y + qc y^2 at the two vertical edges (x0, x1 at their
  // clamped stationary y) and the two horizontal ones, as pairs
  const float2 vx = xd, hy = yd;
  const float2 svy = __fmul2_rn(bcast(sy), vx), shx = __fmul2_rn(bcast(sx), hy);
  const float2 vy = make_float2(fminf(fmaxf(svy.x, y0), y1), fminf(fmaxf(svy.y, y0), y1));
  const float2 hx = make_float2(fminf(fmaxf(shx.x, x0), x1), fminf(fmaxf(shx.y, x0), x1));
  auto Q2 = [&](float2 x, float2 y) {
    return __ffma2_rn(__fmul2_rn(bcast(qa), x), x,
                      __ffma2_rn(__fmul2_rn(bcast(qb), x), y,
                                 __fmul2_rn(__fmul2_rn(bcast(qc), y), y)));
  };
  const float2 qv = Q2(vx, vy), qh = Q2(hx, hy);
  return fminf(fminf(qv.x, qv.y), fminf(qh.x, qh.y)) <= vis;
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
  const uint32_t nt = a.tile_w * a.tile_h;  // == blockDim.x
  const uint32_t D = a.batch ? a.batch : nt;  // splats per staged batch
  const uint32_t tid = threadIdx.x;
  const uint32_t px = g.ox + tid % a.tile_w;
  const uint32_t py = g.oy + tid / a.tile_w;
  const bool in_bounds = px < g.W && py < g.H;
  const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;

  const uint32_t start = __ldg(a.tile_offsets + g.tile);
  const uint32_t end = __ldg(a.tile_offsets + g.tile + 1);
  const uint32_t len = end > start ? end - start : 0u;
  const uint32_t nbatches = (len + D - 1) / D;

  Pixel p{0.f, 0.f, 0.f, 1.0f};
  bool done = !in_bounds;
  uint32_t used = 0;

  if (nbatches > 0) stage_batch(a.proj, a.values, start, end, D, nt, buf0);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage_batch(a.proj, a.values, start + (bi + 1) * D, end, D, nt, (bi & 1) ? buf0 : buf1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const uint32_t cnt = min(D, end - (start + bi * D));
    for (uint32_t k = tid; k < cnt; k += nt) prepare(cur[k]);  // own copies are complete
    __syncthreads();
    if (!done) {
      for (uint32_t j = 0; j < cnt; ++j) {
        if (blend_one<true>(pfx, pfy, cur[j], p, true)) {
          done = true;
          used = bi * D + j + 1;
          break;
        }
      }
      if (!done) used = bi * D + cnt;
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

// Culled variant: warps own compact pixel blocks and skip splats that no
// pixel of their block can blend.  blockDim.x == tile_w * tile_h, a multiple
// of 32.
// The tile's rows [row0, row0 + nthr / tile_w) are shaded by the CTA's nthr
// threads, one pixel each (the whole tile in the one-pixel kernel; half a
// row strip when the two-pixel kernel splits a heavy tile).
__device__ void raster_tile_culled(const RasterArgs& a, const TileGeom& g, uint32_t row0,
                                   uint32_t nthr, SplatStage* buf0, SplatStage* buf1,
                                   uint32_t* s_cost) {
  const uint32_t nt = a.tile_w * a.tile_h;
  const uint32_t D = a.batch ? a.batch : nt;  // splats per staged batch
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t lx, ly;
  if ((a.tile_w % 8 == 0) && ((nthr / a.tile_w) % 4 == 0)) {  // 8x4 pixel block per warp
    const uint32_t bw = a.tile_w / 8;
    lx = (warp % bw) * 8 + (lane & 7);
    ly = row0 + (warp / bw) * 4 + (lane >> 3);
  } else {
    lx = tid % a.tile_w;
    ly = row0 + tid / a.tile_w;
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
  const uint32_t nbatches = (len + D - 1) / D;

  Pixel p{0.f, 0.f, 0.f, 1.0f};
  bool done = !in_bounds;
  uint32_t used = 0;

  if (nbatches > 0) stage_batch(a.proj, a.values, start, end, D, nthr, buf0);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage_batch(a.proj, a.values, start + (bi + 1) * D, end, D, nthr, (bi & 1) ? buf0 : buf1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const uint32_t cnt = min(D, end - (start + bi * D));
    for (uint32_t k = tid; k < cnt; k += nthr) prepare(cur[k]);  // own copies are complete
    __syncthreads();
    if (__any_sync(0xffffffffu, !done)) {
      for (uint32_t k0 = 0; k0 < cnt; k0 += 32) {
        const uint32_t j = k0 + lane;
        const bool hit = j < cnt && rect_may_hit(cur[j], make_float2(xlo, xhi), make_float2(ylo, yhi));
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const uint32_t b0 = __ffs(mask) - 1;
          mask &= mask - 1;
          if (mask) {
            // two hits: both alphas first (independent work for the
            // scheduler), then the blends in order
            const uint32_t b1 = __ffs(mask) - 1;
            mask &= mask - 1;
            bool ok0, ok1;
            const float al0 = splat_alpha(pfx, pfy, cur[k0 + b0], ok0);
            const float al1 = splat_alpha(pfx, pfy, cur[k0 + b1], ok1);
            if (blend_alpha(p, cur[k0 + b0].c, al0, ok0 && !done)) {
              done = true;
              used = bi * D + k0 + b0 + 1;
            }
            if (blend_alpha(p, cur[k0 + b1].c, al1, ok1 && !done)) {
              done = true;
              used = bi * D + k0 + b1 + 1;
            }
          } else if (blend_one<false>(pfx, pfy, cur[k0 + b0], p, !done)) {
            done = true;
            used = bi * D + k0 + b0 + 1;
          }
        }
        if (__all_sync(0xffffffffu, done)) break;
      }
      if (!done) used = bi * D + cnt;
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

// Culled variant with two pixels a thread: each warp owns an 8x8 block,
// lane (x, y) shading rows y and y + 4, so a staged splat is loaded, culled
// and looped over once for 64 pixels.  blockDim.x == tile_w * tile_h / 2;
// tile sides divide by 8.  Per pixel the arithmetic and the splat sequence
// are those of the other variants (bit-identical image).
__device__ void raster_tile_culled2(const RasterArgs& a, const TileGeom& g, uint32_t strip,
                                    SplatStage* buf0, SplatStage* buf1, uint32_t* s_cost) {
  const uint32_t nt = a.tile_w * a.tile_h;
  const uint32_t strip_h = a.tile_h / a.split;  // this CTA shades rows [strip * strip_h, +strip_h)
  const uint32_t nthr = a.tile_w * strip_h / 2;
  const uint32_t D = a.batch ? a.batch : nt;  // splats per staged batch
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t bw = a.tile_w / 8;
  const uint32_t px = g.ox + (warp % bw) * 8 + (lane & 7);
  const uint32_t py0 = g.oy + strip * strip_h + (warp / bw) * 8 + (lane >> 3), py1 = py0 + 4;
  const bool in0 = px < g.W && py0 < g.H, in1 = px < g.W && py1 < g.H;
  const float pfx = (float)px + 0.5f, pfy0 = (float)py0 + 0.5f, pfy1 = (float)py1 + 0.5f;
  float xlo = pfx, xhi = pfx, ylo = pfy0, yhi = pfy1;
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
  const uint32_t nbatches = (len + D - 1) / D;

  const float2 pfy = make_float2(pfy0, pfy1);
  Pixel2 p{bcast(0.f), bcast(0.f), bcast(0.f), bcast(1.0f)};
  bool done0 = !in0, done1 = !in1;
  uint32_t used0 = 0, used1 = 0;

  if (nbatches > 0) stage_batch(a.proj, a.values, start, end, D, nthr, buf0);
  for (uint32_t bi = 0; bi < nbatches; ++bi) {
    SplatStage* cur = (bi & 1) ? buf1 : buf0;
    if (bi + 1 < nbatches) {
      stage_batch(a.proj, a.values, start + (bi + 1) * D, end, D, nthr, (bi & 1) ? buf0 : buf1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const uint32_t cnt = min(D, end - (start + bi * D));
    for (uint32_t k = tid; k < cnt; k += nthr) prepare(cur[k]);  // own copies are complete
    __syncthreads();
    if (__any_sync(0xffffffffu, !(done0 && done1))) {
      for (uint32_t k0 = 0; k0 < cnt; k0 += 32) {
        const uint32_t j = k0 + lane;
        const bool hit = j < cnt && rect_may_hit(cur[j], make_float2(xlo, xhi), make_float2(ylo, yhi));
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
          const uint32_t b = __ffs(mask) - 1;
          mask &= mask - 1;
          const SplatStage& sp = cur[k0 + b];
          bool ok0, ok1;
          const float2 al = splat_alpha2(pfx, pfy, sp, ok0, ok1);
          ok0 = ok0 && !done0;
          ok1 = ok1 && !done1;
          blend_alpha2(p, sp.c, al, ok0, ok1);
          if (ok0 && p.T.x < 1.0e-4f) {
            done0 = true;
            used0 = bi * D + k0 + b + 1;
          }
          if (ok1 && p.T.y < 1.0e-4f) {
            done1 = true;
            used1 = bi * D + k0 + b + 1;
          }
        }
        if (__all_sync(0xffffffffu, done0 && done1)) break;
      }
      if (!done0) used0 = bi * D + cnt;
      if (!done1) used1 = bi * D + cnt;
    }
    if (__syncthreads_and(done0 && done1)) {
      cp_async_wait<0>();
      break;
    }
  }
  if (in0) {
    atomicMax(s_cost, used0);
    store_pixel(g.image, g.W, px, py0, Pixel{p.cr.x, p.cg.x, p.cb.x, p.T.x});
  }
  if (in1) {
    atomicMax(s_cost, used1);
    store_pixel(g.image, g.W, px, py1, Pixel{p.cr.y, p.cg.y, p.cb.y, p.T.y});
  }
}

// Persistent CTAs pull tile indices from the work queue.
// Persistent CTAs over the queue; MODE 0: one thread per pixel, linear;
// 1: culled, 8x4 warp blocks; 2: culled, two pixels a thread, 8x8 blocks.
template <int MODE>
__device__ __forceinline__ void raster_loop(const RasterArgs& a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t D = a.batch ? a.batch : a.tile_w * a.tile_h;
  SplatStage* buf0 = reinterpret_cast<SplatStage*>(smem);
  SplatStage* buf1 = buf0 + D;
  __shared__ uint32_t s_item, s_cost;
  // work items: the first `heavy` tiles of the order as two half-strip items
  // per strip, then one item per strip of the others
  const uint32_t heavy = (MODE == 2 && a.heavy != nullptr) ? min(__ldg(a.heavy), a.num_tiles) : 0u;
  const uint32_t heavy_items = 2u * a.split * heavy;
  const uint32_t items = heavy_items + (a.num_tiles - heavy) * a.split;
  while (true) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(a.queue_counter, 1u);
      s_cost = 0u;
    }
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= items) break;
    uint32_t ti, strip, half;  // half: 0 whole strip, 1 / 2 first / second half
    if (item < heavy_items) {
      ti = item / (2u * a.split);
      const uint32_t sub = item - ti * 2u * a.split;
      strip = sub >> 1;
      half = 1u + (sub & 1u);
    } else {
      const uint32_t j = item - heavy_items;
      ti = heavy + j / a.split;
      strip = j - (ti - heavy) * a.split;
      half = 0u;
    }
    const uint32_t t = a.order != nullptr ? __ldg(a.order + ti) : ti;
    const TileGeom g = tile_geom(a, t);
    if (MODE == 2) {
      if (half == 0u) {
        raster_tile_culled2(a, g, strip, buf0, buf1, &s_cost);
      } else {  // half a row strip, one pixel a thread (the same per-pixel arithmetic)
        const uint32_t strip_h = a.tile_h / a.split;
        raster_tile_culled(a, g, strip * strip_h + (half - 1u) * (strip_h / 2), blockDim.x, buf0,
                           buf1, &s_cost);
      }
    } else if (MODE == 1) {
      raster_tile_culled(a, g, 0u, a.tile_w * a.tile_h, buf0, buf1, &s_cost);
    } else {
      raster_tile_plain(a, g, buf0, buf1, &s_cost);
    }
    __syncthreads();  // s_cost complete; shared buffers free for the next tile
    if (threadIdx.x == 0 && a.tile_costs != nullptr)
      atomicMax(a.tile_costs + t, s_cost);  // zeroed before the launch; max over a tile's items
  }
}

__global__ void raster_kernel_plain(RasterArgs a) { raster_loop<0>(a); }
__global__ void raster_kernel_culled(RasterArgs a) { raster_loop<1>(a); }
// at most 512 threads (a 1024-pixel tile of unsplittable strips)
__global__ void __launch_bounds__(512, 2) raster_kernel_culled2(RasterArgs a) {
  raster_loop<2>(a);
}

// Variant, strips, block size, staged batch and resident CTAs per SM of the
// raster launch for `a` (the occupancy is computed once per device and shape).
struct RasterConfig {
  int mode;
  uint32_t split, threads, D;
  int per_sm;
  void (*kern)(RasterArgs);
};

cudaError_t raster_config(const RasterArgs& a, RasterConfig* cfg) {
  const uint32_t nt = a.tile_w * a.tile_h;
  if (a.batch % 32 != 0 || a.batch > 1024) return cudaErrorInvalidValue;
  const uint32_t D = a.batch ? a.batch : nt;
  const bool culled = a.culled && (nt % 32 == 0);
  // two pixels a thread where the tile splits into 8x8 blocks
  const int mode = !culled ? 0 : (a.tile_w % 8 == 0 && a.tile_h % 8 == 0) ? 2 : 1;
  // two-pixel tiles of more than 512 pixels are shaded by four (else two)
  // CTAs of row strips whose heights divide by 8, so that a block barrier
  // waits for few warps and more CTAs interleave on an SM
  uint32_t split = 1;
  if (mode == 2 && nt > 512) split = (a.tile_h / 4) % 8 == 0 ? 4u : (a.tile_h / 2) % 8 == 0 ? 2u : 1u;
  const uint32_t threads = mode == 2 ? nt / (2 * split) : nt;
  // one thread a pixel up to 1024 pixels; two-pixel strips of at most 512
  // threads (the kernel's launch bound)
  if ((mode != 2 && nt > 1024) || (mode == 2 && threads > 512)) return cudaErrorInvalidValue;
  const size_t smem = 2 * (size_t)D * sizeof(SplatStage);
  auto kern = mode == 2 ? raster_kernel_culled2 : mode == 1 ? raster_kernel_culled
                                                             : raster_kernel_plain;
  // launch configuration per (device, variant, tile area, batch), computed
  // once per process (the shared-memory attribute is a per-device setting)
  static std::mutex mu;
  static std::map<uint64_t, int> cache;
  int dev = 0;
  {
    const cudaError_t e = current_device(&dev);
    if (e != cudaSuccess) return e;
  }
  const uint64_t key = ((uint64_t)dev << 48) | ((uint64_t)mode << 40) |
                       ((uint64_t)threads << 20) | D;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) per_sm = it->second;
  }
  if (per_sm == 0) {
    // one attribute per kernel, set to the largest batch's footprint so that
    // configurations cached earlier keep fitting
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * 1024 * sizeof(SplatStage)));
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, (int)threads, smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(n, 1);
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = per_sm;
  }
  *cfg = RasterConfig{mode, split, threads, D, per_sm, kern};
  return cudaSuccess;
}

}  // namespace

cudaError_t raster_shape(const RasterArgs& a, int sm_count, uint32_t* strips,
                         uint32_t* resident_ctas) {
  RasterConfig cfg;
  const cudaError_t e = raster_config(a, &cfg);
  if (e != cudaSuccess) return e;
  *strips = cfg.split;
  *resident_ctas = (uint32_t)sm_count * (uint32_t)cfg.per_sm;
  return cudaSuccess;
}

cudaError_t launch_raster(const RasterArgs& args, int sm_count, cudaStream_t s) {
  if (args.num_tiles == 0) return cudaSuccess;
  RasterArgs a = args;
  RasterConfig cfg;
  cudaError_t e = raster_config(a, &cfg);
  if (e != cudaSuccess) return e;
  a.split = cfg.split;
  if (cfg.mode != 2) a.heavy = nullptr;  // half strips exist in the two-pixel variant only
  // every work item folds its cost into its tile's by maximum
  if (a.tile_costs != nullptr) {
    e = cudaMemsetAsync(a.tile_costs, 0, (size_t)a.num_tiles * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
  }
  // up to two items per strip when tiles are split
  const uint64_t max_items = (uint64_t)a.num_tiles * a.split * (a.heavy != nullptr ? 2 : 1);
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      max_items, (uint64_t)sm_count * (uint64_t)std::max(cfg.per_sm, 1));
  cfg.kern<<<grid, cfg.threads, 2 * (size_t)cfg.D * sizeof(SplatStage), s>>>(a);
  return cudaGetLastError();
}

}  // namespace gs3d
