// learned.cu - learned raster schedule: per-tile features, a 16-64-64-1 cost
// MLP (warp-level bf16 mma inference, fp32 training kernels) and the work
// order it produces.
//
// The raster's cost per tile is the number of splats its CTA iterates before
// the tile's last pixel terminates (recorded in tile_costs).  The key count
// is a poor proxy for it in dense, opaque regions where pixels terminate
// early.  The MLP predicts log(1 + cost) from 16 features; the persistent
// raster CTAs then take tiles in decreasing predicted cost.  The schedule
// only changes which CTA renders a tile and when, never a pixel's arithmetic.
//
// Parameter vector (f32, kMlpParams entries):
//   W1[64][16] | b1[64] | W2[64][64] | b2[64] | w3[64] | b3
// Features (kFeatures = 16), computed from the tile's key count, its
// neighbours' key counts and its first kSample sorted splats:
//   0 key count / 1000        1 log(1 + key count)     2 mean opacity
//   3 max opacity             4 min depth              5 max depth
//   6 mean depth              7 depth std              8 mean log conic det
//   9 mean radius / tile size 10 tile x / tiles x      11 tile y / tiles y
//   12 coverage sum (sum of min(1, pi r^2 / tile area), scaled to the key
//      count)                 13-15 log(1 + key count) of the left, right
//      and upper neighbour tiles.
#include <cuda_bf16.h>

#include <algorithm>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kSample = 64;  // sorted splats per tile read for the features

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ float warp_max(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ float warp_min(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

__device__ __forceinline__ uint32_t tile_keys(const uint32_t* off, uint32_t t) {
  const uint32_t lo = __ldg(off + t), hi = __ldg(off + t + 1);
  return hi > lo ? hi - lo : 0u;
}

// One warp per tile; writes raw features, or normalized ones when mean/std
// are given.
__global__ void __launch_bounds__(256)
    tile_features_kernel(const ViewDesc* __restrict__ views, uint32_t n_views, uint32_t num_tiles,
                         uint32_t tile_w, uint32_t tile_h,
                         const uint32_t* __restrict__ tile_offsets,
                         const uint32_t* __restrict__ values,
                         const gs3d_projected_splat* __restrict__ proj,
                         const float* __restrict__ mean, const float* __restrict__ inv_std,
                         float* __restrict__ out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= num_tiles) return;
  const uint32_t v =
      find_view(n_views, t, [&](uint32_t k) { return __ldg(&views[k].f.tile_base); });
  const uint32_t base = __ldg(&views[v].f.tile_base);
  const uint32_t tx_count = __ldg(&views[v].f.tile_count[0]);
  const uint32_t ty_count = __ldg(&views[v].f.tile_count[1]);
  const uint32_t lt = t - base, tx = lt % tx_count, ty = lt / tx_count;
  const uint32_t start = __ldg(tile_offsets + t);
  const uint32_t n = tile_keys(tile_offsets, t);
  const uint32_t m = min(n, (uint32_t)kSample);
  const float area = (float)(tile_w * tile_h);

  float s_op = 0.f, mx_op = 0.f, mn_d = 3.0e38f, mx_d = 0.f, s_d = 0.f, s_d2 = 0.f;
  float s_det = 0.f, s_r = 0.f, s_cov = 0.f;
  for (uint32_t j = lane; j < m; j += 32) {
    const uint32_t id = __ldg(values + start + j);
    const float4 r0 = __ldg(reinterpret_cast<const float4*>(proj + id));      // mean, depth, r
    const float4 r1 = __ldg(reinterpret_cast<const float4*>(proj + id) + 1);  // conic, opacity
    const float d = -r0.z;
    s_op += r1.w;
    mx_op = fmaxf(mx_op, r1.w);
    mn_d = fminf(mn_d, d);
    mx_d = fmaxf(mx_d, d);
    s_d += d;
    s_d2 += d * d;
    s_det += __logf(fmaxf(r1.x * r1.z - r1.y * r1.y, 1e-30f));
    s_r += r0.w;
    s_cov += fminf(1.0f, 3.14159265f * r0.w * r0.w / area);
  }
  s_op = warp_sum(s_op);
  mx_op = warp_max(mx_op);
  mn_d = warp_min(mn_d);
  mx_d = warp_max(mx_d);
  s_d = warp_sum(s_d);
  s_d2 = warp_sum(s_d2);
  s_det = warp_sum(s_det);
  s_r = warp_sum(s_r);
  s_cov = warp_sum(s_cov);
  if (lane != 0) return;
  const float inv_m = m > 0 ? 1.0f / (float)m : 0.0f;
  const float md = s_d * inv_m;
  float f[kFeatures];
  f[0] = (float)n * 1e-3f;
  f[1] = __logf(1.0f + (float)n);
  f[2] = s_op * inv_m;
  f[3] = mx_op;
  f[4] = m > 0 ? mn_d : 0.0f;
  f[5] = mx_d;
  f[6] = md;
  f[7] = sqrtf(fmaxf(0.0f, s_d2 * inv_m - md * md));
  f[8] = s_det * inv_m;
  f[9] = s_r * inv_m / (float)tile_w;
  f[10] = ((float)tx + 0.5f) / (float)tx_count;
  f[11] = ((float)ty + 0.5f) / (float)ty_count;
  f[12] = s_cov * inv_m * (float)n * 1e-3f;
  f[13] = tx > 0 ? __logf(1.0f + (float)tile_keys(tile_offsets, t - 1)) : 0.0f;
  f[14] = tx + 1 < tx_count ? __logf(1.0f + (float)tile_keys(tile_offsets, t + 1)) : 0.0f;
  f[15] = ty > 0 ? __logf(1.0f + (float)tile_keys(tile_offsets, t - tx_count)) : 0.0f;
  float* o = out + (size_t)t * kFeatures;
#pragma unroll
  for (int k = 0; k < kFeatures; ++k) o[k] = mean ? (f[k] - mean[k]) * inv_std[k] : f[k];
}

// ---- inference: one warp per 16 tiles, mma.sync m16n8k16 bf16 -> f32 ----

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// D[16x8] += A[16x16] (row) * B[16x8] (col), bf16 inputs, f32 accumulators.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Weights in shared memory as bf16: W1 [64 out][16 in], W2 [64 out][64 in];
// biases and w3 in f32.  The weight matrices are the B operands ("col"
// layout = B[k][n] with n the output unit, read as W[n][k]).
struct MlpSmem {
  __nv_bfloat16 w1[kHidden][kFeatures];
  __nv_bfloat16 w2[kHidden][kHidden];
  float b1[kHidden], b2[kHidden], w3[kHidden];
  float b3;
  float h1[8][16][kHidden + 8];  // per warp, padded rows
};

__global__ void __launch_bounds__(256)
    mlp_infer_kernel(const float* __restrict__ params, const float* __restrict__ x,
                     uint32_t n, float* __restrict__ y) {
  __shared__ MlpSmem sm;
  const float* W1 = params;
  const float* B1 = W1 + kHidden * kFeatures;
  const float* W2 = B1 + kHidden;
  const float* B2 = W2 + kHidden * kHidden;
  const float* W3 = B2 + kHidden;
  const float* B3 = W3 + kHidden;
  for (int i = threadIdx.x; i < kHidden * kFeatures; i += blockDim.x)
    (&sm.w1[0][0])[i] = __float2bfloat16_rn(__ldg(W1 + i));
  for (int i = threadIdx.x; i < kHidden * kHidden; i += blockDim.x)
    (&sm.w2[0][0])[i] = __float2bfloat16_rn(__ldg(W2 + i));
  for (int i = threadIdx.x; i < kHidden; i += blockDim.x) {
    sm.b1[i] = __ldg(B1 + i);
    sm.b2[i] = __ldg(B2 + i);
    sm.w3[i] = __ldg(W3 + i);
  }
  if (threadIdx.x == 0) sm.b3 = __ldg(B3);
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;  // mma fragment coordinates
  const uint32_t row0 = (blockIdx.x * 8 + warp) * 16;
  if (row0 >= n) return;
  auto xin = [&](uint32_t r, int c) -> float {
    return r < n ? __ldg(x + (size_t)r * kFeatures + c) : 0.0f;
  };
  // A fragment of X (16 tiles x 16 features)
  uint32_t a[4];
  a[0] = pack_bf16(xin(row0 + g, 2 * q), xin(row0 + g, 2 * q + 1));
  a[1] = pack_bf16(xin(row0 + g + 8, 2 * q), xin(row0 + g + 8, 2 * q + 1));
  a[2] = pack_bf16(xin(row0 + g, 2 * q + 8), xin(row0 + g, 2 * q + 9));
  a[3] = pack_bf16(xin(row0 + g + 8, 2 * q + 8), xin(row0 + g + 8, 2 * q + 9));
  // layer 1: 8 n-tiles of 8 hidden units
  float (*h1)[kHidden + 8] = sm.h1[warp];
#pragma unroll
  for (int nt = 0; nt < kHidden / 8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int col = nt * 8 + g;  // output unit held by this lane's B fragment
    uint32_t b[2];
    b[0] = *reinterpret_cast<const uint32_t*>(&sm.w1[col][2 * q]);
    b[1] = *reinterpret_cast<const uint32_t*>(&sm.w1[col][2 * q + 8]);
    mma_bf16(d, a, b);
    const int c0 = nt * 8 + 2 * q;
    h1[g][c0] = fmaxf(0.f, d[0] + sm.b1[c0]);
    h1[g][c0 + 1] = fmaxf(0.f, d[1] + sm.b1[c0 + 1]);
    h1[g + 8][c0] = fmaxf(0.f, d[2] + sm.b1[c0]);
    h1[g + 8][c0 + 1] = fmaxf(0.f, d[3] + sm.b1[c0 + 1]);
  }
  __syncwarp();
  // layer 2: K = 64 in 4 steps, 8 n-tiles; layer 3 folded into the epilogue
  float out_lo = 0.f, out_hi = 0.f;  // rows g and g + 8
#pragma unroll
  for (int nt = 0; nt < kHidden / 8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int col = nt * 8 + g;
#pragma unroll
    for (int ks = 0; ks < kHidden / 16; ++ks) {
      const int k0 = ks * 16;
      uint32_t a2[4];
      a2[0] = pack_bf16(h1[g][k0 + 2 * q], h1[g][k0 + 2 * q + 1]);
      a2[1] = pack_bf16(h1[g + 8][k0 + 2 * q], h1[g + 8][k0 + 2 * q + 1]);
      a2[2] = pack_bf16(h1[g][k0 + 2 * q + 8], h1[g][k0 + 2 * q + 9]);
      a2[3] = pack_bf16(h1[g + 8][k0 + 2 * q + 8], h1[g + 8][k0 + 2 * q + 9]);
      uint32_t b[2];
      b[0] = *reinterpret_cast<const uint32_t*>(&sm.w2[col][k0 + 2 * q]);
      b[1] = *reinterpret_cast<const uint32_t*>(&sm.w2[col][k0 + 2 * q + 8]);
      mma_bf16(d, a2, b);
    }
    const int c0 = nt * 8 + 2 * q;
    out_lo += fmaxf(0.f, d[0] + sm.b2[c0]) * sm.w3[c0] + fmaxf(0.f, d[1] + sm.b2[c0 + 1]) * sm.w3[c0 + 1];
    out_hi += fmaxf(0.f, d[2] + sm.b2[c0]) * sm.w3[c0] + fmaxf(0.f, d[3] + sm.b2[c0 + 1]) * sm.w3[c0 + 1];
  }
  // the 4 lanes of a quad hold partial sums of the same two rows
  out_lo += __shfl_xor_sync(0xffffffffu, out_lo, 1);
  out_lo += __shfl_xor_sync(0xffffffffu, out_lo, 2);
  out_hi += __shfl_xor_sync(0xffffffffu, out_hi, 1);
  out_hi += __shfl_xor_sync(0xffffffffu, out_hi, 2);
  if (q == 0) {
    if (row0 + g < n) y[row0 + g] = out_lo + sm.b3;
    if (row0 + g + 8 < n) y[row0 + g + 8] = out_hi + sm.b3;
  }
}

// ---- training (f32): forward keeps activations, backward accumulates ----

// One block of kHidden threads per chunk of samples; thread j owns hidden
// unit j of both layers.  acts[i] = h1 (64) | h2 (64) | y.
__global__ void __launch_bounds__(kHidden)
    mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ x, uint32_t n,
                       float* __restrict__ acts, float* __restrict__ y) {
  const float* W1 = params;
  const float* B1 = W1 + kHidden * kFeatures;
  const float* W2 = B1 + kHidden;
  const float* B2 = W2 + kHidden * kHidden;
  const float* W3 = B2 + kHidden;
  const float* B3 = W3 + kHidden;
  __shared__ float s_x[kFeatures], s_h1[kHidden], s_part[kHidden / 32];
  const int j = threadIdx.x;
  float w1[kFeatures];
#pragma unroll
  for (int k = 0; k < kFeatures; ++k) w1[k] = __ldg(W1 + j * kFeatures + k);
  const float b1 = __ldg(B1 + j), b2 = __ldg(B2 + j), w3 = __ldg(W3 + j), b3 = __ldg(B3);
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    if (j < kFeatures) s_x[j] = __ldg(x + (size_t)i * kFeatures + j);
    __syncthreads();
    float h = b1;
#pragma unroll
    for (int k = 0; k < kFeatures; ++k) h = fmaf(w1[k], s_x[k], h);
    h = fmaxf(0.f, h);
    s_h1[j] = h;
    __syncthreads();
    float h2 = b2;
    for (int k = 0; k < kHidden; ++k) h2 = fmaf(__ldg(W2 + j * kHidden + k), s_h1[k], h2);
    h2 = fmaxf(0.f, h2);
    float* a = acts + (size_t)i * (2 * kHidden + 1);
    a[j] = h;
    a[kHidden + j] = h2;
    const float p = warp_sum(w3 * h2);
    if ((j & 31) == 0) s_part[j >> 5] = p;
    __syncthreads();
    if (j == 0) {
      float out = b3;
      for (int w = 0; w < kHidden / 32; ++w) out += s_part[w];
      a[2 * kHidden] = out;
      y[i] = out;
    }
    __syncthreads();
  }
}

// Gradient of the mean squared error (y - target)^2 over n samples, added
// into grads (same layout as params; must be zeroed by the caller).
__global__ void __launch_bounds__(kHidden)
    mlp_backward_kernel(const float* __restrict__ params, const float* __restrict__ x,
                        const float* __restrict__ acts, const float* __restrict__ target,
                        uint32_t n, float* __restrict__ grads) {
  const float* W2 = params + kHidden * kFeatures + kHidden;
  const float* W3 = W2 + kHidden * kHidden + kHidden;
  float* gW1 = grads;
  float* gB1 = gW1 + kHidden * kFeatures;
  float* gW2 = gB1 + kHidden;
  float* gB2 = gW2 + kHidden * kHidden;
  float* gW3 = gB2 + kHidden;
  float* gB3 = gW3 + kHidden;
  __shared__ float s_x[kFeatures], s_h1[kHidden], s_dh2[kHidden];
  const int j = threadIdx.x;
  float w2col[kHidden];  // W2[i][j] for all i: this thread's column
#pragma unroll
  for (int i = 0; i < kHidden; ++i) w2col[i] = __ldg(W2 + i * kHidden + j);
  const float w3 = __ldg(W3 + j);
  float acc_w1[kFeatures], acc_w2[kHidden];
#pragma unroll
  for (int k = 0; k < kFeatures; ++k) acc_w1[k] = 0.f;
#pragma unroll
  for (int k = 0; k < kHidden; ++k) acc_w2[k] = 0.f;
  float acc_b1 = 0.f, acc_b2 = 0.f, acc_w3 = 0.f, acc_b3 = 0.f;
  const float scale = 2.0f / (float)n;
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const float* a = acts + (size_t)i * (2 * kHidden + 1);
    if (j < kFeatures) s_x[j] = __ldg(x + (size_t)i * kFeatures + j);
    const float h1 = a[j], h2 = a[kHidden + j];
    s_h1[j] = h1;
    const float dy = scale * (a[2 * kHidden] - __ldg(target + i));
    const float dh2 = h2 > 0.f ? dy * w3 : 0.f;
    s_dh2[j] = dh2;
    __syncthreads();
    acc_w3 += dy * h2;
    acc_b3 += dy;
    acc_b2 += dh2;
#pragma unroll
    for (int k = 0; k < kHidden; ++k) acc_w2[k] = fmaf(dh2, s_h1[k], acc_w2[k]);
    float dh1 = 0.f;
#pragma unroll
    for (int r = 0; r < kHidden; ++r) dh1 = fmaf(w2col[r], s_dh2[r], dh1);
    dh1 = h1 > 0.f ? dh1 : 0.f;
    acc_b1 += dh1;
#pragma unroll
    for (int k = 0; k < kFeatures; ++k) acc_w1[k] = fmaf(dh1, s_x[k], acc_w1[k]);
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < kFeatures; ++k) atomicAdd(gW1 + j * kFeatures + k, acc_w1[k]);
  atomicAdd(gB1 + j, acc_b1);
#pragma unroll
  for (int k = 0; k < kHidden; ++k) atomicAdd(gW2 + j * kHidden + k, acc_w2[k]);
  atomicAdd(gB2 + j, acc_b2);
  atomicAdd(gW3 + j, acc_w3);
  if (j == 0) atomicAdd(gB3, acc_b3);
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, uint32_t count, float lr, float beta1,
                            float beta2, float eps, float c1, float c2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
  const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void log_costs_kernel(const uint32_t* __restrict__ costs, uint32_t n,
                                 float* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = log1pf((float)costs[t]);
}

// Schedule keys: larger expected cost first.  While the gate accepts the
// model the expected cost is its prediction, else the key count (the
// key-count schedule's keys).
__global__ void learned_keys_kernel(const float* __restrict__ pred, uint32_t n,
                                    const SchedGate* __restrict__ gate,
                                    const uint32_t* __restrict__ tile_offsets,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ ids,
                                    float* __restrict__ est) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  if (gate->use_learned) {
    // pred = log(1 + cost); 4096 steps per unit of log cost, 16-bit key
    const float c = fminf(fmaxf(pred[t], 0.0f), 15.99f);
    keys[t] = 0xffffu - (uint32_t)(c * 4096.0f);
    est[t] = expm1f(c);
  } else {
    const uint32_t lo = __ldg(tile_offsets + t), hi = __ldg(tile_offsets + t + 1);
    const uint32_t k = hi > lo ? hi - lo : 0u;
    keys[t] = 0xffffu - min(k, 0xffffu);
    est[t] = (float)k;
  }
  ids[t] = t;
}

// One block: the frame's mean |pred - log(1 + cost)| over all tiles (fixed
// reduction order), folded into the running error (weight 1/4 per frame,
// the first frame taken as is); the learned order stays in use while the
// running error is within the bound.
constexpr int kGateThreads = 1024;
__global__ void __launch_bounds__(kGateThreads)
    gate_update_kernel(const float* __restrict__ pred, const uint32_t* __restrict__ costs,
                       uint32_t n, SchedGate* __restrict__ gate) {
  __shared__ float s_sum[kGateThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float sum = 0.0f;
  for (uint32_t t = threadIdx.x; t < n; t += kGateThreads)
    sum += fabsf(pred[t] - log1pf((float)costs[t]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) s_sum[warp] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float total = 0.0f;
    for (int w = 0; w < kGateThreads / 32; ++w) total += s_sum[w];
    const float mae = n ? total / (float)n : 0.0f;
    SchedGate g = *gate;
    g.last_mae = mae;
    g.mae = g.frames == 0 ? mae : 0.75f * g.mae + 0.25f * mae;
    g.frames += 1;
    g.used_learned = g.use_learned;
    if (!g.use_learned) g.fallbacks += 1;
    g.use_learned = g.mae <= g.bound ? 1u : 0u;
    *gate = g;
  }
}

}  // namespace

cudaError_t launch_tile_features(const ViewDesc* views, uint32_t n_views, uint32_t num_tiles,
                                 uint32_t tile_w, uint32_t tile_h, const uint32_t* tile_offsets,
                                 const uint32_t* values, const gs3d_projected_splat* proj,
                                 const float* mean, const float* inv_std, float* out,
                                 cudaStream_t s) {
  if (num_tiles == 0) return cudaSuccess;
  const uint32_t blocks = (uint32_t)(((uint64_t)num_tiles * 32 + 255) / 256);
  tile_features_kernel<<<blocks, 256, 0, s>>>(views, n_views, num_tiles, tile_w, tile_h,
                                              tile_offsets, values, proj, mean, inv_std, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const float* params, const float* x, uint32_t n, float* y,
                             cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  mlp_infer_kernel<<<(n + 127) / 128, 256, 0, s>>>(params, x, n, y);
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const float* params, const float* x, uint32_t n, float* acts,
                               float* y, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  mlp_forward_kernel<<<std::min<uint32_t>(n, 2048), kHidden, 0, s>>>(params, x, n, acts, y);
  return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const float* params, const float* x, const float* acts,
                                const float* target, uint32_t n, float* grads, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  mlp_backward_kernel<<<std::min<uint32_t>(n, 1024), kHidden, 0, s>>>(params, x, acts, target, n,
                                                                      grads);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* p, float* m, float* v, const float* g, uint32_t count, float lr,
                        float beta1, float beta2, float eps, uint32_t step, cudaStream_t s) {
  const float c1 = 1.0f - powf(beta1, (float)step);
  const float c2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<(count + 255) / 256, 256, 0, s>>>(p, m, v, g, count, lr, beta1, beta2, eps, c1,
                                                  c2);
  return cudaGetLastError();
}

cudaError_t launch_log_costs(const uint32_t* costs, uint32_t n, float* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  log_costs_kernel<<<(n + 255) / 256, 256, 0, s>>>(costs, n, out);
  return cudaGetLastError();
}

cudaError_t launch_learned_keys(const float* pred, uint32_t n, const SchedGate* gate,
                                const uint32_t* tile_offsets, uint32_t* keys, uint32_t* ids,
                                float* est, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  learned_keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(pred, n, gate, tile_offsets, keys, ids,
                                                       est);
  return cudaGetLastError();
}

cudaError_t launch_gate_update(const float* pred, const uint32_t* costs, uint32_t n,
                               SchedGate* gate, cudaStream_t s) {
  gate_update_kernel<<<1, kGateThreads, 0, s>>>(pred, costs, n, gate);
  return cudaGetLastError();
}

}  // namespace gs3d
