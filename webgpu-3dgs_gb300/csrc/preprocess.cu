// preprocess.cu - stage 1 of the rebin: EWA projection of every splat.
//
// Follows src/shaders/compute/preprocess_splats.wgsl:76-184.  One thread per
// splat of a scene; the four vec4 splat arrays are read with 128-bit
// coalesced loads and the per-block slice of the SH coefficients (extension,
// SH degree 1..3) is staged into shared memory by one bulk (TMA) copy
// completing on an mbarrier.  In a batch every view of the same scene is
// projected by the same thread, so the splat data leaves HBM once per batch,
// not once per view.
//
// Numerics: this translation unit is compiled with -fmad=false and IEEE
// division / square root, and every expression below is written in the same
// operation order as the CPU oracle (left-to-right sums, zero terms kept), so
// projected means, conics, radii and tile rectangles match it bit for bit.
#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

constexpr int kThreads = 256;

__constant__ float kShC1 = 0.4886025119029199f;
__constant__ float kShC2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                               -1.0925484305920792f, 0.5462742152960396f};
__constant__ float kShC3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                               0.3731763325901154f,  -0.4570457994644658f, 1.445305721320277f,
                               -0.5900435899266435f};

// Colour extension: clamp01(base + sum_k Y_k(dir) * rest[c*K + k-1]), with
// dir = normalize(position - camera position), K = (DEG+1)^2 - 1 and the
// rest coefficients in PLY f_rest order (channel-major); the sum runs
// k = 1..K, each term added by one explicit fused multiply-add (the oracle
// uses std::fma in the same order).
template <int DEG>
__device__ __forceinline__ void sh_color(float px, float py, float pz, const float* campos,
                                         float4 base, const float* rest, float* out) {
  constexpr int K = (DEG + 1) * (DEG + 1) - 1;
  const float dx = px - campos[0];
  const float dy = py - campos[1];
  const float dz = pz - campos[2];
  const float len = sqrtf(dx * dx + dy * dy + dz * dz);
  float x = 0.0f, y = 0.0f, z = 0.0f;
  if (len > 0.0f) {
    x = dx / len;
    y = dy / len;
    z = dz / len;
  }
  float b[16];
  b[1] = -kShC1 * y;
  b[2] = kShC1 * z;
  b[3] = -kShC1 * x;
  if (DEG > 1) {
    const float xx = x * x, yy = y * y, zz = z * z;
    const float xy = x * y, yz = y * z, xz = x * z;
    b[4] = kShC2[0] * xy;
    b[5] = kShC2[1] * yz;
    b[6] = kShC2[2] * (2.0f * zz - xx - yy);
    b[7] = kShC2[3] * xz;
    b[8] = kShC2[4] * (xx - yy);
    if (DEG > 2) {
      b[9] = kShC3[0] * y * (3.0f * xx - yy);
      b[10] = kShC3[1] * xy * z;
      b[11] = kShC3[2] * y * (4.0f * zz - xx - yy);
      b[12] = kShC3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
      b[13] = kShC3[4] * x * (4.0f * zz - xx - yy);
      b[14] = kShC3[5] * z * (xx - yy);
      b[15] = kShC3[6] * x * (xx - 3.0f * yy);
    }
  }
  const float base_c[3] = {base.x, base.y, base.z};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float acc = base_c[c];
#pragma unroll
    for (int k = 1; k <= K; ++k) acc = __fmaf_rn(b[k], rest[c * K + (k - 1)], acc);
    out[c] = fminf(1.0f, fmaxf(0.0f, acc));
  }
}

// preprocess_splats.wgsl:76-184 for the block's 256 splats of one scene, for
// every view of the batch that renders the scene (the chain leader ->
// group_next): the splat arrays, the SH slice and the 3D covariance are read
// and built once, the projection runs per view.
template <int DEG>
__device__ __forceinline__ void preprocess_block(const ViewDesc* __restrict__ views,
                                                 uint32_t leader, uint32_t local_first,
                                                 float* s_sh, uint64_t* s_bar,
                                                 gs3d_projected_splat* __restrict__ out,
                                                 uint32_t* __restrict__ counts,
                                                 uint32_t* __restrict__ depth_keys,
                                                 uint32_t* __restrict__ depth_ids,
                                                 uint32_t* __restrict__ rect8,
                                                 uint32_t* __restrict__ err) {
  constexpr int K = (DEG + 1) * (DEG + 1) - 1;
  constexpr int KC = 3 * K;  // floats of SH rest per splat
  const ViewDesc& lv = views[leader];
  const uint32_t n = lv.f.splat_count;
  const uint32_t li = local_first + threadIdx.x;
  const bool active = li < n;

  // ---- SH slice: one bulk copy per block (issued first, waited on late) ----
  bool bulk = false;
  if (DEG > 0) {
    const uint32_t cnt = min((uint32_t)kThreads, n - local_first);
    const uint32_t bytes = cnt * KC * 4u;
    const float* src = lv.sh + (size_t)local_first * KC;
    bulk = (bytes % 16u) == 0u && (reinterpret_cast<uintptr_t>(src) % 16u) == 0u;
    if (bulk) {
      if (threadIdx.x == 0) {
        mbar_init(s_bar, 1);
        fence_mbar_init();
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        mbar_expect_tx(s_bar, bytes);
        bulk_g2s(s_sh, src, bytes, s_bar);
      }
    } else {
      for (uint32_t k = threadIdx.x; k < cnt * KC; k += kThreads) s_sh[k] = __ldg(src + k);
      __syncthreads();
    }
  }

  // ---- view-independent: the splat and its 3D covariance S = M M^T ----
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f), col = p;
  float S[3][3] = {};
  if (active) {
    p = __ldg(lv.pos + li);
    const float4 s = __ldg(lv.scale + li);
    const float4 q = __ldg(lv.rot + li);
    col = __ldg(lv.color + li);
    const float qw = q.x, qx = q.y, qy = q.z, qz = q.w;
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
    const float xy = qx * qy, xz = qx * qz, yz = qy * qz;
    const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
    float R[3][3];  // [col][row]
    R[0][0] = 1.0f - 2.0f * (yy + zz); R[0][1] = 2.0f * (xy + wz);        R[0][2] = 2.0f * (xz - wy);
    R[1][0] = 2.0f * (xy - wz);        R[1][1] = 1.0f - 2.0f * (xx + zz); R[1][2] = 2.0f * (yz + wx);
    R[2][0] = 2.0f * (xz + wy);        R[2][1] = 2.0f * (yz - wx);        R[2][2] = 1.0f - 2.0f * (xx + yy);
    const float sc[3] = {s.x, s.y, s.z};
    float M[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int r = 0; r < 3; ++r) M[k][r] = R[k][r] * sc[k];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b)
        S[a][b] = M[0][a] * M[0][b] + M[1][a] * M[1][b] + M[2][a] * M[2][b];
  }
  bool sh_ready = true;
  if (DEG > 0 && bulk && !mbar_wait(s_bar, 0)) {
    if (threadIdx.x == 0) latch_error(err, DEVERR_TIMEOUT);
    sh_ready = false;
  }

  for (uint32_t v = leader; v != kNoView; v = views[v].group_next) {
    const ViewDesc& vd = views[v];
    const FrameUniforms* fu = &vd.f;
    const uint32_t gi = vd.splat_base + li;  // global splat-view index
    const float* V = fu->cam.view;
    const float* P = fu->cam.projection;

    bool valid = false;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
    uint4 r3 = make_uint4(0u, 0u, 0u, 0u);
    uint32_t count = 0;

    if (active) {
      float vp[4], cp[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        vp[r] = __ldg(V + 0 * 4 + r) * p.x + __ldg(V + 1 * 4 + r) * p.y +
                __ldg(V + 2 * 4 + r) * p.z + __ldg(V + 3 * 4 + r) * 1.0f;
#pragma unroll
      for (int r = 0; r < 4; ++r)
        cp[r] = __ldg(P + 0 * 4 + r) * vp[0] + __ldg(P + 1 * 4 + r) * vp[1] +
                __ldg(P + 2 * 4 + r) * vp[2] + __ldg(P + 3 * 4 + r) * vp[3];

      bool keep = !(cp[3] <= 0.0f);
      float nx = 0.f, ny = 0.f, nz = 0.f;
      if (keep) {
        nx = cp[0] / cp[3];
        ny = cp[1] / cp[3];
        nz = cp[2] / cp[3];
        keep = !(nx < -1.0f || nx > 1.0f || ny < -1.0f || ny > 1.0f || nz < 0.0f || nz > 1.0f);
      }
      if (keep) {
        const float W = __ldg(&fu->cam.viewport[0]);
        const float H = __ldg(&fu->cam.viewport[1]);
        const float sx = (nx * 0.5f + 0.5f) * W;
        const float sy = (1.0f - (ny * 0.5f + 0.5f)) * H;

        const float fx = __ldg(P + 0) * W * 0.5f;
        const float fy = __ldg(P + 5) * H * 0.5f;
        const float z_cam = -vp[2];
        const float inv_z = 1.0f / z_cam;
        const float inv_z2 = inv_z * inv_z;
        float J[2][3];
        J[0][0] = fx * inv_z;  J[0][1] = 0.0f;        J[0][2] = fx * vp[0] * inv_z2;
        J[1][0] = 0.0f;        J[1][1] = -fy * inv_z; J[1][2] = -fy * vp[1] * inv_z2;
        float T[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            T[r][j] = J[r][0] * __ldg(V + j * 4 + 0) + J[r][1] * __ldg(V + j * 4 + 1) +
                      J[r][2] * __ldg(V + j * 4 + 2);
        float A[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            A[r][j] = T[r][0] * S[0][j] + T[r][1] * S[1][j] + T[r][2] * S[2][j];
        const float c00 = A[0][0] * T[0][0] + A[0][1] * T[0][1] + A[0][2] * T[0][2];
        const float c10 = A[1][0] * T[0][0] + A[1][1] * T[0][1] + A[1][2] * T[0][2];
        const float c11 = A[1][0] * T[1][0] + A[1][1] * T[1][1] + A[1][2] * T[1][2];

        const float a = c00 + 0.3f;
        const float b = c10;
        const float c = c11 + 0.3f;
        const float det = a * c - b * b;
        if (!(det <= 0.0f)) {
          const float inv_det = 1.0f / det;
          const float mid = 0.5f * (a + c);
          const float lambda = mid + sqrtf(fmaxf(0.1f, mid * mid - det));
          const float radius = fmaxf(2.0f, ceilf(3.0f * sqrtf(lambda)));
          const float minx = fmaxf(0.0f, sx - radius);
          const float miny = fmaxf(0.0f, sy - radius);
          const float maxx = fminf(W - 1.0f, sx + radius);
          const float maxy = fminf(H - 1.0f, sy + radius);
          const float itx = __ldg(&fu->inv_tile[0]), ity = __ldg(&fu->inv_tile[1]);
          const uint32_t lastx = __ldg(&fu->tile_count[0]) - 1u;
          const uint32_t lasty = __ldg(&fu->tile_count[1]) - 1u;
          const uint32_t tminx = min(__float2uint_rz(floorf(minx * itx)), lastx);
          const uint32_t tminy = min(__float2uint_rz(floorf(miny * ity)), lasty);
          const uint32_t tmaxx = min(__float2uint_rz(floorf(maxx * itx)), lastx);
          const uint32_t tmaxy = min(__float2uint_rz(floorf(maxy * ity)), lasty);
          if (!(tminx > tmaxx || tminy > tmaxy)) {
            valid = true;
            count = (tmaxx - tminx + 1u) * (tmaxy - tminy + 1u);
            r0 = make_float4(sx, sy, vp[2], radius);
            r1 = make_float4(c * inv_det, -b * inv_det, a * inv_det, col.w);
            r2 = make_float4(col.x, col.y, col.z, 0.0f);
            r3 = make_uint4(tminx, tminy, tmaxx, tmaxy);
          }
        }
      }
    }

    if (DEG > 0) {
      if (!sh_ready) valid = false;
      if (valid) {
        float cc[3];
        sh_color<DEG>(p.x, p.y, p.z, fu->cam.position, col, s_sh + threadIdx.x * KC, cc);
        r2.x = cc[0];
        r2.y = cc[1];
        r2.z = cc[2];
      }
    }

    if (active) {
      if (!valid) {
        r0 = r1 = r2 = make_float4(0.f, 0.f, 0.f, 0.f);
        r3 = make_uint4(0u, 0u, 0u, 0u);
        count = 0u;
      } else {
        r2.w = __uint_as_float(1u);
      }
      float4* o = reinterpret_cast<float4*>(out + gi);
      o[0] = r0;
      o[1] = r1;
      o[2] = r2;
      reinterpret_cast<uint4*>(o)[3] = r3;
      counts[gi] = count;
      if (depth_keys != nullptr) {  // per-splat depth sort keys of the fused rebin
        depth_keys[gi] = valid ? __float_as_uint(-r0.z) : 0xffffffffu;
        depth_ids[gi] = gi;
        // tile rectangle in one word [x0, y0, x1 - x0, y1 - y0] (8 bits each;
        // requested only when every view has at most 256 tiles per axis)
        if (rect8 != nullptr)
          rect8[gi] = r3.x | (r3.y << 8) | ((r3.z - r3.x) << 16) | ((r3.w - r3.y) << 24);
      }
    }
  }
}

template <int MAXDEG>
__global__ void __launch_bounds__(kThreads)
    preprocess_kernel(const ViewDesc* __restrict__ views, uint32_t n_views,
                      gs3d_projected_splat* __restrict__ out, uint32_t* __restrict__ counts,
                      uint32_t* __restrict__ depth_keys, uint32_t* __restrict__ depth_ids,
                      uint32_t* __restrict__ rect8,
                      uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) float s_sh[];
  __shared__ uint64_t s_bar;
  // block_base counts the blocks of the scene groups' leaders only, so the
  // search lands on the leader of this block's group
  const uint32_t v =
      find_view(n_views, blockIdx.x, [&](uint32_t i) { return __ldg(&views[i].block_base); });
  const ViewDesc& vd = views[v];
  const uint32_t local_first = (blockIdx.x - vd.block_base) * kThreads;
  const uint32_t deg = vd.sh == nullptr ? 0u : min(vd.sh_degree, (uint32_t)MAXDEG);
  switch (deg) {  // uniform per block
    case 0:
      preprocess_block<0>(views, v, local_first, s_sh, &s_bar, out, counts, depth_keys,
                          depth_ids, rect8, err);
      break;
    case 1:
      if (MAXDEG >= 1)
        preprocess_block<MAXDEG >= 1 ? 1 : 0>(views, v, local_first, s_sh, &s_bar, out, counts,
                                              depth_keys, depth_ids, rect8, err);
      break;
    case 2:
      if (MAXDEG >= 2)
        preprocess_block<MAXDEG >= 2 ? 2 : 0>(views, v, local_first, s_sh, &s_bar, out, counts,
                                              depth_keys, depth_ids, rect8, err);
      break;
    default:
      if (MAXDEG >= 3)
        preprocess_block<MAXDEG >= 3 ? 3 : 0>(views, v, local_first, s_sh, &s_bar, out, counts,
                                              depth_keys, depth_ids, rect8, err);
      break;
  }
}

}  // namespace

cudaError_t launch_preprocess(const ViewDesc* views, uint32_t n_views, uint32_t total_blocks,
                              uint32_t max_sh_degree, gs3d_projected_splat* out, uint32_t* counts,
                              uint32_t* depth_keys, uint32_t* depth_ids, uint32_t* rect8,
                              uint32_t* err,
                              cudaStream_t s) {
  if (total_blocks == 0) return cudaSuccess;
  const uint32_t kc = 3u * ((max_sh_degree + 1) * (max_sh_degree + 1) - 1);
  // 45 floats x 256 splats = 46,080 B at degree 3: inside the 48 KB default window
  const size_t smem = (size_t)kc * kThreads * sizeof(float);
  switch (max_sh_degree) {
    case 0:
      preprocess_kernel<0><<<total_blocks, kThreads, 0, s>>>(views, n_views, out, counts,
                                                             depth_keys, depth_ids, rect8, err);
      break;
    case 1:
      preprocess_kernel<1><<<total_blocks, kThreads, smem, s>>>(views, n_views, out, counts,
                                                                depth_keys, depth_ids, rect8, err);
      break;
    case 2:
      preprocess_kernel<2><<<total_blocks, kThreads, smem, s>>>(views, n_views, out, counts,
                                                                depth_keys, depth_ids, rect8, err);
      break;
    default:
      preprocess_kernel<3><<<total_blocks, kThreads, smem, s>>>(views, n_views, out, counts,
                                                                depth_keys, depth_ids, rect8, err);
      break;
  }
  return cudaGetLastError();
}

}  // namespace gs3d
