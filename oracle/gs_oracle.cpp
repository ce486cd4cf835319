// gs_oracle.cpp - CPU restatement of the webgpu-3dgs per-frame rebin path.
//
// TEST INFRASTRUCTURE ONLY: what the tests compare the CUDA library with, and
// the timed CPU baseline.  Nothing in the library links or loads this file.
//
// Parity status: UNPINNED against executable reference output (the reference
// is WGSL that needs a WebGPU implementation, unavailable here, and it ships
// no golden vectors).  The restatement is pinned by hand-derived known-answer
// tests in tests/test_oracle_kat.py.
//
// Build: g++ -O3 -fopenmp -ffp-contract=off (no fast-math), so every f32
// operation below is one IEEE-rounded operation in the written order.  WGSL
// leaves contraction and summation order to the shader compiler; this file
// fixes them: matrix-vector and matrix-matrix products sum their terms left
// to right, k = 0, 1, 2(, 3), zero terms included.

#include "gs_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Projected {  // ProjectedSplat, preprocess_splats.wgsl:18-31 (64 bytes)
  float mean_px[2];
  float depth;
  float radius_px;
  float conic[3];
  float opacity;
  float color[3];
  uint32_t valid;
  uint32_t tile_min[2];
  uint32_t tile_max[2];
};
static_assert(sizeof(Projected) == 64, "ProjectedSplat stride is 64 bytes");

int resolve_threads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

// f32 -> u32 conversion that saturates (NaN -> 0), the behaviour WGSL gives
// in-range values and the library's __float2uint_rz gives everywhere.
uint32_t f2u_sat(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

uint32_t f32_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// Real spherical-harmonics basis constants, degree 1..3 (the standard
// orthonormal real SH normalisation used by 3D Gaussian Splatting).
const float SH_C1 = 0.4886025119029199f;
const float SH_C2[5] = {1.0925484305920792f, -1.0925484305920792f,
                        0.31539156525252005f, -1.0925484305920792f,
                        0.5462742152960396f};
const float SH_C3[7] = {-0.5900435899266435f, 2.890611442640554f,
                        -0.4570457994644658f, 0.3731763325901154f,
                        -0.4570457994644658f, 1.445305721320277f,
                        -0.5900435899266435f};

// SH colour extension (not in the reference, whose colour is SH degree 0
// baked at load time, SceneWorker.ts:430-432).  base = splat_colors.rgb;
// colour_c = clamp01(base_c + sum_k basis_k(dir) * rest[c*K + k-1]) with
// dir = normalize(position - camera position) and K = (deg+1)^2 - 1; the
// sum runs k = 1..K, each term added by one fused multiply-add (a single
// rounding, as the GPU's fmaf).
void sh_color(const float* p, const float* cam_pos, const float* base,
              const float* rest, uint32_t deg, float out[3]) {
  const uint32_t K = (deg + 1) * (deg + 1) - 1;
  float dx = p[0] - cam_pos[0];
  float dy = p[1] - cam_pos[1];
  float dz = p[2] - cam_pos[2];
  float len = std::sqrt(dx * dx + dy * dy + dz * dz);
  float x = 0.0f, y = 0.0f, z = 0.0f;
  if (len > 0.0f) {
    x = dx / len;
    y = dy / len;
    z = dz / len;
  }
  float b[16];
  b[1] = -SH_C1 * y;
  b[2] = SH_C1 * z;
  b[3] = -SH_C1 * x;
  if (deg > 1) {
    float xx = x * x, yy = y * y, zz = z * z;
    float xy = x * y, yz = y * z, xz = x * z;
    b[4] = SH_C2[0] * xy;
    b[5] = SH_C2[1] * yz;
    b[6] = SH_C2[2] * (2.0f * zz - xx - yy);
    b[7] = SH_C2[3] * xz;
    b[8] = SH_C2[4] * (xx - yy);
    if (deg > 2) {
      b[9] = SH_C3[0] * y * (3.0f * xx - yy);
      b[10] = SH_C3[1] * xy * z;
      b[11] = SH_C3[2] * y * (4.0f * zz - xx - yy);
      b[12] = SH_C3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
      b[13] = SH_C3[4] * x * (4.0f * zz - xx - yy);
      b[14] = SH_C3[5] * z * (xx - yy);
      b[15] = SH_C3[6] * x * (xx - 3.0f * yy);
    }
  }
  for (int c = 0; c < 3; ++c) {
    float acc = base[c];
    for (uint32_t k = 1; k <= K; ++k) acc = std::fma(b[k], rest[c * K + (k - 1)], acc);
    out[c] = std::min(1.0f, std::max(0.0f, acc));
  }
}

// preprocess_splats.wgsl:76-184 for one splat.
void preprocess_one(uint32_t i, const float* cam, const uint32_t tile_count[2],
                    const float inv_tile[2], const float* positions,
                    const float* scales, const float* rotations,
                    const float* colors, const float* sh_rest,
                    uint32_t sh_degree, Projected* out, uint32_t* counts) {
  Projected rec;
  std::memset(&rec, 0, sizeof(rec));  // valid = 0 (:81); culled records are zero
  out[i] = rec;
  counts[i] = 0u;  // :82

  const float* V = cam;        // view, column-major: V[col*4 + row]
  const float* P = cam + 16;   // projection
  const float* p = positions + 4 * (size_t)i;
  const float* s = scales + 4 * (size_t)i;
  const float* q = rotations + 4 * (size_t)i;
  const float* col = colors + 4 * (size_t)i;

  // :89-90  view = V * (p.xyz, 1); clip = P * view
  float vp[4], cp[4];
  for (int r = 0; r < 4; ++r)
    vp[r] = V[0 * 4 + r] * p[0] + V[1 * 4 + r] * p[1] + V[2 * 4 + r] * p[2] +
            V[3 * 4 + r] * 1.0f;
  for (int r = 0; r < 4; ++r)
    cp[r] = P[0 * 4 + r] * vp[0] + P[1 * 4 + r] * vp[1] + P[2 * 4 + r] * vp[2] +
            P[3 * 4 + r] * vp[3];

  if (cp[3] <= 0.0f) return;  // :92
  float nx = cp[0] / cp[3], ny = cp[1] / cp[3], nz = cp[2] / cp[3];  // :94
  if (nx < -1.0f || nx > 1.0f || ny < -1.0f || ny > 1.0f || nz < 0.0f ||
      nz > 1.0f)
    return;  // :95-97

  const float W = cam[68], H = cam[69];
  const float sx = (nx * 0.5f + 0.5f) * W;          // :100-103
  const float sy = (1.0f - (ny * 0.5f + 0.5f)) * H;

  // :49-65 quaternion (w, x, y, z) -> rotation columns
  const float qw = q[0], qx = q[1], qy = q[2], qz = q[3];
  const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
  const float xy = qx * qy, xz = qx * qz, yz = qy * qz;
  const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
  float R[3][3];  // R[col][row]
  R[0][0] = 1.0f - 2.0f * (yy + zz); R[0][1] = 2.0f * (xy + wz);        R[0][2] = 2.0f * (xz - wy);
  R[1][0] = 2.0f * (xy - wz);        R[1][1] = 1.0f - 2.0f * (xx + zz); R[1][2] = 2.0f * (yz + wx);
  R[2][0] = 2.0f * (xz + wy);        R[2][1] = 2.0f * (yz - wx);        R[2][2] = 1.0f - 2.0f * (xx + yy);
  // :71 M = R * diag(s): column k scaled by s_k.   M[col][row]
  float M[3][3];
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) M[k][r] = R[k][r] * s[k];
  // :72 Sigma = M * M^T: Sigma(i,j) = sum_k M(i,k) M(j,k)
  float S[3][3];  // S[i][j] symmetric
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      S[a][b] = M[0][a] * M[0][b] + M[1][a] * M[1][b] + M[2][a] * M[2][b];

  // :118-132 focal lengths and the projection Jacobian J (rows 0, 1; row 2 = 0)
  const float fx = P[0] * W * 0.5f;
  const float fy = P[5] * H * 0.5f;
  const float z_cam = -vp[2];
  const float inv_z = 1.0f / z_cam;
  const float inv_z2 = inv_z * inv_z;
  float J[2][3];  // J[row][col]
  J[0][0] = fx * inv_z;  J[0][1] = 0.0f;         J[0][2] = fx * vp[0] * inv_z2;
  J[1][0] = 0.0f;        J[1][1] = -fy * inv_z;  J[1][2] = -fy * vp[1] * inv_z2;
  // :134 T = J * W3, W3(k, j) = view[j][k]
  float T[2][3];
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 3; ++j)
      T[r][j] = J[r][0] * V[j * 4 + 0] + J[r][1] * V[j * 4 + 1] +
                J[r][2] * V[j * 4 + 2];
  // :135 cov2d = (T * Sigma) * T^T, rows/cols 0..1 only
  float A[2][3];
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 3; ++j)
      A[r][j] = T[r][0] * S[0][j] + T[r][1] * S[1][j] + T[r][2] * S[2][j];
  const float c00 = A[0][0] * T[0][0] + A[0][1] * T[0][1] + A[0][2] * T[0][2];
  const float c10 = A[1][0] * T[0][0] + A[1][1] * T[0][1] + A[1][2] * T[0][2];
  const float c11 = A[1][0] * T[1][0] + A[1][1] * T[1][1] + A[1][2] * T[1][2];

  const float a = c00 + 0.3f;  // :138-140 low-pass
  const float b = c10;
  const float c = c11 + 0.3f;
  const float det = a * c - b * b;  // :142
  if (det <= 0.0f) return;          // :143
  const float inv_det = 1.0f / det;
  const float conic0 = c * inv_det, conic1 = -b * inv_det, conic2 = a * inv_det;

  const float mid = 0.5f * (a + c);  // :150-152
  const float lambda = mid + std::sqrt(std::max(0.1f, mid * mid - det));
  const float radius = std::max(2.0f, std::ceil(3.0f * std::sqrt(lambda)));

  const float minx = std::max(0.0f, sx - radius);  // :154-155
  const float miny = std::max(0.0f, sy - radius);
  const float maxx = std::min(W - 1.0f, sx + radius);
  const float maxy = std::min(H - 1.0f, sy + radius);

  uint32_t tminx = std::min(f2u_sat(std::floor(minx * inv_tile[0])), tile_count[0] - 1u);
  uint32_t tminy = std::min(f2u_sat(std::floor(miny * inv_tile[1])), tile_count[1] - 1u);
  uint32_t tmaxx = std::min(f2u_sat(std::floor(maxx * inv_tile[0])), tile_count[0] - 1u);
  uint32_t tmaxy = std::min(f2u_sat(std::floor(maxy * inv_tile[1])), tile_count[1] - 1u);
  if (tminx > tmaxx || tminy > tmaxy) return;  // :166

  counts[i] = (tmaxx - tminx + 1u) * (tmaxy - tminy + 1u);  // :169-171

  rec.mean_px[0] = sx;
  rec.mean_px[1] = sy;
  rec.depth = vp[2];
  rec.radius_px = radius;
  rec.conic[0] = conic0;
  rec.conic[1] = conic1;
  rec.conic[2] = conic2;
  rec.opacity = col[3];
  if (sh_degree == 0 || sh_rest == nullptr) {
    rec.color[0] = col[0];
    rec.color[1] = col[1];
    rec.color[2] = col[2];
  } else {
    const uint32_t K = (sh_degree + 1) * (sh_degree + 1) - 1;
    sh_color(p, cam + 64, col, sh_rest + (size_t)i * 3 * K, sh_degree, rec.color);
  }
  rec.valid = 1u;
  rec.tile_min[0] = tminx;
  rec.tile_min[1] = tminy;
  rec.tile_max[0] = tmaxx;
  rec.tile_max[1] = tmaxy;
  out[i] = rec;
}

// One 4x4 inverse in double by Gauss-Jordan elimination with partial pivoting
// (the inverse matrices are part of the uniform but unused by the path).
void invert4(const float* m, float* out) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m[c * 4 + r];
      a[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) {  // singular: zeros
      for (int i = 0; i < 16; ++i) out[i] = 0.0f;
      return;
    }
    if (piv != c)
      for (int k = 0; k < 8; ++k) std::swap(a[piv][k], a[c][k]);
    const double inv = 1.0 / a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      const double f = a[r][c];
      if (f == 0.0) continue;
      for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)a[r][4 + c];
}

}  // namespace

extern "C" {

int orc_max_threads(void) { return resolve_threads(0); }

// Camera.ts:69-79,172-191 with gl-matrix 3.4 lookAt / perspective (OpenGL
// clip-space z in [-1, 1]).  Computed in double, stored as f32, as gl-matrix
// does with its Float32Array outputs.
void orc_camera_uniform(const float eye[3], const float target[3],
                        const float up[3], double fovy, double aspect,
                        double znear, double zfar, double width, double height,
                        float out[72]) {
  std::memset(out, 0, 72 * sizeof(float));
  float* view = out;
  float* proj = out + 16;
  const double e0 = eye[0], e1 = eye[1], e2 = eye[2];
  double z0 = e0 - target[0], z1 = e1 - target[1], z2 = e2 - target[2];
  if (std::fabs(z0) < 1e-6 && std::fabs(z1) < 1e-6 && std::fabs(z2) < 1e-6) {
    for (int i = 0; i < 16; ++i) view[i] = (i % 5 == 0) ? 1.0f : 0.0f;
  } else {
    double len = 1.0 / std::sqrt(z0 * z0 + z1 * z1 + z2 * z2);
    z0 *= len; z1 *= len; z2 *= len;
    const double u0 = up[0], u1 = up[1], u2 = up[2];
    double x0 = u1 * z2 - u2 * z1, x1 = u2 * z0 - u0 * z2, x2 = u0 * z1 - u1 * z0;
    len = std::sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    if (len == 0.0) { x0 = x1 = x2 = 0.0; } else { len = 1.0 / len; x0 *= len; x1 *= len; x2 *= len; }
    double y0 = z1 * x2 - z2 * x1, y1 = z2 * x0 - z0 * x2, y2 = z0 * x1 - z1 * x0;
    len = std::sqrt(y0 * y0 + y1 * y1 + y2 * y2);
    if (len == 0.0) { y0 = y1 = y2 = 0.0; } else { len = 1.0 / len; y0 *= len; y1 *= len; y2 *= len; }
    const double vals[16] = {x0, y0, z0, 0.0, x1, y1, z1, 0.0, x2, y2, z2, 0.0,
                             -(x0 * e0 + x1 * e1 + x2 * e2),
                             -(y0 * e0 + y1 * e1 + y2 * e2),
                             -(z0 * e0 + z1 * e1 + z2 * e2), 1.0};
    for (int i = 0; i < 16; ++i) view[i] = (float)vals[i];
  }
  const double f = 1.0 / std::tan(fovy / 2.0);
  proj[0] = (float)(f / aspect);
  proj[5] = (float)f;
  proj[11] = -1.0f;
  if (std::isfinite(zfar)) {
    const double nf = 1.0 / (znear - zfar);
    proj[10] = (float)((zfar + znear) * nf);
    proj[14] = (float)(2.0 * zfar * znear * nf);
  } else {
    proj[10] = -1.0f;
    proj[14] = (float)(-2.0 * znear);
  }
  invert4(view, out + 32);
  invert4(proj, out + 48);
  out[64] = eye[0];
  out[65] = eye[1];
  out[66] = eye[2];
  out[67] = 1.0f;
  out[68] = (float)width;
  out[69] = (float)height;
  out[70] = (float)(width / height);
  out[71] = 0.0f;
}

// SceneWorker.ts:407-464: activations in double, rounded to f32.
void orc_activate(uint32_t n, const double* xyz, const double* f_dc,
                  const double* opacity, const double* scale_log,
                  const double* rot, float* positions, float* colors,
                  float* scales, float* rotations) {
  const double C0 = 0.28209479177387814;
  auto clamp01 = [](double x) { return std::min(1.0, std::max(0.0, x)); };
  for (uint32_t i = 0; i < n; ++i) {
    const size_t o = 4 * (size_t)i;
    positions[o + 0] = (float)xyz[3 * (size_t)i + 0];
    positions[o + 1] = (float)xyz[3 * (size_t)i + 1];
    positions[o + 2] = (float)xyz[3 * (size_t)i + 2];
    positions[o + 3] = 1.0f;
    for (int c = 0; c < 3; ++c)
      colors[o + c] = (float)clamp01(0.5 + C0 * f_dc[3 * (size_t)i + c]);
    colors[o + 3] = (float)clamp01(1.0 / (1.0 + std::exp(-opacity[i])));
    for (int c = 0; c < 3; ++c)
      scales[o + c] = (float)std::exp(scale_log[3 * (size_t)i + c]);
    scales[o + 3] = 0.0f;
    const double* r = rot + 4 * (size_t)i;
    const double len = std::hypot(std::hypot(r[0], r[1]), std::hypot(r[2], r[3]));
    const double inv = len > 0.0 ? 1.0 / len : 1.0;
    for (int c = 0; c < 4; ++c) rotations[o + c] = (float)(r[c] * inv);
  }
}

void orc_preprocess(uint32_t n, const float cam[72], const uint32_t tile_count[2],
                    const float inv_tile[2], const float* positions,
                    const float* scales, const float* rotations,
                    const float* colors, const float* sh_rest,
                    uint32_t sh_degree, void* projected, uint32_t* ref_counts,
                    int threads) {
  Projected* out = static_cast<Projected*>(projected);
  const int nt = resolve_threads(threads);
  (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long long i = 0; i < (long long)n; ++i)
    preprocess_one((uint32_t)i, cam, tile_count, inv_tile, positions, scales,
                   rotations, colors, sh_rest, sh_degree, out, ref_counts);
}

// prefix_scan_local/blocks/add: exclusive scan with u32 wrap-around,
// offsets[n] = ref_counter[0] = total (prefix_scan_blocks.wgsl:41-42).
uint32_t orc_prefix_scan(uint32_t n, const uint32_t* counts, uint32_t* offsets) {
  uint32_t run = 0;
  for (uint32_t i = 0; i < n; ++i) {
    offsets[i] = run;
    run += counts[i];
  }
  offsets[n] = run;
  return run;
}

// emit_tile_refs.wgsl:57-79
void orc_emit(uint32_t n, uint32_t tiles_x, const void* projected,
              const uint32_t* offsets, uint32_t* keys, uint32_t* values) {
  const Projected* ps = static_cast<const Projected*>(projected);
  for (uint32_t i = 0; i < n; ++i) {
    const Projected& s = ps[i];
    if (s.valid == 0u) continue;
    const uint32_t key_lo = f32_bits(-s.depth);
    uint32_t w = offsets[i];
    for (uint32_t ty = s.tile_min[1]; ty <= s.tile_max[1]; ++ty)
      for (uint32_t tx = s.tile_min[0]; tx <= s.tile_max[0]; ++tx) {
        keys[2 * (size_t)w + 0] = ty * tiles_x + tx;  // hi = tile id
        keys[2 * (size_t)w + 1] = key_lo;              // lo = depth bits
        values[w] = i;
        ++w;
      }
  }
}

// radix_histogram.wgsl + scan_local/scan_add + radix_scatter.wgsl: eight
// stable 8-bit passes, digit (lo >> b) & 0xff for b < 32 else (hi >> (b-32)).
// Per pass: each thread counts its contiguous chunk (a "workgroup"), counts
// are scanned digit-major (bucket * chunks + chunk) and each chunk scatters
// its elements in order - the reference's per-workgroup scheme, which is a
// stable counting sort.
void orc_radix_sort(uint32_t r, uint32_t* keys, uint32_t* values,
                    uint32_t* tmp_keys, uint32_t* tmp_values, int threads) {
  if (r == 0) return;
  const int nt = std::max(1, std::min(resolve_threads(threads), (int)((r + 4095) / 4096)));
  std::vector<uint32_t> hist((size_t)nt * 256);
  uint32_t* src_k = keys;
  uint32_t* src_v = values;
  uint32_t* dst_k = tmp_keys;
  uint32_t* dst_v = tmp_values;
  const size_t chunk = ((size_t)r + nt - 1) / nt;
  for (int pass = 0; pass < 8; ++pass) {
    const int bit = pass * 8;
    const int word = bit < 32 ? 1 : 0;  // lo is element 1 of [hi, lo]
    const int shift = bit < 32 ? bit : bit - 32;
    std::fill(hist.begin(), hist.end(), 0u);
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num();
#else
      const int t = 0;
#endif
      const size_t b = std::min((size_t)r, t * chunk), e = std::min((size_t)r, b + chunk);
      uint32_t* h = hist.data() + (size_t)t * 256;
      for (size_t i = b; i < e; ++i) ++h[(src_k[2 * i + word] >> shift) & 0xffu];
#pragma omp barrier
#pragma omp single
      {
        uint32_t run = 0;  // digit-major exclusive scan
        for (int d = 0; d < 256; ++d)
          for (int c = 0; c < nt; ++c) {
            const uint32_t v = hist[(size_t)c * 256 + d];
            hist[(size_t)c * 256 + d] = run;
            run += v;
          }
      }
      for (size_t i = b; i < e; ++i) {
        const uint32_t d = (src_k[2 * i + word] >> shift) & 0xffu;
        const uint32_t o = h[d]++;
        dst_k[2 * (size_t)o] = src_k[2 * i];
        dst_k[2 * (size_t)o + 1] = src_k[2 * i + 1];
        dst_v[o] = src_v[i];
      }
    }
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
  }
  // eight passes: the result is back in keys/values
}

// identify_tile_ranges.wgsl:31-52
void orc_identify(uint32_t r, const uint32_t* keys, uint32_t* tile_offsets) {
  for (uint32_t i = 0; i < r; ++i) {
    const uint32_t curr = keys[2 * (size_t)i];
    if (i == 0u || keys[2 * (size_t)(i - 1)] != curr) {
      const uint32_t from = (i == 0u) ? 0u : keys[2 * (size_t)(i - 1)] + 1u;
      for (uint32_t t = from; t <= curr; ++t) tile_offsets[t] = i;
    }
    if (i == r - 1u || keys[2 * (size_t)(i + 1)] != curr) tile_offsets[curr + 1u] = i + 1u;
  }
}

// rasterize_tiles.wgsl:44-110, one tile at a time, pixels in order.
void orc_rasterize(uint32_t width, uint32_t height, uint32_t tile_w,
                   uint32_t tile_h, uint32_t tiles_x, uint32_t tiles_y,
                   const void* projected, const uint32_t* tile_offsets,
                   const uint32_t* values, float* image, uint32_t* tile_costs,
                   int threads) {
  const Projected* ps = static_cast<const Projected*>(projected);
  const int nt = resolve_threads(threads);
  (void)nt;
  const long long ntiles = (long long)tiles_x * tiles_y;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
  for (long long t = 0; t < ntiles; ++t) {
    const uint32_t tx = (uint32_t)(t % tiles_x), ty = (uint32_t)(t / tiles_x);
    const uint32_t start = tile_offsets[t], end = tile_offsets[t + 1];
    uint32_t cost = 0;
    bool any_open = false;
    for (uint32_t ly = 0; ly < tile_h; ++ly)
      for (uint32_t lx = 0; lx < tile_w; ++lx) {
        const uint32_t px = tx * tile_w + lx, py = ty * tile_h + ly;
        if (px >= width || py >= height) continue;  // :51,61
        const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;
        float cr = 0.0f, cg = 0.0f, cb = 0.0f, T = 1.0f;
        uint32_t last = start;  // index one past the last splat iterated
        bool done = false;
        for (uint32_t j = start; j < end; ++j) {
          last = j + 1;
          const Projected& s = ps[values[j]];
          const float dx = pfx - s.mean_px[0], dy = pfy - s.mean_px[1];
          if (dx * dx + dy * dy > s.radius_px * s.radius_px) continue;  // :85
          const float power = -0.5f * (s.conic[0] * dx * dx + 2.0f * s.conic[1] * dx * dy +
                                       s.conic[2] * dy * dy);  // :89
          if (power > 0.0f) continue;                           // :90
          const float alpha = std::min(0.99f, s.opacity * std::exp(power));  // :92
          if (alpha < 1.0f / 255.0f) continue;                  // :93
          cr += T * alpha * s.color[0];                          // :95
          cg += T * alpha * s.color[1];
          cb += T * alpha * s.color[2];
          T *= 1.0f - alpha;                                     // :96
          if (T < 1.0e-4f) { done = true; break; }               // :98
        }
        if (!done) any_open = true;
        const uint32_t used = (end > start) ? last - start : 0u;
        cost = std::max(cost, used);
        float* o = image + 4 * ((size_t)py * width + px);
        o[0] = cr; o[1] = cg; o[2] = cb; o[3] = 1.0f - T;  // :106-108
      }
    if (tile_costs) tile_costs[t] = any_open ? (end > start ? end - start : 0u) : cost;
  }
}

// Work counts of rasterize_tiles.wgsl:44-110 over a frame (the same loop as
// orc_rasterize, counting instead of shading): out[0] = (pixel, splat) pairs
// the reference iterates (every splat of the pixel's tile up to the pixel's
// termination), out[1] = pairs inside the radius with power <= 0 (an exp is
// evaluated, :85-92), out[2] = pairs blended (:95-96).
void orc_raster_pairs(uint32_t width, uint32_t height, uint32_t tile_w, uint32_t tile_h,
                      uint32_t tiles_x, uint32_t tiles_y, const void* projected,
                      const uint32_t* tile_offsets, const uint32_t* values, uint64_t out[3],
                      int threads) {
  const Projected* ps = static_cast<const Projected*>(projected);
  const int nt = resolve_threads(threads);
  const long long ntiles = (long long)tiles_x * tiles_y;
  uint64_t it = 0, ev = 0, bl = 0;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt) reduction(+ : it, ev, bl)
  for (long long t = 0; t < ntiles; ++t) {
    const uint32_t tx = (uint32_t)(t % tiles_x), ty = (uint32_t)(t / tiles_x);
    const uint32_t start = tile_offsets[t], end = tile_offsets[t + 1];
    for (uint32_t ly = 0; ly < tile_h; ++ly)
      for (uint32_t lx = 0; lx < tile_w; ++lx) {
        const uint32_t px = tx * tile_w + lx, py = ty * tile_h + ly;
        if (px >= width || py >= height) continue;
        const float pfx = (float)px + 0.5f, pfy = (float)py + 0.5f;
        float T = 1.0f;
        for (uint32_t j = start; j < end; ++j) {
          ++it;
          const Projected& s = ps[values[j]];
          const float dx = pfx - s.mean_px[0], dy = pfy - s.mean_px[1];
          if (dx * dx + dy * dy > s.radius_px * s.radius_px) continue;
          const float power = -0.5f * (s.conic[0] * dx * dx + 2.0f * s.conic[1] * dx * dy +
                                       s.conic[2] * dy * dy);
          if (power > 0.0f) continue;
          ++ev;
          const float alpha = std::min(0.99f, s.opacity * std::exp(power));
          if (alpha < 1.0f / 255.0f) continue;
          ++bl;
          T *= 1.0f - alpha;
          if (T < 1.0e-4f) break;
        }
      }
  }
  out[0] = it;
  out[1] = ev;
  out[2] = bl;
}

uint32_t orc_rebin(uint32_t n, const float cam[72], uint32_t width,
                   uint32_t height, uint32_t tile_w, uint32_t tile_h,
                   const float* positions, const float* scales,
                   const float* rotations, const float* colors,
                   const float* sh_rest, uint32_t sh_degree, void* projected,
                   uint32_t* ref_counts, uint32_t* offsets,
                   uint32_t key_capacity, uint32_t* keys, uint32_t* values,
                   uint32_t* tmp_keys, uint32_t* tmp_values,
                   uint32_t* tile_offsets, float* image, uint32_t* tile_costs,
                   int threads) {
  // GaussianSplatRenderer.ts:1042-1043,1120-1131
  const uint32_t tiles_x = (width + tile_w - 1) / tile_w;
  const uint32_t tiles_y = (height + tile_h - 1) / tile_h;
  const uint32_t tile_count[2] = {tiles_x, tiles_y};
  const float inv_tile[2] = {(float)(1.0 / tile_w), (float)(1.0 / tile_h)};
  orc_preprocess(n, cam, tile_count, inv_tile, positions, scales, rotations,
                 colors, sh_rest, sh_degree, projected, ref_counts, threads);
  const uint32_t r = orc_prefix_scan(n, ref_counts, offsets);
  if (r > key_capacity) return 0xFFFFFFFFu;
  orc_emit(n, tiles_x, projected, offsets, keys, values);
  orc_radix_sort(r, keys, values, tmp_keys, tmp_values, threads);
  std::memset(tile_offsets, 0, ((size_t)tiles_x * tiles_y + 1) * sizeof(uint32_t));
  orc_identify(r, keys, tile_offsets);
  orc_rasterize(width, height, tile_w, tile_h, tiles_x, tiles_y, projected,
                tile_offsets, values, image, tile_costs, threads);
  return r;
}

}  // extern "C"
