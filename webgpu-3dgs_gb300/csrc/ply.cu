// ply.cu - Gaussian-splat PLY ingest (src/workers/SceneWorker.ts:146-550).
//
// Host: the header is parsed and the vertex element laid out (property byte
// offsets and scalar types), with the reference's validation rules and
// messages; an ASCII body is tokenized into f64 rows.  Device: one thread per
// splat reads its row (aligned loads where the layout allows, bytes
// otherwise, swapped for big-endian files), converts every property to f64
// and applies the loader's activations (SceneWorker.ts:407-464) before
// rounding to f32, so the splat arrays match what the reference's
// Float32Arrays receive; position bounds are reduced with ordered-integer
// atomics.
//
// Deviations, all on malformed input: the header ends at the single newline
// (LF or CRLF) after end_header, as the PLY format defines, where the
// reference also swallows any further CR/LF bytes (the first bytes of a
// binary body); element counts must be integers; header keywords are matched
// on bytes, not on decoded UTF-8.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "gs3d_internal.cuh"

namespace gs3d {
namespace {

const char* const kRequired[kPlyRequired] = {
    "x",       "y",       "z",     "opacity", "scale_0", "scale_1", "scale_2",
    "rot_0",   "rot_1",   "rot_2", "rot_3",   "f_dc_0",  "f_dc_1",  "f_dc_2"};

struct Prop {
  std::string name;
  std::string type;
};
struct Elem {
  std::string name;
  uint64_t count = 0;
  std::vector<Prop> props;
};

// PLY scalar type names (SceneWorker.ts:10-18) -> (PlyScalar, bytes)
bool scalar_type(const std::string& t, uint32_t* type, uint32_t* bytes) {
  static const struct {
    const char* name;
    uint32_t type, bytes;
  } kTypes[] = {{"char", PLY_I8, 1},    {"int8", PLY_I8, 1},     {"uchar", PLY_U8, 1},
                {"uint8", PLY_U8, 1},   {"short", PLY_I16, 2},   {"int16", PLY_I16, 2},
                {"ushort", PLY_U16, 2}, {"uint16", PLY_U16, 2},  {"int", PLY_I32, 4},
                {"int32", PLY_I32, 4},  {"uint", PLY_U32, 4},    {"uint32", PLY_U32, 4},
                {"float", PLY_F32, 4},  {"float32", PLY_F32, 4}, {"double", PLY_F64, 8},
                {"float64", PLY_F64, 8}};
  for (const auto& k : kTypes)
    if (t == k.name) {
      *type = k.type;
      *bytes = k.bytes;
      return true;
    }
  return false;
}

std::vector<std::string> split_ws(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && isspace((unsigned char)line[i])) ++i;
    size_t j = i;
    while (j < line.size() && !isspace((unsigned char)line[j])) ++j;
    if (j > i) out.push_back(line.substr(i, j - i));
    i = j;
  }
  return out;
}

bool is_f_rest(const std::string& name, uint32_t* index) {
  if (name.compare(0, 7, "f_rest_") != 0 || name.size() == 7) return false;
  uint64_t v = 0;
  for (size_t i = 7; i < name.size(); ++i) {
    if (name[i] < '0' || name[i] > '9') return false;
    v = v * 10 + (uint32_t)(name[i] - '0');
    if (v > 0xffffffffu) return false;
  }
  *index = (uint32_t)v;
  return true;
}

// inferSphericalHarmonicsDegree (SceneWorker.ts:501-506)
uint32_t infer_degree(uint32_t f_rest) {
  return f_rest >= 45 ? 3 : f_rest >= 24 ? 2 : f_rest >= 9 ? 1 : 0;
}

bool parse_header(const uint8_t* data, size_t size, std::vector<Elem>* elems, uint32_t* format,
                  uint64_t* header_bytes, std::string* err) {
  // parsePlyHeader (SceneWorker.ts:149-253): end_header within the first MB
  const size_t limit = std::min<size_t>(size, 1u << 20);
  static const char kEnd[] = "end_header";
  const size_t kEndLen = sizeof(kEnd) - 1;
  size_t at = std::string::npos;
  for (size_t i = 0; i + kEndLen <= limit; ++i)
    if (std::memcmp(data + i, kEnd, kEndLen) == 0) {
      at = i;
      break;
    }
  if (at == std::string::npos) {
    *err = "Invalid PLY: missing end_header";
    return false;
  }
  size_t hb = at + kEndLen;
  if (hb < size && data[hb] == '\r') ++hb;
  if (hb < size && data[hb] == '\n') ++hb;
  *header_bytes = hb;

  std::vector<std::string> lines;
  {
    std::string cur;
    for (size_t i = 0; i < at + kEndLen; ++i) {
      const char ch = (char)data[i];
      if (ch == '\n') {
        lines.push_back(cur);
        cur.clear();
      } else {
        cur.push_back(ch);
      }
    }
    lines.push_back(cur);
  }
  std::vector<std::string> trimmed;
  for (auto& l : lines) {
    size_t a = 0, b = l.size();
    while (a < b && isspace((unsigned char)l[a])) ++a;
    while (b > a && isspace((unsigned char)l[b - 1])) --b;
    if (b > a) trimmed.push_back(l.substr(a, b - a));
  }
  if (trimmed.empty() || trimmed[0] != "ply") {
    *err = "Invalid PLY: file must start with `ply`";
    return false;
  }
  std::string fmt;
  Elem* cur = nullptr;
  for (size_t li = 1; li < trimmed.size(); ++li) {
    const std::string& line = trimmed[li];
    if (line == "end_header") break;
    if (line.compare(0, 8, "comment ") == 0 || line.compare(0, 9, "obj_info ") == 0) continue;
    const std::vector<std::string> tok = split_ws(line);
    if (tok.empty()) continue;
    if (tok[0] == "format") {
      fmt = tok.size() > 1 ? tok[1] : std::string();
      continue;
    }
    if (tok[0] == "element") {
      Elem e;
      e.name = tok.size() > 1 ? tok[1] : std::string();
      const std::string cs = tok.size() > 2 ? tok[2] : std::string();
      char* end = nullptr;
      const double c = cs.empty() ? NAN : std::strtod(cs.c_str(), &end);
      if (cs.empty() || *end != '\0' || !std::isfinite(c) || c < 0 || c != std::floor(c) ||
          c > 18446744073709549568.0) {
        *err = "Invalid PLY element count for '" + e.name + "'";
        return false;
      }
      e.count = (uint64_t)c;
      elems->push_back(e);
      cur = &elems->back();
      continue;
    }
    if (tok[0] == "property") {
      if (!cur) {
        *err = "Invalid PLY: property declared before element";
        return false;
      }
      if (tok.size() > 1 && tok[1] == "list") {
        *err = "Unsupported PLY: list properties are not expected in Gaussian Splat PLY files";
        return false;
      }
      Prop p;
      p.type = tok.size() > 1 ? tok[1] : std::string();
      p.name = tok.size() > 2 ? tok[2] : std::string();
      cur->props.push_back(p);
    }
  }
  if (fmt.empty()) {
    *err = "Invalid PLY: missing format line";
    return false;
  }
  if (fmt == "ascii") {
    *format = GS3D_PLY_ASCII;
  } else if (fmt == "binary_little_endian") {
    *format = GS3D_PLY_BINARY_LE;
  } else if (fmt == "binary_big_endian") {
    *format = GS3D_PLY_BINARY_BE;
  } else {
    *err = "Unsupported PLY format: " + fmt;
    return false;
  }
  return true;
}

}  // namespace

const char* ply_required_name(int k) { return k >= 0 && k < kPlyRequired ? kRequired[k] : "?"; }

bool ply_parse_layout(const uint8_t* data, size_t size, PlyLayout* out, std::string* err) {
  *out = PlyLayout{};
  if (!data && size) {
    *err = "null PLY data";
    return false;
  }
  std::vector<Elem> elems;
  uint32_t format = 0;
  uint64_t hb = 0;
  if (!parse_header(data, size, &elems, &format, &hb, err)) return false;
  int vi = -1;
  for (size_t i = 0; i < elems.size(); ++i)
    if (elems[i].name == "vertex") {
      vi = (int)i;
      break;
    }
  if (vi < 0) {
    *err = "Invalid Gaussian Splat PLY: missing vertex element";
    return false;
  }
  const Elem& v = elems[vi];
  // validateGaussianSplatHeader (SceneWorker.ts:255-272)
  for (const char* name : kRequired) {
    bool found = false;
    for (const Prop& p : v.props) found = found || p.name == name;
    if (!found) {
      *err = std::string("Invalid Gaussian Splat PLY: missing property '") + name + "'";
      return false;
    }
  }
  const bool ascii = format == GS3D_PLY_ASCII;
  // binary rows: every element's row size (the reference reads all elements)
  uint64_t offset = hb, rows_offset = 0, total = hb;
  uint32_t vstride = 0;
  for (size_t i = 0; i < elems.size(); ++i) {
    uint64_t stride = 0;
    for (const Prop& p : elems[i].props) {
      uint32_t t = 0, b = 0;
      if (!scalar_type(p.type, &t, &b)) {
        if (ascii) continue;  // the ASCII reader never looks at types
        *err = "Unsupported PLY scalar type: " + p.type;
        return false;
      }
      stride += b;
    }
    if ((int)i == vi) {
      rows_offset = offset;
      vstride = (uint32_t)stride;
    }
    if (!ascii) {
      if (stride && elems[i].count > (UINT64_MAX - total) / stride) {
        *err = "Invalid PLY: element data too large";
        return false;
      }
      offset += elems[i].count * stride;
      total = offset;
    }
  }
  if (!ascii && total > size) {
    *err = "Invalid PLY: binary body shorter than its elements";
    return false;
  }
  if (v.count > (1u << 30)) {
    *err = "Gaussian Splat PLY: more than 2^30 splats";
    return false;
  }
  out->count = v.count;
  out->header_bytes = hb;
  out->format = format;
  out->vertex_props = (uint32_t)v.props.size();
  // f_rest_* in index order (createGaussianPropertyLayout, SceneWorker.ts:338-350)
  std::vector<std::pair<uint32_t, uint32_t>> rest;  // (index, property position)
  for (uint32_t i = 0; i < v.props.size(); ++i) {
    uint32_t idx = 0;
    if (is_f_rest(v.props[i].name, &idx)) rest.push_back({idx, i});
  }
  std::stable_sort(rest.begin(), rest.end(),
                   [](const auto& a, const auto& b) { return a.first < b.first; });
  out->f_rest_count = (uint32_t)rest.size();
  out->sh_degree = infer_degree(out->f_rest_count);
  // byte offsets (binary) or f64 slots (ASCII rows built by ply_ascii_rows);
  // a repeated name resolves to its last occurrence, as the reference's
  // row object keeps the last value written
  std::vector<PlyField> fields(v.props.size());
  uint32_t off = 0;
  for (uint32_t i = 0; i < v.props.size(); ++i) {
    uint32_t t = PLY_F64, b = 8;
    if (!ascii) scalar_type(v.props[i].type, &t, &b);
    fields[i] = PlyField{ascii ? 8 * i : off, t};
    off += ascii ? 8 : b;
  }
  for (int r = 0; r < kPlyRequired; ++r)
    for (uint32_t i = 0; i < v.props.size(); ++i)
      if (v.props[i].name == kRequired[r]) out->req[r] = fields[i];
  // SH coefficients used for colour: channel-major f_rest (the 3DGS layout),
  // the first (d+1)^2 - 1 of each channel's f_rest_count / 3
  if (out->sh_degree > 0 && out->f_rest_count % 3 == 0) {
    const uint32_t per = out->f_rest_count / 3;
    out->sh_k = (out->sh_degree + 1) * (out->sh_degree + 1) - 1;  // <= per by the thresholds
    for (uint32_t c = 0; c < 3; ++c)
      for (uint32_t k = 0; k < out->sh_k; ++k)
        out->rest[c * out->sh_k + k] = fields[rest[c * per + k].second];
  }
  out->stride = ascii ? 8 * out->vertex_props : vstride;
  out->rows_offset = ascii ? 0 : rows_offset;
  return true;
}

bool ply_ascii_rows(const uint8_t* data, size_t size, const PlyLayout& lay,
                    std::vector<double>* rows, std::string* err) {
  // createAsciiValueReader (SceneWorker.ts:287-312): whitespace-separated
  // tokens over all elements in order, each a finite number
  std::vector<Elem> elems;
  uint32_t format = 0;
  uint64_t hb = 0;
  if (!parse_header(data, size, &elems, &format, &hb, err)) return false;
  rows->assign((size_t)lay.count * lay.vertex_props, 0.0);
  size_t pos = hb;
  std::string tok;
  auto next = [&](bool keep, double* out) -> bool {
    while (pos < size && isspace(data[pos])) ++pos;
    if (pos >= size) {
      *err = "Unexpected end of ASCII PLY body";
      return false;
    }
    const size_t a = pos;
    while (pos < size && !isspace(data[pos])) ++pos;
    tok.assign(reinterpret_cast<const char*>(data + a), pos - a);
    char* end = nullptr;
    const double v = std::strtod(tok.c_str(), &end);
    if (*end != '\0' || !std::isfinite(v)) {
      *err = "Invalid ASCII PLY value '" + tok + "'";
      return false;
    }
    if (keep) *out = v;
    return true;
  };
  for (const Elem& e : elems) {
    const bool vert = e.name == "vertex";
    for (uint64_t r = 0; r < e.count; ++r)
      for (size_t k = 0; k < e.props.size(); ++k) {
        double* dst = vert ? &(*rows)[(size_t)r * lay.vertex_props + k] : nullptr;
        if (!next(vert, dst)) return false;
      }
  }
  return true;
}

namespace {

__device__ __forceinline__ uint32_t f2ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ double read_scalar(const uint8_t* p, uint32_t type, bool big) {
  const uint32_t bytes = type <= PLY_U8 ? 1 : type <= PLY_U16 ? 2 : type == PLY_F64 ? 8 : 4;
  uint64_t raw = 0;
  if (!big && ((uintptr_t)p & (bytes - 1)) == 0) {
    switch (bytes) {
      case 1: raw = *p; break;
      case 2: raw = *reinterpret_cast<const uint16_t*>(p); break;
      case 4: raw = *reinterpret_cast<const uint32_t*>(p); break;
      default: raw = *reinterpret_cast<const uint64_t*>(p); break;
    }
  } else {
    for (uint32_t i = 0; i < bytes; ++i) {
      const uint64_t byte = p[i];
      raw |= byte << (8 * (big ? bytes - 1 - i : i));
    }
  }
  switch (type) {
    case PLY_I8: return (double)(int8_t)raw;
    case PLY_U8: return (double)(uint8_t)raw;
    case PLY_I16: return (double)(int16_t)raw;
    case PLY_U16: return (double)(uint16_t)raw;
    case PLY_I32: return (double)(int32_t)raw;
    case PLY_U32: return (double)(uint32_t)raw;
    case PLY_F32: return (double)__uint_as_float((uint32_t)raw);
    default: return __longlong_as_double((long long)raw);
  }
}

struct DecodeArgs {
  const uint8_t* rows;
  uint64_t n;
  uint32_t stride, big, sh_k;  // sh_k: coefficients per channel
  PlyField req[kPlyRequired];
  PlyField rest[kPlyMaxRest];
  float4 *pos, *scale, *rot, *color;
  float* sh;
  uint32_t* bad;
  uint32_t* bounds;
};

__global__ void __launch_bounds__(256) ply_decode_kernel(DecodeArgs a) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < a.n;
  float px = 0.f, py = 0.f, pz = 0.f;
  if (live) {
    const uint8_t* row = a.rows + i * a.stride;
    double v[kPlyRequired];
#pragma unroll
    for (int k = 0; k < kPlyRequired; ++k) {
      v[k] = read_scalar(row + a.req[k].offset, a.req[k].type, a.big);
      if (!isfinite(v[k])) atomicCAS(a.bad, 0u, 1u + k);  // required(): not finite
    }
    const double C0 = 0.28209479177387814;
    auto clamp01 = [](double x) { return fmin(1.0, fmax(0.0, x)); };
    px = (float)v[0];
    py = (float)v[1];
    pz = (float)v[2];
    a.pos[i] = make_float4(px, py, pz, 1.0f);
    a.color[i] = make_float4((float)clamp01(0.5 + C0 * v[11]), (float)clamp01(0.5 + C0 * v[12]),
                             (float)clamp01(0.5 + C0 * v[13]),
                             (float)clamp01(1.0 / (1.0 + exp(-v[3]))));
    a.scale[i] = make_float4((float)exp(v[4]), (float)exp(v[5]), (float)exp(v[6]), 0.0f);
    const double len = hypot(hypot(v[7], v[8]), hypot(v[9], v[10]));
    const double inv = len > 0.0 ? 1.0 / len : 1.0;
    a.rot[i] = make_float4((float)(v[7] * inv), (float)(v[8] * inv), (float)(v[9] * inv),
                           (float)(v[10] * inv));
    if (a.sh_k) {
      float* dst = a.sh + i * 3 * a.sh_k;
      for (uint32_t c = 0; c < 3; ++c)
        for (uint32_t k = 0; k < a.sh_k; ++k) {
          const PlyField f = a.rest[c * a.sh_k + k];
          dst[c * a.sh_k + k] = (float)read_scalar(row + f.offset, f.type, a.big);
        }
    }
  }
  // position bounds: warp reduction, one atomic per warp and word
  uint32_t lo[3] = {live ? f2ord(px) : 0xffffffffu, live ? f2ord(py) : 0xffffffffu,
                    live ? f2ord(pz) : 0xffffffffu};
  uint32_t hi[3] = {live ? f2ord(px) : 0u, live ? f2ord(py) : 0u, live ? f2ord(pz) : 0u};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      atomicMin(a.bounds + c, lo[c]);
      atomicMax(a.bounds + 3 + c, hi[c]);
    }
}

}  // namespace

cudaError_t launch_ply_decode(const uint8_t* rows, uint64_t n, const PlyLayout& lay,
                              bool big_endian, float4* pos, float4* scale,
                              float4* rot, float4* color, float* sh, uint32_t* bad,
                              uint32_t* bounds, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  DecodeArgs a{};
  a.rows = rows;
  a.n = n;
  a.stride = lay.stride;
  a.big = big_endian ? 1u : 0u;
  a.sh_k = lay.sh_k;
  for (int k = 0; k < kPlyRequired; ++k) a.req[k] = lay.req[k];
  for (int k = 0; k < kPlyMaxRest; ++k) a.rest[k] = lay.rest[k];
  a.pos = pos;
  a.scale = scale;
  a.rot = rot;
  a.color = color;
  a.sh = sh;
  a.bad = bad;
  a.bounds = bounds;
  const uint64_t blocks = (n + 255) / 256;
  ply_decode_kernel<<<(unsigned)blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gs3d

extern "C" int gs3d_ply_inspect(const void* data, size_t size, gs3d_ply_info* out) {
  if (!data || !out) {
    gs3d::set_context_free_error("null argument");
    return GS3D_ERR_INVALID_ARG;
  }
  gs3d::PlyLayout lay;
  std::string err;
  if (!gs3d::ply_parse_layout(static_cast<const uint8_t*>(data), size, &lay, &err)) {
    gs3d::set_context_free_error(err.c_str());
    return GS3D_ERR_INVALID_ARG;
  }
  *out = gs3d_ply_info{};
  out->splat_count = lay.count;
  out->header_bytes = lay.header_bytes;
  out->format = lay.format;
  out->f_rest_count = lay.f_rest_count;
  out->sh_degree = lay.sh_degree;
  out->vertex_stride = lay.format == GS3D_PLY_ASCII ? 0u : lay.stride;
  return GS3D_OK;
}
