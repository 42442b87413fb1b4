// gltf.cpp -- glTF entry points of include/vlb.h (host code):
//   vlb_gltf_write_light  replaces LightBaker::serialize
//                         (src/baker/light_baker.cpp:375-401)
//   vlb_gltf_read_light   replaces Scene_t::loadBakedLight
//                         (src/scene_manager.cpp:613-648)
//   vlb_gltf_mesh_*       replace the geometry side of Scene_t::loadNodes /
//                         loadNode / fetchVertices / fetchIndices / loadMatrix
//                         (src/scene_manager.cpp:257-337, 445-533, 860-870)
// The document model and its printing follow the reference's JSON library
// (json.h); base64 is the standard alphabet with '=' padding
// (light_baker.cpp:330-373), and decoding stops at the first '=' or
// non-alphabet character as the reference's decoder does
// (scene_manager.cpp:556-611).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "json.h"
#include "vlb_internal.h"

namespace {

const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
const char kDataUri[] = "data:application/octet-stream;base64,";

std::string b64_encode(const uint8_t* p, size_t n) {
  std::string s;
  s.reserve((n + 2) / 3 * 4);
  size_t i = 0;
  for (; i + 3 <= n; i += 3) {
    const uint32_t v = (uint32_t(p[i]) << 16) | (uint32_t(p[i + 1]) << 8) | p[i + 2];
    s += kB64[v >> 18];
    s += kB64[(v >> 12) & 63];
    s += kB64[(v >> 6) & 63];
    s += kB64[v & 63];
  }
  if (i < n) {
    const uint32_t v = (uint32_t(p[i]) << 16) | (i + 1 < n ? uint32_t(p[i + 1]) << 8 : 0u);
    s += kB64[v >> 18];
    s += kB64[(v >> 12) & 63];
    s += i + 1 < n ? kB64[(v >> 6) & 63] : '=';
    s += '=';
  }
  return s;
}

int b64_index(char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '+') return 62;
  if (c == '/') return 63;
  return -1;
}

std::vector<uint8_t> b64_decode(const std::string& s, size_t from) {
  std::vector<uint8_t> out;
  uint32_t acc = 0;
  int nb = 0;
  for (size_t i = from; i < s.size(); ++i) {
    const int x = b64_index(s[i]);
    if (x < 0) break;  // '=' or any other character ends the data
    acc = (acc << 6) | uint32_t(x);
    if (++nb == 4) {
      out.push_back(uint8_t(acc >> 16));
      out.push_back(uint8_t(acc >> 8));
      out.push_back(uint8_t(acc));
      acc = 0;
      nb = 0;
    }
  }
  if (nb >= 2) {  // 2 or 3 leftover characters carry 1 or 2 bytes
    acc <<= 6 * (4 - nb);
    out.push_back(uint8_t(acc >> 16));
    if (nb == 3) out.push_back(uint8_t(acc >> 8));
  }
  return out;
}

thread_local std::string t_gltf_err;
vlb_status gfail(vlb_status st, const std::string& m) {
  t_gltf_err = m;
  return st;
}

// ---- scene geometry ------------------------------------------------------------------
// World-space triangles of glTF scene 0 (the reference loads model.scenes[0],
// scene_manager.cpp:860-870): every node's local matrix is
// T * R * S * M (translation, rotation quaternion, scale, matrix --
// Scene_t::loadMatrix, :466-477) and a mesh's world matrix is the product
// along its parent chain (Node_t::getMatrix, :447-463, which the reference
// hands to the TLAS instances).  Positions are transformed in FP64 and
// rounded once to FP32.  Albedo per triangle: the material's
// pbrMetallicRoughness.baseColorFactor RGB (glTF default 1, also for
// primitives without a material -- the reference's trailing default
// material, :851); textures are not sampled.  Bounds: the exact world AABB
// of all vertices (the reference transforms only the two corners of each
// primitive's local box by the node's local matrix, :495-506).
struct Mesh {
  std::vector<float> pos;
  std::vector<uint32_t> idx;
  std::vector<float> alb;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
};

// 4x4 matrices column-major, like glTF.
void mat_mul(const double* a, const double* b, double* o) {
  double r[16];
  for (int c = 0; c < 4; ++c)
    for (int rr = 0; rr < 4; ++rr) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += a[k * 4 + rr] * b[c * 4 + k];
      r[c * 4 + rr] = s;
    }
  std::memcpy(o, r, sizeof r);
}

bool read_file(const std::string& path, std::vector<uint8_t>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? size_t(n) : 0);
  const bool ok = n >= 0 && std::fread(out->data(), 1, out->size(), f) == out->size();
  std::fclose(f);
  return ok;
}

std::string uri_decode(const std::string& u) {
  std::string o;
  for (size_t i = 0; i < u.size(); ++i) {
    if (u[i] == '%' && i + 2 < u.size()) {
      o += char(std::strtol(u.substr(i + 1, 2).c_str(), nullptr, 16));
      i += 2;
    } else {
      o += u[i];
    }
  }
  return o;
}

struct Loader {
  vlbj::Value doc;
  std::vector<std::vector<uint8_t>> buffers;
  std::string dir, err;
  Mesh mesh;

  bool fail(const std::string& m) {
    err = m;
    return false;
  }
  const vlbj::Value* arr(const char* name, size_t i) const {
    const vlbj::Value* a = doc.get(name);
    return a ? a->at(i) : nullptr;
  }
  static int64_t geti(const vlbj::Value* o, const char* k, int64_t dflt) {
    const vlbj::Value* v = o ? o->get(k) : nullptr;
    return v && v->is_number() ? v->as_int() : dflt;
  }

  bool load_buffers(const std::vector<uint8_t>* glb_bin) {
    const vlbj::Value* bs = doc.get("buffers");
    const size_t nb = bs && bs->type == vlbj::Value::kArray ? bs->a.size() : 0;
    buffers.resize(nb);
    for (size_t i = 0; i < nb; ++i) {
      const vlbj::Value* u = bs->a[i].get("uri");
      const int64_t len = geti(&bs->a[i], "byteLength", -1);
      if (!u) {
        if (!glb_bin || i != 0) return fail("buffer without uri outside a GLB's first buffer");
        buffers[i] = *glb_bin;
      } else if (u->type != vlbj::Value::kString) {
        return fail("buffer uri is not a string");
      } else if (u->s.compare(0, 5, "data:") == 0) {
        const size_t comma = u->s.find(',');
        if (comma == std::string::npos || u->s.rfind(";base64", comma) == std::string::npos)
          return fail("data URI buffers must be base64");
        buffers[i] = b64_decode(u->s, comma + 1);
      } else if (!read_file(dir + uri_decode(u->s), &buffers[i])) {
        return fail("cannot read buffer file " + dir + u->s);
      }
      if (len < 0 || buffers[i].size() < size_t(len)) return fail("buffer shorter than its byteLength");
    }
    return true;
  }

  // Accessor element i -> pointer (bounds-checked), component type, components.
  struct View {
    const uint8_t* base = nullptr;
    size_t stride = 0, count = 0;
    int ctype = 0, ncomp = 0;
  };
  bool accessor(int64_t ai, View* v) {
    const vlbj::Value* a = arr("accessors", size_t(ai));
    if (!a || ai < 0) return fail("accessor index out of range");
    if (a->get("sparse")) return fail("sparse accessors are not supported");
    const vlbj::Value* t = a->get("type");
    const std::string type = t && t->type == vlbj::Value::kString ? t->s : "";
    v->ncomp = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
    if (!v->ncomp) return fail("unsupported accessor type " + type);
    v->ctype = int(geti(a, "componentType", 0));
    const int csize = v->ctype == 5126 || v->ctype == 5125 ? 4 : v->ctype == 5123 || v->ctype == 5122 ? 2
                      : v->ctype == 5121 || v->ctype == 5120 ? 1 : 0;
    if (!csize) return fail("unsupported component type");
    v->count = size_t(geti(a, "count", 0));
    const vlbj::Value* bv = arr("bufferViews", size_t(geti(a, "bufferView", -1)));
    if (!bv) return fail("accessor without a bufferView");
    const int64_t b = geti(bv, "buffer", -1);
    if (b < 0 || size_t(b) >= buffers.size()) return fail("bufferView buffer out of range");
    const size_t off = size_t(geti(bv, "byteOffset", 0)) + size_t(geti(a, "byteOffset", 0));
    const size_t elem = size_t(csize) * size_t(v->ncomp);
    v->stride = size_t(geti(bv, "byteStride", 0));
    if (v->stride == 0) v->stride = elem;
    const size_t view_end = size_t(geti(bv, "byteOffset", 0)) + size_t(geti(bv, "byteLength", 0));
    if (v->count && (off + (v->count - 1) * v->stride + elem > view_end || view_end > buffers[size_t(b)].size()))
      return fail("accessor reads past its bufferView");
    v->base = buffers[size_t(b)].data() + off;
    return true;
  }

  bool primitive(const vlbj::Value& p, const double* world) {
    const int64_t mode = geti(&p, "mode", 4);
    if (mode != 4) return true;  // triangles only (the reference builds triangle BLAS geometry)
    const vlbj::Value* attrs = p.get("attributes");
    const vlbj::Value* pa = attrs ? attrs->get("POSITION") : nullptr;
    if (!pa || !pa->is_number()) return fail("primitive without POSITION");
    View pv;
    if (!accessor(pa->as_int(), &pv)) return false;
    if (pv.ncomp != 3 || pv.ctype != 5126) return fail("POSITION must be float VEC3");
    const uint32_t base = uint32_t(mesh.pos.size() / 3);
    for (size_t i = 0; i < pv.count; ++i) {
      float lp[3];
      std::memcpy(lp, pv.base + i * pv.stride, 12);
      for (int r = 0; r < 3; ++r) {
        const double w = world[r] * lp[0] + world[4 + r] * lp[1] + world[8 + r] * lp[2] + world[12 + r];
        const float f = float(w);
        mesh.pos.push_back(f);
        mesh.lo[r] = std::min(mesh.lo[r], double(f));
        mesh.hi[r] = std::max(mesh.hi[r], double(f));
      }
    }
    std::vector<uint32_t> ix;
    const vlbj::Value* ia = p.get("indices");
    if (ia && ia->is_number()) {
      View iv;
      if (!accessor(ia->as_int(), &iv)) return false;
      if (iv.ncomp != 1) return fail("indices must be SCALAR");
      for (size_t i = 0; i < iv.count; ++i) {
        const uint8_t* q = iv.base + i * iv.stride;
        uint32_t x;
        if (iv.ctype == 5125) std::memcpy(&x, q, 4);
        else if (iv.ctype == 5123) { uint16_t y; std::memcpy(&y, q, 2); x = y; }
        else if (iv.ctype == 5121) x = *q;
        else return fail("index component type not supported");  // scene_manager.cpp:327
        if (x >= pv.count) return fail("index out of range");
        ix.push_back(x);
      }
    } else {
      for (size_t i = 0; i < pv.count; ++i) ix.push_back(uint32_t(i));
    }
    float rgb[3] = {1.f, 1.f, 1.f};
    const vlbj::Value* mat = p.get("material") ? arr("materials", size_t(geti(&p, "material", -1))) : nullptr;
    const vlbj::Value* pbr = mat ? mat->get("pbrMetallicRoughness") : nullptr;
    const vlbj::Value* bc = pbr ? pbr->get("baseColorFactor") : nullptr;
    if (bc && bc->type == vlbj::Value::kArray && bc->a.size() >= 3)
      for (int c = 0; c < 3; ++c) rgb[c] = float(bc->a[size_t(c)].as_double());
    for (size_t t = 0; t + 3 <= ix.size(); t += 3) {
      for (int k = 0; k < 3; ++k) mesh.idx.push_back(base + ix[t + size_t(k)]);
      mesh.alb.insert(mesh.alb.end(), rgb, rgb + 3);
    }
    return true;
  }

  bool node(int64_t ni, const double* parent, int depth, std::set<int64_t>& path) {
    const vlbj::Value* n = arr("nodes", size_t(ni));
    if (!n || ni < 0) return fail("node index out of range");
    if (depth > 256 || path.count(ni)) return fail("node hierarchy has a cycle");
    path.insert(ni);
    // local = T * R * S * M
    double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}, R[16], S[16], M[16], L[16], W[16];
    std::memcpy(R, T, sizeof T);
    std::memcpy(S, T, sizeof T);
    std::memcpy(M, T, sizeof T);
    auto vec = [&](const char* k, size_t nexp, double* out) {
      const vlbj::Value* v = n->get(k);
      if (!v || v->type != vlbj::Value::kArray || v->a.size() != nexp) return false;
      for (size_t i = 0; i < nexp; ++i) out[i] = v->a[i].as_double();
      return true;
    };
    double t[3], q[4], sc[3];
    if (vec("translation", 3, t)) { T[12] = t[0]; T[13] = t[1]; T[14] = t[2]; }
    if (vec("rotation", 4, q)) {  // (x, y, z, w)
      const double x = q[0], y = q[1], z = q[2], w = q[3];
      R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y + z * w);     R[2] = 2 * (x * z - y * w);
      R[4] = 2 * (x * y - z * w);     R[5] = 1 - 2 * (x * x + z * z); R[6] = 2 * (y * z + x * w);
      R[8] = 2 * (x * z + y * w);     R[9] = 2 * (y * z - x * w);     R[10] = 1 - 2 * (x * x + y * y);
    }
    if (vec("scale", 3, sc)) { S[0] = sc[0]; S[5] = sc[1]; S[10] = sc[2]; }
    vec("matrix", 16, M);
    mat_mul(T, R, L);
    mat_mul(L, S, L);
    mat_mul(L, M, L);
    mat_mul(parent, L, W);
    const int64_t mi = geti(n, "mesh", -1);
    if (mi >= 0) {
      const vlbj::Value* m = arr("meshes", size_t(mi));
      const vlbj::Value* prims = m ? m->get("primitives") : nullptr;
      if (!prims || prims->type != vlbj::Value::kArray) return fail("mesh without primitives");
      for (const auto& p : prims->a)
        if (!primitive(p, W)) return false;
    }
    const vlbj::Value* ch = n->get("children");
    if (ch && ch->type == vlbj::Value::kArray)
      for (const auto& c : ch->a)
        if (!node(c.as_int(), W, depth + 1, path)) return false;
    path.erase(ni);
    return true;
  }

  bool load(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    dir = slash == std::string::npos ? "" : path.substr(0, slash + 1);
    std::vector<uint8_t> file, bin;
    if (!read_file(path, &file)) return fail("cannot read " + path);
    const char* json = reinterpret_cast<const char*>(file.data());
    size_t json_len = file.size();
    bool glb = false;
    if (file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0) {  // GLB container
      glb = true;
      uint32_t hdr[3];
      std::memcpy(hdr, file.data(), 12);
      if (hdr[1] != 2 || hdr[2] > file.size()) return fail("bad GLB header");
      size_t pos = 12;
      json = nullptr;
      while (pos + 8 <= hdr[2]) {
        uint32_t ch[2];
        std::memcpy(ch, file.data() + pos, 8);
        if (pos + 8 + ch[0] > hdr[2]) return fail("bad GLB chunk");
        if (ch[1] == 0x4E4F534Au && !json) { json = reinterpret_cast<const char*>(file.data() + pos + 8); json_len = ch[0]; }
        else if (ch[1] == 0x004E4942u && bin.empty()) bin.assign(file.data() + pos + 8, file.data() + pos + 8 + ch[0]);
        pos += 8 + size_t(ch[0]) + ((4 - ch[0] % 4) % 4);
      }
      if (!json) return fail("GLB without a JSON chunk");
    }
    std::string perr;
    if (!vlbj::parse(json, json_len, &doc, &perr)) return fail("glTF JSON: " + perr);
    if (!load_buffers(glb ? &bin : nullptr)) return false;
    const double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::set<int64_t> pathset;
    const vlbj::Value* sc = arr("scenes", 0);
    if (sc) {
      const vlbj::Value* roots = sc->get("nodes");
      if (roots && roots->type == vlbj::Value::kArray)
        for (const auto& r : roots->a)
          if (!node(r.as_int(), I, 0, pathset)) return false;
    } else {  // no scenes: every node that is nobody's child
      const vlbj::Value* ns = doc.get("nodes");
      const size_t nn = ns && ns->type == vlbj::Value::kArray ? ns->a.size() : 0;
      std::vector<bool> child(nn, false);
      for (size_t i = 0; i < nn; ++i) {
        const vlbj::Value* ch = ns->a[i].get("children");
        if (ch && ch->type == vlbj::Value::kArray)
          for (const auto& c : ch->a)
            if (c.as_int() >= 0 && size_t(c.as_int()) < nn) child[size_t(c.as_int())] = true;
      }
      for (size_t i = 0; i < nn; ++i)
        if (!child[i] && !node(int64_t(i), I, 0, pathset)) return false;
    }
    return true;
  }
};

}  // namespace

struct vlb_gltf_mesh {
  Mesh m;
};

extern "C" {

const char* vlb_gltf_last_error(void) { return t_gltf_err.c_str(); }

vlb_status vlb_gltf_mesh_load(const char* path, vlb_gltf_mesh** out) {
  if (!path || !out) return gfail(VLB_ERR_INVALID, "null argument");
  *out = nullptr;
  Loader ld;
  if (!ld.load(path)) return gfail(VLB_ERR_INVALID, ld.err);
  if (ld.mesh.pos.size() / 3 > 0xFFFFFFFFull || ld.mesh.idx.size() / 3 > 0xFFFFFFFFull)
    return gfail(VLB_ERR_INVALID, "mesh too large");
  auto* m = new (std::nothrow) vlb_gltf_mesh();
  if (!m) return gfail(VLB_ERR_OOM, "out of host memory");
  m->m = std::move(ld.mesh);
  *out = m;
  return VLB_OK;
}

void vlb_gltf_mesh_free(vlb_gltf_mesh* m) { delete m; }

vlb_status vlb_gltf_mesh_info(const vlb_gltf_mesh* m, uint32_t* nverts, uint32_t* ntris, float bounds[6]) {
  if (!m) return gfail(VLB_ERR_INVALID, "null mesh");
  if (nverts) *nverts = uint32_t(m->m.pos.size() / 3);
  if (ntris) *ntris = uint32_t(m->m.idx.size() / 3);
  if (bounds) {
    const bool empty = m->m.pos.empty();
    for (int a = 0; a < 3; ++a) {
      bounds[a] = empty ? 0.f : float(m->m.lo[a]);
      bounds[3 + a] = empty ? 0.f : float(m->m.hi[a]);
    }
  }
  return VLB_OK;
}

vlb_status vlb_gltf_mesh_get(const vlb_gltf_mesh* m, float* positions, uint32_t* indices, float* albedo) {
  if (!m) return gfail(VLB_ERR_INVALID, "null mesh");
  if (positions) std::memcpy(positions, m->m.pos.data(), m->m.pos.size() * 4);
  if (indices) std::memcpy(indices, m->m.idx.data(), m->m.idx.size() * 4);
  if (albedo) std::memcpy(albedo, m->m.alb.data(), m->m.alb.size() * 4);
  return VLB_OK;
}

vlb_status vlb_scene_create_gltf(vlb_ctx* ctx, const char* path, vlb_scene** out) {
  if (!ctx || !out) return VLB_ERR_INVALID;
  vlb_gltf_mesh* m = nullptr;
  vlb_status st = vlb_gltf_mesh_load(path, &m);
  if (st) return vlbh::ctx_fail(ctx, st, t_gltf_err.c_str());
  st = vlb_scene_create(ctx, m->m.pos.data(), 12, uint32_t(m->m.pos.size() / 3), m->m.idx.data(),
                        uint32_t(m->m.idx.size() / 3), m->m.alb.data(), out);
  vlb_gltf_mesh_free(m);
  return st;
}

vlb_status vlb_gltf_write_light(const char* gltf_json, size_t json_len, const float* coeffs, uint32_t nprobes,
                                uint32_t coeff_count, const float grid_step[3], char* out, size_t out_cap,
                                size_t* out_len) {
  if (!gltf_json || !grid_step || !out_len || (nprobes && !coeffs)) return gfail(VLB_ERR_INVALID, "null argument");
  if (coeff_count == 0) return gfail(VLB_ERR_INVALID, "coeff_count must be positive");
  vlbj::Value doc;
  std::string err;
  if (!vlbj::parse(gltf_json, json_len, &doc, &err)) return gfail(VLB_ERR_INVALID, "glTF JSON: " + err);
  if (doc.type != vlbj::Value::kObject) return gfail(VLB_ERR_INVALID, "glTF root is not an object");
  const size_t nbytes = size_t(nprobes) * coeff_count * 3 * sizeof(float);
  // buffers[] += {byteLength, uri}
  vlbj::Value& buffers = doc.o["buffers"];
  if (buffers.type == vlbj::Value::kNull) buffers = vlbj::Value::array();
  if (buffers.type != vlbj::Value::kArray) return gfail(VLB_ERR_INVALID, "\"buffers\" is not an array");
  vlbj::Value buf = vlbj::Value::object();
  buf.o["byteLength"] = vlbj::Value::uinteger(nbytes);
  buf.o["uri"] = vlbj::Value::string(kDataUri + b64_encode(reinterpret_cast<const uint8_t*>(coeffs), nbytes));
  buffers.a.push_back(std::move(buf));
  // bufferViews[] += {buffer, byteLength, byteOffset}
  vlbj::Value& views = doc.o["bufferViews"];
  if (views.type == vlbj::Value::kNull) views = vlbj::Value::array();
  if (views.type != vlbj::Value::kArray) return gfail(VLB_ERR_INVALID, "\"bufferViews\" is not an array");
  vlbj::Value view = vlbj::Value::object();
  view.o["buffer"] = vlbj::Value::uinteger(buffers.a.size() - 1);
  view.o["byteLength"] = vlbj::Value::uinteger(nbytes);
  view.o["byteOffset"] = vlbj::Value::integer(0);
  views.a.push_back(std::move(view));
  // light {gridStep {x, y, z}, lmax, bufferView}
  vlbj::Value& light = doc.o["light"];
  if (light.type == vlbj::Value::kNull) light = vlbj::Value::object();
  if (light.type != vlbj::Value::kObject) return gfail(VLB_ERR_INVALID, "\"light\" is not an object");
  vlbj::Value gs = vlbj::Value::object();
  gs.o["x"] = vlbj::Value::number(double(grid_step[0]));
  gs.o["y"] = vlbj::Value::number(double(grid_step[1]));
  gs.o["z"] = vlbj::Value::number(double(grid_step[2]));
  light.o["gridStep"] = std::move(gs);
  light.o["lmax"] = vlbj::Value::uinteger(coeff_count);
  light.o["bufferView"] = vlbj::Value::uinteger(views.a.size() - 1);
  std::string text = vlbj::dump(doc);
  text += '\n';
  *out_len = text.size() + 1;
  if (!out) return VLB_OK;
  if (out_cap < text.size() + 1) return gfail(VLB_ERR_INVALID, "output buffer too small");
  std::memcpy(out, text.c_str(), text.size() + 1);
  return VLB_OK;
}

vlb_status vlb_gltf_read_light(const char* gltf_json, size_t json_len, float grid_step[3], uint32_t* coeff_count,
                               void* coeffs, size_t coeffs_cap, size_t* coeffs_bytes) {
  if (!gltf_json || !grid_step || !coeff_count || !coeffs_bytes) return gfail(VLB_ERR_INVALID, "null argument");
  vlbj::Value doc;
  std::string err;
  if (!vlbj::parse(gltf_json, json_len, &doc, &err)) return gfail(VLB_ERR_INVALID, "glTF JSON: " + err);
  const vlbj::Value* light = doc.get("light");
  if (!light || (light->type == vlbj::Value::kObject && light->o.empty()) || light->type == vlbj::Value::kNull) {
    grid_step[0] = grid_step[1] = grid_step[2] = 0.f;  // no baked light (scene_manager.cpp:639-645)
    *coeff_count = 0;
    *coeffs_bytes = 0;
    return VLB_OK;
  }
  const vlbj::Value* gs = light->get("gridStep");
  const vlbj::Value* lm = light->get("lmax");
  const vlbj::Value* bv = light->get("bufferView");
  if (!gs || !lm || !bv || !lm->is_number() || !bv->is_number())
    return gfail(VLB_ERR_INVALID, "\"light\" needs gridStep, lmax and bufferView");
  const char* axes[3] = {"x", "y", "z"};
  for (int a = 0; a < 3; ++a) {
    const vlbj::Value* c = gs->get(axes[a]);
    if (!c || !c->is_number()) return gfail(VLB_ERR_INVALID, "gridStep needs numeric x, y, z");
    grid_step[a] = float(c->as_double());
  }
  const vlbj::Value* views = doc.get("bufferViews");
  const vlbj::Value* view = views ? views->at(size_t(bv->as_int())) : nullptr;
  const vlbj::Value* bidx = view ? view->get("buffer") : nullptr;
  const vlbj::Value* buffers = doc.get("buffers");
  const vlbj::Value* buf = (buffers && bidx && bidx->is_number()) ? buffers->at(size_t(bidx->as_int())) : nullptr;
  const vlbj::Value* uri = buf ? buf->get("uri") : nullptr;
  const vlbj::Value* len = buf ? buf->get("byteLength") : nullptr;
  if (!uri || uri->type != vlbj::Value::kString || !len || !len->is_number())
    return gfail(VLB_ERR_INVALID, "light bufferView does not lead to a buffer with uri and byteLength");
  const size_t hdr = std::strlen(kDataUri);
  if (uri->s.compare(0, hdr, kDataUri) != 0) return gfail(VLB_ERR_UNSUPPORTED, "light buffer is not a base64 data URI");
  const std::vector<uint8_t> data = b64_decode(uri->s, hdr);
  const size_t n = size_t(len->as_int());
  if (data.size() < n) return gfail(VLB_ERR_INVALID, "light buffer holds fewer bytes than its byteLength");
  *coeff_count = uint32_t(lm->as_int());
  *coeffs_bytes = n;
  if (!coeffs) return VLB_OK;
  if (coeffs_cap < n) return gfail(VLB_ERR_INVALID, "coefficient buffer too small");
  std::memcpy(coeffs, data.data(), n);
  return VLB_OK;
}

}  // extern "C"
