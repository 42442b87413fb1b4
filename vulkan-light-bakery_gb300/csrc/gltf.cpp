// gltf.cpp -- glTF entry points of include/vlb.h (host code):
//   vlb_gltf_write_light  replaces LightBaker::serialize
//                         (src/baker/light_baker.cpp:372-401)
//   vlb_gltf_read_light   replaces Scene_t::loadBakedLight
//                         (src/scene_manager.cpp:614-648)
// The document model and its printing follow the reference's JSON library
// (json.h); base64 is the standard alphabet with '=' padding
// (light_baker.cpp:330-370), and decoding stops at the first '=' or
// non-alphabet character as the reference's decoder does
// (scene_manager.cpp:556-612).
#include <cstring>
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

}  // namespace

extern "C" {

const char* vlb_gltf_last_error(void) { return t_gltf_err.c_str(); }

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
