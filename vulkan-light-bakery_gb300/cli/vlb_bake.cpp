// vlb-bake -- command-line baker over libvlb.so, the replacement of the
// reference's `baker` executable (src/baker/main.cpp:8-45, LightBaker::
// LightBaker / bake / serialize, src/baker/light_baker.cpp:19-401).
//
//   vlb-bake scene.gltf [options]
//
// As the reference: the scene's triangles (glTF scene 0), a probe grid of
// counts (default 7 x 7 x 7) over the scene bounds starting at the origin
// (Scene_t::getBounds), probes in the reference's breadth-first order,
// 16 coefficients (L3) per probe, and the input document re-written with the
// coefficient buffer and the `light` object to baked_<file name> next to the
// input (the reference writes "baked_" + the path it was given).
//
// Options:
//   --counts NX NY NZ    probes per axis (default 7 7 7)
//   --dirs fib:N | equirect:WxH
//                        sample directions (default equirect:3141x1000, the
//                        reference's env map; fib:N = spherical Fibonacci)
//   --lmax 2|3           coefficients 9 or 16 (default 3, the file's layout)
//   --sun X Y Z          direction toward the sun (default 0 1 0)
//   --intensity I        sun intensity (default 5)
//   --precision fp32|fused|mixed|bf16   (default fp32: FP32 trace into a radiance tile,
//                        then the projection -- on the reference's few-probe,
//                        many-ray bake measured faster than fused, the one
//                        kernel without a tile; both within 1e-4 of FP64)
//   --shading sun|ref    sun: Lambert + the sun above (default); ref: the
//                        reference baker's own shading (point light, Phong,
//                        sRGB, 8-bit samples; shaders/env_map.rchit:51-102)
//   --light X Y Z        the ref shading's point light (default 1 10 1)
//   --accumulate         write the reference's running sums (probe i holds
//                        probes 0..i: its coefficient buffer is never cleared)
//   --out PATH           output file (default baked_<name> next to the input)
//   --device N           CUDA device (default 0)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "vlb.h"

namespace {

void check(vlb_ctx* ctx, vlb_status st, const char* what) {
  if (st != VLB_OK)
    throw std::runtime_error(std::string(what) + ": " + (ctx ? vlb_last_error(ctx) : vlb_status_string(st)));
}

std::string read_text(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot read " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc < 2) throw std::runtime_error("Select scene to bake.");
    std::string in = argv[1], out, dirs = "equirect:3141x1000", prec = "fp32";
    uint32_t counts[3] = {7, 7, 7};
    uint32_t lmax = 3;
    int device = 0;
    float sun[3] = {0.f, 1.f, 0.f}, intensity = 5.f, light[3] = {1.f, 10.f, 1.f};
    std::string shading = "sun";
    bool accumulate = false;
    for (int i = 2; i < argc; ++i) {
      const std::string o = argv[i];
      auto need = [&](int n) {
        if (i + n >= argc) throw std::runtime_error("missing value for " + o);
      };
      if (o == "--counts") { need(3); for (int a = 0; a < 3; ++a) counts[a] = uint32_t(std::atoi(argv[++i])); }
      else if (o == "--dirs") { need(1); dirs = argv[++i]; }
      else if (o == "--lmax") { need(1); lmax = uint32_t(std::atoi(argv[++i])); }
      else if (o == "--sun") { need(3); for (float& c : sun) c = float(std::atof(argv[++i])); }
      else if (o == "--intensity") { need(1); intensity = float(std::atof(argv[++i])); }
      else if (o == "--precision") { need(1); prec = argv[++i]; }
      else if (o == "--shading") { need(1); shading = argv[++i]; }
      else if (o == "--light") { need(3); for (float& c : light) c = float(std::atof(argv[++i])); }
      else if (o == "--accumulate") accumulate = true;
      else if (o == "--out") { need(1); out = argv[++i]; }
      else if (o == "--device") { need(1); device = std::atoi(argv[++i]); }
      else throw std::runtime_error("unknown option " + o);
    }
    unsigned dw = 0, dh = 0;
    const bool fib = dirs.rfind("fib:", 0) == 0;
    if (fib ? std::sscanf(dirs.c_str() + 4, "%u", &dw) != 1
            : dirs.rfind("equirect:", 0) != 0 || std::sscanf(dirs.c_str() + 9, "%ux%u", &dw, &dh) != 2)
      throw std::runtime_error("bad --dirs " + dirs);
    if (prec != "fp32" && prec != "fused" && prec != "mixed" && prec != "bf16")
      throw std::runtime_error("bad --precision " + prec);
    if (shading != "sun" && shading != "ref") throw std::runtime_error("bad --shading " + shading);
    const std::string src = read_text(in);  // the document re-written after the bake
    if (src.compare(0, 4, "glTF") == 0)
      throw std::runtime_error("binary glTF input: the baked file is written from a JSON .gltf document");
    if (out.empty()) {
      const size_t slash = in.find_last_of('/');
      out = (slash == std::string::npos ? std::string() : in.substr(0, slash + 1)) + "baked_" +
            (slash == std::string::npos ? in : in.substr(slash + 1));
    }
    vlb_ctx* ctx = nullptr;
    check(nullptr, vlb_ctx_create(device, &ctx), "vlb_ctx_create");
    vlb_scene* scene = nullptr;
    vlb_dirset* ds = nullptr;
    struct Guard {
      vlb_ctx*& c; vlb_scene*& s; vlb_dirset*& d;
      ~Guard() { vlb_dirset_destroy(d); vlb_scene_destroy(s); vlb_ctx_destroy(c); }
    } guard{ctx, scene, ds};
    check(ctx, vlb_scene_create_gltf(ctx, in.c_str(), &scene), "scene");
    float bounds[6];
    check(ctx, vlb_scene_bounds(scene, 1, bounds), "bounds");  // from the origin, as Scene_t::getBounds
    const size_t np = size_t(counts[0]) * counts[1] * counts[2];
    if (np == 0) throw std::runtime_error("probe counts must be positive");
    std::vector<float> probes(np * 3);
    float step[3];
    check(ctx, vlb_probe_grid_ref_order(bounds, counts, probes.data(), step), "probe grid");
    if (fib)
      check(ctx, vlb_dirset_create_fibonacci(ctx, dw, VLB_FRAME_WORLD, &ds), "dirs");
    else
      check(ctx, vlb_dirset_create_equirect(ctx, dw, dh, &ds), "dirs");
    vlb_bake_params p;
    vlb_bake_params_default(&p);
    p.lmax = lmax;
    p.precision = prec == "fp32"    ? VLB_PREC_FP32
                  : prec == "mixed" ? VLB_PREC_MIXED
                  : prec == "bf16"  ? VLB_PREC_BF16
                                    : VLB_PREC_FUSED;
    for (int a = 0; a < 3; ++a) p.sun_dir[a] = sun[a];
    p.sun_intensity = intensity;
    p.shading = shading == "ref" ? VLB_SHADE_REF_PHONG : VLB_SHADE_LAMBERT_SUN;
    for (int a = 0; a < 3; ++a) p.light_pos[a] = light[a];
    if (accumulate) p.flags |= VLB_BAKE_REF_ACCUMULATE;
    p.dirs = ds;
    const uint32_t K = (lmax + 1) * (lmax + 1);
    std::vector<float> sh(np * K * 3);
    check(ctx, vlb_bake(ctx, scene, probes.data(), uint32_t(np), &p, sh.data()), "bake");
    size_t n = 0;
    if (vlb_gltf_write_light(src.data(), src.size(), sh.data(), uint32_t(np), K, step, nullptr, 0, &n) != VLB_OK)
      throw std::runtime_error(std::string("serialize: ") + vlb_gltf_last_error());
    std::string text(n, '\0');
    if (vlb_gltf_write_light(src.data(), src.size(), sh.data(), uint32_t(np), K, step, &text[0], n, &n) != VLB_OK)
      throw std::runtime_error(std::string("serialize: ") + vlb_gltf_last_error());
    std::ofstream o(out, std::ios::binary);
    o << text.c_str();
    if (!o) throw std::runtime_error("cannot write " + out);
    std::printf("baked %zu probes x %u coefficients -> %s\n", np, K, out.c_str());
  } catch (const std::exception& e) {
    std::fprintf(stderr, "std::exception: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
