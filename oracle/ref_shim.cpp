// ref_shim.cpp -- compiles the reference's own shaders/sh_common.h as C++.
//
// TEST INFRASTRUCTURE ONLY (builds oracle/_ref/libshref.so).  The reference
// header is GLSL-flavoured C; this file supplies the few GLSL names it uses
// (vec3, normalize, sin/cos on float) and includes the header from the
// reference checkout, so the reference's basis constants and angle maps run
// unmodified.  Nothing of the header is copied into this repository.  The
// library is used only to pin the FP64 oracle and to generate the golden
// fixtures under tests/golden/.
#include <cmath>

namespace ref {
using std::cos;
using std::sin;

struct vec3 {
  float x, y, z;
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline vec3 normalize(vec3 v) {
  const float n = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  return vec3(v.x / n, v.y / n, v.z / n);
}

#include "sh_common.h"  // found through -I<reference>/shaders
}  // namespace ref

extern "C" {
float ref_sh(int l, int m, float x, float y, float z) { return ref::SH(l, m, ref::vec3(x, y, z)); }
float ref_x2phi(int x, int w) { return ref::x2phi(x, w); }
float ref_y2theta(int y, int h) { return ref::y2theta(y, h); }
void ref_to_vector(float phi, float theta, float* out) {
  const ref::vec3 v = ref::toVector(phi, theta);
  out[0] = v.x; out[1] = v.y; out[2] = v.z;
}
float ref_pi(void) { return PI; }
}
