"""ctypes front end of the FP64 oracle (oracle/vlb_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline / reference legs of bench.py.  It is the checker and the timed
CPU baseline, never part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_PATH = HERE / "_ref" / "libshref.so"


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} missing; build it with __graft_entry__.build() or make -C oracle")
    lib = C.CDLL(str(LIB_PATH))
    P, U32, I32, D, F = C.c_void_p, C.c_uint32, C.c_int, C.c_double, C.c_float
    sig = {
        "orc_version": (I32, []),
        "orc_sh_basis": (None, [I32, P, U32, P]),
        "orc_x2phi_y2theta": (None, [I32, I32, I32, I32, P, P]),
        "orc_to_vector": (None, [D, D, P]),
        "orc_dirs_fibonacci": (None, [U32, P, P]),
        "orc_dirs_equirect": (None, [U32, U32, P, P, P]),
        "orc_cube_solid_angle": (None, [U32, P]),
        "orc_cube_texel_dirs": (None, [U32, P]),
        "orc_cube_select": (None, [P, U32, U32, P]),
        "orc_skybox_sh": (None, [P, I32, I32, U32, U32, I32, U32, P]),
        "orc_project": (None, [P, U32, U32, P, I32, P, I32]),
        "orc_sh_eval_envmap": (None, [P, I32, U32, U32, D, P]),
        "orc_probe_grid_ref_order": (U32, [P, P, P, P]),
        "orc_lbvh_build": (I32, [P, U32, P, U32, P, P, P, P]),
        "orc_scene_create": (P, [P, U32, P, U32, P]),
        "orc_scene_destroy": (None, [P]),
        "orc_bake": (None, [P, P, U32, P, U32, P, I32, P, F, F, F, F, P, U32, P, P, I32, P, P, P, P, P, I32, P]),
        "orc_ray_tri": (I32, [P, P, P, I32, P, P, P, P]),
        "orc_shadow_margin": (D, [P, P, P, D, D]),
        "orc_closest_hit": (None, [P, P, P, D, D, P, P]),
        "orc_probe_eval": (None, [P, P, I32, P, P, P, P, P, U32, F, I32, P, P, P]),
        "orc_synth_box_scene": (I32, [C.c_uint64, U32, P, P, P, C.POINTER(U32), C.POINTER(U32)]),
        "orc_synth_cubemap": (None, [C.c_uint64, U32, P]),
        "orc_synth_sun": (None, [C.c_uint64, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()
NTHREADS = int(os.environ.get("VLB_ORACLE_THREADS", os.cpu_count() or 1))


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def k_of(lmax):
    return (lmax + 1) * (lmax + 1)


def sh_basis(lmax, dirs):
    d = _c(dirs, np.float64).reshape(-1, 3)
    out = np.empty((d.shape[0], k_of(lmax)), np.float64)
    lib.orc_sh_basis(lmax, _p(d), d.shape[0], _p(out))
    return out


def to_vector(phi, theta):
    out = np.empty(3, np.float64)
    lib.orc_to_vector(phi, theta, _p(out))
    return out


def x2phi_y2theta(x, w, y, h):
    a, b = C.c_double(), C.c_double()
    lib.orc_x2phi_y2theta(x, w, y, h, C.byref(a), C.byref(b))
    return a.value, b.value


def dirs_fibonacci(n):
    d = np.empty((n, 3), np.float32)
    w = C.c_double()
    lib.orc_dirs_fibonacci(n, _p(d), C.byref(w))
    return d, np.full(n, w.value)


def dirs_equirect(w, h):
    t = np.empty((w * h, 3), np.float32)
    b = np.empty((w * h, 3), np.float64)
    wt = np.empty(w * h, np.float64)
    lib.orc_dirs_equirect(w, h, _p(t), _p(b), _p(wt))
    return t, b, wt


def basis_matrix(basis_dirs, weights, lmax):
    """S x K FP64 weighted basis w_s * Y_k(b_s)."""
    return sh_basis(lmax, basis_dirs) * np.asarray(weights, np.float64)[:, None]


def cube_solid_angle(n):
    out = np.empty((n, n), np.float64)
    lib.orc_cube_solid_angle(n, _p(out))
    return out


def cube_texel_dirs(n):
    out = np.empty((6, n, n, 3), np.float64)
    lib.orc_cube_texel_dirs(n, _p(out))
    return out


def cube_select(dirs32, n):
    d = _c(dirs32, np.float32).reshape(-1, 3)
    out = np.empty(d.shape[0], np.uint32)
    lib.orc_cube_select(_p(d), d.shape[0], n, _p(out))
    return out


def skybox_sh(texels, fmt, layout, w, h, lmax, flags=0):
    t = _c(texels, np.float32 if fmt == 0 else np.uint8)
    out = np.empty((k_of(lmax), 3), np.float64)
    lib.orc_skybox_sh(_p(t), fmt, layout, w, h, lmax, flags, _p(out))
    return out


def project(radiance, nprobes, S, basis):
    r = _c(radiance, np.float32)
    B = _c(basis, np.float64)
    K = B.shape[1]
    out = np.empty((nprobes, K, 3), np.float64)
    lib.orc_project(_p(r), nprobes * 3, S, _p(B), K, _p(out), NTHREADS)
    return out


def sh_eval_envmap(coeffs, lmax, w, h, scale=1250.0):
    c = _c(coeffs, np.float64)
    out = np.empty((h, w, 3), np.float64)
    lib.orc_sh_eval_envmap(_p(c), lmax, w, h, scale, _p(out))
    return out


def probe_grid_ref_order(bounds, counts):
    b = _c(bounds, np.float32)
    c = _c(counts, np.uint32)
    n = int(np.prod(c))
    out = np.empty((n, 3), np.float32)
    step = np.empty(3, np.float32)
    m = lib.orc_probe_grid_ref_order(_p(b), _p(c), _p(out), _p(step))
    assert m == n
    return out, step


def synth_box_scene(seed, nboxes):
    """The benchmark's seeded box scene (positions, indices, per-triangle albedo)."""
    nv, nt = C.c_uint32(), C.c_uint32()
    lib.orc_synth_box_scene(seed, nboxes, None, None, None, C.byref(nv), C.byref(nt))
    pos = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    alb = np.empty((nt.value, 3), np.float32)
    assert lib.orc_synth_box_scene(seed, nboxes, _p(pos), _p(idx), _p(alb), None, None) == 0
    return pos, idx, alb


def synth_cubemap(seed, n):
    out = np.empty((6, n, n, 3), np.float32)
    lib.orc_synth_cubemap(seed, n, _p(out))
    return out


def synth_sun(seed):
    out = np.empty(3, np.float32)
    lib.orc_synth_sun(seed, _p(out))
    return out


def lbvh_build(pos, idx):
    p = _c(pos, np.float32).reshape(-1, 3)
    i = _c(idx, np.uint32).reshape(-1, 3)
    n = i.shape[0]
    codes = np.empty(n, np.uint32)
    order = np.empty(n, np.uint32)
    child = np.empty(max(0, 2 * (n - 1)), np.int32)
    box = np.empty((max(0, 2 * n - 1), 6), np.float32)
    lib.orc_lbvh_build(_p(p), p.shape[0], _p(i), n, _p(codes), _p(order), _p(child) if child.size else None,
                       _p(box) if box.size else None)
    return {"codes": codes, "order": order, "child": child, "box": box}


class Scene:
    def __init__(self, pos, idx, albedo):
        self.pos = _c(pos, np.float32).reshape(-1, 3)
        self.idx = _c(idx, np.uint32).reshape(-1, 3)
        self.alb = _c(albedo, np.float32).reshape(-1, 3)
        self.h = lib.orc_scene_create(_p(self.pos), self.pos.shape[0], _p(self.idx), self.idx.shape[0], _p(self.alb))

    def __del__(self):
        if getattr(self, "h", None):
            lib.orc_scene_destroy(self.h)
            self.h = None

    def bake(self, probes, dirs32, basis, sun, sun_intensity=5.0, tmin=1e-3, tmax=1e4, bias=5e-3, sky=None,
             sky_n=0, force_hit=None, force_vis=None, per_ray=False, nthreads=None, shading=0, light=(1.0, 10.0, 1.0)):
        """shading 0: Lambert + sun (the configs); 1: the reference baker's
        Phong + sRGB + 8-bit UNORM samples with the point light `light`."""
        pr = _c(probes, np.float32).reshape(-1, 3)
        d = _c(dirs32, np.float32).reshape(-1, 3)
        B = _c(basis, np.float64)
        np_, S, K = pr.shape[0], d.shape[0], B.shape[1]
        sunv = _c(sun, np.float32)
        skyv = None if sky is None else _c(sky, np.float32)
        fh = None if force_hit is None else _c(force_hit, np.int32)
        fv = None if force_vis is None else _c(force_vis, np.uint8)
        out = np.empty((np_, K, 3), np.float64)
        hit = vis = edge = rad = None
        if per_ray:
            hit = np.empty((np_, S), np.int32)
            vis = np.empty((np_, S), np.uint8)
            edge = np.empty((np_, S), np.float64)
            rad = np.empty((np_, S, 3), np.float32)
        lib.orc_bake(self.h, _p(pr), np_, _p(d), S, _p(B), K, _p(sunv), sun_intensity, tmin, tmax, bias, _p(skyv),
                     sky_n, _p(fh), _p(fv), nthreads or NTHREADS, _p(out), _p(hit), _p(vis), _p(edge), _p(rad),
                     int(shading), _p(_c(light, np.float32)))
        if per_ray:
            return out, hit, vis, edge, rad
        return out

    def ray_tri(self, o, d, tri):
        o = _c(o, np.float64)
        d = _c(d, np.float64)
        t, b1, b2, e = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        ok = lib.orc_ray_tri(self.h, _p(o), _p(d), int(tri), C.byref(t), C.byref(b1), C.byref(b2), C.byref(e))
        return (t.value, b1.value, b2.value, e.value) if ok else None

    def shadow_margin(self, o, d, tmin, tmax):
        o = _c(o, np.float64)
        d = _c(d, np.float64)
        return lib.orc_shadow_margin(self.h, _p(o), _p(d), tmin, tmax)

    def closest_hit(self, o, d, tmin=1e-3, tmax=1e4):
        o = _c(o, np.float64)
        d = _c(d, np.float64)
        tri, t = C.c_int(), C.c_double()
        lib.orc_closest_hit(self.h, _p(o), _p(d), tmin, tmax, C.byref(tri), C.byref(t))
        return tri.value, t.value


def probe_eval(scene, coeffs, lmax, origin, step, counts, points, normals, bias=5e-3, margins=False,
               nthreads=None):
    """FP64 probe evaluation (main.rchit:124-168 / sh.rmiss:23-39, intended math).
    scene: Scene or None (every probe visible).  Returns (rgb [n,3] f64,
    visibility mask [n] u8 (bit c = corner c), shadow margins [n,8] or None)."""
    c = _c(coeffs, np.float32)
    o = _c(origin, np.float32)
    st = _c(step, np.float32)
    cn = _c(counts, np.uint32)
    pt = _c(points, np.float32).reshape(-1, 3)
    nm = _c(normals, np.float32).reshape(-1, 3)
    n = pt.shape[0]
    out = np.empty((n, 3), np.float64)
    vis = np.empty(n, np.uint8)
    mg = np.empty((n, 8), np.float64) if margins else None
    lib.orc_probe_eval(None if scene is None else scene.h, _p(c), lmax, _p(o), _p(st), _p(cn), _p(pt), _p(nm), n,
                       bias, nthreads or NTHREADS, _p(out), _p(vis), _p(mg))
    return out, vis, mg


def load_ref():
    """The reference's own sh_common.h compiled in place (None if not built)."""
    if not REF_PATH.exists():
        return None
    r = C.CDLL(str(REF_PATH))
    r.ref_sh.restype = C.c_float
    r.ref_sh.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]
    r.ref_x2phi.restype = C.c_float
    r.ref_x2phi.argtypes = [C.c_int, C.c_int]
    r.ref_y2theta.restype = C.c_float
    r.ref_y2theta.argtypes = [C.c_int, C.c_int]
    r.ref_to_vector.restype = None
    r.ref_to_vector.argtypes = [C.c_float, C.c_float, C.c_void_p]
    r.ref_pi.restype = C.c_float
    return r
