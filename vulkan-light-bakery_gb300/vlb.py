"""ctypes binding of libvlb.so (include/vlb.h) for tests, bench.py and scripts.

Arrays may be numpy arrays (host memory) or torch tensors (host or CUDA); the
library reads each pointer's residency itself.  Every failed call raises
VlbError carrying the status code and the context's message.  The library
must exist: importing this module on a machine where libvlb.so was not built
raises immediately -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("VLB_LIB", _PKG / "_build" / "libvlb.so"))

OK, ERR_INVALID, ERR_OOM, ERR_TIMEOUT, ERR_CUDA, ERR_UNSUPPORTED, ERR_INTERNAL = range(7)
FRAME_WORLD, FRAME_XZY = 0, 1
SKY_CUBEMAP, SKY_PANORAMA, SKY_ENVMAP = 0, 1, 2
TEXEL_RGB32F, TEXEL_RGBA8 = 0, 1
SKY_REF_BGRA_SWAP = 1
PREC_FP32, PREC_FUSED, PREC_MIXED, PREC_BF16 = 0, 1, 2, 3
BAKE_FORCE_FUSED_KERNEL = 1
BAKE_TRAVERSAL_PACKET, BAKE_TRAVERSAL_LANE, BAKE_TRAVERSAL_GRID = 2, 4, 8
BAKE_REF_ACCUMULATE = 16
HOOK_HOLD_PRODUCER = 1
SHADE_LAMBERT_SUN, SHADE_REF_PHONG = 0, 1
SCENE_TRAVERSAL_LBVH, SCENE_TRAVERSAL_WIDE = 1, 2
DTYPE_F32, DTYPE_BF16, DTYPE_BF16_SPLIT = 0, 1, 2


class VlbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"vlb status {status}: {message}")
        self.status = status
        self.message = message


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("total_ms", C.c_double)]


class BakeParams(C.Structure):
    _fields_ = [
        ("lmax", C.c_uint32), ("precision", C.c_uint32), ("flags", C.c_uint32),
        ("sun_dir", C.c_float * 3), ("sun_intensity", C.c_float),
        ("tmin", C.c_float), ("tmax", C.c_float), ("shadow_bias", C.c_float),
        ("dirs", C.c_void_p), ("sky", C.c_void_p), ("shading", C.c_uint32), ("light_pos", C.c_float * 3),
    ]


class BakeDebug(C.Structure):
    _fields_ = [("hit_tri", C.c_void_p), ("shadow", C.c_void_p), ("radiance", C.c_void_p)]


class ProbeGrid(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("step", C.c_float * 3), ("counts", C.c_uint32 * 3)]


class BakeJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("probe_xyz", C.c_void_p), ("nprobes", C.c_uint32),
                ("params", C.c_void_p), ("out", C.c_void_p)]


class BatchSchedule(C.Structure):
    _fields_ = [("dirs_per_item", C.c_uint32), ("cost_order", C.c_uint32), ("graph", C.c_uint32),
                ("ctas_per_sm", C.c_uint32), ("node_steps", C.c_uint32), ("refill_idle", C.c_uint32)]


class TuneTrial(C.Structure):
    _fields_ = [("schedule", BatchSchedule), ("ms", C.c_float)]


class ServiceConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("lmax", C.c_uint32), ("precision", C.c_uint32),
                ("max_batch_probes", C.c_uint32), ("max_inflight", C.c_uint32), ("slice_probes", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("probe_xyz", C.c_void_p), ("nprobes", C.c_uint32), ("params", C.c_void_p),
                ("relight_of", C.c_uint64), ("keep_hits", C.c_uint32)]


class ServiceStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "failed", "batches", "relights",
                                          "relights_rebaked", "evictions", "probes", "rays", "bytes_in_use",
                                          "bytes_peak")]


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"libvlb.so not found at {LIB_PATH}; run __graft_entry__.build() first")
    lib = C.CDLL(str(LIB_PATH))
    P, U32, I32, U64, F32 = C.c_void_p, C.c_uint32, C.c_int, C.c_uint64, C.c_float
    sig = {
        "vlb_version": (U32, []),
        "vlb_status_string": (C.c_char_p, [I32]),
        "vlb_ctx_create": (I32, [I32, C.POINTER(P)]),
        "vlb_ctx_destroy": (None, [P]),
        "vlb_ctx_set_stream": (I32, [P, P]),
        "vlb_ctx_get_stream": (P, [P]),
        "vlb_ctx_synchronize": (I32, [P]),
        "vlb_last_error": (C.c_char_p, [P]),
        "vlb_ctx_set_profiling": (I32, [P, I32]),
        "vlb_ctx_profile_read": (I32, [P, P, U32, C.POINTER(U32)]),
        "vlb_ctx_profile_reset": (I32, [P]),
        "vlb_ctx_launch_count": (U64, [P]),
        "vlb_ctx_test_hook": (I32, [P, U32, U32]),
        "vlb_build_flags": (U32, []),
        "vlb_probe_grid_ref_order": (I32, [P, P, P, P]),
        "vlb_scene_create": (I32, [P, P, U32, U32, P, U32, P, C.POINTER(P)]),
        "vlb_scene_create_ex": (I32, [P, P, U32, U32, P, U32, P, U32, C.POINTER(P)]),
        "vlb_scene_destroy": (None, [P]),
        "vlb_scene_triangle_count": (U32, [P]),
        "vlb_scene_bounds": (I32, [P, I32, P]),
        "vlb_scene_bvh_export": (I32, [P, P, P, P, P]),
        "vlb_scene_device_bytes": (U64, [P]),
        "vlb_dirset_create_fibonacci": (I32, [P, U32, I32, C.POINTER(P)]),
        "vlb_dirset_create_equirect": (I32, [P, U32, U32, C.POINTER(P)]),
        "vlb_dirset_create": (I32, [P, P, P, P, U32, C.POINTER(P)]),
        "vlb_dirset_destroy": (None, [P]),
        "vlb_dirset_count": (U32, [P]),
        "vlb_dirset_export": (I32, [P, P, P]),
        "vlb_skybox_sh": (I32, [P, P, I32, I32, U32, U32, U32, U32, P]),
        "vlb_skybox_sh_batched": (I32, [P, P, I32, I32, U32, U32, U32, U32, U32, P]),
        "vlb_skybox_sh_noalloc": (I32, [P, I32, I32, U32, U32, U32, U32, P, P]),
        "vlb_sky_create": (I32, [P, P, U32, C.POINTER(P)]),
        "vlb_sky_destroy": (None, [P]),
        "vlb_bake_params_default": (None, [P]),
        "vlb_bake": (I32, [P, P, P, U32, P, P]),
        "vlb_bake_ex": (I32, [P, P, P, U32, P, P, P]),
        "vlb_bake_async": (I32, [P, P, P, U32, P, P, P]),
        "vlb_bake_trace_stats": (I32, [P, P, P, U32, P, P]),
        "vlb_bake_batch": (I32, [P, P, U32, P, P]),
        "vlb_batch_autotune": (I32, [P, P, U32, P, U32, P, P]),
        "vlb_batch_tune_log": (I32, [P, P, U32, C.POINTER(U32), C.POINTER(U32)]),
        "vlb_service_create": (I32, [P, P, C.POINTER(P)]),
        "vlb_service_destroy": (None, [P]),
        "vlb_service_submit": (I32, [P, P, C.POINTER(U64)]),
        "vlb_service_wait": (I32, [P, U64, U32, P, C.POINTER(C.c_double)]),
        "vlb_service_release": (I32, [P, U64]),
        "vlb_service_stats_read": (I32, [P, P]),
        "vlb_service_last_error": (C.c_char_p, []),
        "vlb_service_plan": (I32, [P, P, U32, U64, U64, P, C.POINTER(U32)]),
        "vlb_gltf_write_light": (I32, [C.c_char_p, C.c_size_t, P, U32, U32, P, P, C.c_size_t,
                                       C.POINTER(C.c_size_t)]),
        "vlb_gltf_read_light": (I32, [C.c_char_p, C.c_size_t, P, C.POINTER(U32), P, C.c_size_t,
                                      C.POINTER(C.c_size_t)]),
        "vlb_gltf_last_error": (C.c_char_p, []),
        "vlb_gltf_mesh_load": (I32, [C.c_char_p, C.POINTER(P)]),
        "vlb_gltf_mesh_free": (None, [P]),
        "vlb_gltf_mesh_info": (I32, [P, C.POINTER(U32), C.POINTER(U32), P]),
        "vlb_gltf_mesh_get": (I32, [P, P, P, P]),
        "vlb_scene_create_gltf": (I32, [P, C.c_char_p, C.POINTER(P)]),
        "vlb_probe_eval": (I32, [P, P, P, U32, P, P, P, U32, F32, P, P]),
        "vlb_sh_eval_dirs": (I32, [P, P, U32, P, U32, P]),
        "vlb_encode_rgba8": (I32, [P, P, U32, F32, U32, P]),
        "vlb_render_envmap": (I32, [P, P, P, P, U32, U32, P]),
        "vlb_image_write_png": (I32, [C.c_char_p, P, U32, U32]),
        "vlb_image_write_ppm": (I32, [C.c_char_p, P, U32, U32]),
        "vlb_image_last_error": (C.c_char_p, []),
        "vlb_project": (I32, [P, P, I32, U32, P, U32, P]),
        "vlb_sh_eval_envmap": (I32, [P, P, U32, U32, U32, F32, P]),
        "vlb_synth_box_scene": (I32, [U64, U32, P, P, P, C.POINTER(U32), C.POINTER(U32)]),
        "vlb_synth_cubemap": (I32, [U64, U32, P]),
        "vlb_synth_sun": (I32, [U64, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def _ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (contiguous), or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)}")


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def k_of(lmax: int) -> int:
    return (lmax + 1) * (lmax + 1)


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib.vlb_ctx_create(device, C.byref(h))
        if st != OK:
            raise VlbError(st, f"vlb_ctx_create(device={device}) failed: {lib.vlb_status_string(st).decode()}")
        self.h = h
        self._objects = weakref.WeakSet()  # scenes, direction sets, skies, services made on this context

    def check(self, st: int) -> None:
        if st != OK:
            raise VlbError(st, lib.vlb_last_error(self.h).decode())

    def _own(self, obj) -> None:
        self._objects.add(obj)

    def close(self) -> None:
        """Destroys the context, after every object still open on it (the C ABI
        wants a context's objects destroyed before the context).  Services go
        first: destroying one finishes its submitted requests and joins its
        worker, which may still be baking with the scenes, direction sets and
        skies those requests name; those objects are destroyed after that."""
        if getattr(self, "h", None):
            objs = list(getattr(self, "_objects", ()))
            for obj in objs:
                if isinstance(obj, Service):
                    obj.close()
            for obj in objs:
                if not isinstance(obj, Service):
                    obj.close()
            lib.vlb_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # stream / timing
    def set_stream(self, stream_handle: int | None) -> None:
        self.check(lib.vlb_ctx_set_stream(self.h, stream_handle))

    @property
    def stream(self) -> int:
        return lib.vlb_ctx_get_stream(self.h) or 0

    def synchronize(self) -> None:
        self.check(lib.vlb_ctx_synchronize(self.h))

    def set_profiling(self, on: bool) -> None:
        self.check(lib.vlb_ctx_set_profiling(self.h, 1 if on else 0))

    def profile(self) -> dict:
        buf = (KernelTime * 64)()
        n = C.c_uint32()
        self.check(lib.vlb_ctx_profile_read(self.h, buf, 64, C.byref(n)))
        return {buf[i].name.decode(): (buf[i].launches, buf[i].total_ms) for i in range(n.value)}

    def profile_reset(self) -> None:
        self.check(lib.vlb_ctx_profile_reset(self.h))

    @property
    def launch_count(self) -> int:
        return int(lib.vlb_ctx_launch_count(self.h))

    def test_hook(self, hook: int, wait_polls: int = 0) -> None:
        """vlb_ctx_test_hook: HOOK_HOLD_PRODUCER makes the TMA pipelines' waits
        give up (VLB_ERR_TIMEOUT) without a copy in flight; 0 clears it."""
        self.check(lib.vlb_ctx_test_hook(self.h, hook, wait_polls))

    # objects
    def scene(self, positions, indices, albedo=None, stride_bytes: int = 12, flags: int = 0) -> "Scene":
        return Scene(self, positions, indices, albedo, stride_bytes, flags)

    def scene_gltf(self, path) -> "Scene":
        """Device scene straight from a .gltf / .glb file."""
        h = C.c_void_p()
        self.check(lib.vlb_scene_create_gltf(self.h, str(path).encode(), C.byref(h)))
        return Scene._wrap(self, h)

    def fibonacci(self, n: int, frame: int = FRAME_WORLD) -> "DirSet":
        h = C.c_void_p()
        self.check(lib.vlb_dirset_create_fibonacci(self.h, n, frame, C.byref(h)))
        return DirSet(self, h)

    def equirect(self, w: int, h: int) -> "DirSet":
        hh = C.c_void_p()
        self.check(lib.vlb_dirset_create_equirect(self.h, w, h, C.byref(hh)))
        return DirSet(self, hh)

    def dirset(self, trace_dirs, weights, basis_dirs=None) -> "DirSet":
        td = _f32(trace_dirs).reshape(-1, 3)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        bd = None if basis_dirs is None else _f32(basis_dirs).reshape(-1, 3)
        h = C.c_void_p()
        self.check(lib.vlb_dirset_create(self.h, _ptr(td), _ptr(bd), _ptr(w), td.shape[0], C.byref(h)))
        return DirSet(self, h)

    def sky(self, cubemap, n: int) -> "Sky":
        cm = cubemap if hasattr(cubemap, "data_ptr") else _f32(cubemap)
        h = C.c_void_p()
        self.check(lib.vlb_sky_create(self.h, _ptr(cm), n, C.byref(h)))
        return Sky(self, h, n)

    # entry points
    def skybox_sh(self, texels, layout: int, w: int, h: int, lmax: int = 3, fmt: int = TEXEL_RGB32F,
                  flags: int = 0, count: int = 1, out=None):
        K = k_of(lmax)
        ret = out if out is not None else np.empty((count, K, 3), np.float32)
        self.check(lib.vlb_skybox_sh_batched(self.h, _ptr(texels), fmt, layout, w, h, count, lmax, flags, _ptr(ret)))
        if out is None and count == 1:
            return ret[0]
        return ret

    def bake(self, scene: "Scene", probes, params: BakeParams, out=None, debug: bool = False):
        n = int(probes.shape[0]) if hasattr(probes, "shape") else len(probes) // 3
        K = k_of(params.lmax)
        if not hasattr(probes, "data_ptr"):
            probes = _f32(probes).reshape(-1, 3)
        ret = out if out is not None else np.empty((n, K, 3), np.float32)
        if not debug:
            self.check(lib.vlb_bake(self.h, scene.h, _ptr(probes), n, C.byref(params), _ptr(ret)))
            return ret
        S = params_dirs_count(params)
        hit = np.empty(n * S, np.int32)
        vis = np.empty(n * S, np.uint8)
        packet_fused = params.precision == PREC_FUSED and params.flags & BAKE_FORCE_FUSED_KERNEL
        rad = None if packet_fused else np.empty(n * S * 3, np.float32)
        dbg = BakeDebug(_ptr(hit), _ptr(vis), _ptr(rad))
        self.check(lib.vlb_bake_ex(self.h, scene.h, _ptr(probes), n, C.byref(params), _ptr(ret), C.byref(dbg)))
        return ret, hit.reshape(n, S), vis.reshape(n, S), (None if rad is None else rad.reshape(n, S, 3))

    def bake_async(self, scene: "Scene", probes, params: BakeParams, out, done_event=None) -> None:
        """Enqueues a bake of device probes into the device tensor `out` on the
        context's stream; `done_event` (a recorded-once torch.cuda.Event or a raw
        cudaEvent_t) is recorded after the bake."""
        ev = done_event.cuda_event if hasattr(done_event, "cuda_event") else done_event
        self.check(lib.vlb_bake_async(self.h, scene.h, _ptr(probes), int(probes.shape[0]), C.byref(params),
                                      _ptr(out), ev))

    def bake_batch(self, jobs, params: BakeParams, schedule: "BatchSchedule | None" = None):
        """jobs: list of (scene, probes, out-or-None[, job params]); returns the outputs."""
        arr, keep, outs = _job_array(jobs, params)
        self.check(lib.vlb_bake_batch(self.h, arr, len(jobs), C.byref(params),
                                      None if schedule is None else C.byref(schedule)))
        del keep
        return outs

    def batch_autotune(self, jobs, params: BakeParams, reps: int = 2):
        """Times the candidate schedules; returns (BatchSchedule, ms per batch)."""
        arr, keep, _ = _job_array(jobs, params)
        best = BatchSchedule()
        ms = C.c_float()
        self.check(lib.vlb_batch_autotune(self.h, arr, len(jobs), C.byref(params), reps, C.byref(best), C.byref(ms)))
        del keep
        return best, float(ms.value)

    def batch_tune_log(self):
        """(trials of the last batch_autotune as [(schedule dict, ms)], scene-size class)."""
        n, cls = C.c_uint32(), C.c_uint32()
        self.check(lib.vlb_batch_tune_log(self.h, None, 0, C.byref(n), C.byref(cls)))
        buf = (TuneTrial * max(n.value, 1))()
        self.check(lib.vlb_batch_tune_log(self.h, buf, n.value, C.byref(n), C.byref(cls)))
        return [({f: getattr(buf[i].schedule, f) for f, _ in BatchSchedule._fields_}, float(buf[i].ms))
                for i in range(n.value)], int(cls.value)

    def probe_eval(self, scene, coeffs, lmax: int, origin, step, counts, points, normals, shadow_bias: float = 0.005):
        """Evaluate a baked grid at shading points; returns (rgb [n,3], visibility mask [n])."""
        g = ProbeGrid()
        for a in range(3):
            g.origin[a], g.step[a], g.counts[a] = float(origin[a]), float(step[a]), int(counts[a])
        c = coeffs if hasattr(coeffs, "data_ptr") else _f32(coeffs)
        pt = points if hasattr(points, "data_ptr") else _f32(points).reshape(-1, 3)
        nm = normals if hasattr(normals, "data_ptr") else _f32(normals).reshape(-1, 3)
        n = int(pt.shape[0])
        out = np.empty((n, 3), np.float32)
        vis = np.empty(n, np.uint8)
        self.check(lib.vlb_probe_eval(self.h, None if scene is None else scene.h, _ptr(c), lmax, C.byref(g), _ptr(pt),
                                      _ptr(nm), n, shadow_bias, _ptr(out), _ptr(vis)))
        return out, vis

    def encode_rgba8(self, rgb, scale: float = 1.0, srgb: bool = True):
        x = _f32(rgb)
        n = x.size // 3
        out = np.empty(x.shape[:-1] + (4,), np.uint8)
        self.check(lib.vlb_encode_rgba8(self.h, _ptr(x), n, scale, 1 if srgb else 0, _ptr(out)))
        return out

    def render_envmap(self, scene, probe, params: BakeParams, w: int, h: int):
        """The reference's per-probe debug image: [h, w, 4] RGBA8 (sRGB)."""
        pr = _f32(probe).reshape(3)
        out = np.empty((h, w, 4), np.uint8)
        self.check(lib.vlb_render_envmap(self.h, scene.h, _ptr(pr), C.byref(params), w, h, _ptr(out)))
        return out

    def sh_eval_dirs(self, coeffs, lmax: int, dirs):
        c = _f32(coeffs).reshape(-1)
        d = _f32(dirs).reshape(-1, 3)
        out = np.empty((d.shape[0], 3), np.float32)
        self.check(lib.vlb_sh_eval_dirs(self.h, _ptr(c), lmax, _ptr(d), d.shape[0], _ptr(out)))
        return out

    def project(self, radiance, nprobes: int, dirs: "DirSet", lmax: int, dtype: int = DTYPE_F32, out=None):
        K = k_of(lmax)
        ret = out if out is not None else np.empty((nprobes, K, 3), np.float32)
        self.check(lib.vlb_project(self.h, _ptr(radiance), dtype, nprobes, dirs.h, lmax, _ptr(ret)))
        return ret

    def sh_eval_envmap(self, coeffs, lmax: int, w: int, h: int, scale: float = 1250.0):
        c = _f32(coeffs).reshape(-1)
        out = np.empty((h, w, 3), np.float32)
        self.check(lib.vlb_sh_eval_envmap(self.h, _ptr(c), lmax, w, h, scale, _ptr(out)))
        return out


class Service:
    """Resident bake service (vlb_service_*): submit from any thread, wait by ticket."""

    def __init__(self, ctx: Context, budget_bytes: int = 0, lmax: int = 2, precision: int = PREC_MIXED,
                 max_batch_probes: int = 0, max_inflight: int = 0, slice_probes: int = 0):
        cfg = ServiceConfig(budget_bytes, lmax, precision, max_batch_probes, max_inflight, slice_probes)
        h = C.c_void_p()
        self.ctx = ctx
        self.lmax = lmax
        self._check(lib.vlb_service_create(ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        ctx._own(self)
        self._keep = {}  # ticket -> objects the request names (kept alive until collected)
        self._n = {}

    @staticmethod
    def _check(st: int) -> None:
        if st != OK:
            raise VlbError(st, lib.vlb_service_last_error().decode())

    def submit(self, scene, probes, params: BakeParams, keep_hits: bool = False, relight_of: int = 0) -> int:
        if relight_of:
            pr, n = None, self._n.get(relight_of, 0)
        else:
            pr = _f32(probes).reshape(-1, 3)
            n = pr.shape[0]
        req = Request(None if scene is None else getattr(scene.h, "value", scene.h), _ptr(pr), 0 if relight_of else n,
                      C.addressof(params), relight_of, 1 if keep_hits else 0)
        t = C.c_uint64()
        self._check(lib.vlb_service_submit(self.h, C.byref(req), C.byref(t)))
        self._keep[t.value] = (scene, params)
        self._n[t.value] = n
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000):
        """Returns (sh [n, K, 3], latency_ms); raises VlbError (ERR_TIMEOUT if not done)."""
        n = self._n[ticket]
        out = np.empty((n, k_of(self.lmax), 3), np.float32)
        lat = C.c_double()
        st = lib.vlb_service_wait(self.h, ticket, timeout_ms, _ptr(out) if n else None, C.byref(lat))
        if st == ERR_TIMEOUT:
            raise VlbError(st, "not done")
        self._keep.pop(ticket, None)
        self._check(st)
        return out, lat.value

    def release(self, ticket: int) -> None:
        self._check(lib.vlb_service_release(self.h, ticket))

    def stats(self) -> dict:
        s = ServiceStats()
        self._check(lib.vlb_service_stats_read(self.h, C.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in ServiceStats._fields_}

    def close(self) -> None:
        if getattr(self, "h", None):
            lib.vlb_service_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def service_plan(probes, nbytes, max_batch_probes: int, budget_bytes: int):
    """The service's admission rule on the host: batch index per request (-1 refused)."""
    p = np.ascontiguousarray(probes, dtype=np.uint64)
    b = np.ascontiguousarray(nbytes, dtype=np.uint64)
    out = np.zeros(len(p), np.uint32)
    nb = C.c_uint32()
    st = lib.vlb_service_plan(_ptr(p) if len(p) else None, _ptr(b) if len(b) else None, len(p), max_batch_probes,
                              budget_bytes, _ptr(out) if len(p) else None, C.byref(nb))
    if st != OK:
        raise VlbError(st, "vlb_service_plan")
    return np.where(out == 0xFFFFFFFF, -1, out.astype(np.int64)), nb.value


def image_write(path, rgba) -> None:
    """Writes [h, w, 4] RGBA8 as PNG (".png") or PPM (anything else); host only."""
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = a.shape[:2]
    fn = lib.vlb_image_write_png if str(path).endswith(".png") else lib.vlb_image_write_ppm
    st = fn(str(path).encode(), _ptr(a), w, h)
    if st != OK:
        raise VlbError(st, lib.vlb_image_last_error().decode())


def gltf_write_light(gltf_text: str, coeffs, grid_step) -> str:
    """The reference's baked_<name>.gltf text for coefficients [n, K, 3] (host only)."""
    src = gltf_text.encode()
    c = _f32(coeffs)
    n, K = (c.shape[0], c.shape[1]) if c.ndim == 3 else (0, 16)
    g = _f32(grid_step).reshape(3)
    size = C.c_size_t()
    args = (src, len(src), _ptr(c) if c.size else None, n, K, _ptr(g))
    st = lib.vlb_gltf_write_light(*args, None, 0, C.byref(size))
    if st != OK:
        raise VlbError(st, lib.vlb_gltf_last_error().decode())
    buf = C.create_string_buffer(size.value)
    st = lib.vlb_gltf_write_light(*args, buf, size.value, C.byref(size))
    if st != OK:
        raise VlbError(st, lib.vlb_gltf_last_error().decode())
    return buf.value.decode()


def gltf_load_mesh(path):
    """(positions [nv,3], indices [nt,3], albedo [nt,3], bounds[6]) of a .gltf/.glb (host only)."""
    h = C.c_void_p()
    st = lib.vlb_gltf_mesh_load(str(path).encode(), C.byref(h))
    if st != OK:
        raise VlbError(st, lib.vlb_gltf_last_error().decode())
    try:
        nv, nt = C.c_uint32(), C.c_uint32()
        b = np.zeros(6, np.float32)
        lib.vlb_gltf_mesh_info(h, C.byref(nv), C.byref(nt), _ptr(b))
        pos = np.empty((nv.value, 3), np.float32)
        idx = np.empty((nt.value, 3), np.uint32)
        alb = np.empty((nt.value, 3), np.float32)
        lib.vlb_gltf_mesh_get(h, _ptr(pos) if pos.size else None, _ptr(idx) if idx.size else None,
                              _ptr(alb) if alb.size else None)
        return pos, idx, alb, b
    finally:
        lib.vlb_gltf_mesh_free(h)


def gltf_read_light(gltf_text: str):
    """(grid_step[3], coeff_count, coefficient bytes) of a baked glTF (host only)."""
    src = gltf_text.encode()
    g = np.zeros(3, np.float32)
    k = C.c_uint32()
    nb = C.c_size_t()
    st = lib.vlb_gltf_read_light(src, len(src), _ptr(g), C.byref(k), None, 0, C.byref(nb))
    if st != OK:
        raise VlbError(st, lib.vlb_gltf_last_error().decode())
    data = np.zeros(nb.value, np.uint8)
    if nb.value:
        st = lib.vlb_gltf_read_light(src, len(src), _ptr(g), C.byref(k), _ptr(data), nb.value, C.byref(nb))
        if st != OK:
            raise VlbError(st, lib.vlb_gltf_last_error().decode())
    return g, int(k.value), data.tobytes()


def _job_array(jobs, params: BakeParams):
    """vlb_bake_job[] for (scene, probes, out[, params]) tuples; outputs made when None."""
    arr = (BakeJob * max(1, len(jobs)))()
    keep, outs = [], []
    for i, j in enumerate(jobs):
        scene, probes, out = j[0], j[1], j[2]
        jp = j[3] if len(j) > 3 else None
        if not hasattr(probes, "data_ptr"):
            probes = _f32(probes).reshape(-1, 3)
        n = int(probes.shape[0])
        K = k_of((jp or params).lmax)
        if out is None:
            out = np.empty((n, K, 3), np.float32)
        keep += [probes, out, jp]
        outs.append(out)
        arr[i] = BakeJob(getattr(scene.h, "value", scene.h), _ptr(probes), n, None if jp is None else C.addressof(jp), _ptr(out))
    return arr, keep, outs


def params_dirs_count(p: BakeParams) -> int:
    return int(lib.vlb_dirset_count(p.dirs))


def trace_stats(ctx: Context, scene: "Scene", probes, params: BakeParams) -> dict:
    """Rays, shadow rays, BVH nodes fetched and triangles tested for one bake."""
    pr = probes if hasattr(probes, "data_ptr") else _f32(probes).reshape(-1, 3)
    n = int(pr.shape[0])
    out = np.zeros(6, np.uint64)
    ctx.check(lib.vlb_bake_trace_stats(ctx.h, scene.h, _ptr(pr), n, C.byref(params), _ptr(out)))
    return {"rays": int(out[0]), "shadow_rays": int(out[1]), "node_fetches": int(out[2]),
            "tri_fetches": int(out[3]), "node_tests": int(out[4]), "node_bytes": int(out[5])}


class Scene:
    def __init__(self, ctx: Context, positions, indices, albedo, stride_bytes: int, flags: int = 0):
        self.ctx = ctx
        pos = positions if hasattr(positions, "data_ptr") else _f32(positions)
        idx = indices if hasattr(indices, "data_ptr") else np.ascontiguousarray(indices, dtype=np.uint32)
        alb = None if albedo is None else (albedo if hasattr(albedo, "data_ptr") else _f32(albedo))
        nverts = (pos.numel() if hasattr(pos, "numel") else pos.size) * 4 // stride_bytes
        ntris = (idx.numel() if hasattr(idx, "numel") else idx.size) // 3
        h = C.c_void_p()
        ctx.check(lib.vlb_scene_create_ex(ctx.h, _ptr(pos), stride_bytes, nverts, _ptr(idx), ntris, _ptr(alb),
                                          flags, C.byref(h)))
        self.h = h
        self.ntris = ntris
        ctx._own(self)

    @classmethod
    def _wrap(cls, ctx: Context, h) -> "Scene":
        s = cls.__new__(cls)
        s.ctx, s.h = ctx, h
        s.ntris = int(lib.vlb_scene_triangle_count(h))
        ctx._own(s)
        return s

    def bounds(self, include_origin: bool = True) -> np.ndarray:
        b = np.empty(6, np.float32)
        self.ctx.check(lib.vlb_scene_bounds(self.h, 1 if include_origin else 0, _ptr(b)))
        return b

    def bvh_export(self) -> dict:
        n = self.ntris
        codes = np.empty(n, np.uint32)
        order = np.empty(n, np.uint32)
        child = np.empty(max(0, 2 * (n - 1)), np.int32)
        box = np.empty(max(0, (2 * n - 1) * 6), np.float32)
        self.ctx.check(lib.vlb_scene_bvh_export(self.h, _ptr(codes), _ptr(order), _ptr(child) if child.size else None,
                                                _ptr(box) if box.size else None))
        return {"codes": codes, "order": order, "child": child, "box": box.reshape(-1, 6)}

    @property
    def device_bytes(self) -> int:
        return int(lib.vlb_scene_device_bytes(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            lib.vlb_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DirSet:
    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self.h = h
        self.n = int(lib.vlb_dirset_count(h))
        ctx._own(self)

    def export(self):
        d = np.empty((self.n, 3), np.float32)
        b = np.empty((self.n, 16), np.float32)
        self.ctx.check(lib.vlb_dirset_export(self.h, _ptr(d), _ptr(b)))
        return d, b

    def close(self) -> None:
        if getattr(self, "h", None):
            lib.vlb_dirset_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sky:
    def __init__(self, ctx: Context, h, n: int):
        self.ctx = ctx
        self.h = h
        self.n = n
        ctx._own(self)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib.vlb_sky_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bake_params(dirs: DirSet, lmax: int = 2, precision: int = PREC_FP32, sun=(0.0, 1.0, 0.0),
                sun_intensity: float = 5.0, sky: Sky | None = None, shading: int = SHADE_LAMBERT_SUN,
                light_pos=None, flags: int = 0) -> BakeParams:
    p = BakeParams()
    lib.vlb_bake_params_default(C.byref(p))
    p.lmax = lmax
    p.precision = precision
    p.shading = shading
    p.flags = flags
    if light_pos is not None:
        for i in range(3):
            p.light_pos[i] = float(light_pos[i])
    for i in range(3):
        p.sun_dir[i] = float(sun[i])
    p.sun_intensity = sun_intensity
    p.dirs = dirs.h
    p.sky = sky.h if sky is not None else None
    # the struct carries raw handles: keep their owners alive as long as it lives
    p._owners = (dirs, sky)
    return p


# ---- host-only helpers (no GPU needed) ------------------------------------------------
def probe_grid_ref_order(bounds, counts):
    b = _f32(bounds)
    c = np.ascontiguousarray(counts, dtype=np.uint32)
    n = int(np.prod(c))
    out = np.empty((n, 3), np.float32)
    step = np.empty(3, np.float32)
    st = lib.vlb_probe_grid_ref_order(_ptr(b), _ptr(c), _ptr(out), _ptr(step))
    if st != OK:
        raise VlbError(st, "vlb_probe_grid_ref_order")
    return out, step


def synth_box_scene(seed: int, nboxes: int):
    nv, nt = C.c_uint32(), C.c_uint32()
    lib.vlb_synth_box_scene(seed, nboxes, None, None, None, C.byref(nv), C.byref(nt))
    pos = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    alb = np.empty((nt.value, 3), np.float32)
    st = lib.vlb_synth_box_scene(seed, nboxes, _ptr(pos), _ptr(idx), _ptr(alb), C.byref(nv), C.byref(nt))
    if st != OK:
        raise VlbError(st, "vlb_synth_box_scene")
    return pos, idx, alb


def synth_cubemap(seed: int, n: int) -> np.ndarray:
    out = np.empty((6, n, n, 3), np.float32)
    st = lib.vlb_synth_cubemap(seed, n, _ptr(out))
    if st != OK:
        raise VlbError(st, "vlb_synth_cubemap")
    return out


def synth_sun(seed: int) -> np.ndarray:
    out = np.empty(3, np.float32)
    st = lib.vlb_synth_sun(seed, _ptr(out))
    if st != OK:
        raise VlbError(st, "vlb_synth_sun")
    return out
