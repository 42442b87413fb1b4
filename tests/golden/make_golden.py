"""Generates tests/golden/reference_golden.npz from the reference's own code.

Run in a checkout that has the reference project next to it (the shim library
oracle/_ref/libshref.so is built from <reference>/shaders/sh_common.h by
`make -C oracle` or __graft_entry__.build()).  The fixture is committed so the
tests need neither the reference checkout nor the shim.

What is recorded, all computed by the reference header's own functions in
FP32 (as the shaders run them):
  * basis:     SH(l, m, dir) for l <= 4 at 96 seeded unit directions
               (shaders/sh_common.h:154-223)
  * angles:    x2phi, y2theta, toVector over a 24 x 12 grid (sh_common.h:8-22)
  * skybox:    the skybox_sh.comp:27-41 sum over a seeded 32 x 16 RGBA8 image,
               each texel's term computed with the reference functions in
               FP32, the terms accumulated in FP64 (the shader's own
               accumulation is an unordered race, so only the per-texel terms
               are pinned exactly)
  * envmap:    the same for sh.comp:27-41 (no -PI/2, basis at dir)
  * sh_sum:    sh_sum.comp:39-51 reconstruction (x1250) of seeded coefficients
  * grid:      the probe order of light_baker.cpp:80-101 for a 3x3x3 grid
               over the unit box, written out from that loop by hand
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import oracle as O  # noqa: E402


def main() -> None:
    ref = O.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libshref.so missing: build it from the reference checkout first")
    rng = np.random.default_rng(20221)
    f32 = np.float32

    # basis at seeded directions
    v = rng.normal(size=(96, 3))
    dirs = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(f32)
    basis = np.zeros((96, 25), f32)
    for i, d in enumerate(dirs):
        for l in range(5):
            for m in range(-l, l + 1):
                basis[i, l * (l + 1) + m] = ref.ref_sh(l, m, float(d[0]), float(d[1]), float(d[2]))

    # angle maps
    W, H = 24, 12
    phi = np.array([ref.ref_x2phi(x, W) for x in range(W)], f32)
    theta = np.array([ref.ref_y2theta(y, H) for y in range(H)], f32)
    tv = np.zeros((H, W, 3), f32)
    buf = (C.c_float * 3)()
    for y in range(H):
        for x in range(W):
            ref.ref_to_vector(float(phi[x]), float(theta[y]), buf)
            tv[y, x] = list(buf)

    # skybox_sh.comp / sh.comp over a seeded RGBA8 image
    PW, PH = 32, 16
    img = rng.integers(0, 256, size=(PH, PW, 4), dtype=np.uint8)
    pi = ref.ref_pi()

    def project(shift: bool, swz: bool) -> np.ndarray:
        acc = np.zeros((16, 3), np.float64)
        area = f32(f32(2.0 * pi / PW) * f32(pi / PH))
        for y in range(PH):
            for x in range(PW):
                ph = f32(ref.ref_x2phi(x, PW))
                if shift:
                    ph = f32(ph - f32(pi / 2.0))
                th = f32(ref.ref_y2theta(y, PH))
                ref.ref_to_vector(float(ph), float(th), buf)
                d = [buf[0], buf[1], buf[2]]
                if swz:
                    d = [d[0], d[2], d[1]]
                col = img[y, x, :3].astype(f32) / f32(255.0)
                w = f32(area * f32(np.sin(th)))
                for l in range(4):
                    for m in range(-l, l + 1):
                        s = f32(ref.ref_sh(l, m, *map(float, d)))
                        acc[l * (l + 1) + m] += (s * col * w).astype(f32)
        return acc

    skybox = project(True, True)
    envmap = project(False, False)

    # sh_sum.comp reconstruction
    coeffs = rng.normal(size=(16, 3)).astype(f32) * f32(0.01)
    SW, SH = 16, 8
    recon = np.zeros((SH, SW, 3), f32)
    for y in range(SH):
        for x in range(SW):
            ref.ref_to_vector(ref.ref_x2phi(x, SW), ref.ref_y2theta(y, SH), buf)
            c = np.zeros(3, f32)
            for l in range(4):
                for m in range(-l, l + 1):
                    c += coeffs[l * (l + 1) + m] * f32(ref.ref_sh(l, m, buf[0], buf[1], buf[2]))
            recon[y, x] = f32(1250.0) * c

    # light_baker.cpp:80-101 for bounds [0,1]^3, counts 3x3x3: positions grow
    # one axis at a time (x run, then each existing probe stepped along y,
    # then along z); step (b1-b0)/(n-1) = 0.5 accumulated in FP32.
    grid = []
    pos = [(0.0, 0.0, 0.0)]
    for dim in range(3):
        for p in list(pos):
            q = list(p)
            for _ in range(2):
                q[dim] = float(f32(q[dim]) + f32(0.5))
                pos.append(tuple(q))
    grid = np.array(pos, f32)

    np.savez_compressed(
        HERE / "reference_golden.npz",
        dirs=dirs, basis=basis, W=W, H=H, phi=phi, theta=theta, to_vector=tv, pi=np.float32(pi),
        img=img, skybox=skybox, envmap=envmap, coeffs=coeffs, recon=recon, recon_wh=np.array([SW, SH]),
        grid=grid)
    print("wrote", HERE / "reference_golden.npz")


if __name__ == "__main__":
    main()
