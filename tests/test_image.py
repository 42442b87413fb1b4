"""Debug env-map images: the PNG / PPM writers (host only) and the RGBA8
encoding (GPU), against independent decoders / a numpy restatement."""
import struct
import zlib

import numpy as np
import pytest

import vlb


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        chunks.append((typ, body))
        pos += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])  # checks the Adler-32 too
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("w,h", [(1, 1), (3141 // 8, 1000 // 8), (200, 400)])
def test_png_round_trip(tmp_path, w, h):
    img = np.random.default_rng(w).integers(0, 256, (h, w, 4), dtype=np.uint8)
    p = tmp_path / "probe.png"
    vlb.image_write(p, img)
    assert np.array_equal(_read_png(p), img)


def test_ppm(tmp_path):
    img = np.random.default_rng(5).integers(0, 256, (7, 9, 4), dtype=np.uint8)
    p = tmp_path / "probe.ppm"
    vlb.image_write(p, img)
    data = open(p, "rb").read()
    assert data.startswith(b"P6\n9 7\n255\n")
    assert np.array_equal(np.frombuffer(data[len(b"P6\n9 7\n255\n"):], np.uint8).reshape(7, 9, 3), img[..., :3])


def test_image_errors(tmp_path):
    with pytest.raises(vlb.VlbError):
        vlb.image_write(tmp_path / "missing_dir" / "x.png", np.zeros((2, 2, 4), np.uint8))


def srgb_encode(rgb, scale=1.0, srgb=True):
    """numpy restatement of the shaders' sRGB() + R8G8B8A8 UNORM store."""
    v = scale * rgb.astype(np.float64)
    if srgb:
        v = np.where(v < 0.0031308, v * 12.92, 1.055 * np.power(np.maximum(v, 0), 1 / 2.4) - 0.055)
    v = np.nan_to_num(np.clip(v, 0, 1))
    out = np.empty(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.rint(v * 255)
    out[..., 3] = 255
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("srgb", [True, False])
def test_encode_rgba8(ctx, srgb):
    rgb = np.random.default_rng(1).uniform(-0.2, 1.3, (100000, 3)).astype(np.float32)
    rgb[:5] = [[0, 0, 0], [1, 1, 1], [0.0031308, 0.5, 2.0], [np.nan, -1, 1e-9], [0.002, 0.004, 0.9999]]
    got = ctx.encode_rgba8(rgb, 1.0, srgb)
    exp = srgb_encode(rgb, 1.0, srgb)
    d = np.abs(got.astype(int) - exp.astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3  # FP32 powf vs FP64 at the rounding midpoints


@pytest.mark.gpu
def test_render_envmap_matches_the_traced_radiance(ctx, tmp_path):
    pos, idx, alb = vlb.synth_box_scene(2, 32)
    scene = ctx.scene(pos, idx, alb)
    w, h = 96, 48
    sky = ctx.sky(vlb.synth_cubemap(2, 32), 32)
    p = vlb.bake_params(ctx.equirect(w, h), 2, vlb.PREC_FP32, vlb.synth_sun(2), sky=sky)
    probe = np.float32([0.5, 0.3, 0.45])
    img = ctx.render_envmap(scene, probe, p, w, h)
    sh, hit, vis, rad = ctx.bake(scene, probe[None], p, debug=True)
    assert np.array_equal(img, ctx.encode_rgba8(rad[0], 1.0, True).reshape(h, w, 4))
    assert np.abs(img.astype(int) - srgb_encode(rad[0]).reshape(h, w, 4).astype(int)).max() <= 1
    assert np.all(img[..., 3] == 255) and img[..., :3].std() > 0
    vlb.image_write(tmp_path / "0.png", img)
    assert np.array_equal(_read_png(tmp_path / "0.png"), img)
    # the reference's reconstruction image (sh_sum.comp): 1250 x SH, no sRGB
    rec = ctx.sh_eval_envmap(sh[0], 2, w, h, scale=1.0)
    assert ctx.encode_rgba8(rec, 1250.0, False).shape == (h, w, 4)
