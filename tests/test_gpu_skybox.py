"""Skybox SH kernel (skybox_sh.comp / sh.comp forms and the cubemap) vs the FP64 oracle."""
import numpy as np
import pytest

import oracle as O
import vlb

pytestmark = pytest.mark.gpu
TOL = 1e-5  # FP32 per-texel arithmetic + FP32 slab sums, FP64 final sum


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("lmax", [2, 3])
def test_cubemap_config0_matches_oracle(ctx, lmax):
    cm = vlb.synth_cubemap(2022, 128)
    got = ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 128, 128, lmax)
    ref = O.skybox_sh(cm, 0, 0, 128, 128, lmax)
    assert got.shape == (vlb.k_of(lmax), 3)
    assert rel(got, ref) < TOL


@pytest.mark.parametrize("layout,key", [(vlb.SKY_PANORAMA, "skybox"), (vlb.SKY_ENVMAP, "envmap")])
def test_rgba8_panorama_matches_reference_golden(ctx, golden, layout, key):
    img = golden["img"]
    got = ctx.skybox_sh(img, layout, img.shape[1], img.shape[0], 3, fmt=vlb.TEXEL_RGBA8)
    assert rel(got, golden[key]) < TOL
    assert rel(got, O.skybox_sh(img, 1, layout, img.shape[1], img.shape[0], 3)) < TOL


def test_bgra_swap_flag(ctx, golden):
    img = golden["img"]
    got = ctx.skybox_sh(img, vlb.SKY_PANORAMA, 32, 16, 3, fmt=vlb.TEXEL_RGBA8, flags=vlb.SKY_REF_BGRA_SWAP)
    ref = O.skybox_sh(img, 1, 1, 32, 16, 3, flags=1)
    assert rel(got, ref) < TOL
    plain = ctx.skybox_sh(img, vlb.SKY_PANORAMA, 32, 16, 3, fmt=vlb.TEXEL_RGBA8)
    assert np.allclose(got[:, 0], plain[:, 2]) and np.allclose(got[:, 2], plain[:, 0])


@pytest.mark.parametrize("lmax", [2, 3])
@pytest.mark.parametrize("n,count", [(64, 5), (40, 21)])
def test_batched_equals_single_bit_exact(ctx, lmax, n, count):
    """A map's result is the same bits alone, in a batch, and at any place in
    it (21 maps: a group of 16 and a partial one; face 40: a partial last
    chunk of 256 texels)."""
    maps = np.stack([vlb.synth_cubemap(s, n) for s in range(count)])
    batch = ctx.skybox_sh(maps, vlb.SKY_CUBEMAP, n, n, lmax, count=count)
    shifted = ctx.skybox_sh(maps[1:], vlb.SKY_CUBEMAP, n, n, lmax, count=count - 1)
    for i in range(count):
        one = ctx.skybox_sh(maps[i], vlb.SKY_CUBEMAP, n, n, lmax)
        assert np.array_equal(batch[i], one)
        if i:
            assert np.array_equal(shifted[i - 1], one)
        if i < 3:
            assert rel(one, O.skybox_sh(maps[i], 0, 0, n, n, lmax)) < TOL


def test_repeatable(ctx):
    cm = vlb.synth_cubemap(5, 128)
    a = ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 128, 128, 3)
    b = ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 128, 128, 3)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("w,h", [(33, 17), (1, 1), (3, 2), (1000, 3)])
def test_ragged_panorama_sizes(ctx, w, h):
    rng = np.random.default_rng(w * 7 + h)
    img = rng.random((h, w, 3)).astype(np.float32)
    got = ctx.skybox_sh(img, vlb.SKY_ENVMAP, w, h, 3)
    ref = O.skybox_sh(img, 0, 2, w, h, 3)
    assert rel(got, ref) < TOL


@pytest.mark.parametrize("n", [1, 3, 130])
def test_odd_cube_sizes(ctx, n):
    cm = vlb.synth_cubemap(n, n)
    got = ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, n, n, 3)
    assert rel(got, O.skybox_sh(cm, 0, 0, n, n, 3)) < TOL


def test_device_input_and_output(ctx):
    torch = pytest.importorskip("torch")
    cm = vlb.synth_cubemap(77, 128)
    dev = torch.from_numpy(cm).cuda()
    out = torch.empty((1, 16, 3), dtype=torch.float32, device="cuda")
    ctx.skybox_sh(dev, vlb.SKY_CUBEMAP, 128, 128, 3, out=out)
    ctx.synchronize()
    assert rel(out.cpu().numpy()[0], O.skybox_sh(cm, 0, 0, 128, 128, 3)) < TOL


def test_invalid_arguments_are_reported(ctx):
    cm = vlb.synth_cubemap(1, 8)
    with pytest.raises(vlb.VlbError) as e:
        ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 8, 8, lmax=5)
    assert e.value.status == vlb.ERR_INVALID
    with pytest.raises(vlb.VlbError):
        ctx.skybox_sh(cm, vlb.SKY_CUBEMAP, 8, 4, lmax=2)
