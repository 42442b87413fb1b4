"""vlb_skybox_sh_noalloc: the skybox projection for callers that cannot
allocate device memory at call time (its scratch is an array inside the
library).  Called through the C ABI with device buffers and compared with the
allocating entry point vlb_skybox_sh, within the skybox tests' tolerance, on
two calls in a row -- the second, smaller call reuses the array that the
first one left behind.  This file is collected last on purpose."""
import numpy as np
import pytest

import oracle as O
import vlb

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


def _noalloc(torch, texels, fmt, layout, w, h, lmax, flags=0):
    dev_in = texels if hasattr(texels, "data_ptr") else torch.from_numpy(np.ascontiguousarray(texels)).cuda()
    dev_out = torch.full((vlb.k_of(lmax), 3), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = vlb.lib.vlb_skybox_sh_noalloc(dev_in.data_ptr(), fmt, layout, w, h, lmax, flags, dev_out.data_ptr(), None)
    assert st == vlb.OK, vlb.lib.vlb_status_string(st)
    return dev_out.cpu().numpy()


def test_two_calls_match_allocating_entry(ctx):
    torch = pytest.importorskip("torch")
    big = vlb.synth_cubemap(31, 128)
    small = vlb.synth_cubemap(32, 64)
    first = _noalloc(torch, big, vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 128, 128, 3)
    second = _noalloc(torch, small, vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 64, 64, 2)
    assert rel(first, ctx.skybox_sh(big, vlb.SKY_CUBEMAP, 128, 128, 3)) < TOL
    assert rel(second, ctx.skybox_sh(small, vlb.SKY_CUBEMAP, 64, 64, 2)) < TOL
    # and against the FP64 oracle directly
    assert rel(first, O.skybox_sh(big, 0, vlb.SKY_CUBEMAP, 128, 128, 3)) < TOL
    assert rel(second, O.skybox_sh(small, 0, vlb.SKY_CUBEMAP, 64, 64, 2)) < TOL


def test_documented_maximum_sizes(ctx):
    """The largest maps the array is sized for: 6 x 256^2 cubemap faces (the
    oracle checks it) and an 8192 x 8192 RGBA8 panorama (checked against the
    allocating entry), the panorama with the reference's R/B swap."""
    torch = pytest.importorskip("torch")
    cube = vlb.synth_cubemap(41, 256)
    got = _noalloc(torch, cube, vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 256, 256, 3)
    assert rel(got, O.skybox_sh(cube, 0, vlb.SKY_CUBEMAP, 256, 256, 3)) < TOL
    g = torch.Generator(device="cuda").manual_seed(7)
    pano = torch.randint(0, 256, (8192, 8192, 4), dtype=torch.uint8, device="cuda", generator=g)
    got = _noalloc(torch, pano, vlb.TEXEL_RGBA8, vlb.SKY_PANORAMA, 8192, 8192, 3, flags=vlb.SKY_REF_BGRA_SWAP)
    ref = ctx.skybox_sh(pano, vlb.SKY_PANORAMA, 8192, 8192, 3, fmt=vlb.TEXEL_RGBA8, flags=vlb.SKY_REF_BGRA_SWAP)
    assert rel(got, ref) < TOL
    del pano
    torch.cuda.empty_cache()


def test_panorama_layouts_match_allocating_entry(ctx, golden):
    torch = pytest.importorskip("torch")
    img = golden["img"]
    for layout in (vlb.SKY_PANORAMA, vlb.SKY_ENVMAP):
        got = _noalloc(torch, img, vlb.TEXEL_RGBA8, layout, 32, 16, 3)
        ref = ctx.skybox_sh(img, layout, 32, 16, 3, fmt=vlb.TEXEL_RGBA8)
        assert rel(got, ref) < TOL


def test_rejects_host_memory_and_oversize(ctx):
    torch = pytest.importorskip("torch")
    host = vlb.synth_cubemap(1, 16)
    out = torch.empty((9, 3), dtype=torch.float32, device="cuda")
    st = vlb.lib.vlb_skybox_sh_noalloc(host.ctypes.data, vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 16, 16, 2, 0,
                                       out.data_ptr(), None)
    assert st == vlb.ERR_INVALID
    big = torch.zeros((6, 257, 257, 3), dtype=torch.float32, device="cuda")
    st = vlb.lib.vlb_skybox_sh_noalloc(big.data_ptr(), vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 257, 257, 2, 0,
                                       out.data_ptr(), None)
    assert st == vlb.ERR_INVALID
    ok = torch.zeros((6, 16, 16, 3), dtype=torch.float32, device="cuda")
    st = vlb.lib.vlb_skybox_sh_noalloc(ok.data_ptr(), vlb.TEXEL_RGB32F, vlb.SKY_CUBEMAP, 16, 16, 2, 0x80,
                                       out.data_ptr(), None)
    assert st == vlb.ERR_INVALID  # unknown flag bits
