"""vlb_skybox_sh_noalloc: the skybox projection for callers that cannot
allocate device memory at call time (its scratch is an array inside the
library).  Called through the C ABI with device buffers and compared with the
allocating entry point vlb_skybox_sh, within the skybox tests' tolerance, on
two calls in a row -- the second, smaller call reuses the array that the
first one left behind.  This file is collected last on purpose."""
import numpy as np
import pytest

import vlb

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


def _noalloc(torch, texels, fmt, layout, w, h, lmax):
    dev_in = torch.from_numpy(np.ascontiguousarray(texels)).cuda()
    dev_out = torch.full((vlb.k_of(lmax), 3), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = vlb.lib.vlb_skybox_sh_noalloc(dev_in.data_ptr(), fmt, layout, w, h, lmax, 0, dev_out.data_ptr(), None)
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
