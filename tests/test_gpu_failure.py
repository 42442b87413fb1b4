"""Failure paths on the GPU, made without faulting it.

- A traversal stack overflow: a scene whose traversal tree is a chain about
  99 nodes deep (triangles at geometrically growing distances and sizes, so
  the clustering merges one triangle at a time), walked by rays that enter
  every node's two children.  Every push is bounds-checked; the overflow is
  counted on the device and the bake returns VLB_ERR_INTERNAL.
- Bounded mbarrier waits that run out: the test hook holds the producer of
  the TMA pipelines (it issues no copy, so none is in flight), the waiting
  threads give up after a short bound and the call returns VLB_ERR_TIMEOUT.

In both cases the next call on the same context succeeds and returns what a
fresh context returns.
"""
import numpy as np
import pytest

import vlb

pytestmark = pytest.mark.gpu


def chain_scene(n=100, ratio=1.3):
    """Triangle k lies in the plane x = ratio^k, spans 6 ratio^k in y and z
    and contains the x axis; the union box of the cluster below it is always
    smaller than its union with the next triangle, so every clustering round
    merges the lowest pair only: a chain n - 1 nodes deep.  (ratio^n stays
    near 2e11, so the FP32 triangle test's products stay finite.)"""
    x = ratio ** np.arange(n, dtype=np.float64)
    s = 2.0 * x
    tri = np.zeros((n, 3, 3), np.float64)
    tri[:, :, 0] = x[:, None]
    tri[:, 0, 1], tri[:, 0, 2] = -s, -s
    tri[:, 1, 1], tri[:, 1, 2] = 2 * s, -s
    tri[:, 2, 1], tri[:, 2, 2] = -s, 2 * s
    pos = tri.reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    alb = np.full((n, 3), 0.5, np.float32)
    return pos, idx, alb


def small_scene():
    pos, idx, alb = vlb.synth_box_scene(2, 8)
    probes = np.array([[0.5, 0.5, -0.5], [-0.2, 0.4, 0.3]], np.float32)
    return pos, idx, alb, probes


@pytest.mark.parametrize("prec,flags", [(vlb.PREC_FP32, vlb.BAKE_TRAVERSAL_LANE),
                                        (vlb.PREC_FP32, vlb.BAKE_TRAVERSAL_PACKET),
                                        (vlb.PREC_FUSED, 0)])
def test_stack_overflow_is_an_internal_error(ctx, prec, flags):
    pos, idx, alb = chain_scene()
    scene = ctx.scene(pos, idx, alb)
    probes = np.zeros((32, 3), np.float32)
    ds = ctx.fibonacci(256)
    p = vlb.bake_params(ds, 2, prec, (0.0, 1.0, 0.0), flags=flags)
    p.tmax = 1e13  # the chain reaches 1.3^99 ~ 2e11
    with pytest.raises(vlb.VlbError) as e:
        ctx.bake(scene, probes, p)
    assert e.value.status == vlb.ERR_INTERNAL and "stack overflow" in e.value.message, e.value
    # the context stays usable: a normal scene bakes as on a fresh context
    spos, sidx, salb, sprobes = small_scene()
    sp = vlb.bake_params(ds, 2, prec, (0.3, 0.8, 0.2), flags=flags)
    got = ctx.bake(ctx.scene(spos, sidx, salb), sprobes, sp)
    fresh = vlb.Context(0)
    try:
        want = fresh.bake(fresh.scene(spos, sidx, salb), sprobes,
                          vlb.bake_params(fresh.fibonacci(256), 2, prec, (0.3, 0.8, 0.2), flags=flags))
    finally:
        fresh.close()
    assert np.array_equal(got, want)


def test_skybox_wait_runs_out(ctx):
    sky = vlb.synth_cubemap(3, 64)
    good = ctx.skybox_sh(sky, vlb.SKY_CUBEMAP, 64, 64, lmax=3)
    ctx.test_hook(vlb.HOOK_HOLD_PRODUCER, 1024)
    try:
        with pytest.raises(vlb.VlbError) as e:
            ctx.skybox_sh(sky, vlb.SKY_CUBEMAP, 64, 64, lmax=3)
        assert e.value.status == vlb.ERR_TIMEOUT, e.value
    finally:
        ctx.test_hook(0)
    assert np.array_equal(ctx.skybox_sh(sky, vlb.SKY_CUBEMAP, 64, 64, lmax=3), good)


def test_tensor_core_projection_wait_runs_out(ctx):
    """The tcgen05 projection: its MMA thread and epilogue warps give up, the
    kernel frees its tensor memory (the next launch allocates it again)."""
    torch = pytest.importorskip("torch")
    n, S = 100, 1024
    ds = ctx.fibonacci(S)
    g = torch.Generator().manual_seed(9)
    bits = (torch.rand((n, 3, S), generator=g) * 5).to(torch.bfloat16).view(torch.int16).numpy().copy()
    good = ctx.project(bits, n, ds, 3, dtype=vlb.DTYPE_BF16)
    ctx.test_hook(vlb.HOOK_HOLD_PRODUCER, 1024)
    try:
        with pytest.raises(vlb.VlbError) as e:
            ctx.project(bits, n, ds, 3, dtype=vlb.DTYPE_BF16)
        assert e.value.status == vlb.ERR_TIMEOUT, e.value
    finally:
        ctx.test_hook(0)
    for _ in range(3):
        assert np.array_equal(ctx.project(bits, n, ds, 3, dtype=vlb.DTYPE_BF16), good)


def test_fp32_projection_wait_runs_out(ctx):
    """The TMA-staged FP32 projection (the default bake's, for tiles of at
    least one 256-row tile per SM): its consumer warps give up when the
    producer is held."""
    n, S = 16384, 1024
    ds = ctx.fibonacci(S)
    rad = np.random.default_rng(11).random((n, 3, S)).astype(np.float32)
    good = ctx.project(rad, n, ds, 2)
    ctx.test_hook(vlb.HOOK_HOLD_PRODUCER, 1024)
    try:
        with pytest.raises(vlb.VlbError) as e:
            ctx.project(rad, n, ds, 2)
        assert e.value.status == vlb.ERR_TIMEOUT, e.value
    finally:
        ctx.test_hook(0)
    assert np.array_equal(ctx.project(rad, n, ds, 2), good)


def test_hook_is_validated(ctx):
    with pytest.raises(vlb.VlbError) as e:
        ctx.test_hook(7)
    assert e.value.status == vlb.ERR_INVALID
