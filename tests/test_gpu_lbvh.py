"""Device LBVH build is bit-exact with the CPU build of the oracle."""
import numpy as np
import pytest

import oracle as O
import vlb

pytestmark = pytest.mark.gpu


def _compare(ctx, pos, idx, alb=None):
    sc = ctx.scene(pos, idx, alb)
    got = sc.bvh_export()
    ref = O.lbvh_build(pos, idx)
    assert np.array_equal(got["codes"], ref["codes"])
    assert np.array_equal(got["order"], ref["order"])
    assert np.array_equal(got["child"], ref["child"])
    assert np.array_equal(got["box"].view(np.uint32), ref["box"].view(np.uint32))
    return sc


@pytest.mark.parametrize("nboxes", [0, 1, 64, 4096])
def test_box_scenes_bit_exact(ctx, nboxes):
    pos, idx, alb = vlb.synth_box_scene(nboxes + 1, nboxes)
    _compare(ctx, pos, idx, alb)


@pytest.mark.parametrize("n", [1, 2, 3, 255, 4096, 4097, 100_003])
def test_random_soups_bit_exact(ctx, n):
    rng = np.random.default_rng(n)
    pos = (rng.random((3 * n, 3)) * 10 - 5).astype(np.float32)
    idx = rng.permutation(3 * n).astype(np.uint32).reshape(n, 3)
    _compare(ctx, pos, idx)


def test_duplicate_centroids_tie_break(ctx):
    n = 5000
    pos = np.tile(np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]]), (n, 1))
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    _compare(ctx, pos, idx)


def test_strided_reference_vertex_layout(ctx):
    """Positions inside the reference's 48-byte shader::Vertex (structures.h:20-26)."""
    pos, idx, alb = vlb.synth_box_scene(3, 16)
    verts = np.zeros((pos.shape[0], 12), np.float32)
    verts[:, :3] = pos
    verts[:, 3] = 1.0
    sc = ctx.scene(verts, idx, alb, stride_bytes=48)
    ref = O.lbvh_build(pos, idx)
    got = sc.bvh_export()
    assert np.array_equal(got["child"], ref["child"]) and np.array_equal(got["box"], ref["box"])


def test_bad_index_rejected(ctx):
    pos = np.zeros((3, 3), np.float32)
    with pytest.raises(vlb.VlbError) as e:
        ctx.scene(pos, np.uint32([[0, 1, 3]]))
    assert e.value.status == vlb.ERR_INVALID


def test_bounds(ctx):
    pos = np.float32([[1, 2, 3], [2, 3, 4], [1.5, 2.5, 5]])
    sc = ctx.scene(pos, np.uint32([[0, 1, 2]]))
    assert np.array_equal(sc.bounds(False), np.float32([1, 2, 3, 2, 3, 5]))
    assert np.array_equal(sc.bounds(True), np.float32([0, 0, 0, 2, 3, 5]))
