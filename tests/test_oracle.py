"""The FP64 oracle against the reference's own code and analytic known answers.

The golden fixture was produced by the reference header shaders/sh_common.h
compiled in place (tests/golden/make_golden.py); when the shim library is
present (a checkout with the reference next to it) the oracle is also checked
against it directly.
"""
import numpy as np
import pytest

import oracle as O


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300)


# ---- pinned against the reference ----------------------------------------------------
def test_basis_matches_reference_golden(golden):
    got = O.sh_basis(4, golden["dirs"].astype(np.float64))
    ref = golden["basis"].astype(np.float64)
    # the shader evaluates in FP32: agreement to FP32 rounding of the products
    assert np.max(np.abs(got - ref) / np.maximum(1.0, np.abs(ref))) < 3e-6


def test_angle_maps_match_reference_golden(golden):
    W, H = int(golden["W"]), int(golden["H"])
    for x in range(W):
        phi, _ = O.x2phi_y2theta(x, W, 0, H)
        assert abs(phi - golden["phi"][x]) < 1e-6
    for y in range(H):
        _, th = O.x2phi_y2theta(0, W, y, H)
        assert abs(th - golden["theta"][y]) < 1e-6
    for y in range(H):
        for x in range(W):
            v = O.to_vector(float(golden["phi"][x]), float(golden["theta"][y]))
            assert np.max(np.abs(v - golden["to_vector"][y, x])) < 1e-6


def test_skybox_panorama_matches_reference_golden(golden):
    img = golden["img"]
    got = O.skybox_sh(img, 1, 1, img.shape[1], img.shape[0], 3)
    assert rel(got, golden["skybox"]) < 2e-6


def test_envmap_projection_matches_reference_golden(golden):
    img = golden["img"]
    got = O.skybox_sh(img, 1, 2, img.shape[1], img.shape[0], 3)
    assert rel(got, golden["envmap"]) < 2e-6


def test_sh_sum_matches_reference_golden(golden):
    w, h = (int(v) for v in golden["recon_wh"])
    got = O.sh_eval_envmap(golden["coeffs"].astype(np.float64), 3, w, h, 1250.0)
    assert rel(got, golden["recon"]) < 1e-5


def test_probe_grid_matches_reference_order(golden):
    pos, step = O.probe_grid_ref_order([0, 0, 0, 1, 1, 1], [3, 3, 3])
    assert np.array_equal(pos, golden["grid"])
    assert np.array_equal(step, np.float32([0.5, 0.5, 0.5]))


def test_oracle_against_reference_shim_directly():
    ref = O.load_ref()
    if ref is None:
        pytest.skip("reference shim not built (reference checkout absent)")
    rng = np.random.default_rng(7)
    v = rng.normal(size=(500, 3))
    d = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    ours = O.sh_basis(4, d.astype(np.float64))
    for i in range(d.shape[0]):
        for l in range(5):
            for m in range(-l, l + 1):
                r = ref.ref_sh(l, m, *map(float, d[i]))
                assert abs(ours[i, l * (l + 1) + m] - r) <= 3e-6 * max(1.0, abs(r))
    assert abs(ref.ref_pi() - np.float32(3.1415926538)) == 0.0


# ---- analytic known answers ---------------------------------------------------------
def test_cube_solid_angles_sum_to_4pi():
    for n in (1, 2, 7, 64):
        assert abs(6 * O.cube_solid_angle(n).sum() - 4 * np.pi) < 1e-12


def test_constant_radiance_projects_to_dc_only():
    n = 16
    tex = np.full((6, n, n, 3), 2.0, np.float32)
    c = O.skybox_sh(tex, 0, 0, n, n, 3)
    assert np.allclose(c[0], 2.0 * 0.282095 * 4 * np.pi, rtol=1e-12)
    assert np.max(np.abs(c[1:])) < 1e-12


def test_equirect_weights_approach_4pi():
    _, _, w = O.dirs_equirect(3141, 1000)
    assert abs(w.sum() - 4 * np.pi) < 1e-5


def test_fibonacci_set_is_unit_and_equal_weight():
    d, w = O.dirs_fibonacci(1024)
    assert np.max(np.abs(np.linalg.norm(d.astype(np.float64), axis=1) - 1)) < 1e-7
    assert np.allclose(w.sum(), 4 * np.pi)


def test_basis_nearly_orthonormal_under_fine_quadrature():
    d, w = O.dirs_fibonacci(200_000)
    B = O.sh_basis(3, d.astype(np.float64))
    G = (B * w[:, None]).T @ B
    # the reference's 6-digit constants limit orthonormality to ~1e-6
    assert np.max(np.abs(G - np.eye(16))) < 2e-5


def test_cubemap_round_trip_of_band_limited_signal():
    n = 64
    rng = np.random.default_rng(3)
    coeffs = rng.normal(size=(9, 3))
    dirs = O.cube_texel_dirs(n).reshape(-1, 3)
    tex = (O.sh_basis(2, dirs) @ coeffs).astype(np.float32).reshape(6, n, n, 3)
    got = O.skybox_sh(tex, 0, 0, n, n, 2)
    assert rel(got, coeffs) < 2e-4


def test_reconstruction_inverts_envmap_projection():
    rng = np.random.default_rng(5)
    coeffs = rng.normal(size=(16, 3))
    W, H = 512, 256
    img = O.sh_eval_envmap(coeffs, 3, W, H, 1.0).astype(np.float32)
    back = O.skybox_sh(img, 0, 2, W, H, 3)
    assert rel(back, coeffs) < 1e-4


# ---- LBVH structure --------------------------------------------------------------------
def _check_lbvh(pos, idx, L):
    n = idx.shape[0]
    codes, order, child, box = L["codes"], L["order"], L["child"], L["box"]
    assert np.all(np.diff(codes.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(order), np.arange(n))
    # stability: equal codes keep triangle order
    same = codes[1:] == codes[:-1]
    assert np.all(order[1:][same] > order[:-1][same])
    tri_lo = pos[idx].min(axis=1)
    tri_hi = pos[idx].max(axis=1)
    leaf0 = n - 1
    assert np.array_equal(box[leaf0:, :3], tri_lo[order]) and np.array_equal(box[leaf0:, 3:], tri_hi[order])
    if n == 1:
        return
    seen = np.zeros(2 * n - 1, np.int32)
    for i in range(n - 1):
        kids = [c if c >= 0 else leaf0 + ~c for c in child[2 * i:2 * i + 2]]
        for k in kids:
            seen[k] += 1
        assert np.array_equal(box[i, :3], np.minimum(box[kids[0], :3], box[kids[1], :3]))
        assert np.array_equal(box[i, 3:], np.maximum(box[kids[0], 3:], box[kids[1], 3:]))
    assert seen[0] == 0 and np.all(seen[1:] == 1)


def test_oracle_lbvh_is_a_valid_tree():
    import vlb

    pos, idx, _ = vlb.synth_box_scene(1, 64)
    _check_lbvh(pos, idx, O.lbvh_build(pos, idx))
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 17, 300):
        p = rng.random((3 * n, 3)).astype(np.float32)
        i = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
        _check_lbvh(p, i, O.lbvh_build(p, i))
    # all centroids identical: every code equal, ties broken by index
    p = np.tile(np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]]), (40, 1))
    i = np.arange(120, dtype=np.uint32).reshape(40, 3)
    _check_lbvh(p, i, O.lbvh_build(p, i))


# ---- bake known answers ------------------------------------------------------------------
def test_bake_open_sky_equals_sky_projection():
    """No geometry: every ray sees the sky texel in its direction."""
    n = 16
    sky = np.full((6, n, n, 3), 0.7, np.float32)
    sc = O.Scene(np.zeros((3, 3), np.float32), np.zeros((0, 3), np.uint32), np.zeros((0, 3), np.float32))
    d, w = O.dirs_fibonacci(256)
    B = O.basis_matrix(d.astype(np.float64), w, 2)
    sh = sc.bake(np.float32([[0.5, 0.5, 0.5]]), d, B, [0, 1, 0], sky=sky, sky_n=n)
    assert np.allclose(sh[0, 0], float(np.float32(0.7)) * 0.282095 * 4 * np.pi, rtol=1e-12)


def test_bake_lit_floor_lambert():
    """A huge floor under the probe, sun overhead, black sky: hits carry albedo*5/pi."""
    big = 1e3
    pos = np.float32([[-big, 0, -big], [big, 0, -big], [0, 0, big]])
    sc = O.Scene(pos, np.uint32([[0, 1, 2]]), np.float32([[0.5, 0.25, 1.0]]))
    d, w = O.dirs_fibonacci(512)
    B = O.basis_matrix(d.astype(np.float64), w, 2)
    sh, hit, vis, edge, rad = sc.bake(np.float32([[0, 1, 0]]), d, B, [0, 1, 0], per_ray=True)
    down = d[:, 1] < 0
    assert np.array_equal(hit[0] >= 0, down)
    assert np.all(vis[0][down] == 1)
    L = np.where(down[:, None], np.float64([0.5, 0.25, 1.0]) * 5 / np.pi, 0.0)
    assert np.allclose(sh[0], B.T @ L, rtol=1e-12)


def test_bake_probe_inside_closed_box_is_dark():
    import vlb

    pos, idx, alb = vlb.synth_box_scene(11, 1)
    box = pos[8:16]
    c = (box.min(0) + box.max(0)) / 2
    sc = O.Scene(pos, idx, alb)
    d, w = O.dirs_fibonacci(128)
    B = O.basis_matrix(d.astype(np.float64), w, 3)
    sh = sc.bake(c[None].astype(np.float32), d, B, vlb.synth_sun(1))
    assert np.max(np.abs(sh)) == 0.0


def test_probe_eval_oracle_indexes_the_bake_grid_order():
    """With no occluders the oracle's probe evaluation is a weighted mean of the
    8 corner probes, looked up in the bake's breadth-first order: give every
    probe a DC coefficient equal to its x (resp. y, z) position and the
    evaluation at a cell's centre returns the centre's coordinate."""
    import vlb

    bounds = np.float32([-1.0, 0.0, 2.0, 3.0, 1.5, 4.0])
    counts = np.uint32([5, 3, 4])
    pos, step = vlb.probe_grid_ref_order(bounds, counts)
    K = 9
    y00 = 0.282095
    rng = np.random.default_rng(1)
    pts = (bounds[:3] + rng.random((64, 3)) * (bounds[3:] - bounds[:3])).astype(np.float32)
    cell = np.clip(np.floor((pts - bounds[:3]) / step), 0, counts - 2)
    nrm = rng.standard_normal((64, 3)).astype(np.float32)
    for axis in range(3):
        coeffs = np.zeros((pos.shape[0], K, 3), np.float32)
        coeffs[:, 0, :] = (pos[:, axis] / y00)[:, None]
        out, vis, _ = O.probe_eval(None, coeffs, 2, bounds[:3], step, counts, pts, nrm)
        assert np.all(vis == 255)
        # expected: the distance-weighted mean of the 8 corner positions along the axis
        wmax = np.linalg.norm(step.astype(np.float64))
        exp = np.zeros(len(pts))
        for i, (p, c) in enumerate(zip(pts, cell)):
            num = den = 0.0
            for corner in range(8):
                bits = np.array([(corner >> 2) & 1, (corner >> 1) & 1, corner & 1])
                ijk = np.minimum(c + bits, counts - 1)
                q = (bounds[:3] + step * ijk.astype(np.float32)).astype(np.float64)
                w = wmax - np.linalg.norm(q - p)
                num += w * q[axis]
                den += w
            exp[i] = num / den
        assert np.allclose(out[:, 0], exp, rtol=0, atol=1e-5)


@pytest.mark.parametrize("seed,nboxes", [(1, 64), (1, 4096), (7, 0), (31, 700)])
def test_oracle_workload_generators_match_library(seed, nboxes):
    """The oracle's restated seeded generators (the CPU baseline builds its
    inputs with them, without the product library) give the library's inputs
    bit for bit."""
    import vlb

    for a, b in zip(O.synth_box_scene(seed, nboxes), vlb.synth_box_scene(seed, nboxes)):
        assert a.dtype == b.dtype and np.array_equal(a.reshape(b.shape), b)
    assert np.array_equal(O.synth_cubemap(seed, 32).reshape(-1), vlb.synth_cubemap(seed, 32).reshape(-1))
    assert np.array_equal(O.synth_sun(seed), vlb.synth_sun(seed))
