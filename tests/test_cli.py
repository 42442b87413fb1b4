"""vlb-bake, the command-line baker (replaces the reference's `baker`,
src/baker/main.cpp:8-45 with LightBaker::bake / serialize,
src/baker/light_baker.cpp:19-401): argument errors on the host, and on the GPU
a bake of a glTF scene whose written file carries exactly the coefficients of
vlb_bake over the reference's 7x7x7 grid (same library path: bit-exact)."""
import base64
import json
import subprocess

import numpy as np
import pytest

import vlb
import vlb_build


def run_cli(*args):
    return subprocess.run([str(vlb_build.CLI), *map(str, args)], capture_output=True, text=True, timeout=300)


def write_scene(path, seed=3, nboxes=12):
    """A box scene as .gltf with its buffer in a data URI, one material per box
    colour so the albedo survives the round trip through the file."""
    pos, idx, alb = vlb.synth_box_scene(seed, nboxes)
    prims, mats, accs, views, blobs = [], [], [], [], []
    off = 0

    def add(arr, typ, ctype, count):
        nonlocal off
        data = arr.tobytes()
        blobs.append(data + b"\0" * ((4 - len(data) % 4) % 4))
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(data)})
        off += len(blobs[-1])
        accs.append({"bufferView": len(views) - 1, "componentType": ctype, "count": count, "type": typ})
        return len(accs) - 1

    a_pos = add(pos, "VEC3", 5126, len(pos))
    colours = {}
    for t, c in enumerate(map(tuple, alb)):
        colours.setdefault(c, []).append(t)
    for c, tris in colours.items():
        a_idx = add(np.ascontiguousarray(idx[tris]).astype(np.uint32), "SCALAR", 5125, 3 * len(tris))
        mats.append({"pbrMetallicRoughness": {"baseColorFactor": [*map(float, c), 1.0]}})
        prims.append({"attributes": {"POSITION": a_pos}, "indices": a_idx, "material": len(mats) - 1})
    binary = b"".join(blobs)
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": prims}], "materials": mats, "accessors": accs, "bufferViews": views,
           "buffers": [{"byteLength": len(binary),
                        "uri": "data:application/octet-stream;base64," + base64.b64encode(binary).decode()}]}
    path.write_text(json.dumps(doc))
    return path


def test_cli_built():
    assert vlb_build.CLI.exists()


def test_cli_no_scene():
    r = run_cli()
    assert r.returncode == 1 and "Select scene to bake." in r.stderr


@pytest.mark.parametrize("args, msg", [(("--counts", "7"), "missing value"), (("--bogus",), "unknown option"),
                                       (("--dirs", "grid:3"), "bad --dirs"),
                                       (("--precision", "fp16"), "bad --precision")])
def test_cli_bad_arguments(tmp_path, args, msg):
    scene = write_scene(tmp_path / "s.gltf")
    r = run_cli(scene, *args)
    assert r.returncode == 1 and msg in r.stderr


def test_cli_missing_file(tmp_path):
    r = run_cli(tmp_path / "nope.gltf")
    assert r.returncode == 1 and "cannot read" in r.stderr


def test_cli_rejects_glb(tmp_path):
    p = tmp_path / "s.glb"
    p.write_bytes(b"glTF" + b"\0" * 16)
    r = run_cli(p)
    assert r.returncode == 1 and "binary glTF" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("dirs, lmax, prec", [("fib:2048", 3, "fp32"), ("equirect:64x32", 3, "fused"),
                                              ("fib:1000", 2, "mixed")])
def test_cli_bake_matches_library(ctx, tmp_path, dirs, lmax, prec):
    scene_path = write_scene(tmp_path / "boxes.gltf")
    r = run_cli(scene_path, "--dirs", dirs, "--lmax", lmax, "--precision", prec, "--sun", 0.3, 0.8, 0.2,
                "--intensity", 4)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "baked_boxes.gltf"
    text = out.read_text()
    step, K, data = vlb.gltf_read_light(text)
    got = np.frombuffer(data, np.float32).reshape(-1, K, 3)

    scene = ctx.scene_gltf(scene_path)
    probes, ref_step = vlb.probe_grid_ref_order(scene.bounds(include_origin=True), (7, 7, 7))
    if dirs.startswith("fib:"):
        ds = ctx.fibonacci(int(dirs[4:]))
    else:
        w, h = map(int, dirs[9:].split("x"))
        ds = ctx.equirect(w, h)
    p = vlb.bake_params(ds, lmax=lmax, precision={"fp32": vlb.PREC_FP32, "fused": vlb.PREC_FUSED,
                                                  "mixed": vlb.PREC_MIXED}[prec],
                        sun=(0.3, 0.8, 0.2), sun_intensity=4.0)
    want = ctx.bake(scene, probes, p)
    assert K == (lmax + 1) ** 2 and got.shape == (343, K, 3)
    np.testing.assert_array_equal(step, ref_step)
    np.testing.assert_array_equal(got, want)
    assert np.abs(want).max() > 0
    assert text == vlb.gltf_write_light(scene_path.read_text(), want, ref_step)


@pytest.mark.gpu
def test_cli_reference_shading_and_running_sums(ctx, tmp_path):
    """--shading ref --light --accumulate: the library's bake with the
    reference's shading and its carry-over sums."""
    scene_path = write_scene(tmp_path / "r.gltf", seed=2)
    r = run_cli(scene_path, "--dirs", "equirect:64x32", "--shading", "ref", "--light", 0.5, 4, 0.5, "--accumulate",
                "--precision", "fp32")
    assert r.returncode == 0, r.stderr
    step, K, data = vlb.gltf_read_light((tmp_path / "baked_r.gltf").read_text())
    got = np.frombuffer(data, np.float32).reshape(-1, K, 3)
    scene = ctx.scene_gltf(scene_path)
    probes, _ = vlb.probe_grid_ref_order(scene.bounds(include_origin=True), (7, 7, 7))
    p = vlb.bake_params(ctx.equirect(64, 32), 3, vlb.PREC_FP32, shading=vlb.SHADE_REF_PHONG,
                        light_pos=(0.5, 4, 0.5), flags=vlb.BAKE_REF_ACCUMULATE)
    np.testing.assert_array_equal(got, ctx.bake(scene, probes, p))
    assert run_cli(scene_path, "--shading", "phong").returncode == 1


@pytest.mark.gpu
def test_cli_counts_and_out(ctx, tmp_path):
    scene_path = write_scene(tmp_path / "s.gltf", seed=5, nboxes=4)
    out = tmp_path / "sub" / "x.gltf"
    out.parent.mkdir()
    r = run_cli(scene_path, "--counts", 3, 2, 5, "--dirs", "fib:256", "--out", out)
    assert r.returncode == 0, r.stderr
    step, K, data = vlb.gltf_read_light(out.read_text())
    assert K == 16 and len(data) == 3 * 2 * 5 * 16 * 12
    b = ctx.scene_gltf(scene_path).bounds(include_origin=True)
    np.testing.assert_array_equal(step, vlb.probe_grid_ref_order(b, (3, 2, 5))[1])
