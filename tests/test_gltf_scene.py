"""glTF scene ingestion (vlb_gltf_mesh_*, host only) against a numpy
restatement of the node transforms: world = parent chain of T * R * S * M
(scene_manager.cpp:463-477), positions in FP64 rounded once to FP32,
triangles of scene 0, baseColorFactor albedo."""
import base64
import json
import struct

import numpy as np
import pytest

import vlb


def quat_mat(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w), 0],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w), 0],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y), 0],
                     [0, 0, 0, 1]])


def local(node):
    T = np.eye(4)
    T[:3, 3] = node.get("translation", [0, 0, 0])
    R = quat_mat(node["rotation"]) if "rotation" in node else np.eye(4)
    S = np.diag(list(node.get("scale", [1, 1, 1])) + [1.0])
    M = np.array(node["matrix"], np.float64).reshape(4, 4).T if "matrix" in node else np.eye(4)
    return T @ R @ S @ M


def build_case(tmp_path, kind):
    """A 2-mesh, 4-node glTF: nested TRS / quaternion / matrix transforms,
    u8, u16, u32 and missing indices, interleaved positions, two materials."""
    rng = np.random.default_rng(7)
    blobs, views, accs = [], [], []

    def add(arr, target_type, ctype, count, stride=0):
        off = sum(len(b) for b in blobs)
        data = arr.tobytes()
        data += b"\0" * ((4 - len(data) % 4) % 4)
        blobs.append(data)
        v = {"buffer": 0, "byteOffset": off, "byteLength": len(arr.tobytes())}
        if stride:
            v["byteStride"] = stride
        views.append(v)
        accs.append({"bufferView": len(views) - 1, "componentType": ctype, "count": count, "type": target_type})
        return len(accs) - 1

    p0 = rng.uniform(-1, 1, (6, 3)).astype(np.float32)
    inter = np.zeros((5, 6), np.float32)  # position + something else, 24-byte stride
    p1 = rng.uniform(-2, 2, (5, 3)).astype(np.float32)
    inter[:, :3] = p1
    a_p0 = add(p0, "VEC3", 5126, 6)
    a_p1 = add(inter, "VEC3", 5126, 5, stride=24)
    i8 = np.uint8([0, 1, 2, 3, 4, 5])
    i16 = np.uint16([0, 1, 2, 2, 3, 4, 4, 1, 0])
    i32 = np.uint32([5, 4, 3])
    a_i8, a_i16, a_i32 = add(i8, "SCALAR", 5121, 6), add(i16, "SCALAR", 5123, 9), add(i32, "SCALAR", 5125, 3)
    meshes = [{"primitives": [{"attributes": {"POSITION": a_p0}, "indices": a_i8, "material": 0},
                              {"attributes": {"POSITION": a_p0}, "indices": a_i32}]},
              {"primitives": [{"attributes": {"POSITION": a_p1}, "indices": a_i16, "material": 1},
                              {"attributes": {"POSITION": a_p1}, "material": 1, "mode": 1},
                              {"attributes": {"POSITION": a_p1}}]}]  # no indices: 5 vertices, 1 triangle
    nodes = [{"translation": [1, 2, 3], "rotation": [0.2, 0.3, 0.1, 0.927], "scale": [1, 2, 0.5], "children": [1, 2],
              "mesh": 0},
             {"matrix": [1, 0, 0, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0.5, 0.25, -1, 1], "mesh": 1, "children": [3]},
             {"translation": [-4, 0, 0], "mesh": 1},
             {"scale": [3, 3, 3], "mesh": 0},
             {"mesh": 1}]  # not in scene 0: ignored
    mats = [{"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1]}},
            {"pbrMetallicRoughness": {"metallicFactor": 0}}]
    binary = b"".join(blobs)
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": nodes, "meshes": meshes,
           "materials": mats, "accessors": accs, "bufferViews": views,
           "buffers": [{"byteLength": len(binary)}]}
    if kind == "bin":
        (tmp_path / "my scene.bin").write_bytes(binary)
        doc["buffers"][0]["uri"] = "my%20scene.bin"
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(doc))
    elif kind == "datauri":
        doc["buffers"][0]["uri"] = "data:application/gltf-buffer;base64," + base64.b64encode(binary).decode()
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(doc))
    else:
        js = json.dumps(doc).encode()
        js += b" " * ((4 - len(js) % 4) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(binary), 0x004E4942) + binary
        path = tmp_path / "scene.glb"
        path.write_bytes(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)

    # expected: depth-first from scene 0's roots
    pos, idx, alb = [], [], []

    def visit(ni, parent):
        W = parent @ local(nodes[ni])
        for prim in meshes[nodes[ni]["mesh"]]["primitives"] if "mesh" in nodes[ni] else []:
            if prim.get("mode", 4) != 4:
                continue
            src = p0 if prim["attributes"]["POSITION"] == a_p0 else p1
            base = sum(len(p) for p in pos)
            w = (W[:3, :3] @ src.astype(np.float64).T).T + W[:3, 3]
            pos.append(w.astype(np.float32))
            ind = {a_i8: i8, a_i16: i16, a_i32: i32}.get(prim.get("indices"), np.arange(len(src)))
            tri = ind[: len(ind) // 3 * 3].astype(np.uint32).reshape(-1, 3) + base
            idx.append(tri)
            m = prim.get("material")
            rgb = mats[m]["pbrMetallicRoughness"].get("baseColorFactor", [1, 1, 1])[:3] if m is not None else [1, 1, 1]
            alb.append(np.tile(np.float32(rgb), (len(tri), 1)))
        for c in nodes[ni].get("children", []):
            visit(c, W)

    visit(0, np.eye(4))
    return path, np.concatenate(pos), np.concatenate(idx), np.concatenate(alb)


@pytest.mark.parametrize("kind", ["bin", "datauri", "glb"])
def test_gltf_scene_geometry(tmp_path, kind):
    path, epos, eidx, ealb = build_case(tmp_path, kind)
    pos, idx, alb, bounds = vlb.gltf_load_mesh(path)
    assert np.array_equal(idx, eidx) and np.array_equal(alb, ealb)
    assert pos.shape == epos.shape
    assert np.abs(pos - epos).max() <= 4e-7 * max(1.0, np.abs(epos).max())
    assert np.allclose(bounds, np.concatenate([pos.min(0), pos.max(0)]))


def test_gltf_scene_errors(tmp_path):
    path, *_ = build_case(tmp_path, "bin")
    doc = json.loads(path.read_text())
    doc["accessors"][0]["count"] = 1000  # reads past its bufferView
    bad = tmp_path / "bad.gltf"
    bad.write_text(json.dumps(doc))
    with pytest.raises(vlb.VlbError):
        vlb.gltf_load_mesh(bad)
    doc = json.loads(path.read_text())
    doc["nodes"][3]["children"] = [0]  # a cycle
    bad.write_text(json.dumps(doc))
    with pytest.raises(vlb.VlbError):
        vlb.gltf_load_mesh(bad)
    with pytest.raises(vlb.VlbError):
        vlb.gltf_load_mesh(tmp_path / "nope.gltf")


@pytest.mark.gpu
def test_scene_from_gltf_bakes_like_arrays(ctx, tmp_path):
    path, epos, eidx, ealb = build_case(tmp_path, "glb")
    s1 = ctx.scene_gltf(path)
    pos, idx, alb, _ = vlb.gltf_load_mesh(path)
    s2 = ctx.scene(pos, idx, alb)
    assert s1.ntris == len(idx)
    probes = np.random.default_rng(1).uniform(-3, 3, (64, 3)).astype(np.float32)
    p = vlb.bake_params(ctx.fibonacci(64), 2, vlb.PREC_FP32, (0.3, 1, 0.2))
    assert np.array_equal(ctx.bake(s1, probes, p), ctx.bake(s2, probes, p))
