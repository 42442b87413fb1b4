"""Baked-light glTF files (host only): vlb_gltf_write_light / vlb_gltf_read_light.

The reference re-prints the whole glTF through its JSON library after adding
the coefficient buffer (src/baker/light_baker.cpp:375-401): sorted keys,
4-space indentation, shortest round-trip doubles, UTF-8 passed through.
Python's json module prints with the same conventions (sort_keys, indent=4,
ensure_ascii=False, repr floats), so for documents without numbers in
[1e15, 1e16) -- where the two libraries switch to exponent notation at
different points -- the expected file is built with it, byte for byte.
"""
import base64
import json

import numpy as np
import pytest

import vlb

DOC = """{
  "asset": {"version": "2.0", "generator": "caf\\u00e9 \\"test\\" \\t tab / \\/ slash \\ud83d\\ude00"},
  "scene": 0, "scenes": [{"nodes": [0, 1]}],
  "nodes": [{"mesh": 0, "translation": [1.0, -0.0, 2.5e-7], "scale": [1e-5, 0.0001, 123456.75]},
            {"mesh": 0, "matrix": [1,0,0,0, 0,1,0,0, 0,0,1,0, 0.1,0.2,0.3,1], "extras": {}}],
  "meshes": [{"primitives": [{"attributes": {"POSITION": 1}, "indices": 0}], "weights": []}],
  "accessors": [{"bufferView": 0, "componentType": 5125, "count": 3, "type": "SCALAR", "max": [2], "min": [0]},
                {"bufferView": 1, "componentType": 5126, "count": 3, "type": "VEC3",
                 "max": [1.0, 1.0, 0.0], "min": [-1.5, 0.0, -3.14159265358979]}],
  "bufferViews": [{"buffer": 0, "byteLength": 12, "byteOffset": 0},
                  {"buffer": 0, "byteLength": 36, "byteOffset": 12}],
  "buffers": [{"byteLength": 48, "uri": "data:application/octet-stream;base64,AAAAAAEAAAACAAAA"}],
  "zeta": -17, "alpha": 18446744073709551615, "big": 3.5e+300, "tiny": -2.2250738585072014e-308,
  "flag": true, "none": null
}"""


def expected_text(doc_text, coeffs, grid):
    doc = json.loads(doc_text)
    raw = np.ascontiguousarray(coeffs, np.float32).tobytes()
    doc.setdefault("buffers", []).append(
        {"byteLength": len(raw), "uri": "data:application/octet-stream;base64," + base64.b64encode(raw).decode()})
    doc.setdefault("bufferViews", []).append({"buffer": len(doc["buffers"]) - 1, "byteLength": len(raw),
                                              "byteOffset": 0})
    light = doc.setdefault("light", {})
    light["bufferView"] = len(doc["bufferViews"]) - 1
    light["gridStep"] = {a: float(np.float32(v)) for a, v in zip("xyz", grid)}
    light["lmax"] = coeffs.shape[1]
    return json.dumps(doc, indent=4, sort_keys=True, ensure_ascii=False) + "\n"


@pytest.mark.parametrize("nprobes,K", [(7 ** 3, 16), (5, 9), (1, 16), (0, 16)])
def test_write_matches_reference_printing(nprobes, K):
    rng = np.random.default_rng(nprobes)
    coeffs = (rng.standard_normal((nprobes, K, 3)) * 10).astype(np.float32)
    grid = np.float32([1.0 / 6.0, 0.25, 1e-3])
    got = vlb.gltf_write_light(DOC, coeffs, grid)
    assert got == expected_text(DOC, coeffs, grid)


def test_round_trip_and_reader_rules():
    rng = np.random.default_rng(3)
    coeffs = rng.standard_normal((343, 16, 3)).astype(np.float32)
    grid = np.float32([0.5, 1.0 / 3.0, 2.0])
    text = vlb.gltf_write_light(DOC, coeffs, grid)
    g, k, raw = vlb.gltf_read_light(text)
    assert k == 16 and np.array_equal(g, grid)
    assert np.array_equal(np.frombuffer(raw, np.float32).reshape(343, 16, 3), coeffs)
    # writing twice appends a second buffer; the reader follows the light's bufferView to the newest
    text2 = vlb.gltf_write_light(text, coeffs[:10] * 2, grid)
    g, k, raw = vlb.gltf_read_light(text2)
    assert np.array_equal(np.frombuffer(raw, np.float32).reshape(10, 16, 3), coeffs[:10] * 2)
    assert len(json.loads(text2)["buffers"]) == 3
    # no light: zeros (scene_manager.cpp:639-645)
    g, k, raw = vlb.gltf_read_light(DOC)
    assert k == 0 and raw == b"" and not g.any()


def test_base64_padding_and_decoder_stop():
    for n in range(0, 7):  # every padding case, via whole floats and a final partial triple
        coeffs = np.arange(n * 3, dtype=np.float32).reshape(n, 1, 3) + 0.5
        text = vlb.gltf_write_light("{}", coeffs, [1, 1, 1])
        raw = np.ascontiguousarray(coeffs).tobytes()
        assert base64.b64encode(raw).decode() in text
        assert vlb.gltf_read_light(text)[2] == raw
    # the reference's decoder stops at '=' or any non-alphabet character; byteLength bytes are used
    payload = base64.b64encode(b"\x01\x02\x03\x04\x05\x06").decode()
    doc = {"buffers": [{"byteLength": 3, "uri": "data:application/octet-stream;base64," + payload[:4] + "!!garbage"}],
           "bufferViews": [{"buffer": 0, "byteLength": 3, "byteOffset": 0}],
           "light": {"bufferView": 0, "gridStep": {"x": 1, "y": 2, "z": 3}, "lmax": 16}}
    g, k, raw = vlb.gltf_read_light(json.dumps(doc))
    assert raw == b"\x01\x02\x03" and list(g) == [1, 2, 3]


def test_invalid_documents():
    c = np.zeros((1, 16, 3), np.float32)
    for bad in ("", "[1,2]", '{"a": }', '{"buffers": 3}', '{"light": []}', '{"a": "\\ud800"}', '{"a": 1} x'):
        with pytest.raises(vlb.VlbError) as e:
            vlb.gltf_write_light(bad, c, [1, 1, 1])
        assert e.value.status == vlb.ERR_INVALID
    with pytest.raises(vlb.VlbError):
        vlb.gltf_read_light('{"light": {"bufferView": 4, "gridStep": {"x": 1, "y": 1, "z": 1}, "lmax": 16}}')
