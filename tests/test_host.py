"""Host-side logic of libvlb.so that needs no GPU: ABI exports, the reference
probe order, the seeded workload generators."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import vlb

ROOT = Path(__file__).resolve().parents[1]


def _header_functions():
    text = (ROOT / "include" / "vlb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vlb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_function():
    names = _header_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(vlb.lib, n)]
    assert not missing, missing


def test_version_and_status_strings():
    assert vlb.lib.vlb_version() == 1
    assert vlb.lib.vlb_status_string(vlb.ERR_INVALID) == b"invalid argument"


def test_probe_grid_matches_oracle_bit_exact():
    rng = np.random.default_rng(1)
    for _ in range(20):
        lo = rng.uniform(-5, 5, 3).astype(np.float32)
        hi = (lo + rng.uniform(0.1, 9, 3)).astype(np.float32)
        counts = rng.integers(2, 9, 3)
        a, sa = vlb.probe_grid_ref_order(np.concatenate([lo, hi]), counts)
        b, sb = O.probe_grid_ref_order(np.concatenate([lo, hi]), counts)
        assert np.array_equal(a, b) and np.array_equal(sa, sb)


def test_probe_grid_reference_breadth_first_order(golden):
    pos, step = vlb.probe_grid_ref_order([0, 0, 0, 1, 1, 1], [3, 3, 3])
    assert np.array_equal(pos, golden["grid"])


def test_probe_grid_single_count_axis():
    # counts of 1 divide by zero in the reference too; the positions stay at b0
    a, sa = vlb.probe_grid_ref_order([0, 0, 0, 1, 2, 3], [1, 2, 1])
    b, sb = O.probe_grid_ref_order([0, 0, 0, 1, 2, 3], [1, 2, 1])
    assert np.array_equal(a, b)
    assert np.array_equal(sa, sb, equal_nan=True)


def test_probe_grid_rejects_zero_counts():
    with pytest.raises(vlb.VlbError):
        vlb.probe_grid_ref_order([0, 0, 0, 1, 1, 1], [0, 2, 2])


def test_box_scene_generator_matches_config_ranges():
    pos, idx, alb = vlb.synth_box_scene(123, 64)
    assert idx.shape == (778, 3) and pos.shape == (520, 3)
    assert pos.min() >= 0.0 and pos.max() <= 1.0
    boxes = pos[8:].reshape(64, 8, 3)
    lo, hi = boxes.min(1), boxes.max(1)
    c, e = (lo + hi) / 2, hi - lo
    assert np.all((c >= 0.1 - 1e-6) & (c <= 0.9 + 1e-6))
    assert np.all((e >= 0.05 - 1e-6) & (e <= 0.2 + 1e-6))
    a = alb[10:]
    assert np.all((a >= 0.2) & (a <= 0.8))
    assert np.all(alb[:10] == 0.5)
    # 12 triangles per box share one albedo
    assert np.all(a.reshape(64, 12, 3) == a.reshape(64, 12, 3)[:, :1])
    p2, i2, a2 = vlb.synth_box_scene(123, 64)
    assert np.array_equal(pos, p2) and np.array_equal(idx, i2) and np.array_equal(alb, a2)
    p3, _, _ = vlb.synth_box_scene(124, 64)
    assert not np.array_equal(pos, p3)


def test_box_scene_scales_to_config2():
    pos, idx, alb = vlb.synth_box_scene(7, 4096)
    assert idx.shape[0] == 49162


def test_cubemap_generator():
    cm = vlb.synth_cubemap(9, 32)
    assert cm.shape == (6, 32, 32, 3)
    assert cm.min() >= 0.3 - 1e-6
    assert cm.max() > 1.0  # the lobes
    assert np.array_equal(cm, vlb.synth_cubemap(9, 32))


def test_sun_generator_upper_hemisphere():
    for s in range(50):
        d = vlb.synth_sun(s)
        assert d[1] > 0 and abs(np.linalg.norm(d.astype(np.float64)) - 1) < 1e-6


def test_context_creation_fails_cleanly_without_gpu():
    from conftest import HAS_GPU

    if HAS_GPU:
        pytest.skip("a GPU is present")
    with pytest.raises(vlb.VlbError):
        vlb.Context(0)


def test_service_admission_plan():
    """The service's batch cut rule (pure host code): FIFO, probe cap, budget,
    oversize requests refused, a request larger than the cap goes alone."""
    b, n = vlb.service_plan([10, 20, 30, 5, 100], [1, 2, 3, 1, 50], 40, 10)
    assert list(b) == [0, 0, 1, 1, -1] and n == 2
    b, n = vlb.service_plan([100, 1, 1], [1, 1, 1], 40, 10)
    assert list(b) == [0, 1, 1] and n == 2
    b, n = vlb.service_plan([1, 1, 1, 1], [4, 4, 4, 4], 1000, 10)
    assert list(b) == [0, 0, 1, 1] and n == 2
    b, n = vlb.service_plan([1], [11], 1000, 10)
    assert list(b) == [-1] and n == 0
    b, n = vlb.service_plan([], [], 1, 1)
    assert len(b) == 0 and n == 0
    rng = np.random.default_rng(4)
    p = rng.integers(1, 5000, 500)
    by = rng.integers(1, 1 << 20, 500)
    b, n = vlb.service_plan(p, by, 16384, 1 << 22)
    assert np.all(np.diff(b[b >= 0]) >= 0) and b.max() == n - 1  # batches in queue order
    for k in range(n):  # each batch within the caps, and no batch could take the next request
        sel = b == k
        assert by[sel].sum() <= 1 << 22 and (p[sel].sum() <= 16384 or sel.sum() == 1)


def test_node_layout_round_trip(tmp_path):
    """The binary node layout (boxes grouped by axis for the packed box tests):
    pack_node then unpack_node returns both boxes and both references, and the
    packed FMA operands sit where the walk reads them -- (lo x, lo y) and
    (hi x, hi y) of each child in one float4, the four z planes in the third."""
    import shutil
    import subprocess

    import vlb_build

    try:
        cuda_inc = vlb_build._cuda_home() / "include"
    except RuntimeError:
        pytest.skip("needs nvcc's CUDA headers")
    if not shutil.which("g++") or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    src = tmp_path / "node.cpp"
    src.write_text(r'''
#include <cstdio>
#include "vlb_internal.h"
int main() {
  const float b0[6] = {1, 2, 3, 4, 5, 6}, b1[6] = {-1, -2, -3, 7, 8, 9};
  float4 q[4];
  vlbk::pack_node(q, b0, b1, 5, ~7);
  float c0[6], c1[6];
  int32_t r0, r1;
  vlbk::unpack_node(q, c0, c1, &r0, &r1);
  for (int i = 0; i < 6; ++i) if (c0[i] != b0[i] || c1[i] != b1[i]) return 1;
  if (r0 != 5 || r1 != ~7) return 2;
  if (q[0].x != 1 || q[0].y != 2 || q[0].z != 4 || q[0].w != 5) return 3;
  if (q[1].x != -1 || q[1].y != -2 || q[1].z != 7 || q[1].w != 8) return 4;
  if (q[2].x != 3 || q[2].y != 6 || q[2].z != -3 || q[2].w != 9) return 5;
  std::puts("ok");
  return 0;
}
''')
    exe = tmp_path / "node"
    csrc = ROOT / "vulkan-light-bakery_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", f"-I{csrc}", f"-I{cuda_inc}", str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout)
