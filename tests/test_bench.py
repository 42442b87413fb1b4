"""bench.py's CPU-only parts: the reference arm runs the FP64 restatement on
inputs from the oracle's own generators and never loads the product library;
its config equals the GPU arm's."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_loads_no_product_library():
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', "
            "'--ref-probes', '16']; sys.path.insert(0, '.'); import bench; bench.main(); "
            "mods = [m for m in sys.modules if m == 'vlb' or m.startswith('vlb.')]; "
            "print(json.dumps({'mods': mods}))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    ref, mods = lines[0], lines[1]["mods"]
    assert mods == []
    assert ref["impl"] == "reference" and ref["value"] > 0 and ref["cpu_baseline"]["kind"] == "port"
    sys.path.insert(0, str(ROOT))
    import bench

    assert ref["config"] == bench.config_dict(262144, 49162)


def test_trace_roofline_is_the_live_issue_view():
    """The trace kernel's roofline: the committed capture's warp instructions
    per launch over the live launch time, against 4 issue slots per SM clock;
    the capture's DRAM bytes are the traffic."""
    sys.path.insert(0, str(ROOT))
    import bench

    stats = {"bytes": 1.5e12, "node_tests_per_ray": 58.0, "node_fetches_per_ray": 58.0}
    for kname in ("trace_tile", "trace_fused_lane"):
        ncu = bench.TRACE_NCU[kname]
        r = bench.trace_roofline(kname, 125.0, stats, {"sm_max_mhz": 2070.0}, 152, 6788.6, True, 262144, 49162, 9,
                                 4, kname == "trace_tile")
        assert r["bound"] == "issue" and r["unit"] == "warp instructions/s"
        assert abs(r["achieved"] - ncu["warp_instructions"] / 0.125) <= 1e-9 * r["achieved"]
        assert abs(r["frac"] - r["achieved"] / (152 * 4 * 2070e6)) <= 1e-12
        assert 0 < r["frac"] < 1.2 and r["traffic"] == ncu["dram_bytes"]
        assert r["l1"]["requested_bytes_per_launch"] == stats["bytes"]
