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
