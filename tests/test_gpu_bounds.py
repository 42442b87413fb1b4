"""The bounds-check build: every data-dependent device index of the trace
kernels (tree nodes, triangle slots, probe and direction permutations, sky
texels, the fused walk's ring slots, grid entries) is checked and a
violation counted instead of used.  The edge cases of bounds_cases.py run
under this build and under the normal one: no violation may be counted (a
count would turn a case into VLB_ERR_INTERNAL) and every output must be the
normal build's, bit for bit.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import vlb_build

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


def run_cases(lib: Path, out: Path) -> dict:
    env = dict(os.environ, VLB_LIB=str(lib))
    r = subprocess.run([sys.executable, str(HERE / "bounds_cases.py"), str(out)], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return dict(np.load(out))


def test_bounds_checked_build_matches_and_counts_nothing(tmp_path):
    bounds_lib = vlb_build.build_library(bounds_check=True)
    normal = run_cases(vlb_build.LIB, tmp_path / "normal.npz")
    checked = run_cases(bounds_lib, tmp_path / "checked.npz")
    assert int(normal.pop("build_flags")[0]) == 0
    assert int(checked.pop("build_flags")[0]) == 1  # VLB_BUILD_BOUNDS_CHECK
    assert normal.keys() == checked.keys()
    failed = sorted(k for k in normal if k.endswith("/status"))
    print(f"{len(normal)} outputs; calls refused in both builds: {failed}")
    # a refusal must be an argument check, never a device-side error
    for k in failed:
        assert int(normal[k][0]) in (1, 5), (k, normal[k])  # VLB_ERR_INVALID, VLB_ERR_UNSUPPORTED
    assert len(failed) < len(normal) // 4
    diff = [k for k in normal if not np.array_equal(normal[k], checked[k])]
    assert not diff, diff[:10]
