"""The bounds-checked build (libwoxel_gb300_checked.so, WX_BOUNDS_CHECK): the parity suites run
again in a child process that loads it, and every node-pool index and pixel index their kernels
used must have been in range (the session's context reports zero violations at teardown). This
stands in for a memory checker: out-of-range indices are counted and skipped, never accessed."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

import woxel_gb300 as wx

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_normal_build_has_no_counter(cuda_ctx):
    if os.environ.get("WOXEL_GB300_BOUNDS_CHECK") == "1":
        pytest.skip("this process loaded the bounds-checked build")
    with pytest.raises(wx.WxError, match="not a bounds-checked build"):
        cuda_ctx.bounds_violations()


def test_parity_suites_in_the_bounds_checked_build():
    if os.environ.get("WOXEL_GB300_BOUNDS_CHECK") == "1":
        pytest.skip("already the bounds-checked build")
    env = dict(os.environ, WOXEL_GB300_BOUNDS_CHECK="1")
    suites = ["tests/test_render_gpu.py", "tests/test_fuzz_gpu.py", "tests/test_batch_gpu.py",
              "tests/test_surface_gpu.py", "tests/test_chain_gpu.py", "tests/test_wgsl_golden_gpu.py"]
    r = subprocess.run([sys.executable, "-m", "pytest", *suites, "-m", "gpu", "-q", "-x", "-p", "no:cacheprovider"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and " error" not in r.stdout
