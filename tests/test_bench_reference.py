"""bench.py's reference arm: the oracle alone, no product code.

It builds the workload's grid with the oracle's restated generator, compute_sdf and
atlas(), makes the uniforms with the oracle's ComputeState::build and renders with the
oracle; libwoxel_gb300.so must never be mapped into that process, and its `config` must
equal the one the GPU arm reports for the same workload (built here from the product's
grid and frames).
"""
import json
import subprocess
import sys
from pathlib import Path

import bench
import woxel_gb300 as wx  # noqa: F401
from woxel_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent

RUN = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "sphere", "--steps", "2", "--warmup", "1"]
runpy.run_path(sys.argv_path, run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED", "libwoxel_gb300" in maps, "woxel_gb300" in sys.modules, file=sys.stderr)
"""


def test_reference_arm_loads_no_product_code():
    code = RUN.replace("sys.argv_path", repr(str(ROOT / "bench.py")))
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert p.returncode == 0, p.stderr
    assert "MAPPED False False" in p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    topo = W.sphere_topology()
    ours = bench.workload_config("sphere", topo.counts, topo.active_voxels,
                                 [(f.width, f.height) for f in W.sphere_frames()])
    assert line["config"] == ours
