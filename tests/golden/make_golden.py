"""Regenerate the golden fixtures in this directory.

  python tests/golden/make_golden.py [ASSETS_DIR]

ASSETS_DIR holds woxel's level-set fixtures cube.vdb and icosahedron.vdb (the
reference checkout's assets/ directory). For each fixture this writes
  <name>_topology.npz  the grid topology read by the product's OpenVDB reader
                       (masks/origins in DFS order) plus the file's
                       file_voxel_count metadata, which the reference's own test
                       (src/vdb/read.rs:733-807) compares with the voxel count;
  <name>_values.npz    its leaf values (float16, as the half-float file stores them)
                       and the grid's background, read by the product's reader;
  <name>_render.npz    oracle renders of that topology (uniform bytes, RGBA8 and
                       hit records) for a few cameras and modes.
It also writes sphere64_render.npz (the 64-voxel sphere of the benchmark's small
configuration). The renders are oracle outputs: they pin the oracle against drift
and give the GPU kernels a fixed target.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as orc  # noqa: E402
import woxel_gb300 as wx  # noqa: E402

# (eye, mode, width, height) per render; target is the origin, fovy 60.
CAMERAS = {
    "cube": [((260.0, 190.0, 310.0), 3, 96, 72), ((-300.0, 40.0, 120.0), 0, 96, 72),
             ((10.0, -330.0, 60.0), 2, 64, 48)],
    "icosahedron": [((180.0, 150.0, 240.0), 3, 96, 72), ((-230.0, -90.0, -170.0), 1, 96, 72),
                    ((0.5, 0.5, 260.0), 4, 64, 48)],
    "sphere64": [((0.0, 0.0, 200.0), 3, 128, 96), ((120.0, 90.0, 100.0), 0, 128, 96)],
}


def render_set(name: str, view: dict) -> dict:
    out = {}
    for k, (eye, mode, w, h) in enumerate(CAMERAS[name]):
        st = wx.state_build(eye=eye, target=(0.0, 0.0, 0.0), aspect=w / h, fovy=60.0, width=float(w), mode=mode)
        sb = wx.state_bytes(st)
        rgba, hits, _ = orc.render(view, sb, w, h, nthreads=8, hits=True)
        out[f"state{k}"] = np.frombuffer(sb, np.uint8)
        out[f"size{k}"] = np.array([w, h], np.int32)
        out[f"rgba{k}"] = rgba
        out[f"hits{k}"] = hits.view(np.uint8).reshape(h, w, 32)
    return out


def main(assets: Path) -> None:
    for name in ("cube", "icosahedron"):
        topo, meta = wx.Topology.read_vdb(assets / f"{name}.vdb", f"ls_{name}")
        m = topo.masks()
        np.savez_compressed(HERE / f"{name}_topology.npz", **m,
                            file_voxel_count=np.array(meta["file_voxel_count"], np.int64),
                            file_version=np.array(meta["file_version"], np.int32))
        vals, bg = wx.Topology.read_vdb_values(assets / f"{name}.vdb", f"ls_{name}")
        half = vals.astype(np.float16)
        assert np.array_equal(half.astype(np.float32), vals)  # half-float files: exact
        np.savez_compressed(HERE / f"{name}_values.npz", values=half, background=np.float32(bg))
        view = orc.Tree.from_masks(m).view()
        np.savez_compressed(HERE / f"{name}_render.npz", **render_set(name, view))
        print(name, topo.counts, topo.active_voxels, meta)
    sphere = wx.Topology.sphere((0.0, 0.0, 0.0), 64.0, 3.0)
    view = orc.Tree.from_masks(sphere.masks()).view()
    np.savez_compressed(HERE / "sphere64_render.npz", **render_set("sphere64", view))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py ASSETS_DIR")
    main(Path(sys.argv[1]))
