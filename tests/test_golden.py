"""Golden fixtures (tests/golden/, written by tests/golden/make_golden.py).

The reference's own test of its reader (src/vdb/read.rs:733-807) checks that the
voxels read from assets/cube.vdb and assets/icosahedron.vdb equal the files'
file_voxel_count metadata: 1,452,218 and 364,741. The frozen topologies carry
those counts; the frozen renders are oracle outputs for fixed cameras.
"""
import os
from pathlib import Path

import numpy as np
import pytest

import oracle as orc
import woxel_gb300 as wx

GOLDEN = Path(__file__).resolve().parent / "golden"
# woxel's assets/ directory (cube.vdb, icosahedron.vdb); the reader tests skip without it.
ASSETS = Path(os.environ["WOXEL_ASSETS"]) if os.environ.get("WOXEL_ASSETS") else None
KAT = {"cube": 1452218, "icosahedron": 364741}
MASK_KEYS = ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")


def frozen_masks(name):
    d = np.load(GOLDEN / f"{name}_topology.npz")
    return {k: d[k] for k in MASK_KEYS}, int(d["file_voxel_count"])


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_fixture_voxel_count_kat(name):
    m, meta_count = frozen_masks(name)
    active = int(np.unpackbits(m["vals3"].view(np.uint8)).sum())
    assert active == KAT[name] == meta_count
    assert wx.Topology.from_masks(m).active_voxels == KAT[name]
    assert orc.Tree.from_masks(m).counts[2] == m["vals3"].size // 16


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_reader_reproduces_frozen_topology(name):
    path = ASSETS / f"{name}.vdb" if ASSETS else None
    if path is None or not path.exists():
        pytest.skip("set WOXEL_ASSETS to woxel's assets/ directory to read the .vdb fixtures")
    topo, meta = wx.Topology.read_vdb(path, f"ls_{name}")
    assert meta["file_voxel_count"] == KAT[name] and topo.active_voxels == KAT[name]
    assert meta["file_version"] == 222 and meta["half_float"]
    m, _ = frozen_masks(name)
    got = topo.masks()
    for k in MASK_KEYS:
        np.testing.assert_array_equal(got[k], m[k], err_msg=k)


def frozen_values(name):
    d = np.load(GOLDEN / f"{name}_values.npz")
    return d["values"].astype(np.float32), float(d["background"])


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_reader_reproduces_frozen_values(name):
    """Leaf values of the tree-data section (read.rs:571-629), half floats converted exactly."""
    path = ASSETS / f"{name}.vdb" if ASSETS else None
    if path is None or not path.exists():
        pytest.skip("set WOXEL_ASSETS to woxel's assets/ directory to read the .vdb fixtures")
    vals, bg = wx.Topology.read_vdb_values(path, f"ls_{name}")
    want, want_bg = frozen_values(name)
    assert bg == want_bg
    np.testing.assert_array_equal(vals, want)


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_frozen_values_are_a_level_set(name):
    """Active voxels lie inside the narrow band; inactive ones hold +-background (outside/inside)."""
    m, _ = frozen_masks(name)
    v, bg = frozen_values(name)
    v = v.reshape(-1, 512)
    bits = np.unpackbits(m["vals3"].view(np.uint8), bitorder="little").reshape(-1, 512).astype(bool)
    assert (np.abs(v[bits]) <= bg).all() and (np.abs(v[bits]) < bg).mean() > 0.999
    assert np.array_equal(np.abs(v[~bits]), np.full((~bits).sum(), bg, np.float32))
    assert 0.3 < (v[~bits] < 0).mean() < 0.6  # both sides of the surface are present


def test_reader_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.vdb"
    p.write_bytes(b"\x00" * 64)
    with pytest.raises(wx.WxError, match="magic"):
        wx.Topology.read_vdb(p)
    with pytest.raises(wx.WxError):
        wx.Topology.read_vdb(tmp_path / "missing.vdb")


@pytest.mark.parametrize("name", ["cube", "icosahedron", "sphere64"])
def test_oracle_reproduces_golden_renders(name):
    if name == "sphere64":
        m = wx.Topology.sphere((0, 0, 0), 64.0, 3.0).masks()
    else:
        m, _ = frozen_masks(name)
    view = orc.Tree.from_masks(m).view()
    g = np.load(GOLDEN / f"{name}_render.npz")
    k = 0
    while f"state{k}" in g:
        w, h = (int(x) for x in g[f"size{k}"])
        rgba, hits, _ = orc.render(view, g[f"state{k}"].tobytes(), w, h, nthreads=4, hits=True)
        np.testing.assert_array_equal(rgba, g[f"rgba{k}"])
        np.testing.assert_array_equal(hits.view(np.uint8).reshape(h, w, 32), g[f"hits{k}"])
        k += 1
    assert k >= 2


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_product_sdf_matches_oracle_on_fixtures(name):
    m, _ = frozen_masks(name)
    pv = wx.Topology.from_masks(m).view()
    ov = orc.Tree.from_masks(m).view()
    for i in range(3):
        np.testing.assert_array_equal(pv["atlas"][i], ov["atlas"][i], err_msg=f"atlas {i}")
