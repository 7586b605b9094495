"""Zip-compressed OpenVDB files: the reader decodes zlib buffers (as the reference does
with flate2, src/vdb/read.rs:546-563) and gives the same topology and leaf values as
for the uncompressed file; blosc grids are reported as unsupported; damaged zip data
is an error, never a crash.

The files come from tests/vdb_writer.py (one float grid over leaves in three N5 nodes,
negative coordinates included), written raw, with zlib at several levels and
strategies (stored, fixed and dynamic Huffman blocks), with zip blocks that store
their values raw (negative byte count), and with and without active-mask value
compression."""
import zlib

import numpy as np
import pytest

import woxel_gb300 as wx
from vdb_writer import ACTIVE_MASK, BLOSC, ZIP, Block, write


@pytest.fixture(scope="module")
def leaves():
    rng = np.random.default_rng(12)
    out = {}
    for _ in range(60):
        c = rng.integers(-5000, 5000, 3)
        o = tuple(int(x) & ~7 for x in c)
        m = rng.random(512) < rng.uniform(0.05, 0.9)
        m[rng.integers(0, 512)] = True
        v = np.where(m, rng.normal(0.0, 1.0, 512), 3.0).astype(np.float32)
        out[o] = (m, v)
    return out


def read(path):
    topo, info = wx.Topology.read_vdb(path)
    vals, bg = wx.Topology.read_vdb_values(path)
    return topo.masks(), info, vals, bg


def assert_same(a, b):
    for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins"):
        np.testing.assert_array_equal(np.asarray(a[0][k]), np.asarray(b[0][k]), err_msg=k)
    np.testing.assert_array_equal(a[2], b[2])
    assert a[3] == b[3]


@pytest.mark.parametrize("active_mask", [True, False])
def test_zip_equals_uncompressed(tmp_path, leaves, active_mask):
    base = ACTIVE_MASK if active_mask else 0
    write(tmp_path / "raw.vdb", leaves, compression=base)
    ref = read(tmp_path / "raw.vdb")
    assert ref[1]["compression"] == base
    # the uncompressed file's values are the written ones (DFS leaf order) and its leaf
    # masks the written masks
    nleaves = ref[2].size // 512
    assert nleaves == len(leaves)
    written = sorted(np.where(m, v, 3.0).tobytes() for m, v in leaves.values())
    assert sorted(ref[2].reshape(-1, 512)[i].tobytes() for i in range(nleaves)) == written
    cases = [Block("zlib", 0), Block("zlib", 1), Block("zlib", 9), Block("zlib", 6, zlib.Z_FIXED),
             Block("zlib", 6, zlib.Z_HUFFMAN_ONLY), Block("zlib", 6, zlib.Z_RLE), Block("zip-stored")]
    for i, blk in enumerate(cases):
        p = tmp_path / f"zip{i}.vdb"
        write(p, leaves, compression=base | ZIP, block=blk)
        got = read(p)
        assert got[1]["compression"] == base | ZIP
        assert_same(ref, got)


def test_zip_with_all_values_stored(tmp_path, leaves):
    """Metadata 6 (every value written) for the nodes and the leaves."""
    write(tmp_path / "raw.vdb", leaves, all_values=True)
    write(tmp_path / "zip.vdb", leaves, compression=ACTIVE_MASK | ZIP, block=Block("zlib", 9), all_values=True)
    assert_same(read(tmp_path / "raw.vdb"), read(tmp_path / "zip.vdb"))


def test_zip_half_float(tmp_path, leaves):
    """Half-float values (2-byte elements in the zip blocks), converted exactly."""
    write(tmp_path / "raw.vdb", leaves, half=True)
    write(tmp_path / "zip.vdb", leaves, compression=ACTIVE_MASK | ZIP, block=Block("zlib", 9), half=True)
    a, b = read(tmp_path / "raw.vdb"), read(tmp_path / "zip.vdb")
    assert a[1]["half_float"] and b[1]["half_float"]
    assert_same(a, b)
    written = sorted(np.where(m, v.astype(np.float16).astype(np.float32), 3.0).tobytes() for m, v in leaves.values())
    assert sorted(a[2].reshape(-1, 512)[i].tobytes() for i in range(len(leaves))) == written


def test_blosc_is_unsupported(tmp_path, leaves):
    write(tmp_path / "blosc.vdb", leaves, compression=ACTIVE_MASK | BLOSC, block=Block("zlib", 6))
    with pytest.raises(wx.WxError, match="blosc"):
        wx.Topology.read_vdb(tmp_path / "blosc.vdb")


def test_damaged_zip_data_is_an_error(tmp_path, leaves):
    p = tmp_path / "zip.vdb"
    write(p, leaves, compression=ACTIVE_MASK | ZIP, block=Block("zlib", 6))
    good = p.read_bytes()
    vals, _ = wx.Topology.read_vdb_values(p)
    rng = np.random.default_rng(3)
    errors = 0
    for _ in range(20):  # flip bytes in the tree-data section (leaf buffers)
        b = bytearray(good)
        i = int(rng.integers(len(good) - 8000, len(good)))
        b[i] ^= 0x5A
        q = tmp_path / "bad.vdb"
        q.write_bytes(bytes(b))
        try:
            got, _ = wx.Topology.read_vdb_values(q)
            assert got.size == vals.size  # a flip inside a value mask can still parse
        except wx.WxError:
            errors += 1
    assert errors > 0
    for cut in (len(good) - 1, len(good) - 100, len(good) - 3000):
        q.write_bytes(good[:cut])
        with pytest.raises(wx.WxError):
            wx.Topology.read_vdb_values(q)
