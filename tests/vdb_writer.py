"""A minimal OpenVDB file writer for reader tests: one float grid of a VDB345 tree
(5-4-3), file version 224, written uncompressed or with zip (zlib) buffers.

The layout is the one woxel's reader walks (src/vdb/read.rs): archive header,
one grid descriptor, the grid's compression flags and metadata, a uniform-scale
transform, the topology (N5 masks and node values, each N4's masks and node values,
each leaf's value mask), then the tree-data section (each leaf's value mask and
values). Node values use the OpenVDB per-node metadata byte: 0 (no inactive values
stored, the rest are +background) with only the active values written when the
active-mask flag is set, or 6 (all values).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

ZIP, ACTIVE_MASK, BLOSC = 0x1, 0x2, 0x4


def _lstr(s: str) -> bytes:
    b = s.encode()
    return struct.pack("<I", len(b)) + b


def _bits(offsets, nbits: int) -> np.ndarray:
    w = np.zeros(nbits // 64, np.uint64)
    for o in offsets:
        w[o >> 6] |= np.uint64(1) << np.uint64(o & 63)
    return w


class Block:
    """How a buffer of values is stored: raw, zlib at a level, or zip with a negative
    byte count (values stored as they are)."""

    def __init__(self, kind: str = "raw", level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY):
        self.kind, self.level, self.strategy = kind, level, strategy

    def encode(self, data: bytes) -> bytes:
        if self.kind == "raw":
            return data
        if self.kind == "zip-stored":
            return struct.pack("<q", -len(data)) + data
        c = zlib.compressobj(self.level, zlib.DEFLATED, 15, 9, self.strategy)
        z = c.compress(data) + c.flush()
        return struct.pack("<q", len(z)) + z


def write(path, leaves: dict, background: float = 3.0, compression: int = ACTIVE_MASK,
          block: Block = Block(), all_values: bool = False, voxel_count: int = -1, half: bool = False) -> None:
    """leaves: {(x, y, z) leaf origin (multiples of 8): (value mask bool[512], values float32[512])},
    voxel offset (x & 7) << 6 | (y & 7) << 3 | (z & 7). half: values stored as IEEE binary16
    (grid metadata is_saved_as_half_float)."""
    vt = np.float16 if half else np.float32
    n5 = {}
    for o in leaves:
        k5 = tuple(c & ~4095 for c in o)
        k4 = tuple(c & ~127 for c in o)
        n5.setdefault(k5, {}).setdefault(k4, []).append(o)

    def slot5(k4):
        return (((k4[0] & 4095) >> 7) << 10) | (((k4[1] & 4095) >> 7) << 5) | ((k4[2] & 4095) >> 7)

    def slot4(k3):
        return (((k3[0] & 127) >> 3) << 8) | (((k3[1] & 127) >> 3) << 4) | ((k3[2] & 127) >> 3)

    def node_values(nslots: int, vmask_words: np.ndarray) -> bytes:
        if all_values:  # metadata 6: every slot's value (the background here)
            return bytes([6]) + block.encode(np.full(nslots, background, vt).tobytes())
        n = int(sum(bin(int(w)).count("1") for w in vmask_words)) if compression & ACTIVE_MASK else nslots
        return bytes([0]) + block.encode(np.full(n, background, vt).tobytes())

    topo = bytearray()
    topo += struct.pack("<I", 1) + struct.pack("<f", background) + struct.pack("<II", 0, len(n5))
    order = []
    for k5, n4s in n5.items():
        topo += struct.pack("<3i", *k5)
        kid5 = _bits([slot5(k4) for k4 in n4s], 32768)
        val5 = np.zeros(512, np.uint64)
        topo += kid5.tobytes() + val5.tobytes()
        topo += node_values(32768, val5)
        for k4 in sorted(n4s, key=slot5):
            ls = sorted(n4s[k4], key=slot4)
            kid4 = _bits([slot4(o) for o in ls], 4096)
            val4 = np.zeros(64, np.uint64)
            topo += kid4.tobytes() + val4.tobytes()
            topo += node_values(4096, val4)
            for o in ls:
                m, _ = leaves[o]
                topo += _bits(np.flatnonzero(m), 512).tobytes()
                order.append(o)
    data = bytearray()
    for o in order:
        m, v = leaves[o]
        mw = _bits(np.flatnonzero(m), 512)
        data += mw.tobytes()
        vals = np.asarray(v, np.float32).astype(vt)
        if all_values or not (compression & ACTIVE_MASK):
            data += bytes([6]) + block.encode(vals.tobytes())
        else:
            data += bytes([0]) + block.encode(vals[np.asarray(m, bool)].tobytes())

    meta = struct.pack("<I", 2 if half else 1) + _lstr("file_voxel_count") + _lstr("int64") + \
        struct.pack("<Iq", 8, voxel_count)
    if half:
        meta += _lstr("is_saved_as_half_float") + _lstr("bool") + struct.pack("<IB", 1, 1)
    transform = _lstr("UniformScaleMap") + struct.pack("<15d", *([0.0] * 3 + [1.0] * 3 + [1.0] * 3 + [1.0] * 3 + [0.0] * 3))
    head = struct.pack("<QIIIB", 0x56444220, 224, 10, 0, 1) + b"0" * 36 + struct.pack("<I", 0) + struct.pack("<I", 1)
    desc = _lstr("ls") + _lstr("Tree_float_5_4_3") + _lstr("")
    grid_pos = len(head) + len(desc) + 24
    grid = struct.pack("<I", compression) + meta + transform + bytes(topo)
    block_pos = grid_pos + len(grid)
    end_pos = block_pos + len(data)
    with open(path, "wb") as f:
        f.write(head + desc + struct.pack("<QQQ", grid_pos, block_pos, end_pos) + grid + bytes(data))
