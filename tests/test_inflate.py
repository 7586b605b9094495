"""The zlib decoder of the VDB reader (woxel_gb300/csrc/inflate.cpp) against Python's
zlib: every DEFLATE block type (stored at level 0, fixed Huffman, dynamic Huffman),
every compression strategy, data from incompressible to all-zero, early stop when the
caller needs fewer bytes than the stream holds, and rejection of damaged streams."""
import ctypes as C
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

CSRC = Path(__file__).resolve().parent.parent / "woxel_gb300" / "csrc"

SHIM = r"""
#include "inflate.h"
#include <cstring>
extern "C" long long shim_inflate(const unsigned char *src, unsigned long long n, unsigned char *dst,
                                  unsigned long long cap, char *err, int errcap) {
    std::string e;
    long long r = wx::zlib_inflate(src, n, dst, cap, &e);
    std::strncpy(err, e.c_str(), errcap - 1);
    err[errcap - 1] = 0;
    return r;
}
"""


@pytest.fixture(scope="module")
def inflate(tmp_path_factory):
    d = tmp_path_factory.mktemp("inflate")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(CSRC), "-o", str(so),
                    str(d / "shim.cpp"), str(CSRC / "inflate.cpp")], check=True)
    lib = C.CDLL(str(so))
    lib.shim_inflate.restype = C.c_longlong
    lib.shim_inflate.argtypes = [C.c_char_p, C.c_ulonglong, C.c_void_p, C.c_ulonglong, C.c_char_p, C.c_int]

    def run(stream: bytes, cap: int):
        out = np.zeros(max(cap, 1), np.uint8)
        err = C.create_string_buffer(256)
        r = lib.shim_inflate(stream, len(stream), out.ctypes.data, cap, err, 256)
        return r, out[:max(r, 0)].tobytes(), err.value.decode()

    return run


def datasets():
    rng = np.random.default_rng(5)
    yield "random", rng.integers(0, 256, 70000, dtype=np.uint8).tobytes()
    yield "zeros", bytes(100000)
    yield "floats", (np.sin(np.arange(30000, dtype=np.float32) * 0.01) * 3.0).astype(np.float32).tobytes()
    yield "text", b"the quick brown fox jumps over the lazy dog " * 900
    yield "runs", bytes(np.repeat(rng.integers(0, 4, 3000, dtype=np.uint8), rng.integers(1, 40, 3000)))
    yield "tiny", b"a"
    yield "empty", b""


STRATEGIES = [("default", zlib.Z_DEFAULT_STRATEGY), ("filtered", zlib.Z_FILTERED),
              ("huffman", zlib.Z_HUFFMAN_ONLY), ("rle", zlib.Z_RLE), ("fixed", zlib.Z_FIXED)]


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_matches_python_zlib(inflate, level):
    for name, data in datasets():
        for sname, strat in STRATEGIES:
            c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strat)
            stream = c.compress(data) + c.flush()
            r, out, err = inflate(stream, len(data))
            assert r == len(data) and out == data, (name, sname, err)


def test_stops_when_the_caller_has_enough(inflate):
    data = b"".join(bytes([i % 251]) * (i % 7 + 1) for i in range(20000))
    stream = zlib.compress(data, 9)
    for cap in (1, 100, 4096, len(data) // 2, len(data) - 1):
        r, out, err = inflate(stream, cap)
        assert r == cap and out == data[:cap], (cap, err)


def test_short_stream_reports_fewer_bytes(inflate):
    data = bytes(range(256)) * 10
    r, out, _ = inflate(zlib.compress(data), len(data) + 100)
    assert r == len(data) and out == data  # the reader then rejects the block as too short


def _fixed_block(codes, payload=b""):
    """A zlib stream of one final fixed-Huffman block from (huffman code, bit length) and
    (raw value, bit count, "raw") items: Huffman codes go most significant bit first,
    header fields and extra bits least significant bit first (RFC 1951 section 3.1.1)."""
    bits = [1, 1, 0]  # BFINAL = 1, BTYPE = 01
    for v, n, *kind in codes:
        if kind:
            bits += [(v >> k) & 1 for k in range(n)]
        else:
            bits += [(v >> (n - 1 - k)) & 1 for k in range(n)]
    bits += [0] * (-len(bits) % 8)
    body = bytes(sum(b << k for k, b in enumerate(bits[i:i + 8])) for i in range(0, len(bits), 8))
    return b"\x78\x01" + body + zlib.adler32(payload).to_bytes(4, "big")


@pytest.mark.parametrize("damage", ["header", "checksum", "truncated", "block type"])
def test_damaged_streams_are_rejected(inflate, damage):
    data = (b"0123456789abcdef" * 64) + bytes(range(256))
    s = bytearray(zlib.compress(data, 6))
    if damage == "header":
        s[1] ^= 0x01  # header check fails
    elif damage == "checksum":
        s[-1] ^= 0xFF
    elif damage == "truncated":
        s = s[: len(s) // 2]
    elif damage == "block type":
        s = bytearray(b"\x78\x9c") + bytearray([0x07])  # BFINAL=1, BTYPE=3
    r, _, err = inflate(bytes(s), len(data))
    assert r == -1 and err.startswith("zlib:"), err


def test_back_reference_before_any_output_is_rejected(inflate):
    # length 3 (symbol 257: 7-bit code 0000001), distance 1 (code 0: 00000), end of block
    stream = _fixed_block([(0b0000001, 7), (0, 5), (0, 7)])
    r, _, err = inflate(stream, 16)
    assert r == -1 and err == "zlib: distance beyond the output"
    # the same pair after one literal 'a' (8-bit code 0x30 + 0x61) copies it: "aaaa"
    stream = _fixed_block([(0x30 + 0x61, 8), (0b0000001, 7), (0, 5), (0, 7)], b"aaaa")
    r, out, err = inflate(stream, 4)
    assert r == 4 and out == b"aaaa", err
