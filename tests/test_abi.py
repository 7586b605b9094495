"""The C-ABI library loads and exports every function include/*.h declares (no GPU calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import woxel_gb300 as wx
from woxel_gb300 import _ffi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(wx_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_core_entry_points():
    names = declared_functions()
    for n in ("wx_ctx_create", "wx_grid_upload", "wx_grid_build", "wx_render", "wx_render_batch",
              "wx_batch_create", "wx_batch_launch", "wx_state_build"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_ffi.LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_exports_are_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_ffi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert declared_functions() <= exported


def test_binding_covers_header():
    assert declared_functions() <= set(_ffi.SIGNATURES)


def test_struct_sizes():
    assert C.sizeof(wx.wx_state_uniform) == 256
    assert C.sizeof(wx.wx_hit) == 32
    assert C.sizeof(wx.wx_tuning) == 24
    assert wx.HIT_DTYPE.itemsize == 32


def test_status_strings_and_errors_without_gpu():
    L = _ffi.lib()
    assert L.wx_status_string(0) == b"ok"
    assert L.wx_status_string(1) == b"invalid argument"
    rc = L.wx_topology_from_voxels(None, 5, None)
    assert rc == 1 and b"null" in L.wx_thread_last_error()
    assert b"sm_103a" in L.wx_version()
