"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arms of bench.py, to check and to time. The product never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

HIT_DTYPE = np.dtype([("p", "<f4", (3,)), ("t", "<f4"), ("node", "<u4"), ("info", "<u4"),
                      ("shadow", "<u4"), ("reserved", "<u4")])
STATS_DTYPE = np.dtype([("steps", "<u4"), ("bytes", "<u4"), ("shadow_steps", "<u4"), ("shadow_bytes", "<u4"),
                        ("grazing", "<u4"), ("reserved", "<u4", (3,))])


class orc_view(C.Structure):
    _fields_ = [("kids5", C.c_void_p), ("vals5", C.c_void_p), ("kids4", C.c_void_p), ("vals4", C.c_void_p),
                ("vals3", C.c_void_p), ("origins", C.c_void_p), ("n5", C.c_uint64), ("n4", C.c_uint64),
                ("n3", C.c_uint64), ("atlas", C.c_void_p * 3), ("dims", (C.c_uint32 * 3) * 3),
                ("values", C.c_void_p), ("band", C.c_float)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        L = C.CDLL(str(LIB_PATH))
        P, U64, I = C.c_void_p, C.c_uint64, C.c_int
        sig = {
            "orc_global_to_node": (None, [P, I, P]),
            "orc_global_to_offset": (U64, [P, I, I]),
            "orc_offset_to_child": (None, [U64, I, P]),
            "orc_child_to_offset": (U64, [P, I]),
            "orc_tree_new": (P, []),
            "orc_tree_free": (None, [P]),
            "orc_set_voxel": (None, [P, P, C.c_uint32]),
            "orc_get_voxel": (I, [P, P, P, P]),
            "orc_tree_from_masks": (P, [P, P, U64, P, P, U64, P, U64, P]),
            "orc_count_nodes": (None, [P, P]),
            "orc_compute_sdf": (None, [P]),
            "orc_masks": (None, [P, P, P, P, P, P, P]),
            "orc_atlas": (None, [P, P, P, P, P]),
            "orc_state_build": (None, [P, P, P, C.c_float, C.c_float, C.c_float, C.c_uint32, P, P, P,
                                       C.c_float, P]),
            "orc_render": (I, [P, P, C.c_uint32, C.c_uint32, P, P, P, I]),
            "orc_render_tiles": (I, [P, P, C.c_uint32, C.c_uint32, U64, U64, P, P, P, I]),
            "orc_render_tile_list": (I, [P, P, C.c_uint32, C.c_uint32, P, U64, P, P, P, I]),
            "orc_sun_default": (None, [P, P, P]),
            "orc_sphere_list": (None, [C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, U64, P]),
            "orc_gen_spheres": (I, [P, P, C.c_uint32, C.c_double]),
            "orc_set_leaf": (None, [P, P, P]),
            "orc_gen_spheres_values": (I, [P, P, C.c_uint32, C.c_double, P]),
            "orc_gen_noise_leaves": (C.c_int64, [P, C.c_int32, C.c_uint32, C.c_double, C.c_double, U64,
                                                 C.c_int32, C.c_int32]),
            "orc_orbit_eyes": (None, [C.c_uint32, C.c_float, U64, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# ---- coordinate maths (data_structure.rs:43-91) ----
def global_to_node(g, total_log2: int):
    a = np.asarray(g, np.int32)
    out = np.zeros(3, np.int32)
    lib().orc_global_to_node(a.ctypes.data, total_log2, out.ctypes.data)
    return tuple(int(x) for x in out)


def global_to_offset(g, log2d: int, total_log2: int) -> int:
    a = np.asarray(g, np.int32)
    return int(lib().orc_global_to_offset(a.ctypes.data, log2d, total_log2))


def offset_to_child(off: int, log2d: int):
    out = np.zeros(3, np.uint32)
    lib().orc_offset_to_child(off, log2d, out.ctypes.data)
    return tuple(int(x) for x in out)


def child_to_offset(c, log2d: int) -> int:
    a = np.asarray(c, np.uint32)
    return int(lib().orc_child_to_offset(a.ctypes.data, log2d))


class Tree:
    """The reference VDB345 tree restated in C (vdb345.rs)."""

    def __init__(self, handle=None):
        self._h = C.c_void_p(handle if handle is not None else lib().orc_tree_new())

    def __del__(self):
        try:
            if self._h and self._h.value:
                lib().orc_tree_free(self._h)
        except Exception:
            pass

    @classmethod
    def from_voxels(cls, ijk, values=None) -> "Tree":
        t = cls()
        a = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        vals = np.ones(a.shape[0], np.uint32) if values is None else np.asarray(values, np.uint32)
        for i in range(a.shape[0]):
            t.set_voxel(a[i], int(vals[i]))
        return t

    @classmethod
    def from_masks(cls, m: dict) -> "Tree":
        k5, v5, k4, v4, v3 = (np.ascontiguousarray(m[k], np.uint32) for k in ("kids5", "vals5", "kids4", "vals4", "vals3"))
        org = np.ascontiguousarray(m["origins"], np.int32).reshape(-1, 4)
        h = lib().orc_tree_from_masks(k5.ctypes.data, v5.ctypes.data, k5.size // 1024, k4.ctypes.data,
                                      v4.ctypes.data, k4.size // 128, v3.ctypes.data, v3.size // 16, org.ctypes.data)
        if not h:
            raise ValueError("masks do not describe a consistent tree")
        return cls(h)

    @classmethod
    def spheres(cls, spheres: np.ndarray, band: float) -> "Tree":
        """Narrow-band union of spheres (rows cx, cy, cz, r): every voxel with
        |min_s(|ijk - c_s| - r_s)| < band set through set_voxel."""
        t = cls()
        sp = np.ascontiguousarray(spheres, np.float64).reshape(-1, 4)
        if lib().orc_gen_spheres(t._h, sp.ctypes.data, sp.shape[0], float(band)) != 0:
            raise MemoryError("orc_gen_spheres: out of memory")
        return t

    @classmethod
    def noise_leaves(cls, lo: int, extent: int, occupancy: float, p_voxel: float, seed: int,
                     box=None) -> "Tree":
        """Value-noise leaves of [lo, lo + extent)^3; box=(b0, b1) keeps the leaves whose
        origin lies in [b0, b1) on every axis."""
        t = cls()
        b0, b1 = box if box is not None else (0, 0)
        if lib().orc_gen_noise_leaves(t._h, lo, extent, occupancy, p_voxel, seed, b0, b1) < 0:
            raise ValueError("orc_gen_noise_leaves: bad arguments or out of memory")
        return t

    def spheres_values(self, spheres: np.ndarray, band: float) -> np.ndarray:
        """Level-set values of every leaf voxel (n3 * 512 float32, DFS leaf order)."""
        sp = np.ascontiguousarray(spheres, np.float64).reshape(-1, 4)
        out = np.empty(self.counts[2] * 512, np.float32)
        if lib().orc_gen_spheres_values(self._h, sp.ctypes.data, sp.shape[0], float(band), out.ctypes.data) != 0:
            raise MemoryError("orc_gen_spheres_values: out of memory")
        return out

    def set_voxel(self, p, value: int = 1) -> None:
        a = np.asarray(p, np.int32)
        lib().orc_set_voxel(self._h, a.ctypes.data, value)

    def get_voxel(self, p):
        a = np.asarray(p, np.int32)
        v, lvl = C.c_uint64(), C.c_int()
        kind = lib().orc_get_voxel(self._h, a.ctypes.data, C.byref(v), C.byref(lvl))
        return ["Offs", "Leaf", "Innr", "Root", "Bkgr"][kind], int(v.value), int(lvl.value)

    @property
    def counts(self):
        c = np.zeros(3, np.uint64)
        lib().orc_count_nodes(self._h, c.ctypes.data)
        return tuple(int(x) for x in c)

    def compute_sdf(self) -> None:
        lib().orc_compute_sdf(self._h)

    def masks(self) -> dict:
        n5, n4, n3 = self.counts
        out = {"kids5": np.zeros(n5 * 1024, np.uint32), "vals5": np.zeros(n5 * 1024, np.uint32),
               "kids4": np.zeros(n4 * 128, np.uint32), "vals4": np.zeros(n4 * 128, np.uint32),
               "vals3": np.zeros(n3 * 16, np.uint32), "origins": np.zeros((n5, 4), np.int32)}
        lib().orc_masks(self._h, *(out[k].ctypes.data for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")))
        return out

    def atlas(self):
        side = np.zeros(3, np.uint32)
        lib().orc_atlas(self._h, side.ctypes.data, None, None, None)
        a = [np.zeros(int(s) ** 3, np.uint32) for s in side]
        lib().orc_atlas(self._h, side.ctypes.data, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data)
        return a, [int(s) for s in side]

    def view(self, sdf: bool = True) -> dict:
        """compute_sdf() then the flattened view (masks, origins, atlases)."""
        if sdf:
            self.compute_sdf()
        v = self.masks()
        a, s = self.atlas()
        v["atlas"] = a
        v["dims"] = [(x, x, x) for x in s]
        return v


def state_build(eye, target, up, aspect, fovy, width, mode, show_345, sun_dir, sun_color, intensity) -> bytes:
    f3 = C.c_float * 3
    out = C.create_string_buffer(256)
    lib().orc_state_build(f3(*eye), f3(*target), f3(*up), aspect, fovy, width, mode, (C.c_uint32 * 3)(*show_345),
                          f3(*sun_dir), f3(*sun_color), intensity, out)
    return out.raw


def sun_default():
    """(dir, colour, intensity) of the reference app's default sun (egui_dev.rs:355-368)."""
    d, c, i = (C.c_float * 3)(), (C.c_float * 3)(), C.c_float()
    lib().orc_sun_default(d, c, C.byref(i))
    return tuple(d), tuple(c), i.value


def sphere_list(count: int, rmin: float, rmax: float, lo: float, hi: float, seed: int) -> np.ndarray:
    out = np.zeros((count, 4), np.float64)
    lib().orc_sphere_list(count, rmin, rmax, lo, hi, seed, out.ctypes.data)
    return out


def orbit_eyes(count: int, radius: float, seed: int) -> np.ndarray:
    out = np.zeros((count, 3), np.float32)
    lib().orc_orbit_eyes(count, radius, seed, out.ctypes.data)
    return out


def frame_state(eye, width: int, height: int, mode: int, fovy: float = 60.0) -> bytes:
    """Uniform of a camera at eye looking at the origin (up +y) with the default sun."""
    sd, sc, si = sun_default()
    return state_build(tuple(float(x) for x in eye), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), width / height, fovy,
                       float(width), mode, (0, 0, 0), sd, sc, si)


def _view_struct(v: dict):
    keep = {k: np.ascontiguousarray(v[k], np.uint32) for k in ("kids5", "vals5", "kids4", "vals4", "vals3")}
    org = np.ascontiguousarray(v["origins"], np.int32).reshape(-1, 4)
    atl = [np.ascontiguousarray(a, np.uint32) for a in v["atlas"]]
    s = orc_view()
    for k, a in keep.items():
        setattr(s, k, a.ctypes.data)
    s.origins = org.ctypes.data
    s.n5, s.n4, s.n3 = keep["kids5"].size // 1024, keep["kids4"].size // 128, keep["vals3"].size // 16
    for i in range(3):
        s.atlas[i] = atl[i].ctypes.data
        for j in range(3):
            s.dims[i][j] = int(v["dims"][i][j])
    vals = None
    if v.get("values") is not None:  # zero-crossing mode: n3 * 512 level-set values and their band
        vals = np.ascontiguousarray(v["values"], np.float32)
        assert vals.size == s.n3 * 512
        s.values = vals.ctypes.data
        s.band = float(v["band"])
    return s, (keep, org, atl, vals)


def render(v: dict, state: bytes, width: int, height: int, nthreads: int = 1, hits: bool = True,
           stats: bool = False, tiles=None):
    """Run the oracle's raycast pass. Returns (rgba[h,w,4] u8, hits[h,w] or None, stats[h,w] or None)."""
    s, keep = _view_struct(v)
    rgba = np.zeros((height, width, 4), np.uint8)
    h = np.zeros((height, width), HIT_DTYPE) if hits else None
    st = np.zeros((height, width), STATS_DTYPE) if stats else None
    sb = C.create_string_buffer(bytes(state), 256)
    if tiles is None:
        rc = lib().orc_render(C.byref(s), sb, width, height, rgba.ctypes.data,
                              None if h is None else h.ctypes.data, None if st is None else st.ctypes.data, nthreads)
    elif isinstance(tiles, np.ndarray):
        tl = np.ascontiguousarray(tiles, np.uint64)
        rc = lib().orc_render_tile_list(C.byref(s), sb, width, height, tl.ctypes.data, tl.size, rgba.ctypes.data,
                                        None if h is None else h.ctypes.data,
                                        None if st is None else st.ctypes.data, nthreads)
    else:
        rc = lib().orc_render_tiles(C.byref(s), sb, width, height, tiles[0], tiles[1], rgba.ctypes.data,
                                    None if h is None else h.ctypes.data, None if st is None else st.ctypes.data,
                                    nthreads)
    if rc != 0:
        raise RuntimeError(f"orc_render failed: {rc}")
    del keep
    return rgba, h, st


# ---- The benchmark workloads, built by the oracle alone (no product code) ----
# Same parameters as the product's seeded generators: one r=64 sphere at the origin;
# 2000 spheres r ~ U[4,40], centres U[-1024,1024)^3, seed 2; value-noise leaves over
# [-2048,2048)^3 at 2% occupancy, voxels p=0.5, seed 3; band 3 voxels.
def workload_spheres(name: str) -> np.ndarray:
    """Rows (cx, cy, cz, r) of the sphere workloads' spheres."""
    if name == "sphere":
        return np.array([[0.0, 0.0, 0.0, 64.0]])
    if name == "spheres":
        return sphere_list(2000, 4.0, 40.0, -1024.0, 1024.0, 2)
    raise ValueError(f"{name!r} is not a sphere workload")


def workload_tree(name: str, box=None) -> Tree:
    if name in ("sphere", "spheres"):
        return Tree.spheres(workload_spheres(name), 3.0)
    if name == "noise":
        return Tree.noise_leaves(-2048, 4096, 0.02, 0.5, 3, box)
    raise ValueError(f"unknown workload {name!r}")


def workload_frames(name: str) -> list:
    """[(width, height, uniform bytes)] of the workload's cameras: the 640x480 view from
    (0,0,200); 16 orbit eyes at radius 3000 (seed 16), 1920x1080, Lambert mode 3; 8 orbit
    eyes at radius 3500 (seed 8), 3840x2160, mode 0. All 60 degree, looking at the origin."""
    if name == "sphere":
        return [(640, 480, frame_state((0.0, 0.0, 200.0), 640, 480, 3))]
    if name == "spheres":
        return [(1920, 1080, frame_state(e, 1920, 1080, 3)) for e in orbit_eyes(16, 3000.0, 16)]
    if name == "noise":
        return [(3840, 2160, frame_state(e, 3840, 2160, 0)) for e in orbit_eyes(8, 3500.0, 8)]
    raise ValueError(f"unknown workload {name!r}")


def workload_view(name: str, box=None, values: bool = False) -> dict:
    """The workload's flattened view (compute_sdf, masks, atlas) built by the oracle; with
    values=True (sphere workloads) also its level-set values and band for render mode 5."""
    t = workload_tree(name, box)
    v = t.view()
    if values:
        v["values"], v["band"] = t.spheres_values(workload_spheres(name), 3.0), 3.0
    del t
    return v
