"""woxel_gb300 — GB300 (sm_103a) primary-ray pass for woxel's VDB345 grids.

Host-side mirror of the reference's raycast-pass interface: a grid is
uploaded once (WgpuContext::new / change_vdb_model, src/render/wgpu_context.rs:
101-159, 506-573), then every frame takes the 256-byte ComputeState uniform
(src/render/gpu_types/compute_state.rs:9-29) and produces RGBA8 plus an
optional hit buffer (the compute pass of src/render/wgpu_context.rs:270-282).
All work runs in libwoxel_gb300.so through its C ABI (include/woxel_gb300.h);
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from ._ffi import (WX_OK, WxError, check, lib, wx_frame, wx_grid_info, wx_hit, wx_state_uniform,  # noqa: F401
                   wx_tuning, wx_vdb345_view)

HIT_DTYPE = np.dtype([("p", "<f4", (3,)), ("t", "<f4"), ("node", "<u4"), ("info", "<u4"),
                      ("shadow", "<u4"), ("reserved", "<u4")])
assert HIT_DTYPE.itemsize == 32

MODE_GRAY, MODE_RGB, MODE_RAY, MODE_DIFFUSE, MODE_GLOSSY, MODE_SURFACE = 0, 1, 2, 3, 4, 5


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch.Tensor
        return a.data_ptr()
    return int(a)


def hit_fields(hits: np.ndarray) -> dict:
    """Decode wx_hit records: state, level, mask, steps, node, ijk = floor(p), t, shadow.

    ijk of a position outside the int32 range (a ray that left the grid after a long
    jump) or of a non-finite one is -2^31.
    """
    info = hits["info"]
    fp = np.floor(hits["p"].astype(np.float64))
    ok = np.isfinite(fp) & (fp >= -2.0 ** 31) & (fp < 2.0 ** 31)
    ijk = np.where(ok, fp, -2.0 ** 31).astype(np.int32)
    return {
        "state": info & 3, "level": (info >> 2) & 3, "mask": (info >> 4) & 7, "steps": (info >> 8) & 0x7FF,
        "node": hits["node"], "ijk": ijk, "t": hits["t"],
        "p": hits["p"], "shadow": hits["shadow"],
    }


# --------------------------------------------------------------------------
# Topology (host): node structure of a VDB345 grid in DFS order.
# --------------------------------------------------------------------------
class Topology:
    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @staticmethod
    def _make(fn, *args) -> "Topology":
        out = C.c_void_p()
        check(fn(*args, C.byref(out)))
        return Topology(out.value)

    @classmethod
    def sphere(cls, center=(0.0, 0.0, 0.0), radius=64.0, band=3.0) -> "Topology":
        return cls._make(lib().wx_gen_sphere, *map(float, center), float(radius), float(band))

    @classmethod
    def spheres(cls, count=2000, rmin=4.0, rmax=40.0, lo=-1024.0, hi=1024.0, band=3.0, seed=2) -> "Topology":
        return cls._make(lib().wx_gen_spheres, count, rmin, rmax, lo, hi, band, seed)

    @classmethod
    def noise_leaves(cls, lo=-2048, extent=4096, occupancy=0.02, p_voxel=0.5, seed=3, nthreads=0) -> "Topology":
        return cls._make(lib().wx_gen_noise_leaves, lo, extent, occupancy, p_voxel, seed, nthreads)

    @classmethod
    def read_vdb(cls, path, grid_name: Optional[str] = None) -> tuple:
        """Topology of one grid of an OpenVDB file, and the file's info (version, voxel-count metadata)."""
        from ._ffi import wx_vdb_info

        out, info = C.c_void_p(), wx_vdb_info()
        check(lib().wx_vdb_read_topology(str(path).encode(), grid_name.encode() if grid_name else None,
                                         C.byref(out), C.byref(info)))
        meta = {"file_version": info.file_version, "compression": info.compression,
                "half_float": bool(info.half_float), "file_voxel_count": info.file_voxel_count,
                "grid_name": info.grid_name.decode()}
        return Topology(out.value), meta

    @staticmethod
    def read_vdb_values(path, grid_name: Optional[str] = None) -> tuple:
        """Leaf values of one grid of an OpenVDB file (n3 * 512 float32, wx_grid_set_values layout)
        and the grid's background value."""
        n, bg = C.c_uint64(), C.c_float()
        g = grid_name.encode() if grid_name else None
        check(lib().wx_vdb_read_leaf_values(str(path).encode(), g, None, 0, C.byref(n), C.byref(bg)))
        out = np.empty(n.value, np.float32)
        check(lib().wx_vdb_read_leaf_values(str(path).encode(), g, out.ctypes.data, out.size, C.byref(n), C.byref(bg)))
        return out, bg.value

    @classmethod
    def from_voxels(cls, ijk) -> "Topology":
        a = np.ascontiguousarray(ijk, dtype=np.int32).reshape(-1, 3)
        return cls._make(lib().wx_topology_from_voxels, a.ctypes.data, a.shape[0])

    @classmethod
    def from_leaves(cls, origins, masks) -> "Topology":
        o = np.ascontiguousarray(origins, dtype=np.int32).reshape(-1, 3)
        m = np.ascontiguousarray(masks, dtype=np.uint64).reshape(-1, 8)
        return cls._make(lib().wx_topology_from_leaves, o.ctypes.data, m.ctypes.data, o.shape[0])

    @classmethod
    def from_masks(cls, m: dict) -> "Topology":
        arrs = {k: np.ascontiguousarray(m[k], dtype=np.uint32) for k in ("kids5", "vals5", "kids4", "vals4", "vals3")}
        org = np.ascontiguousarray(m["origins"], dtype=np.int32)
        stride = org.shape[1] if org.ndim == 2 else 4
        n5, n4, n3 = arrs["kids5"].size // 1024, arrs["kids4"].size // 128, arrs["vals3"].size // 16
        return cls._make(lib().wx_topology_from_masks, arrs["kids5"].ctypes.data, arrs["vals5"].ctypes.data, n5,
                         arrs["kids4"].ctypes.data, arrs["vals4"].ctypes.data, n4, arrs["vals3"].ctypes.data, n3,
                         org.ctypes.data, stride)

    def sphere_values(self, center=(0.0, 0.0, 0.0), radius=64.0, band=3.0) -> np.ndarray:
        """Level-set values (n3 * 512 float32, wx_grid_set_values layout) of Topology.sphere's grid."""
        out = np.empty(self.counts[2] * 512, np.float32)
        check(lib().wx_gen_sphere_values(self._h, *map(float, center), float(radius), float(band), out.ctypes.data))
        return out

    def spheres_values(self, count=2000, rmin=4.0, rmax=40.0, lo=-1024.0, hi=1024.0, band=3.0, seed=2) -> np.ndarray:
        """Level-set values of Topology.spheres' grid (same arguments)."""
        out = np.empty(self.counts[2] * 512, np.float32)
        check(lib().wx_gen_spheres_values(self._h, count, rmin, rmax, lo, hi, band, seed, out.ctypes.data))
        return out

    def close(self) -> None:
        if self._h and self._h.value:
            lib().wx_topology_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def counts(self) -> tuple:
        c = (C.c_uint64 * 3)()
        check(lib().wx_topology_counts(self._h, c))
        return int(c[0]), int(c[1]), int(c[2])

    @property
    def active_voxels(self) -> int:
        return int(lib().wx_topology_active_voxels(self._h))

    def masks(self) -> dict:
        """masks()/origins() of the reference (src/vdb/vdb345.rs:108-161)."""
        n5, n4, n3 = self.counts
        out = {"kids5": np.zeros(n5 * 1024, np.uint32), "vals5": np.zeros(n5 * 1024, np.uint32),
               "kids4": np.zeros(n4 * 128, np.uint32), "vals4": np.zeros(n4 * 128, np.uint32),
               "vals3": np.zeros(n3 * 16, np.uint32), "origins": np.zeros((n5, 4), np.int32)}
        check(lib().wx_topology_masks(self._h, *(out[k].ctypes.data for k in
                                                 ("kids5", "vals5", "kids4", "vals4", "vals3", "origins"))))
        return out

    def sdf(self, nthreads: int = 0) -> None:
        check(lib().wx_topology_sdf(self._h, nthreads))

    def atlas(self, value_texel: int = 1) -> tuple:
        """atlas() in the uploaded texture layout: three flat u32 arrays and their cube sides."""
        side = (C.c_uint32 * 3)()
        check(lib().wx_topology_atlas(self._h, side, None, None, None, 0))
        s = [int(x) for x in side]
        a = [np.zeros(x ** 3, np.uint32) for x in s]
        check(lib().wx_topology_atlas(self._h, side, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data,
                                      value_texel))
        return a, s

    def view(self, value_texel: int = 1) -> dict:
        """The flattened reference view (masks + origins + atlases), computing the SDF first."""
        self.sdf()
        v = self.masks()
        a, s = self.atlas(value_texel)
        v["atlas"] = a
        v["dims"] = [(x, x, x) for x in s]
        return v


# --------------------------------------------------------------------------
# Uniform and cameras
# --------------------------------------------------------------------------
def sun_default() -> tuple:
    d, c, i = (C.c_float * 3)(), (C.c_float * 3)(), C.c_float()
    lib().wx_sun_default(d, c, C.byref(i))
    return tuple(d), tuple(c), i.value


def state_build(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), aspect=4.0 / 3.0, fovy=60.0, width=640.0,
                mode=MODE_DIFFUSE, show_345=(0, 0, 0), sun=None) -> wx_state_uniform:
    sd, sc, si = sun if sun is not None else sun_default()
    f3 = C.c_float * 3
    out = wx_state_uniform()
    check(lib().wx_state_build(f3(*eye), f3(*target), f3(*up), aspect, fovy, width, mode,
                               (C.c_uint32 * 3)(*show_345), f3(*sd), f3(*sc), si, C.byref(out)))
    return out


def state_bytes(s: wx_state_uniform) -> bytes:
    return C.string_at(C.addressof(s), 256)


def state_from_bytes(b: bytes) -> wx_state_uniform:
    s = wx_state_uniform()
    C.memmove(C.addressof(s), b, 256)
    return s


def orbit_eyes(count: int, radius: float, seed: int) -> np.ndarray:
    out = np.zeros((count, 3), np.float32)
    check(lib().wx_orbit_eyes(count, radius, seed, out.ctypes.data))
    return out


# --------------------------------------------------------------------------
# Device context and grids
# --------------------------------------------------------------------------
class Grid:
    def __init__(self, ctx: "Context", handle: int):
        self.ctx = ctx
        self._h = C.c_void_p(handle)

    @property
    def info(self) -> dict:
        i = wx_grid_info()
        check(lib().wx_grid_get_info(self._h, C.byref(i)))
        return {k: int(getattr(i, k)) for k, _ in wx_grid_info._fields_}

    def set_values(self, values: np.ndarray, band: float) -> None:
        """Level-set values for MODE_SURFACE (n3 * 512 float32, DFS leaf order)."""
        v = np.ascontiguousarray(values, np.float32)
        if v.size != self.info["n3"] * 512:
            raise ValueError("need n3 * 512 values")
        check(lib().wx_grid_set_values(self.ctx._h, self._h, v.ctypes.data, float(band)), self.ctx._h)

    def pools(self) -> dict:
        """Copies of the device pools: slot5, slot4 (u32), leaf (u8) and ovf ((key, distance) u32 pairs)."""
        i = self.info
        n = C.c_uint64()
        check(lib().wx_grid_read_pools(self.ctx._h, self._h, None, None, None, None, C.byref(n)), self.ctx._h)
        out = {"slot5": np.empty(i["n5"] * 32768, np.uint32), "slot4": np.empty(i["n4"] * 4096, np.uint32),
               "leaf": np.empty(i["n3"] * 512, np.uint8), "ovf": np.empty((n.value, 2), np.uint32)}
        check(lib().wx_grid_read_pools(self.ctx._h, self._h, out["slot5"].ctypes.data, out["slot4"].ctypes.data,
                                       out["leaf"].ctypes.data, out["ovf"].ctypes.data, C.byref(n)), self.ctx._h)
        return out

    def release(self) -> None:
        if self._h and self._h.value:
            check(lib().wx_grid_release(self.ctx._h, self._h), self.ctx._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Context:
    def __init__(self, device: int = 0):
        out = C.c_void_p()
        check(lib().wx_ctx_create(device, C.byref(out)))
        self._h = out
        self.device = device

    def close(self) -> None:
        if self._h and self._h.value:
            lib().wx_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_grid(self, topo: Topology, gpu: bool = False) -> Grid:
        """Compute the SDF and pack the device pools from a topology: on the host
        (wx_grid_build) or on the GPU (wx_grid_build_gpu); both give the same pools."""
        out = C.c_void_p()
        fn = lib().wx_grid_build_gpu if gpu else lib().wx_grid_build
        check(fn(self._h, topo._h, C.byref(out)), self._h)
        return Grid(self, out.value)

    def upload_view(self, v: dict) -> Grid:
        """Drop-in upload of the Rust side's flattened view (masks, origins, atlases)."""
        keep = {k: np.ascontiguousarray(v[k], dtype=np.uint32) for k in ("kids5", "vals5", "kids4", "vals4", "vals3")}
        org = np.ascontiguousarray(v["origins"], dtype=np.int32)
        atl = [np.ascontiguousarray(a, dtype=np.uint32) for a in v["atlas"]]
        view = wx_vdb345_view()
        for k, a in keep.items():
            setattr(view, k, a.ctypes.data)
        view.origins = org.ctypes.data
        view.origin_stride = org.shape[1] if org.ndim == 2 else 4
        view.n5, view.n4, view.n3 = keep["kids5"].size // 1024, keep["kids4"].size // 128, keep["vals3"].size // 16
        for i in range(3):
            view.atlas[i] = atl[i].ctypes.data
            for j in range(3):
                view.dims[i][j] = int(v["dims"][i][j])
        out = C.c_void_p()
        check(lib().wx_grid_upload(self._h, C.byref(view), C.byref(out)), self._h)
        return Grid(self, out.value)

    def render(self, grid: Grid, state: wx_state_uniform, width: int, height: int, rgba, hits=None,
               stream=None) -> None:
        """One frame: rgba (w*h*4 bytes) and hits (w*h records) are device tensors or host arrays."""
        check(lib().wx_render(self._h, grid._h, C.byref(state), width, height, _ptr(rgba), _ptr(hits),
                              None if stream is None else int(stream)), self._h)

    @property
    def tuning(self) -> dict:
        t = wx_tuning()
        check(lib().wx_ctx_get_tuning(self._h, C.byref(t)), self._h)
        return {k: int(getattr(t, k)) for k, _ in wx_tuning._fields_}

    def set_tuning(self, **kw) -> None:
        cur = self.tuning
        cur.update(kw)
        t = wx_tuning(**cur)
        check(lib().wx_ctx_set_tuning(self._h, C.byref(t)), self._h)

    def set_sdf_wait_limit(self, polls: int) -> None:
        """Bound of the GPU SDF build's dependency waits (polls 256 ns apart; 0 = default, about 2 s)."""
        check(lib().wx_ctx_set_sdf_wait_limit(self._h, polls), self._h)

    def autotune(self, frames: Sequence, candidates: Optional[Sequence[dict]] = None, reps: int = 3) -> dict:
        """Time candidate launch shapes on `frames` ((grid, state, w, h, rgba_dev, hits_dev) tuples) and
        install the fastest. Returns {"best": tuning, "table": [(tuning, ms), ...]}."""
        arr = self._frames(frames)
        if candidates is None:
            cands = []
            for o in (1, 0):  # the built-in set of wx_autotune, in its order
                cands += [dict(kernel=k, warps_per_block=w, blocks_per_sm=0, tile_width=t, tile_order=o, rays_per_lane=1)
                          for k in (0, 1) for t in (4, 8, 16) for w in (2, 4, 8)]
                cands += [dict(kernel=0, warps_per_block=4, blocks_per_sm=4, tile_width=t, tile_order=o,
                               rays_per_lane=1) for t in (4, 8)]
                cands += [dict(kernel=1, warps_per_block=w, blocks_per_sm=0, tile_width=t, tile_order=o,
                               rays_per_lane=r) for r in (2, 4, 8) for t in (4, 8) for w in (2, 4)]
        else:
            cands = [dict(self.tuning, **c) for c in candidates]
        carr = (wx_tuning * len(cands))(*[wx_tuning(**c) for c in cands])
        times = (C.c_double * len(cands))()
        best = wx_tuning()
        check(lib().wx_autotune(self._h, arr, len(frames), carr, len(cands), reps, C.byref(best), times), self._h)
        return {"best": {k: int(getattr(best, k)) for k, _ in wx_tuning._fields_},
                "table": [(c, float(times[i])) for i, c in enumerate(cands)]}

    def check_division(self, max_m: int = 4096) -> tuple:
        out = (C.c_uint64 * 3)()
        check(lib().wx_check_division(self._h, max_m, out), self._h)
        return int(out[0]), int(out[1]), int(out[2])

    def bounds_violations(self) -> int:
        """Out-of-range indices counted by the bounds-checked build (WOXEL_GB300_BOUNDS_CHECK=1)
        since the last call; raises WxError in the normal build."""
        n = C.c_uint64()
        check(lib().wx_bounds_violations(self._h, C.byref(n)), self._h)
        return int(n.value)

    @staticmethod
    def _frames(frames: Sequence) -> "C.Array":
        arr = (wx_frame * len(frames))()
        for i, (grid, state, w, h, rgba, hits) in enumerate(frames):
            arr[i].grid = grid._h.value
            arr[i].state = state
            arr[i].width, arr[i].height = w, h
            arr[i].rgba8 = _ptr(rgba)
            arr[i].hits = _ptr(hits)
        return arr

    def render_batch(self, frames: Sequence, stream=None) -> None:
        """frames: (grid, state, width, height, rgba_dev, hits_dev_or_None) tuples; one persistent launch."""
        arr = self._frames(frames)
        check(lib().wx_render_batch(self._h, arr, len(frames), None if stream is None else int(stream)), self._h)

    def batch(self, frames: Sequence) -> "Batch":
        arr = self._frames(frames)
        out = C.c_void_p()
        check(lib().wx_batch_create(self._h, arr, len(frames), C.byref(out)), self._h)
        return Batch(self, out.value, [f[0] for f in frames])


NOALLOC_MAX_FRAMES = 256


def render_batch_noalloc(frames: Sequence, stream=None) -> None:
    """wx_render_batch_noalloc: a batch rendered without any allocation or context.

    For callers that cannot allocate device memory while rendering; scratch is a
    fixed 98,560-byte device array inside the library (at most 256 frames a call).
    The first call on a device sets that device up; overlapping calls race.
    """
    arr = Context._frames(frames)
    check(lib().wx_render_batch_noalloc(arr, len(frames), None if stream is None else int(stream)))


def inject_alloc_failures(count: int) -> None:
    """wx_inject_alloc_failures: the library's next `count` device or page-locked allocations fail
    as out of memory (testing error paths); 0 stops injecting."""
    check(lib().wx_inject_alloc_failures(count))


class Batch:
    """A batched launch captured in a CUDA graph (wx_batch_create / wx_batch_launch)."""

    def __init__(self, ctx: Context, handle: int, grids: list):
        self.ctx = ctx
        self._h = C.c_void_p(handle)
        self._grids = grids  # keep the grids alive while the plan exists

    def launch(self, stream=None) -> None:
        check(lib().wx_batch_launch(self._h, None if stream is None else int(stream)), self.ctx._h)

    @property
    def info(self) -> dict:
        f, t, r = C.c_uint32(), C.c_uint32(), C.c_uint64()
        check(lib().wx_batch_info(self._h, C.byref(f), C.byref(t), C.byref(r)))
        return {"frames": f.value, "tiles": t.value, "rays": r.value}

    def close(self) -> None:
        if self._h and self._h.value:
            lib().wx_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# Serving: continuous batching of render requests (wx_server_*)
# --------------------------------------------------------------------------
from ._ffi import wx_request, wx_result, wx_server_config, wx_server_stats  # noqa: E402

SERVE_FIFO = 1


class Server:
    """Continuous-batching render server over resident grids (see include/woxel_gb300.h).

    Results live in the server's device arena until release(ticket)."""

    def __init__(self, ctx: Context, budget_bytes: int, max_inflight: int = 2, slice_tiles: int = 0,
                 max_frames: int = 0, fifo: bool = False):
        cfg = wx_server_config(budget_bytes, max_inflight, slice_tiles, max_frames, SERVE_FIFO if fifo else 0)
        out = C.c_void_p()
        check(lib().wx_server_create(ctx._h, C.byref(cfg), C.byref(out)))
        self.ctx = ctx
        self._h = out
        self._grids = []

    def add_grid(self, grid: Grid) -> int:
        gid = C.c_uint32()
        check(lib().wx_server_add_grid(self._h, grid._h, C.byref(gid)))
        self._grids.append(grid)
        return gid.value

    @staticmethod
    def request(grid_id: int, state: wx_state_uniform, width: int, height: int, hits: bool = False,
                user: int = 0) -> wx_request:
        return wx_request(grid_id, 1 if hits else 0, width, height, state, user)

    def submit(self, req: wx_request) -> int:
        t = C.c_uint64()
        check(lib().wx_server_submit(self._h, C.byref(req), C.byref(t)))
        return t.value

    def cancel(self, ticket: int) -> None:
        check(lib().wx_server_cancel(self._h, ticket))

    def poll(self, max_results: int = 64, wait_ms: int = 0) -> list:
        out = (wx_result * max_results)()
        n = C.c_uint32()
        check(lib().wx_server_poll(self._h, out, max_results, C.byref(n), wait_ms))
        return [out[i] for i in range(n.value)]

    def release(self, ticket: int) -> None:
        check(lib().wx_server_release(self._h, ticket))

    def fetch(self, result: wx_result, hits: bool = False) -> tuple:
        """Host copies of a polled result: rgba[h, w, 4] and (optionally) hits[h, w]."""
        w, h = result.width, result.height
        rgba = np.zeros((h, w, 4), np.uint8)
        hb = np.zeros((h, w), HIT_DTYPE) if hits else None
        check(lib().wx_server_copy_result(self._h, result.ticket, rgba.ctypes.data,
                                          None if hb is None else hb.ctypes.data))
        return rgba, hb

    @property
    def stats(self) -> dict:
        s = wx_server_stats()
        check(lib().wx_server_get_stats(self._h, C.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in wx_server_stats._fields_}

    def replay(self, reqs: Sequence, arrivals: Sequence, release: bool = True, timeout_s: float = 600.0) -> list:
        n = len(reqs)
        ra = (wx_request * n)(*reqs)
        ta = (C.c_double * n)(*arrivals)
        res = (wx_result * n)()
        check(lib().wx_server_replay(self._h, ra, ta, n, res, 1 if release else 0, timeout_s))
        return [res[i] for i in range(n)]

    def close(self) -> None:
        if self._h and self._h.value:
            lib().wx_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
