"""Generate tests/golden/wgsl_raycast.npz: RGBA8 frames rendered by the reference's own
raycast shader (src/shaders/raycast.comp.wgsl of woxel), translated to C++ by
oracle/wgsl_ref.py and run on the host, over grids and cameras built by the oracle.

    WOXEL_REFERENCE=/path/to/woxel python tests/golden/make_wgsl_golden.py

The frames pin the C oracle (tests/test_wgsl_golden.py) and the CUDA kernels
(tests/test_wgsl_golden_gpu.py) to the shader source. Each frame is stored with its
256-byte uniform; the grids are rebuilt by the tests from the recipes below (the
random-sphere list is stored too).
"""
from __future__ import annotations

import struct
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402
import wgsl_ref as W  # noqa: E402

OUT = HERE / "wgsl_raycast.npz"

# Grids: 0 the r=64 sphere, 1 the 2000-sphere grid, 2 40 small spheres spread over
# [-6000, 6000)^3 (several N5 nodes, negative coordinates), 3 the noise grid's leaves
# with origins in [0, 1024)^3, 4 spheres cut by the planes of the 345 grid tints
# (coordinates that are multiples of 4096, 2048, 128 and 8), 5 and 6 the reference's
# own cube and icosahedron models (their topology as the reader took it from the
# reference's assets, frozen in tests/golden/*_topology.npz), with the cameras of
# tests/golden/*_render.npz.
RANDOM_SPHERES = dict(count=40, rmin=3.0, rmax=12.0, lo=-6000.0, hi=6000.0, seed=11)
NOISE_BOX = (0, 1024)
MODELS = {5: "cube", 6: "icosahedron"}
PLANE_SPHERES = np.array([[4096.0, 100.0, 100.0, 16.0], [2048.0, -50.0, 300.0, 16.0],
                          [-4096.0, 10.0, -4096.0, 20.0], [640.0, 384.0, 60.0, 10.0]])


def random_spheres() -> np.ndarray:
    return O.sphere_list(**RANDOM_SPHERES)


def grid_view(g: int) -> dict:
    if g == 0:
        return O.workload_view("sphere")
    if g == 1:
        return O.workload_view("spheres")
    if g == 2:
        return O.Tree.spheres(random_spheres(), 3.0).view()
    if g == 3:
        return O.workload_view("noise", box=NOISE_BOX)
    if g == 4:
        return O.Tree.spheres(PLANE_SPHERES, 3.0).view()
    if g in MODELS:
        t = np.load(HERE / f"{MODELS[g]}_topology.npz")
        return O.Tree.from_masks({k: t[k] for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")}).view()
    raise ValueError(g)


def _state(eye, target, w, h, mode, show=(0, 0, 0), up=(0.0, 1.0, 0.0)) -> bytes:
    sd, sc, si = O.sun_default()
    return O.state_build(tuple(float(x) for x in eye), tuple(float(x) for x in target), up, w / h, 60.0, float(w),
                         mode, show, sd, sc, si)


def _patch(st: bytes, off: int, vals) -> bytes:
    b = bytearray(st)
    struct.pack_into(f"<{len(vals)}f", b, off, *vals)
    return bytes(b)


def frames():
    """[(grid, width, height, uniform, large)]; large frames are checked on the GPU only."""
    rng = np.random.default_rng(2024)
    out = []
    # r=64 sphere: the 640x480 benchmark camera; the same view at 160x120 in every
    # mode with and without the 345 grid tints; random eyes around and inside it.
    out.append((0, 640, 480, O.frame_state((0.0, 0.0, 200.0), 640, 480, 3), False))
    for mode in range(5):
        for show in ((0, 0, 0), (1, 1, 1)):
            out.append((0, 160, 120, _state((0.0, 0.0, 200.0), (0.0, 0.0, 0.0), 160, 120, mode, show), False))
    for k in range(15):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        eye = d * rng.uniform(70.0, 300.0)
        out.append((0, 96, 64, _state(eye, rng.uniform(-40, 40, 3), 96, 64, k % 5, (k % 2,) * 3), False))
    out.append((0, 64, 48, _state((0.0, 0.0, 0.0), (1.0, 0.3, 0.2), 64, 48, 4), False))
    # Rays with zero direction components and a -0 eye coordinate (the shader's inf / NaN paths).
    base = _state((0.5, 0.5, 200.0), (0.0, 0.0, 0.0), 64, 32, 2)
    st = _patch(base, 144, (0.0, 0.0, 0.0, 0.0))           # u = 0: dir.x = 0 for every pixel
    st = _patch(st, 160, (0.0, 0.01, 0.0, 0.0))
    out.append((0, 64, 32, _patch(st, 176, (0.0, -0.15, -1.0, 0.0)), False))
    st = _patch(base, 144, (0.0, 0.0, 0.0, 0.0))           # dir = (0, 0, -1) exactly
    st = _patch(st, 160, (0.0, 0.0, 0.0, 0.0))
    out.append((0, 16, 8, _patch(st, 176, (0.0, 0.0, -1.0, 0.0)), False))
    for mode in (0, 3, 4):
        st = _state((0.0, 0.25, 150.0), (0.0, 0.0, 0.0), 64, 48, mode)
        out.append((0, 64, 48, _patch(st, 128, (-0.0,)), False))  # eye.x = -0
    # 2000-sphere grid: orbit cameras of the benchmark at reduced size, one eye inside;
    # the benchmark's first 1920x1080 frame (GPU only).
    eyes = O.orbit_eyes(16, 3000.0, 16)
    for k, mode in enumerate((3, 2, 0, 4)):
        out.append((1, 192, 108, _state(eyes[k], (0.0, 0.0, 0.0), 192, 108, mode), False))
    out.append((1, 128, 72, _state((0.0, 0.0, 0.0), (500.0, 200.0, 100.0), 128, 72, 4), False))
    out.append((1, 1920, 1080, O.frame_state(eyes[0], 1920, 1080, 3), True))
    # small spheres over several N5 nodes
    sp = random_spheres()
    for k in range(12):
        c = sp[rng.integers(0, len(sp)), :3]
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        out.append((2, 64, 48, _state(c + d * rng.uniform(20.0, 120.0), c, 64, 48, k % 5), False))
    out.append((2, 96, 64, _state((0.0, 0.0, 0.0), (1.0, 0.5, 0.25), 96, 64, 2), False))
    # noise leaves: views from outside and inside the box
    out.append((3, 128, 72, _state((2500.0, 1800.0, 2200.0), (512.0, 512.0, 512.0), 128, 72, 0), False))
    out.append((3, 128, 72, _state((-900.0, 700.0, 1500.0), (512.0, 512.0, 512.0), 128, 72, 2), False))
    out.append((3, 96, 64, _state((512.0, 512.0, 512.0), (900.0, 100.0, 300.0), 96, 64, 3), False))
    # spheres on the tint planes, all tints on, and with only the 128 or the 8 tint
    for k, c in enumerate(PLANE_SPHERES):
        eye = c[:3] + np.array([45.0, 25.0, 60.0])
        for mode, show in ((0, (1, 1, 1)), (1, (0, 1, 0)), (2, (1, 0, 1))):
            out.append((4, 64, 48, _state(eye, c[:3], 64, 48, mode, show), False))
    # the reference's models: each frozen camera, and the first one in every mode
    for g, name in MODELS.items():
        r = np.load(HERE / f"{name}_render.npz")
        k = 0
        while f"state{k}" in r:
            w, h = (int(x) for x in r[f"size{k}"])
            st = r[f"state{k}"].tobytes()
            modes = range(5) if k == 0 else (struct.unpack_from("<I", st, 192)[0],)
            for mode in modes:
                b = bytearray(st)
                struct.pack_into("<I", b, 192, mode)
                out.append((g, w, h, bytes(b), False))
            k += 1
    return out


def main():
    so = W.build()
    shader = W.Shader(so)
    fr = frames()
    views = {}
    arrays = {"random_spheres": random_spheres(), "plane_spheres": PLANE_SPHERES}
    meta = []
    mism = 0
    for i, (g, w, h, st, large) in enumerate(fr):
        if g not in views:
            t0 = time.time()
            views[g] = grid_view(g)
            print(f"grid {g}: view in {time.time() - t0:.1f} s", flush=True)
        rgba = shader.render(views[g], st, w, h)
        arrays[f"rgba_{i}"] = rgba
        arrays[f"state_{i}"] = np.frombuffer(st, np.uint8)
        meta.append((g, w, h, int(large)))
        if not large:
            ref = O.render(views[g], st, w, h, nthreads=8, hits=False)[0]
            d = int((ref != rgba).any(axis=2).sum())
            mism += d
            if d:
                print(f"frame {i}: the oracle differs on {d} pixels", flush=True)
    arrays["meta"] = np.array(meta, np.int64)
    np.savez_compressed(OUT, **arrays)
    print(f"{len(fr)} frames -> {OUT} ({OUT.stat().st_size} bytes); oracle mismatches {mism}")


if __name__ == "__main__":
    main()
