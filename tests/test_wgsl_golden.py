"""The C oracle against frames rendered by the reference's own raycast shader.

tests/golden/wgsl_raycast.npz holds RGBA8 frames of src/shaders/raycast.comp.wgsl
(woxel), translated mechanically to C++ by oracle/wgsl_ref.py and run on the host
(tests/golden/make_wgsl_golden.py made them): 80 frames over seven grids the oracle
builds (the r=64 sphere, the 2000-sphere grid, small spheres over several N5 nodes,
noise leaves, spheres on the planes of the 345 grid tints, and the reference's own
cube and icosahedron models as its reader's topology), render modes 0-4, grid
tints, cameras outside and inside the grids, rays with zero direction components and
a -0 eye coordinate. Every frame must be equal byte for byte: the oracle's control
flow, constants, index arithmetic and FP32 operation order are those of the shader
text. Planted changes in the translated shader (the nudge, the shadow offset, the
mask logic, the scale table, sign11, the shading constants, the tints, the bounds
test) each change at least two of these frames.
"""
import os
from pathlib import Path

import numpy as np
import pytest

import oracle as orc

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "golden" / "wgsl_raycast.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(FIXTURE)


def _frames(golden):
    for i, (g, w, h, large) in enumerate(golden["meta"]):
        yield i, int(g), int(w), int(h), bool(large), bytes(golden[f"state_{i}"]), golden[f"rgba_{i}"]


def _make():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_wgsl_golden", HERE / "golden" / "make_wgsl_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fixture_recipes(golden):
    """The grids the frames were rendered over are the ones the recipes rebuild."""
    mk = _make()
    assert np.array_equal(golden["random_spheres"], mk.random_spheres())
    assert np.array_equal(golden["plane_spheres"], mk.PLANE_SPHERES)
    meta = golden["meta"]
    assert len(meta) == 80 and set(int(g) for g in meta[:, 0]) == {0, 1, 2, 3, 4, 5, 6}
    assert sum(int(x) for x in meta[:, 3]) == 1  # the 1920x1080 frame, checked on the GPU


@pytest.mark.parametrize("grid", [0, 2, 3, 4, 5, 6])
def test_oracle_matches_reference_shader(golden, grid):
    mk = _make()
    view = mk.grid_view(grid)
    n = 0
    for i, g, w, h, large, st, want in _frames(golden):
        if g != grid or large:
            continue
        got = orc.render(view, st, w, h, nthreads=os.cpu_count() or 4, hits=False)[0]
        bad = np.argwhere((got != want).any(axis=2))
        assert bad.size == 0, f"frame {i} ({w}x{h}): {len(bad)} pixels differ, first at {bad[:3].tolist()}"
        n += 1
    assert n >= 3


def test_oracle_matches_reference_shader_spheres_grid(golden, oracle_spheres_view):
    n = 0
    for i, g, w, h, large, st, want in _frames(golden):
        if g != 1 or large:
            continue
        got = orc.render(oracle_spheres_view, st, w, h, nthreads=os.cpu_count() or 4, hits=False)[0]
        bad = np.argwhere((got != want).any(axis=2))
        assert bad.size == 0, f"frame {i} ({w}x{h}): {len(bad)} pixels differ, first at {bad[:3].tolist()}"
        n += 1
    assert n == 5


def _shader():
    import wgsl_ref

    if not wgsl_ref.shader_path().exists():
        pytest.skip("the reference checkout (WOXEL_REFERENCE) is not present on this machine")
    return wgsl_ref.Shader(wgsl_ref.build())


def test_translated_shader_reproduces_fixture(golden):
    """Where the reference checkout is present: translating its shader again gives the
    stored frames (the fixture is the shader's output, not a copy of the oracle's)."""
    sh = _shader()
    mk = _make()
    views = {}
    for i, g, w, h, large, st, want in _frames(golden):
        if large or g == 1:
            continue
        if g not in views:
            views[g] = mk.grid_view(g)
        assert np.array_equal(sh.render(views[g], st, w, h), want), f"frame {i}"


def test_translator_on_a_small_shader(tmp_path):
    """The translator itself on a shader with a known answer: vector arithmetic and
    swizzles, switch, for, struct constructors, integer and float %, shifts, select."""
    import wgsl_ref

    src = """
struct P { v: vec3<f32>, k: u32, }
@group(0) @binding(0) var out_tex: texture_storage_2d<rgba8unorm, write>;
fn f(p: P) -> P { var q = p; q.v = q.v.zxy * 0.5; q.k += 1u; return q; }
@compute @workgroup_size(4, 2)
fn main(@builtin(global_invocation_id) gid: vec3<u32>) {
    var acc = 0.0;
    for (var i: u32 = 0u; i < gid.x; i++) { acc += f32(i % 3u); }
    var c = vec3<f32>(0.0);
    switch gid.y % 2u {
        case 0u: { c = vec3(acc / 8.0, 0.25, 1.0); }
        default: { let p = f(P(vec3(1.0, 0.5, 0.25), 7u)); c = vec3<f32>(p.v.x, f32(p.k) / 16.0, select(0.0, 1.0, (i32(-7) % 4) == -3)); }
    }
    let s = f32((gid.x << 2u) >> 1u) / 16.0;
    textureStore(out_tex, gid.xy, vec4(c.xy, s, 1.0));
}
"""
    cpp, table = wgsl_ref.translate(src, entry="main")
    assert table == {"out_tex": (0, 0, "texture_storage_2d")}
    import subprocess

    so = tmp_path / "lib.so"
    cpp_file = tmp_path / "s.cpp"
    cpp_file.write_text(cpp)
    subprocess.run(["g++", "-O1", "-std=c++20", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                    "-I", str(Path(wgsl_ref.__file__).parent), "-o", str(so), str(cpp_file)], check=True)
    import ctypes as C
    lib = C.CDLL(str(so))
    lib.wref_bind.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
    out = np.zeros((4, 8, 4), np.uint8)
    assert lib.wref_bind(0, 0, out.ctypes.data, out.nbytes, 8, 4, 1) == 0
    lib.wref_dispatch(2, 2, 1, 2)

    def u8(x):
        return 0 if x <= 0 else 255 if x >= 1 else int(np.floor(np.float32(x) * np.float32(255) + np.float32(0.5)))

    for y in range(4):
        for x in range(8):
            acc = float(sum(i % 3 for i in range(x)))
            if y % 2 == 0:
                c = (acc / 8.0, 0.25)
            else:
                c = (0.25 * 0.5, 8 / 16.0)  # q.v = (1, .5, .25).zxy * .5 -> x = .125; k = 8
            s = ((x << 2) >> 1) / 16.0
            assert tuple(out[y, x]) == (u8(c[0]), u8(c[1]), u8(s), 255), (x, y)
