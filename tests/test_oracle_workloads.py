"""The benchmark workloads built twice: by the product's generators and by the oracle alone.

The oracle restates the seeded generators (splitmix64 sphere lists, narrow-band spheres
set voxel by voxel, value-noise leaves, orbit eyes, the reference app's default sun) and
builds its grids through its own set_voxel, so a CPU run that uses only the oracle sees
the same grids and cameras the GPU renders. Checked here:

* masks and origins of the r=64 sphere, of the full 2000-sphere grid and of value-noise
  grids (a 1024^3 domain at two voxel probabilities; the [-2048,0)^3 octant of the
  benchmark's 4096^3 noise grid) are identical word for word;
* the uniforms of every benchmark camera (the 640x480 sphere view, the 16 orbit views of
  the 2000-sphere grid, the 8 noise views and the 256 mixed requests) are identical
  byte for byte between wx_state_build and the oracle's restatement of
  ComputeState::build (compute_state.rs:87-131), so eye, u, mv and wp agree exactly.
"""
import numpy as np
import pytest

import oracle as orc
import woxel_gb300 as wx
from woxel_gb300 import workloads as W

MASK_KEYS = ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")


def assert_masks_equal(a: dict, b: dict):
    for k in MASK_KEYS:
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)


def first_n5_slice(m: dict) -> dict:
    """masks() restricted to the first N5 in DFS order (its N4s and leaves come first)."""
    n4 = int(sum(bin(int(x)).count("1") for x in m["kids5"][:1024]))
    n3 = int(sum(bin(int(x)).count("1") for x in m["kids4"][:128 * n4]))
    return {"kids5": m["kids5"][:1024], "vals5": m["vals5"][:1024], "kids4": m["kids4"][:128 * n4],
            "vals4": m["vals4"][:128 * n4], "vals3": m["vals3"][:16 * n3], "origins": m["origins"][:1]}


def test_sphere_grid_masks_equal():
    t = orc.workload_tree("sphere")
    assert t.counts == (8, 8, 1706)
    assert_masks_equal(t.masks(), W.sphere_topology().masks())


def test_spheres_grid_masks_equal():
    np.testing.assert_array_equal(orc.sphere_list(2000, 4.0, 40.0, -1024.0, 1024.0, 2)[:, 3].min() >= 4.0, True)
    t = orc.workload_tree("spheres")
    topo = W.spheres_topology()
    assert t.counts == topo.counts == (8, 3037, 476014)
    assert_masks_equal(t.masks(), topo.masks())


@pytest.mark.parametrize("p_voxel,seed", [(0.5, 3), (0.3, 5)])
def test_noise_grid_masks_equal_small_domain(p_voxel, seed):
    t = orc.Tree.noise_leaves(-512, 1024, 0.02, p_voxel, seed)
    topo = wx.Topology.noise_leaves(-512, 1024, 0.02, p_voxel, seed)
    assert t.counts == topo.counts
    assert t.counts[2] == round(0.02 * 128 ** 3)
    assert_masks_equal(t.masks(), topo.masks())


def test_noise_grid_octant_masks_equal():
    """The benchmark's noise grid: its [-2048,0)^3 octant is the first N5 of the product's grid."""
    t = orc.workload_tree("noise", box=(-2048, 0))
    assert t.counts[0] == 1
    assert_masks_equal(t.masks(), first_n5_slice(W.noise_topology().masks()))


def test_orbit_eyes_and_sun_equal():
    for count, radius, seed in ((16, 3000.0, 16), (8, 3500.0, 8), (64, 200.0, 12345)):
        np.testing.assert_array_equal(orc.orbit_eyes(count, radius, seed), wx.orbit_eyes(count, radius, seed))
    assert orc.sun_default() == wx.sun_default()


@pytest.mark.parametrize("name", ["sphere", "spheres", "noise"])
def test_benchmark_uniforms_bit_exact(name):
    ours = W.workload(name).frames
    theirs = orc.workload_frames(name)
    assert len(ours) == len(theirs)
    for f, (w, h, sb) in zip(ours, theirs):
        assert (f.width, f.height) == (w, h)
        assert wx.state_bytes(f.state()) == sb


def test_mixed_request_uniforms_bit_exact():
    """The 256 mixed requests: every pose and resolution, wx_state_build against the oracle's
    ComputeState::build, all 256 bytes (view, camera_to_world, eye, u, mv, wp, sun)."""
    frames = W.mixed_frames()
    assert len(frames) == 256
    for f in frames:
        ours = wx.state_bytes(f.state())
        assert ours == orc.frame_state(f.eye, f.width, f.height, f.mode), (f.width, f.height, f.eye)
        u = np.frombuffer(ours, np.float32)
        assert np.isfinite(u[:64]).all()


def test_random_cameras_uniforms_bit_exact():
    """Seeded random cameras (eye, target, fov, aspect, width, mode): the same 256 bytes."""
    rng = np.random.default_rng(11)
    sun = orc.sun_default()
    for _ in range(200):
        eye = tuple(float(x) for x in rng.uniform(-5000, 5000, 3).astype(np.float32))
        target = tuple(float(x) for x in rng.uniform(-100, 100, 3).astype(np.float32))
        fovy = float(np.float32(rng.uniform(20, 100)))
        w, h = int(rng.integers(8, 4096)), int(rng.integers(4, 2160))
        mode = int(rng.integers(0, 6))
        ours = wx.state_bytes(wx.state_build(eye=eye, target=target, aspect=w / h, fovy=fovy, width=float(w),
                                             mode=mode))
        theirs = orc.state_build(eye, target, (0.0, 1.0, 0.0), w / h, fovy, float(w), mode, (0, 0, 0), *sun)
        assert ours == theirs


@pytest.mark.parametrize("name", ["sphere", "spheres"])
def test_level_set_values_equal(name):
    """Render mode 5's level-set values (one float per leaf voxel): the oracle's restatement
    of the sphere distance against wx_gen_sphere(s)_values, bit for bit."""
    t = orc.workload_tree(name)
    ov = t.spheres_values(orc.workload_spheres(name), 3.0)
    topo = W.workload(name).grids[name]()
    pv = W.sphere_values(topo) if name == "sphere" else W.spheres_values(topo)
    assert ov.size == topo.counts[2] * 512
    np.testing.assert_array_equal(ov.view(np.uint32), pv.view(np.uint32))
    assert (ov < 0).any() and (ov == 3.0).any()
