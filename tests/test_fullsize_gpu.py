"""Parity at the benchmark's full sizes, on sampled tiles and size-independent properties.

The oracle side is built by the oracle alone: its restated generator sets the voxels,
its compute_sdf and atlas() flatten the grid, its ComputeState::build makes the
uniforms (asserted byte-equal to the product's). The GPU side is the product's
generator, SDF, pools and kernels.

* 2000-sphere grid (476k leaves), 1920x1080 frames: random 8x4 tiles against the
  oracle-built view; batched launch == per-frame launches; repeated renders identical.
* noise grid, 3840x2160, mode 0 (first active voxel): the [-2048,0)^3 octant of the
  benchmark's 4096^3 grid (367,660 leaves) against the oracle-built view of that octant;
  and the whole 2.68M-leaf grid (GPU SDF build) against the oracle's own view of it, built
  on a host thread while the other GPU tests run.
"""
import numpy as np
import pytest
import torch

import oracle as orc
import woxel_gb300 as wx
from parity import compare, gpu_render
from woxel_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def tile_mask(w, h, tiles):
    m = np.zeros((h, w), bool)
    tx = w // 8
    for t in tiles:
        x0, y0 = (int(t) % tx) * 8, (int(t) // tx) * 4
        m[y0:y0 + 4, x0:x0 + 8] = True
    return m


def sampled_parity(ctx, grid, view, frame, ntiles, seed, oracle_state=None):
    """GPU frame vs the oracle on `ntiles` random tiles; the oracle renders with its own
    uniform (oracle_state) when given, which must equal the product's byte for byte."""
    st = frame.state()
    sb = wx.state_bytes(st)
    if oracle_state is not None:
        assert oracle_state == sb, "uniform differs from the oracle's"
        sb = oracle_state
    rg, hg = gpu_render(ctx, grid, st, frame.width, frame.height)
    rng = np.random.default_rng(seed)
    tiles = np.sort(rng.choice((frame.width // 8) * (frame.height // 4), size=ntiles, replace=False)).astype(np.uint64)
    ro, ho, _ = orc.render(view, sb, frame.width, frame.height, nthreads=16, hits=True, tiles=tiles)
    m = tile_mask(frame.width, frame.height, tiles)
    compare(rg, hg, ro, ho, where=m, label=f"{frame.grid} {frame.width}x{frame.height}")
    return rg, hg


@pytest.fixture(scope="module")
def spheres(cuda_ctx, oracle_spheres_view):
    topo = W.spheres_topology()
    grid = cuda_ctx.build_grid(topo)
    return topo, oracle_spheres_view, grid


def test_spheres_1080p_sampled_tiles(cuda_ctx, spheres):
    topo, view, grid = spheres
    frames = W.spheres_frames()
    ostates = orc.workload_frames("spheres")
    for k in (0, 7, 12):
        rg, hg = sampled_parity(cuda_ctx, grid, view, frames[k], ntiles=1500, seed=k, oracle_state=ostates[k][2])
        assert (wx.hit_fields(hg)["state"] == 0).mean() > 0.05


def test_spheres_batched_equals_plain_and_repeatable(cuda_ctx, spheres):
    _, _, grid = spheres
    frames = W.spheres_frames()[:4]
    outs = [torch.zeros(f.width * f.height * 4, dtype=torch.uint8, device="cuda") for f in frames]
    cuda_ctx.render_batch([(grid, f.state(), f.width, f.height, o, None) for f, o in zip(frames, outs)])
    torch.cuda.synchronize()
    for f, o in zip(frames, outs):
        a, _ = gpu_render(cuda_ctx, grid, f.state(), f.width, f.height, hits=False)
        b, _ = gpu_render(cuda_ctx, grid, f.state(), f.width, f.height, hits=False)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(o.cpu().numpy().reshape(f.height, f.width, 4), a)


@pytest.mark.parametrize("mode", [3, 0])
def test_spheres_all_kernels_agree(cuda_ctx, spheres, mode):
    """Whole 1080p frames: the per-tile kernel, other tile shapes, both tile-row orders and 2, 4 and 8
    rays per lane (lanes that refill) write the same RGBA8 and hit records as the tile-queue kernel,
    bit for bit."""
    _, _, grid = spheres
    before = cuda_ctx.tuning
    try:
        for f in W.spheres_frames()[:4]:
            st = f.state()
            st.render_mode[0] = mode
            outs = []
            for k, tw, order, rays in ((0, 8, 1, 1), (1, 4, 1, 1), (0, 16, 0, 1), (1, 32, 1, 1), (1, 4, 0, 1),
                                       (0, 4, 0, 1), (1, 4, 1, 4), (1, 8, 0, 2), (1, 4, 1, 8)):
                cuda_ctx.set_tuning(kernel=k, tile_width=tw, tile_order=order, rays_per_lane=rays)
                outs.append(gpu_render(cuda_ctx, grid, st, f.width, f.height))
            for rg, hg in outs[1:]:
                np.testing.assert_array_equal(rg, outs[0][0])
                np.testing.assert_array_equal(hg.view(np.uint8), outs[0][1].view(np.uint8))
    finally:
        cuda_ctx.set_tuning(**before)


def test_noise_octant_4k_sampled_tiles(cuda_ctx):
    """The noise grid's first octant: product generator (first N5 of its masks), product SDF
    and pools on the GPU; oracle generator, compute_sdf and atlas() on the CPU."""
    from test_oracle_workloads import first_n5_slice

    topo = wx.Topology.from_masks(first_n5_slice(W.noise_topology().masks()))
    assert topo.counts == (1, 443, 367660)
    grid = cuda_ctx.build_grid(topo)
    view = orc.workload_view("noise", box=(-2048, 0))
    frames, ostates = W.noise_frames(), orc.workload_frames("noise")
    hits = 0
    for k in (0, 5):
        rg, hg = sampled_parity(cuda_ctx, grid, view, frames[k], ntiles=800, seed=40 + k, oracle_state=ostates[k][2])
        f = wx.hit_fields(hg)
        hits += int((f["state"] == 0).sum())
        assert (f["level"][f["state"] == 0] == 3).all()
    assert hits > 10000


def test_noise_4k_sampled_tiles(cuda_ctx, oracle_noise_view):
    """The whole noise grid: product generator, GPU SDF build and pools against the oracle's
    generator, compute_sdf and atlas() (built on a host thread while the other tests ran)."""
    topo = W.noise_topology()
    n5, n4, n3 = topo.counts
    assert abs(n3 / (512 ** 3) - 0.02) < 0.001  # 2.0% of the 8^3 leaf lattice
    grid = cuda_ctx.build_grid(topo, gpu=True)
    assert grid.info["n3"] == n3
    view = oracle_noise_view
    assert view["vals3"].size // 16 == n3
    frame = W.noise_frames()[0]
    ostate = orc.workload_frames("noise")[0][2]
    rg, hg = sampled_parity(cuda_ctx, grid, view, frame, ntiles=600, seed=3, oracle_state=ostate)
    f = wx.hit_fields(hg)
    hit = f["state"] == 0
    assert hit.mean() > 0.05 and (f["level"][hit] == 3).all()  # first active voxel, always inside a leaf
