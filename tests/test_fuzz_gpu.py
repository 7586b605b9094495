"""Seeded random cases, GPU against the oracle: random grids (sparse voxels, sphere unions,
leaf-aligned blocks, voxels at the +-4096 bound, active tiles), random cameras (outside,
inside and across the grid), ragged resolutions, every render mode (mode 5 with level-set
values where the grid has them) and every launch shape. Bit-exact as in the other parity
tests, the zero-crossing t included."""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, dispatch_mask, gpu_render, oracle_render, oracle_view

pytestmark = pytest.mark.gpu

TUNINGS = [dict(kernel=0, tile_width=8, warps_per_block=4, blocks_per_sm=0, tile_order=1, rays_per_lane=1),
           dict(kernel=1, tile_width=4, warps_per_block=2, blocks_per_sm=0, tile_order=0, rays_per_lane=1),
           dict(kernel=0, tile_width=16, warps_per_block=8, blocks_per_sm=0, tile_order=0, rays_per_lane=1),
           dict(kernel=1, tile_width=32, warps_per_block=4, blocks_per_sm=0, tile_order=1, rays_per_lane=1),
           dict(kernel=0, tile_width=4, warps_per_block=4, blocks_per_sm=4, tile_order=1, rays_per_lane=1),
           dict(kernel=1, tile_width=8, warps_per_block=4, blocks_per_sm=0, tile_order=1, rays_per_lane=4),
           dict(kernel=1, tile_width=4, warps_per_block=2, blocks_per_sm=0, tile_order=0, rays_per_lane=8),
           dict(kernel=1, tile_width=16, warps_per_block=8, blocks_per_sm=0, tile_order=1, rays_per_lane=2)]


def random_grid(rng):
    """(topology, values or None, a point of interest)."""
    kind = rng.integers(5)
    if kind == 0:
        r = int(rng.integers(50, 600))
        ijk = rng.integers(-r, r, size=(int(rng.integers(50, 3000)), 3))
        return wx.Topology.from_voxels(ijk.astype(np.int32)), None, (0.0, 0.0, 0.0)
    if kind == 1:
        args = dict(count=int(rng.integers(3, 40)), rmin=3.0, rmax=float(rng.uniform(6, 40)),
                    lo=-300.0, hi=300.0, band=3.0, seed=int(rng.integers(1 << 30)))
        topo = wx.Topology.spheres(**args)
        return topo, (topo.spheres_values(**args), 3.0), (0.0, 0.0, 0.0)
    if kind == 2:
        n = int(rng.integers(2, 7))
        o = rng.integers(-20, 20, 3) * 8
        g = (np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3) * 8 + o)
        masks = rng.integers(0, 1 << 62, size=(g.shape[0], 8), dtype=np.uint64) * (rng.random((g.shape[0], 8)) < 0.3)
        topo = wx.Topology.from_leaves(g.astype(np.int32), masks.astype(np.uint64))
        return topo, None, tuple(float(x) for x in o + 4 * n)
    if kind == 3:
        ijk = np.concatenate([rng.integers(4000, 4096, size=(300, 3)), rng.integers(-4096, -4000, size=(300, 3))])
        return wx.Topology.from_voxels(ijk.astype(np.int32)), None, (4050.0, 4050.0, 4050.0)
    topo = wx.Topology.from_voxels(rng.integers(-200, 200, size=(800, 3)).astype(np.int32))
    m = topo.masks()
    for _ in range(3):
        m["vals4"][rng.integers(m["vals4"].size)] |= np.uint32(1 << int(rng.integers(32)))
        m["vals5"][rng.integers(m["vals5"].size)] |= np.uint32(1 << int(rng.integers(32)))
    return wx.Topology.from_masks(m), None, (0.0, 0.0, 0.0)


def random_camera(rng, poi):
    where = rng.integers(3)
    if where == 0:  # outside, looking at the point of interest
        d = rng.normal(size=3)
        eye = np.array(poi) + d / np.linalg.norm(d) * rng.uniform(100, 3000)
        return tuple(float(x) for x in eye), poi
    if where == 1:  # inside the grid's box
        eye = np.array(poi) + rng.uniform(-150, 150, 3)
        return tuple(float(x) for x in eye), tuple(float(x) for x in eye + rng.normal(size=3))
    eye = rng.uniform(-5000, 5000, 3)  # anywhere, possibly beyond the +-4096 bound
    return tuple(float(x) for x in eye), poi


@pytest.mark.parametrize("seed", range(24))
def test_fuzz(cuda_ctx, seed):
    rng = np.random.default_rng(1000 + seed)
    topo, vals, poi = random_grid(rng)
    view = oracle_view(topo)
    grid = cuda_ctx.build_grid(topo, gpu=bool(rng.integers(2)))
    if vals is not None:
        view["values"], view["band"] = vals
        grid.set_values(*vals)
    before = cuda_ctx.tuning
    cuda_ctx.set_tuning(**TUNINGS[seed % len(TUNINGS)])
    try:
        for _ in range(2):
            w, h = int(rng.integers(8, 160)), int(rng.integers(4, 120))
            eye, target = random_camera(rng, poi)
            mode = int(rng.integers(6))
            st = wx.state_build(eye=eye, target=target, aspect=w / h, fovy=float(rng.uniform(20, 120)),
                                width=float(w), mode=mode, show_345=tuple(int(x) for x in rng.integers(0, 2, 3)))
            rg, hg = gpu_render(cuda_ctx, grid, st, w, h)
            ro, ho = oracle_render(view, st, w, h)
            m = dispatch_mask(w, h)
            label = f"seed {seed} mode {mode} {w}x{h} eye {eye}"
            compare(rg, hg, ro, ho, where=m, label=label)
            np.testing.assert_array_equal(hg["reserved"][m], ho["reserved"][m], err_msg=label)
    finally:
        cuda_ctx.set_tuning(**before)
