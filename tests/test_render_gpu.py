"""GPU parity: the sm_103a raycast kernel (through the C ABI) against the CPU oracle."""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, dispatch_mask, gpu_render, oracle_render, oracle_view

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["persistent", "pixel", "pixel-16x2", "persistent-4x8", "persistent-4blocks", "pixel-rows",
                        "wave4", "wave2-4x8", "wave8-16x2-rows"],
                autouse=True)
def kernel(request, cuda_ctx):
    """Run every parity test on both kernels, on non-default pixel tile shapes, at reduced occupancy,
    with tile rows handed out top to bottom, and with 2, 4 and 8 rays per lane (lanes that refill)."""
    before = cuda_ctx.tuning
    p = request.param
    tw = {"pixel-16x2": 16, "persistent-4x8": 4, "wave2-4x8": 4, "wave8-16x2-rows": 16}.get(p, 8)
    bps = 4 if p == "persistent-4blocks" else 0
    rays = {"wave4": 4, "wave2-4x8": 2, "wave8-16x2-rows": 8}.get(p, 1)
    cuda_ctx.set_tuning(kernel=0 if p.startswith("persistent") else 1, tile_width=tw, blocks_per_sm=bps,
                        warps_per_block=4, tile_order=0 if p.endswith("rows") else 1, rays_per_lane=rays)
    yield request.param
    cuda_ctx.set_tuning(**before)


def test_fast_division_matches_ieee(cuda_ctx, kernel):
    """Every divisor m < 4096 and every significand of [1,2) and [-2,-1): bit-equal to IEEE x/m."""
    if kernel != "persistent":
        pytest.skip("kernel independent")
    bad, m, xbits = cuda_ctx.check_division(4096)
    assert bad == 0, f"{bad} mismatches, first m={m} x=0x{xbits:08x}"


@pytest.fixture(scope="module")
def sphere64(cuda_ctx):
    topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    view = oracle_view(topo)
    return topo, view, cuda_ctx.build_grid(topo)


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_sphere_640x480_all_modes(cuda_ctx, sphere64, mode):
    """Config 1: sphere r=64 at the origin, band 3, camera (0,0,200) -> origin, 60 deg, 640x480."""
    _, view, grid = sphere64
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=640 / 480, fovy=60.0, width=640.0, mode=mode)
    rg, hg = gpu_render(cuda_ctx, grid, st, 640, 480)
    ro, ho = oracle_render(view, st, 640, 480)
    s = compare(rg, hg, ro, ho, label=f"mode{mode}")
    assert s["rgba_exact"] and s["t_exact"]
    assert (wx.hit_fields(hg)["state"] == 0).sum() > 50000  # the sphere is in view


def test_show_345_grid_tint(cuda_ctx, sphere64):
    _, view, grid = sphere64
    st = wx.state_build(eye=(30, 90, 150), target=(0, 0, 0), aspect=1.0, fovy=50.0, width=256.0, mode=1,
                        show_345=(1, 1, 1))
    rg, hg = gpu_render(cuda_ctx, grid, st, 256, 256)
    ro, ho = oracle_render(view, st, 256, 256)
    compare(rg, hg, ro, ho, label="show345")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_sparse_grids(cuda_ctx, seed):
    rng = np.random.default_rng(seed)
    ijk = rng.integers(-400, 400, size=(3000, 3)).astype(np.int32)
    topo = wx.Topology.from_voxels(ijk)
    view = oracle_view(topo)
    grid = cuda_ctx.build_grid(topo)
    eye = tuple(float(x) for x in rng.uniform(-700, 700, 3))
    for mode in (0, 3):
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=1.5, fovy=70.0, width=192.0, mode=mode)
        rg, hg = gpu_render(cuda_ctx, grid, st, 192, 128)
        ro, ho = oracle_render(view, st, 192, 128)
        compare(rg, hg, ro, ho, label=f"rand{seed}/mode{mode}")


def test_dropin_view_upload_equals_native_build(cuda_ctx):
    """wx_grid_upload (Rust-side view) and wx_grid_build (native SDF) render identically."""
    rng = np.random.default_rng(11)
    ijk = rng.integers(-150, 150, size=(5000, 3)).astype(np.int32)
    topo = wx.Topology.from_voxels(ijk)
    view = topo.view(value_texel=0x40400000)  # value texels carry f32 bits, as in the reference
    g1 = cuda_ctx.build_grid(topo)
    g2 = cuda_ctx.upload_view(view)
    assert g1.info["n3"] == g2.info["n3"] and g1.info["active_voxels"] == g2.info["active_voxels"]
    st = wx.state_build(eye=(200, 130, -260), target=(0, 0, 0), aspect=1.0, fovy=60.0, width=160.0, mode=3)
    r1, h1 = gpu_render(cuda_ctx, g1, st, 160, 160)
    r2, h2 = gpu_render(cuda_ctx, g2, st, 160, 160)
    np.testing.assert_array_equal(r1, r2)
    np.testing.assert_array_equal(h1.view(np.uint8), h2.view(np.uint8))
    ro, ho = oracle_render(view, st, 160, 160)
    compare(r1, h1, ro, ho, label="dropin")


def test_large_leaf_distances_use_the_overflow_table(cuda_ctx):
    """Leaf texels >= 255 (possible in a hand-made view) are stored exactly beside the byte pool."""
    rng = np.random.default_rng(12)
    topo = wx.Topology.from_voxels(rng.integers(-120, 120, size=(3000, 3)).astype(np.int32))
    marker = 0x7FFFFFFF
    view = topo.view(value_texel=marker)
    a3 = view["atlas"][2].copy()
    inactive = np.nonzero(a3 != marker)[0]
    pick = rng.choice(inactive, size=min(4000, inactive.size), replace=False)
    a3[pick] = rng.choice(np.array([254, 255, 256, 300, 4097, 70000, 4000000000], np.uint32), size=pick.size)
    view["atlas"] = [view["atlas"][0], view["atlas"][1], a3]
    grid = cuda_ctx.upload_view(view)
    for eye, mode in [((150.0, 90.0, -200.0), 3), ((-40.0, 180.0, 160.0), 0)]:
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=1.0, fovy=70.0, width=96.0, mode=mode)
        rg, hg = gpu_render(cuda_ctx, grid, st, 96, 96)
        ro, ho = oracle_render(view, st, 96, 96)
        compare(rg, hg, ro, ho, label=f"overflow/mode{mode}")


def test_root_table_and_root_scan(cuda_ctx):
    """N5 lookup through the dense root-key table (keys with holes) and through the scan that
    replaces it when the box of root keys exceeds 2^20 entries: both match the oracle."""
    cube = np.stack(np.mgrid[0:40, 0:40, 0:40], -1).reshape(-1, 3)
    near = np.concatenate([cube + 1500, cube - 1540])            # N5 keys (0,0,0) and (-1,-1,-1) only
    far = np.array([[4096 * 1500, 4096 * 1500, 0]])              # key box 1501 x 1501 x 1
    views = [((3500.0, 3400.0, 3600.0), (1500, 1500, 1500), 3),
             ((-3900.0, -200.0, -3900.0), (-1500, -1500, -1500), 0),
             ((10.0, -20.0, 30.0), (1500, 1500, 1500), 3)]     # eye in key (0,-1,0): no N5 there
    for ijk in (near, np.concatenate([near, far])):
        topo = wx.Topology.from_voxels(ijk.astype(np.int32))
        view = oracle_view(topo)
        grid = cuda_ctx.build_grid(topo)
        for eye, target, mode in views:
            st = wx.state_build(eye=eye, target=target, aspect=1.0, fovy=3.0, width=96.0, mode=mode)
            rg, hg = gpu_render(cuda_ctx, grid, st, 96, 96)
            ro, ho = oracle_render(view, st, 96, 96)
            compare(rg, hg, ro, ho, label=f"root n5={topo.counts[0]} eye={eye}")
            assert (wx.hit_fields(hg)["state"] == 0).mean() > 0.01


def test_host_buffers_match_device_buffers(cuda_ctx, sphere64):
    _, view, grid = sphere64
    st = wx.state_build(eye=(100, 40, 120), target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=320.0, mode=3)
    rd, hd = gpu_render(cuda_ctx, grid, st, 320, 240)
    rh, hh = gpu_render(cuda_ctx, grid, st, 320, 240, host=True)
    np.testing.assert_array_equal(rd, rh)
    np.testing.assert_array_equal(hd.view(np.uint8), hh.view(np.uint8))


def test_pinned_host_buffers_are_written_directly(cuda_ctx, sphere64):
    """Page-locked host outputs (written by the kernel through their device alias) equal device outputs,
    and pixels outside the dispatched region keep their contents."""
    import torch

    _, view, grid = sphere64
    w, h = 101, 77
    st = wx.state_build(eye=(100, 40, 120), target=(0, 0, 0), aspect=w / h, fovy=60.0, width=float(w), mode=3)
    rd, hd = gpu_render(cuda_ctx, grid, st, w, h)
    rgba = torch.full((h * w * 4,), 7, dtype=torch.uint8).pin_memory()
    hits = torch.zeros(h * w * 32, dtype=torch.uint8).pin_memory()
    cuda_ctx.render(grid, st, w, h, rgba, hits, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    r = rgba.numpy().reshape(h, w, 4)
    hh = hits.numpy().view(wx.HIT_DTYPE).reshape(h, w)
    m = dispatch_mask(w, h)
    np.testing.assert_array_equal(r[m], rd[m])
    np.testing.assert_array_equal(hh[m].view(np.uint8), hd[m].view(np.uint8))
    assert (r[~m] == 7).all()


def test_ragged_resolution_leaves_border_untouched(cuda_ctx, sphere64):
    """Dispatch covers 8*floor(w/8) x 4*floor(h/4) pixels (wgpu_context.rs:281); the rest is not written."""
    _, view, grid = sphere64
    w, h = 103, 37
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=w / h, fovy=60.0, width=float(w), mode=0)
    rgba = np.full((h, w, 4), 7, np.uint8)
    hits = np.zeros((h, w), wx.HIT_DTYPE)
    cuda_ctx.render(grid, st, w, h, rgba, hits)
    import torch

    torch.cuda.synchronize()
    m = dispatch_mask(w, h)
    assert (rgba[~m] == 7).all()
    ro, ho = oracle_render(view, st, w, h)
    compare(rgba, hits, ro, ho, where=m, label="ragged")


def test_edge_cameras(cuda_ctx, sphere64):
    """Eye inside the band (hit at i=0, zero mask), far outside the +-4096 bound, on node boundaries."""
    _, view, grid = sphere64
    for eye, target in [((64.0, 0.5, 0.5), (0, 0, 0)),       # inside an active voxel
                        ((9000.0, 10.0, 5.0), (0, 0, 0)),    # beyond the bound: state 1 at step 0
                        ((0.0, 0.0, 128.0), (0, 0, 0)),      # on N4/N5 boundaries
                        ((-128.0, 4096.0, -8.0), (0, 0, 0))]:
        for mode in (0, 3, 4):
            st = wx.state_build(eye=eye, target=target, aspect=1.0, fovy=75.0, width=64.0, mode=mode)
            rg, hg = gpu_render(cuda_ctx, grid, st, 64, 64)
            ro, ho = oracle_render(view, st, 64, 64)
            compare(rg, hg, ro, ho, label=f"eye{eye}/mode{mode}")


def test_nodes_beyond_the_bound(cuda_ctx):
    """N5 nodes outside [-4096, 4096)^3: the bounds test then runs on every step (it is skipped
    inside N5s only when all N5s lie in that box). Rays cross voxels on both sides of +-4096."""
    rng = np.random.default_rng(17)
    ijk = np.concatenate([rng.integers(4080, 4112, size=(3000, 3)), rng.integers(-4112, -4080, size=(3000, 3)),
                          rng.integers(5000, 5100, size=(500, 3))]).astype(np.int32)
    topo = wx.Topology.from_voxels(ijk)
    view = topo.view()
    grid = cuda_ctx.build_grid(topo)
    for eye, target in [((4000.0, 4000.0, 3950.0), (4100.0, 4100.0, 4100.0)),
                        ((4200.0, 4150.0, 4300.0), (4096.0, 4096.0, 4096.0)),
                        ((-4000.0, -4010.0, -3900.0), (-4100.0, -4100.0, -4100.0)),
                        ((4500.0, 4500.0, 4500.0), (5050.0, 5050.0, 5050.0))]:
        for mode in (0, 3):
            st = wx.state_build(eye=eye, target=target, aspect=1.0, fovy=70.0, width=64.0, mode=mode)
            rg, hg = gpu_render(cuda_ctx, grid, st, 64, 64)
            ro, ho = oracle_render(view, st, 64, 64)
            compare(rg, hg, ro, ho, label=f"beyond/{eye}/mode{mode}")
    grid.release()


def test_zero_direction_components(cuda_ctx, sphere64):
    """Rays with an exactly-zero direction component (1/dir = inf) take the NaN-aware step."""
    _, view, grid = sphere64
    w, h = 64, 64
    st = wx.state_build(eye=(0.5, 0.0, 150.0), target=(0, 0, 0), aspect=1.0, fovy=60.0, width=float(w), mode=3,
                        sun=((0.0, -1.0, 0.0), (1.0, 0.8, 0.6), 1.0))
    # Hand-made ray basis: dir = (x - 32, 0, -40) for every pixel, so dir.y == 0 exactly.
    for i in range(4):
        st.u[i], st.mv[i], st.wp[i] = (1.0, 0.0, 0.0, 0.0)[i], 0.0, (-32.0, 0.0, -40.0, 0.0)[i]
    for mode in (0, 3, 4):
        st.render_mode[0] = mode
        rg, hg = gpu_render(cuda_ctx, grid, st, w, h)
        ro, ho = oracle_render(view, st, w, h)
        compare(rg, hg, ro, ho, label=f"zero-dir/mode{mode}")
    assert (wx.hit_fields(hg)["state"] == 0).any()


def test_empty_grid(cuda_ctx):
    topo = wx.Topology.from_voxels(np.zeros((0, 3), np.int32))
    assert topo.counts == (0, 0, 0)
    grid = cuda_ctx.build_grid(topo)
    view = {"kids5": np.zeros(0, np.uint32), "vals5": np.zeros(0, np.uint32), "kids4": np.zeros(0, np.uint32),
            "vals4": np.zeros(0, np.uint32), "vals3": np.zeros(0, np.uint32), "origins": np.zeros((0, 4), np.int32),
            "atlas": [np.zeros(1, np.uint32)] * 3, "dims": [(0, 0, 0)] * 3}
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=1.0, fovy=60.0, width=32.0, mode=3)
    rg, hg = gpu_render(cuda_ctx, grid, st, 32, 32)
    ro, ho = oracle_render(view, st, 32, 32)
    compare(rg, hg, ro, ho, label="empty")
    assert (wx.hit_fields(hg)["state"] == 1).all()
