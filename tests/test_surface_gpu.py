"""Zero-crossing hit mode (render mode 5) on the GPU against the oracle's specification:
RGBA8 and hit records bit for bit, including the crossing's t and sample index."""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, gpu_render, oracle_render, oracle_view
from woxel_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def compare_surface(rg, hg, ro, ho, label, where=None):
    compare(rg, hg, ro, ho, where=where, label=label)
    a, b = hg["reserved"], ho["reserved"]
    if where is not None:
        a, b = a[where], b[where]
    np.testing.assert_array_equal(a, b, err_msg=f"{label}: crossing t bits")


@pytest.fixture(scope="module")
def sphere_surface(cuda_ctx):
    """The r=64 sphere: the oracle's view and values built by the oracle alone; the GPU grid
    and values by the product."""
    import oracle as orc

    topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    view = orc.workload_view("sphere", values=True)
    grid = cuda_ctx.build_grid(topo)
    grid.set_values(W.sphere_values(topo), 3.0)
    return view, grid


@pytest.mark.parametrize("kernel", [0, 1])
def test_sphere_surface_matches_oracle(cuda_ctx, sphere_surface, kernel):
    view, grid = sphere_surface
    before = cuda_ctx.tuning
    cuda_ctx.set_tuning(kernel=kernel)
    try:
        for eye in [(0.0, 0.0, 200.0), (30.0, 50.0, 200.0), (-150.0, 20.0, -90.0), (64.5, 0.5, 0.5)]:
            st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=320.0, mode=5)
            rg, hg = gpu_render(cuda_ctx, grid, st, 320, 240)
            ro, ho = oracle_render(view, st, 320, 240)
            compare_surface(rg, hg, ro, ho, f"surface eye={eye}")
        assert ((hg["shadow"] & 1) == 1).any() or eye == (64.5, 0.5, 0.5)
    finally:
        cuda_ctx.set_tuning(**before)


def test_grid_without_values(cuda_ctx):
    topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    view = oracle_view(topo)
    grid = cuda_ctx.build_grid(topo)
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=1.0, fovy=40.0, width=64.0, mode=5)
    rg, hg = gpu_render(cuda_ctx, grid, st, 64, 64)
    ro, ho = oracle_render(view, st, 64, 64)
    compare_surface(rg, hg, ro, ho, "no values")
    assert np.isnan(hg["reserved"].view(np.float32)).all()


def test_spheres_1080p_surface_sampled_tiles(cuda_ctx, oracle_spheres_view):
    """The 2000-sphere grid with its level-set values, 1080p, 800 random tiles per frame. The
    oracle's view, values and uniforms are its own (restated generators, compute_sdf,
    atlas(), ComputeState::build); the GPU's are the product's."""
    import oracle as orc

    topo = W.spheres_topology()
    view = oracle_spheres_view
    grid = cuda_ctx.build_grid(topo)
    grid.set_values(W.spheres_values(topo), 3.0)
    for k, (f, (_, _, osb)) in enumerate(zip(W.spheres_frames()[:2], orc.workload_frames("spheres")[:2])):
        st = f.state()
        st.render_mode[0] = 5
        ob = bytearray(osb)
        ob[192:196] = (5).to_bytes(4, "little")  # render_mode, after two matrices and four vec4s
        assert bytes(ob) == wx.state_bytes(st)
        rg, hg = gpu_render(cuda_ctx, grid, st, f.width, f.height)
        rng = np.random.default_rng(k)
        tiles = np.sort(rng.choice((f.width // 8) * (f.height // 4), 800, replace=False)).astype(np.uint64)
        ro, ho, _ = orc.render(view, bytes(ob), f.width, f.height, nthreads=16, hits=True, tiles=tiles)
        m = np.zeros((f.height, f.width), bool)
        for t in tiles:
            x0, y0 = (int(t) % (f.width // 8)) * 8, (int(t) // (f.width // 8)) * 4
            m[y0:y0 + 4, x0:x0 + 8] = True
        compare_surface(rg, hg, ro, ho, f"spheres surface frame {k}", where=m)
        assert ((hg["shadow"][m] & 1) == 1).sum() > 1000


@pytest.mark.parametrize("name", ["cube", "icosahedron"])
def test_fixture_level_sets(cuda_ctx, name):
    """The reference's own level sets with the values its files store (tests/golden)."""
    from pathlib import Path

    golden = Path(__file__).resolve().parent / "golden"
    d = np.load(golden / f"{name}_topology.npz")
    m = {k: d[k] for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")}
    vd = np.load(golden / f"{name}_values.npz")
    vals, bg = vd["values"].astype(np.float32), float(vd["background"])
    topo = wx.Topology.from_masks(m)
    view = oracle_view(topo)
    view["values"], view["band"] = vals, bg
    grid = cuda_ctx.build_grid(topo, gpu=True)
    grid.set_values(vals, bg)
    for eye in [(0.5, 0.5, 260.0), (180.0, 150.0, 240.0), (-230.0, -90.0, -170.0)]:
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=4 / 3, fovy=50.0, width=128.0, mode=5)
        rg, hg = gpu_render(cuda_ctx, grid, st, 128, 96)
        ro, ho = oracle_render(view, st, 128, 96)
        compare_surface(rg, hg, ro, ho, f"{name} surface eye={eye}")
        assert ((hg["shadow"] & 1) == 1).sum() > 500
