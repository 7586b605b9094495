"""Zero-crossing hit mode (render mode 5, an extension with no reference counterpart): the
oracle's specification against ground truth, and the level-set value generators against the
activity masks they must agree with. CPU only."""
import numpy as np

import oracle as orc
import woxel_gb300 as wx


def sphere_view():
    """The r=64 sphere as the oracle builds it alone: its generator, compute_sdf, atlas()
    and level-set values."""
    return wx.Topology.sphere((0, 0, 0), 64.0, 3.0), orc.workload_view("sphere", values=True)


def test_values_agree_with_activity():
    """A leaf voxel is active exactly where |value| < band (the generators' rule)."""
    one = wx.Topology.sphere((5, -7, 3), 30.0, 3.0)
    many = wx.Topology.spheres(60, 4.0, 20.0, -200.0, 200.0, 3.0, 9)
    for topo, vals in [(one, one.sphere_values((5, -7, 3), 30.0, 3.0)),
                       (many, many.spheres_values(60, 4.0, 20.0, -200.0, 200.0, 3.0, 9))]:
        words = topo.masks()["vals3"].reshape(-1, 16)
        bits = np.unpackbits(words.view(np.uint8), bitorder="little").reshape(-1, 512).astype(bool)
        v = vals.reshape(-1, 512)
        assert (np.abs(v) <= 3.0).all()
        np.testing.assert_array_equal(bits, np.abs(v) < 3.0)


def test_crossing_matches_the_analytic_sphere():
    """t* of the oracle's zero-crossing search lies within 0.05 voxel of the exact ray-sphere
    intersection (trilinear interpolation of a sampled distance field)."""
    _, view = sphere_view()
    eye = np.array([30.0, 50.0, 200.0])
    st = wx.state_build(eye=tuple(eye), target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=160.0, mode=5)
    rgba, hits, _ = orc.render(view, wx.state_bytes(st), 160, 120, nthreads=8, hits=True)
    f = wx.hit_fields(hits)
    found = (hits["shadow"] & 1) == 1
    ts = hits["reserved"].view(np.float32)
    assert found.sum() > 3000 and (f["state"][found] == 0).all()
    assert np.isnan(ts[~found]).all()
    d = hits["p"].astype(np.float64) - eye
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    b = (d * eye).sum(-1)
    disc = b * b - ((eye * eye).sum() - 64.0 ** 2)
    m = found & (disc > 0)
    err = np.abs(ts[m] - (-b[m] - np.sqrt(disc[m])))
    assert err.max() < 0.05, err.max()
    # The crossing lies beyond the HDDA's first active voxel (within its 1-voxel back-off).
    assert (ts[found] >= hits["t"][found] - 1.0).all()


def test_without_values_no_crossing_is_found():
    view = orc.workload_view("sphere")
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=1.0, fovy=40.0, width=64.0, mode=5)
    rgba, hits, _ = orc.render(view, wx.state_bytes(st), 64, 64, nthreads=4, hits=True)
    assert ((hits["shadow"] & 1) == 0).all()
    assert np.isnan(hits["reserved"].view(np.float32)).all()
    st0 = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=1.0, fovy=40.0, width=64.0, mode=0)
    rgba0, _, _ = orc.render(view, wx.state_bytes(st0), 64, 64, nthreads=4, hits=True)
    np.testing.assert_array_equal(rgba, rgba0)  # mode 0's colour where no crossing is found


def test_crossings_on_the_cube_fixture():
    """The reference's cube level set with its own values: crossings are found for almost all HDDA
    hits, a little beyond them (the band is 3 voxels wide), with axis-aligned normals on the faces."""
    from pathlib import Path

    golden = Path(__file__).resolve().parent / "golden"
    d = np.load(golden / "cube_topology.npz")
    m = {k: d[k] for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")}
    vd = np.load(golden / "cube_values.npz")
    view = orc.Tree.from_masks(m).view()
    view["values"], view["band"] = vd["values"].astype(np.float32), float(vd["background"])
    st = wx.state_build(eye=(0.5, 0.5, 260.0), target=(0, 0, 0), aspect=1.0, fovy=40.0, width=96.0, mode=5)
    rgba, hits, _ = orc.render(view, wx.state_bytes(st), 96, 96, nthreads=8, hits=True)
    f = wx.hit_fields(hits)
    hit = f["state"] == 0
    found = (hits["shadow"] & 1) == 1
    assert hit.sum() > 1000 and found[hit].mean() > 0.95
    ts = hits["reserved"].view(np.float32)
    dt = ts[found] - hits["t"][found]
    assert (dt >= -1.0).all() and (dt < 8.0).all()
