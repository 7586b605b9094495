"""The CUDA kernels against frames rendered by the reference's own raycast shader.

The frames of tests/golden/wgsl_raycast.npz come from src/shaders/raycast.comp.wgsl
(woxel) translated mechanically to C++ and run on the host (see test_wgsl_golden.py).
Here the product renders the same uniforms over the same grids, handed to it as the
reference's flattened view (masks, origins, atlases built by the oracle) through the
drop-in upload, with and without hit records, through every kernel (one pixel per
lane, persistent warps, lanes that refill, one batched launch and its CUDA-graph plan);
every RGBA8 byte must be equal. The bounds-checked build reruns this file
(tests/test_bounds_gpu.py). This includes the benchmark's first 1920x1080 frame of the
2000-sphere grid, which the fixture holds whole.
"""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import gpu_render
from test_wgsl_golden import FIXTURE, _make

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return np.load(FIXTURE)


@pytest.fixture(scope="module")
def grids(cuda_ctx, oracle_spheres_view):
    mk = _make()
    views = {g: (oracle_spheres_view if g == 1 else mk.grid_view(g)) for g in range(7)}
    return {g: cuda_ctx.upload_view(v) for g, v in views.items()}


def _check(golden, ctx, grids, hits):
    n = 0
    for i, (g, w, h, large) in enumerate(golden["meta"]):
        st = wx.state_from_bytes(bytes(golden[f"state_{i}"]))
        rgba, _ = gpu_render(ctx, grids[int(g)], st, int(w), int(h), hits=hits)
        want = golden[f"rgba_{i}"]
        bad = np.argwhere((rgba != want).any(axis=2))
        assert bad.size == 0, f"frame {i} (grid {g}, {w}x{h}): {len(bad)} pixels differ, first at {bad[:3].tolist()}"
        n += 1
    assert n == len(golden["meta"])


@pytest.mark.parametrize("kernel,rays", [(1, 1), (0, 1), (1, 2), (1, 4)])
def test_kernels_match_reference_shader(golden, cuda_ctx, grids, kernel, rays):
    """k_pixel, the persistent kernel, and k_wave's lane refill (2 and 4 rays per lane)."""
    old = cuda_ctx.tuning
    cuda_ctx.set_tuning(kernel=kernel, rays_per_lane=rays)
    try:
        _check(golden, cuda_ctx, grids, hits=False)
    finally:
        cuda_ctx.set_tuning(**old)


def test_kernels_with_hit_records_match_reference_shader(golden, cuda_ctx, grids):
    _check(golden, cuda_ctx, grids, hits=True)


def test_batched_launch_matches_reference_shader(golden, cuda_ctx, grids):
    """All 80 frames over the seven grids in one batched launch (the persistent kernel over
    a job table, the path of wx_batch_* plans and the server), and again as a CUDA-graph
    plan replayed twice."""
    import torch

    meta = golden["meta"]
    outs, frames = [], []
    for i, (g, w, h, large) in enumerate(meta):
        st = wx.state_from_bytes(bytes(golden[f"state_{i}"]))
        o = torch.zeros(int(w) * int(h) * 4, dtype=torch.uint8, device="cuda")
        outs.append(o)
        frames.append((grids[int(g)], st, int(w), int(h), o, None))
    stream = torch.cuda.current_stream().cuda_stream
    cuda_ctx.render_batch(frames, stream=stream)
    torch.cuda.synchronize()

    def check_all():
        for i, (g, w, h, large) in enumerate(meta):
            got = outs[i].cpu().numpy().reshape(int(h), int(w), 4)
            assert np.array_equal(got, golden[f"rgba_{i}"]), f"frame {i} (grid {g}, {w}x{h})"

    check_all()
    plan = cuda_ctx.batch(frames)
    for _ in range(2):
        for o in outs:
            o.zero_()
        plan.launch(stream=stream)
        torch.cuda.synchronize()
        check_all()
