"""GPU kernels against the frozen golden renders of woxel's level-set fixtures."""
from pathlib import Path

import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, gpu_render

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
MASK_KEYS = ("kids5", "vals5", "kids4", "vals4", "vals3", "origins")


@pytest.mark.parametrize("name", ["cube", "icosahedron", "sphere64"])
@pytest.mark.parametrize("kernel", [0, 1])
def test_gpu_matches_golden(cuda_ctx, name, kernel):
    if name == "sphere64":
        topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    else:
        d = np.load(GOLDEN / f"{name}_topology.npz")
        topo = wx.Topology.from_masks({k: d[k] for k in MASK_KEYS})
    grid = cuda_ctx.build_grid(topo)
    before = cuda_ctx.tuning
    cuda_ctx.set_tuning(kernel=kernel)
    try:
        g = np.load(GOLDEN / f"{name}_render.npz")
        k = 0
        while f"state{k}" in g:
            w, h = (int(x) for x in g[f"size{k}"])
            st = wx.state_from_bytes(g[f"state{k}"].tobytes())
            rg, hg = gpu_render(cuda_ctx, grid, st, w, h)
            ho = g[f"hits{k}"].reshape(h, w * 32).view(wx.HIT_DTYPE).reshape(h, w)
            compare(rg, hg, g[f"rgba{k}"], ho, label=f"{name}/{k}")
            k += 1
    finally:
        cuda_ctx.set_tuning(**before)
