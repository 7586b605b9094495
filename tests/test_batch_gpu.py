"""Batched rendering: many frames over several resident grids in one persistent launch.

Each frame of a batch must equal the same frame rendered alone (wx_render) bit for bit,
and the oracle within the parity tolerance; the CUDA-graph plan must replay identically.
"""
import numpy as np
import pytest
import torch

import woxel_gb300 as wx
from parity import compare, dispatch_mask, gpu_render, oracle_render, oracle_view

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(cuda_ctx):
    rng = np.random.default_rng(21)
    t1 = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    t2 = wx.Topology.from_voxels(rng.integers(-300, 300, size=(4000, 3)).astype(np.int32))
    views = [oracle_view(t1), oracle_view(t2)]
    grids = [cuda_ctx.build_grid(t1), cuda_ctx.build_grid(t2)]
    frames = []
    sizes = [(64, 48), (120, 64), (96, 96), (33, 17), (160, 120), (8, 4), (7, 3), (200, 52)]
    for i in range(24):
        gi = i % 2
        w, h = sizes[i % len(sizes)]
        eye = tuple(float(x) for x in rng.uniform(-450, 450, 3))
        mode = [3, 0, 1, 2, 3, 4][i % 6]
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=max(w, 1) / max(h, 1), fovy=65.0, width=float(w),
                            mode=mode)
        frames.append((gi, st, w, h))
    return views, grids, frames


def alloc(frames):
    outs = []
    for gi, st, w, h in frames:
        outs.append((torch.zeros(max(w * h * 4, 4), dtype=torch.uint8, device="cuda"),
                     torch.zeros(max(w * h * 32, 32), dtype=torch.uint8, device="cuda")))
    return outs


def fetch(out, w, h):
    r, hb = out
    return (r.cpu().numpy()[: w * h * 4].reshape(h, w, 4),
            hb.cpu().numpy()[: w * h * 32].view(wx.HIT_DTYPE).reshape(h, w))


def test_batch_equals_single_frames_and_oracle(cuda_ctx, scene):
    views, grids, frames = scene
    outs = alloc(frames)
    cuda_ctx.render_batch([(grids[gi], st, w, h, o[0], o[1]) for (gi, st, w, h), o in zip(frames, outs)],
                          stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for k, ((gi, st, w, h), o) in enumerate(zip(frames, outs)):
        rb, hb = fetch(o, w, h)
        rs, hs = gpu_render(cuda_ctx, grids[gi], st, w, h)
        m = dispatch_mask(w, h)
        np.testing.assert_array_equal(rb[m], rs[m], err_msg=f"frame {k} rgba")
        np.testing.assert_array_equal(hb[m].view(np.uint8), hs[m].view(np.uint8), err_msg=f"frame {k} hits")
        if m.any():
            ro, ho = oracle_render(views[gi], st, w, h)
            compare(rb, hb, ro, ho, where=m, label=f"batch frame {k}")


def test_batch_graph_plan_replays(cuda_ctx, scene):
    views, grids, frames = scene
    outs = alloc(frames)
    plan = cuda_ctx.batch([(grids[gi], st, w, h, o[0], o[1]) for (gi, st, w, h), o in zip(frames, outs)])
    info = plan.info
    assert info["frames"] == sum(1 for _, _, w, h in frames if (w // 8) * (h // 4) > 0)
    stream = torch.cuda.current_stream().cuda_stream
    plan.launch(stream)
    torch.cuda.synchronize()
    first = [fetch(o, w, h) for (gi, st, w, h), o in zip(frames, outs)]
    for o in outs:
        o[0].zero_()
        o[1].zero_()
    plan.launch(stream)
    plan.launch(stream)
    torch.cuda.synchronize()
    for k, ((gi, st, w, h), o) in enumerate(zip(frames, outs)):
        r, hh = fetch(o, w, h)
        np.testing.assert_array_equal(r, first[k][0])
        np.testing.assert_array_equal(hh.view(np.uint8), first[k][1].view(np.uint8))
    plan.close()


def test_autotune_installs_a_candidate_and_keeps_results(cuda_ctx, scene):
    views, grids, frames = scene
    before = cuda_ctx.tuning
    big = [f for f in frames if f[2] * f[3] >= 96 * 96]
    outs = alloc(big)
    res = cuda_ctx.autotune([(grids[gi], st, w, h, o[0], None) for (gi, st, w, h), o in zip(big, outs)],
                            candidates=[dict(kernel=0, tile_width=8), dict(kernel=1, tile_width=16, warps_per_block=2),
                                        dict(kernel=0, tile_width=4, warps_per_block=8)], reps=1)
    assert res["best"] == cuda_ctx.tuning and len(res["table"]) == 3 and all(ms > 0 for _, ms in res["table"])
    gi, st, w, h = big[0]
    rg, hg = gpu_render(cuda_ctx, grids[gi], st, w, h)
    ro, ho = oracle_render(views[gi], st, w, h)
    compare(rg, hg, ro, ho, label="after autotune")
    cuda_ctx.set_tuning(**before)


def test_batch_rejects_host_outputs(cuda_ctx, scene):
    _, grids, frames = scene
    gi, st, w, h = frames[0]
    host = np.zeros(w * h * 4, np.uint8)
    with pytest.raises(wx.WxError):
        cuda_ctx.render_batch([(grids[gi], st, w, h, host, None)])
