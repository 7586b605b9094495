"""wx_render_batch_noalloc: batched rendering for callers that cannot allocate device memory.

Such callers (engines that reserve all GPU memory at start-up, code on a frame
deadline) get one entry point whose scratch is a fixed device array inside the
library. It must give the same frames as the context-based wx_render_batch
(bit-exact here, so within the parity tolerance of the other tests), on two
calls in a row: the second call reuses the array left by the first, so the
work-queue counter must be cleared by every call. This file is collected last
so that a run stopping at the first failure has already run every other test;
it also passes alone in a fresh process, where its first call does the
per-device set-up.
"""
import numpy as np
import pytest
import torch

import woxel_gb300 as wx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frames(cuda_ctx):
    rng = np.random.default_rng(5)
    grids = [cuda_ctx.build_grid(wx.Topology.sphere((0, 0, 0), 64.0, 3.0)),
             cuda_ctx.build_grid(wx.Topology.from_voxels(rng.integers(-250, 250, size=(3000, 3)).astype(np.int32)))]
    out = []
    for i, (w, h) in enumerate([(64, 48), (120, 64), (33, 17), (160, 120), (8, 4), (200, 52), (96, 96), (7, 3)]):
        eye = tuple(float(x) for x in rng.uniform(-400, 400, 3))
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=w / h, fovy=65.0, width=float(w), mode=[3, 0, 1, 4][i % 4])
        out.append((grids[i % 2], st, w, h))
    return out


def buffers(frames):
    return [(torch.zeros(w * h * 4 + 4, dtype=torch.uint8, device="cuda"),
             torch.zeros(w * h * 32 + 32, dtype=torch.uint8, device="cuda")) for _, _, w, h in frames]


def host(bufs):
    return [(r.cpu().numpy(), h.cpu().numpy()) for r, h in bufs]


def test_noalloc_matches_context_batch_on_two_calls(cuda_ctx, frames):
    stream = torch.cuda.current_stream().cuda_stream
    ref = buffers(frames)
    cuda_ctx.render_batch([(g, st, w, h, r, hb) for (g, st, w, h), (r, hb) in zip(frames, ref)], stream=stream)
    torch.cuda.synchronize()
    expect = host(ref)
    got = buffers(frames)
    for call in range(2):
        for r, hb in got:
            r.zero_()
            hb.zero_()
        wx.render_batch_noalloc([(g, st, w, h, r, hb) for (g, st, w, h), (r, hb) in zip(frames, got)], stream=stream)
        torch.cuda.synchronize()
        for k, ((e_r, e_h), (g_r, g_h)) in enumerate(zip(expect, host(got))):
            np.testing.assert_array_equal(g_r, e_r, err_msg=f"call {call} frame {k} rgba")
            np.testing.assert_array_equal(g_h, e_h, err_msg=f"call {call} frame {k} hits")


def test_noalloc_rejects_more_than_the_maximum(frames):
    g, st, w, h = frames[0]
    r = torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda")
    too_many = [(g, st, w, h, r, None)] * (wx.NOALLOC_MAX_FRAMES + 1)
    with pytest.raises(wx.WxError, match="256"):
        wx.render_batch_noalloc(too_many)


def test_noalloc_calls_queued_back_to_back(cuda_ctx, frames):
    """Two calls on one stream with different frames and outputs, the second enqueued before the
    first has run: each call keeps its own frame table (it travels in the table kernels'
    launch parameters), so both match the context-based batch."""
    stream = torch.cuda.current_stream().cuda_stream
    first, second = frames[:5], frames[3:]
    expect = []
    for part in (first, second):
        ref = buffers(part)
        cuda_ctx.render_batch([(g, st, w, h, r, hb) for (g, st, w, h), (r, hb) in zip(part, ref)], stream=stream)
        torch.cuda.synchronize()
        expect.append(host(ref))
    got = [buffers(first), buffers(second)]
    torch.cuda._sleep(20_000_000)  # keep the GPU busy so that both calls are queued before either runs
    for part, bufs in zip((first, second), got):
        wx.render_batch_noalloc([(g, st, w, h, r, hb) for (g, st, w, h), (r, hb) in zip(part, bufs)], stream=stream)
    torch.cuda.synchronize()
    for p, (exp, bufs) in enumerate(zip(expect, got)):
        for k, ((e_r, e_h), (g_r, g_h)) in enumerate(zip(exp, host(bufs))):
            np.testing.assert_array_equal(g_r, e_r, err_msg=f"call {p} frame {k} rgba")
            np.testing.assert_array_equal(g_h, e_h, err_msg=f"call {p} frame {k} hits")


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs a second GPU for a stream of another device")
def test_noalloc_rejects_a_stream_of_another_device(frames):
    g, st, w, h = frames[0]
    r = torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda:0")
    with torch.cuda.device(1):
        other = torch.cuda.Stream(device=1)
    with pytest.raises(wx.WxError, match="another device"):
        wx.render_batch_noalloc([(g, st, w, h, r, None)], stream=other.cuda_stream)
