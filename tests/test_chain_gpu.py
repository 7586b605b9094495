"""Back-to-back k_pixel frames on one stream (programmatic dependent launches).

A frame may start while earlier frames on its stream finish. Its blocks write
without waiting for the previous kernel only when every earlier frame whose
outputs overlap theirs has finished. These tests queue 1080p frames of the
2000-sphere grid without synchronising, into output layouts that do and do not
overlap, from one and from two contexts and streams, and compare every buffer
with the frames rendered one at a time.
"""
import numpy as np
import pytest
import torch

import woxel_gb300 as wx
from woxel_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NPIX = 1920 * 1080


@pytest.fixture(scope="module", params=[1, 4], ids=["rays1", "rays4"])
def scene(cuda_ctx, request):
    """The frames and their references; every test runs with one ray per lane (k_pixel) and with
    four (lanes that refill)."""
    grid = cuda_ctx.build_grid(W.spheres_topology())
    frames = W.spheres_frames()[:8]
    states = [f.state() for f in frames]
    before = cuda_ctx.tuning
    refs = []
    for st in states:  # one at a time, synchronised
        o = torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda")
        h = torch.zeros(NPIX * 32, dtype=torch.uint8, device="cuda")
        cuda_ctx.render(grid, st, 1920, 1080, o, h)
        torch.cuda.synchronize()
        refs.append((o.cpu().numpy(), h.cpu().numpy()))
    cuda_ctx.set_tuning(kernel=1, tile_width=4, warps_per_block=4, rays_per_lane=request.param)
    yield grid, states, refs
    cuda_ctx.set_tuning(**before)


def test_disjoint_outputs_rotating(cuda_ctx, scene):
    """As the benchmark: frames into rotating buffers, three rounds, hit records included."""
    grid, states, refs = scene
    outs = [torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda") for _ in states]
    hits = [torch.zeros(NPIX * 32, dtype=torch.uint8, device="cuda") for _ in states]
    for _ in range(3):
        for st, o, h in zip(states, outs, hits):
            cuda_ctx.render(grid, st, 1920, 1080, o, h)
    torch.cuda.synchronize()
    for k, (o, h) in enumerate(zip(outs, hits)):
        np.testing.assert_array_equal(o.cpu().numpy(), refs[k][0], err_msg=f"frame {k}")
        np.testing.assert_array_equal(h.cpu().numpy(), refs[k][1], err_msg=f"frame {k} hits")


def test_one_buffer_and_alternating_buffers(cuda_ctx, scene):
    grid, states, refs = scene
    one = torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda")
    ab = [torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
    for r in range(2):
        for k, st in enumerate(states):
            cuda_ctx.render(grid, st, 1920, 1080, one, None)
            cuda_ctx.render(grid, st, 1920, 1080, ab[k % 2], None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(one.cpu().numpy(), refs[-1][0])
    np.testing.assert_array_equal(ab[0].cpu().numpy(), refs[-2][0])
    np.testing.assert_array_equal(ab[1].cpu().numpy(), refs[-1][0])


def test_partly_overlapping_outputs(cuda_ctx, scene):
    """Frame k writes at byte offset (k % 4) half frames into a buffer 2.5 frames long, so that it
    overlaps half of the frame before it. Expected: the frames' writes applied in order."""
    grid, states, refs = scene
    step = NPIX // 2 * 4  # bytes
    buf = torch.zeros(step * 5, dtype=torch.uint8, device="cuda")
    want = np.zeros(step * 5, np.uint8)
    for k, st in enumerate(states * 2):
        off = (k % 4) * step
        view = buf[off:off + NPIX * 4]
        cuda_ctx.render(grid, st, 1920, 1080, view, None)
        want[off:off + NPIX * 4] = refs[k % len(states)][0]
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy(), want)


def test_colour_of_one_frame_over_hit_records_of_the_last(cuda_ctx, scene):
    """Frames alternate between two layouts in one buffer, so that each frame's RGBA8
    and hit records land on the previous frame's hit records. Expected: the writes applied
    in order."""
    grid, states, refs = scene
    n4, n32 = NPIX * 4, NPIX * 32
    buf = torch.zeros(n4 + n4 + n32, dtype=torch.uint8, device="cuda")
    want = np.zeros(n4 + n4 + n32, np.uint8)
    layouts = [(0, n4), (n4, n4 + n4)]  # (rgba offset, hits offset)
    for k, st in enumerate(states):
        ro, ho = layouts[k % 2]
        cuda_ctx.render(grid, st, 1920, 1080, buf[ro:ro + n4], buf[ho:ho + n32])
        want[ro:ro + n4] = refs[k][0]
        want[ho:ho + n32] = refs[k][1]
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy(), want)


def test_two_contexts_on_one_stream(cuda_ctx, scene):
    grid, states, refs = scene
    other = wx.Context(0)
    other.set_tuning(**cuda_ctx.tuning)
    grid2 = other.build_grid(W.spheres_topology())
    torch.cuda.synchronize()
    buf = torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda")
    side = [torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
    for k, st in enumerate(states):
        cuda_ctx.render(grid, st, 1920, 1080, side[k % 2], None)
        (cuda_ctx if k % 2 else other).render(grid if k % 2 else grid2, st, 1920, 1080, buf, None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy(), refs[-1][0])
    np.testing.assert_array_equal(side[0].cpu().numpy(), refs[-2][0])
    np.testing.assert_array_equal(side[1].cpu().numpy(), refs[-1][0])
    grid2.release()
    other.close()


def test_two_streams_and_kernel_switches(cuda_ctx, scene):
    """Frames on two streams at once, and the tile-queue kernel between k_pixel frames."""
    grid, states, refs = scene
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    a = [torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
    b = torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda")
    for k, st in enumerate(states):
        cuda_ctx.set_tuning(kernel=1 if k % 3 else 0)
        cuda_ctx.render(grid, st, 1920, 1080, a[k % 2], None, stream=s1.cuda_stream)
        cuda_ctx.set_tuning(kernel=1)
        cuda_ctx.render(grid, st, 1920, 1080, b, None, stream=s2.cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a[0].cpu().numpy(), refs[-2][0])
    np.testing.assert_array_equal(a[1].cpu().numpy(), refs[-1][0])
    np.testing.assert_array_equal(b.cpu().numpy(), refs[-1][0])


def test_two_threads_on_the_per_thread_default_stream(cuda_ctx, scene):
    """Two host threads, each with its own context, render on cudaStreamPerThread: one handle
    value that names a different stream in every thread. Each thread writes all frames into
    one buffer of its own, so every frame must wait for the one before it on its thread's
    stream; the record of one thread's last frame must never let the other thread's frames skip
    that wait. Repeated rounds; each buffer ends as the last frame."""
    import threading

    grid, states, refs = scene
    per_thread = 2  # cudaStreamPerThread
    ctxs = [wx.Context(0) for _ in range(2)]
    for c in ctxs:
        c.set_tuning(**cuda_ctx.tuning)
    bufs = [torch.zeros(NPIX * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    start = threading.Barrier(2)
    errors = []

    def work(i):
        try:
            start.wait()
            for _ in range(4):
                for st in states:
                    ctxs[i].render(grid, st, 1920, 1080, bufs[i], None, stream=per_thread)
            torch.cuda.synchronize()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    torch.cuda.synchronize()
    for i, b in enumerate(bufs):
        np.testing.assert_array_equal(b.cpu().numpy(), refs[-1][0], err_msg=f"thread {i}")
    for c in ctxs:
        c.close()
