"""Benchmark: primary-ray Grays/s of the raycast pass on one GB300.

Default workload (one "step"): the 2000-sphere narrow-band grid (1.0 GB of
node pools, resident in HBM) rendered from 16 orbit cameras at 1920x1080 in
Lambert mode (primary + shadow rays), one plain per-frame launch per camera.
value = primary rays / device time; e2e = the same through wx_render with
host output buffers (device->host copy of every frame inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm's CPU implementation (the C
restatement of raycast.comp.wgsl in oracle/, all host threads) on a bounded
sample of the same frames; the reference itself (Rust + wgpu) cannot run here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MEASURED = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def hbm_peak():
    try:
        d = json.loads(MEASURED.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def l2_copy_peak(dev, mib: int = 32, reps: int = 300) -> float:
    """L2 bandwidth measured here: GB/s of back-to-back device copies between two buffers
    that together fit in L2 (2 x 32 MiB of the 129 MB)."""
    import torch

    a = torch.ones(mib << 18, dtype=torch.float32, device=dev)
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    return 2 * a.numel() * 4 * reps / (e0.elapsed_time(e1) / 1e3) / 1e9


def max_over_ranks(ms: float, dist=None, device=None) -> float:
    """The slowest rank's step time (every rank gets it); ms itself without a process group."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(rays_per_rank: int, world: int, ms: float) -> float:
    """Whole-job Grays/s of `world` replicas that each trace rays_per_rank rays in ms (weak scaling)."""
    return world * rays_per_rank / (ms / 1e3) / 1e9


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
# capture of the benchmark's kernel on each workload, with the commit it was taken on.
# Reported as roofline.traffic_from_profile: a recorded capture, not a figure of this run.
NCU_TRAFFIC = {
    ("k_pixel", "spheres"): (142257408, "5c05830"),
}


class ClockSampler:
    """SM clock and throttle-reason samples during the timed region, from two sources:
    `nvidia-smi -lms 200` (the process is started, and its first sample awaited, before
    the region begins) and NVML itself, polled every 10 ms from a thread through ctypes
    (libnvidia-ml: nvmlDeviceGetClockInfo / nvmlDeviceGetCurrentClocksEventReasons, read
    only), which gives tens of samples even in a sub-second region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason bits (nvml.h)
    NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                    0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int, period_s: float = 0.01):
        self.device = device
        self.period = period_s
        self.proc = None
        self.lines = []
        self.first = threading.Event()
        self.nv = []          # (sm MHz, reason bits)
        self.nv_max = None
        self.stop = threading.Event()
        self.nt = None
        self.sample = None
        self.nvml_shutdown = None
        self.bracket = []     # one sample just before and one just after the region

    def _nvml_index(self) -> int:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if ids and all(v.isdigit() for v in ids) and self.device < len(ids):
            return int(ids[self.device])
        return self.device

    def _nvml_start(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return
        h = C.c_void_p()
        if lib.nvmlInit_v2() != 0 or lib.nvmlDeviceGetHandleByIndex_v2(self._nvml_index(), C.byref(h)) != 0:
            return
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
        mx = C.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.nv_max = float(mx.value)

        def sample():
            clk, rs = C.c_uint(), C.c_ulonglong()
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) != 0:
                return None
            bits = rs.value if get_reasons is not None and get_reasons(h, C.byref(rs)) == 0 else 0
            return float(clk.value), int(bits)

        def poll():
            while not self.stop.is_set():
                v = sample()
                if v is not None:
                    self.nv.append(v)
                self.stop.wait(self.period)

        self.sample = sample
        self.nvml_shutdown = lib.nvmlShutdown
        self.nt = threading.Thread(target=poll, daemon=True)
        self.nt.start()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self._nvml_index()), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(5.0)
        except FileNotFoundError:
            self.proc = None
        self._nvml_start()
        if self.nt is not None:
            t0 = time.time()
            while not self.nv and time.time() - t0 < 1.0:
                time.sleep(0.001)
            del self.nv[:]   # samples from the timed region only
        if self.sample is not None:
            self.bracket.append(self.sample())
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()

    def __exit__(self, *exc):
        if self.sample is not None:
            self.bracket.append(self.sample())
        self.stop.set()
        if self.nt is not None:
            self.nt.join(timeout=2)
            self.nvml_shutdown()  # balances this sampler's nvmlInit_v2
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
               "samples": len(sm), "source": "nvidia-smi -lms 200"}
        nv = self.nv
        src = "NVML every 10 ms; nvidia-smi -lms 200"
        if not nv:  # a region shorter than the sampling period
            nv = [b for b in self.bracket if b is not None]
            src = "NVML just before and just after the timed region (shorter than 10 ms)"
        if nv:
            nv_sm = [c for c, _ in nv]
            for _, bits in nv:
                reasons.update(n for b, n in self.NVML_REASONS.items() if bits & b)
            out.update({"sm_mhz": statistics.median(nv_sm), "sm_min_mhz": min(nv_sm),
                        "sm_max_mhz": self.nv_max if self.nv_max is not None else smax,
                        "reasons": sorted(reasons), "samples": len(nv_sm),
                        "source": src,
                        "nvidia_smi": {"sm_mhz": out["sm_mhz"], "samples": len(sm)}})
        return out


# --------------------------------------------------------------------------
# CPU side: the oracle (restated reference algorithm) on tiles of the same frames.
# --------------------------------------------------------------------------
def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    return orc


def tile_chunks(width: int, height: int, parts: int, seed: int) -> list:
    """The 8x4 tiles of a frame in a seeded random order, split into `parts` chunks of equal
    size (to one tile): chunk k of every frame is one step's sample, and `parts` consecutive
    steps cover every tile once."""
    n = (width // 8) * (height // 4)
    perm = np.random.default_rng(seed).permutation(n)
    return [np.sort(c) for c in np.array_split(perm, parts)]


def oracle_sample(view, frames, chunk, parts, nthreads, seed=5, stats=False):
    """Render chunk `chunk` of `parts` (tile_chunks) of every frame [(width, height, uniform
    bytes)] on the CPU oracle.

    Returns (rays, seconds, mean node-visit bytes per primary ray incl. its shadow ray, grazing
    fraction of the primary rays); the last two only with stats=True."""
    import ctypes as C

    orc = _oracle()
    L = orc.lib()
    s, keep = orc._view_struct(view)
    rays, secs, byte_sum, grazing = 0, 0.0, 0.0, 0
    for i, (w, h, sb_bytes) in enumerate(frames):
        sb = C.create_string_buffer(sb_bytes, 256)
        tiles = tile_chunks(w, h, parts, seed + i)[chunk % parts]
        rgba = np.zeros((h, w, 4), np.uint8)
        stt = np.zeros((h, w), orc.STATS_DTYPE) if stats else None
        tl = np.ascontiguousarray(tiles, np.uint64)
        t0 = time.perf_counter()
        rc = L.orc_render_tile_list(C.byref(s), sb, w, h, tl.ctypes.data, tl.size, rgba.ctypes.data,
                                    None, None if stt is None else stt.ctypes.data, nthreads)
        secs += time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError("oracle tile list out of range")
        rays += len(tiles) * 32
        if stats:
            m = np.zeros((h // 4, w // 8), bool)
            m.ravel()[tiles] = True
            m = np.repeat(np.repeat(m, 4, axis=0), 8, axis=1)
            m = np.pad(m, ((0, h - m.shape[0]), (0, w - m.shape[1])))
            byte_sum += float(stt["bytes"][m].sum() + stt["shadow_bytes"][m].sum())
            grazing += int(stt["grazing"][m].sum())
    del keep
    return rays, secs, (byte_sum / rays if stats else None), (grazing / rays if stats else None)


def active_voxels(view) -> int:
    """Active voxels of a view without active tiles: set bits of the leaf value masks."""
    return int(np.unpackbits(np.ascontiguousarray(view["vals3"], np.uint32).view(np.uint8)).sum())


def workload_config(name: str, counts, voxels: int, frames) -> dict:
    """`config` of both arms: the workload, its grid and its frames [(width, height, ...)]."""
    w, h = frames[0][0], frames[0][1]
    mode = {"sphere": 3, "spheres": 3, "noise": 0}[name]
    return {"workload": f"{name}: {len(frames)} x {w}x{h} frames, one plain per-frame raycast pass each",
            "grid": {"n5": int(counts[0]), "n4": int(counts[1]), "n3": int(counts[2]), "active_voxels": int(voxels)},
            "frames": len(frames), "resolution": f"{w}x{h}", "render_mode": mode}


def run_reference(args, wl_name):
    """--impl reference: the reference algorithm on the host cores (rank 0 only), built from
    the oracle alone: the oracle's restated generator makes the grid through set_voxel, its
    compute_sdf and atlas() flatten it, its ComputeState::build makes the uniforms, and its
    restatement of raycast.comp.wgsl renders. No product code is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    orc = _oracle()
    t0 = time.perf_counter()
    view = orc.workload_view(wl_name)
    t_view = time.perf_counter() - t0
    frames = orc.workload_frames(wl_name)
    counts = (view["kids5"].size // 1024, view["kids4"].size // 128, view["vals3"].size // 16)
    nthreads = os.cpu_count() or 1
    parts = max(1, int(round(1.0 / args.cpu_fraction)))
    log(f"[reference] {wl_name}: grid {counts} built by the oracle in {t_view:.1f}s; {nthreads} threads")
    for k in range(max(0, min(args.warmup, 1))):  # one warm-up step
        oracle_sample(view, frames, k, parts * 4, nthreads, seed=99)
    times, rays_tot = [], 0
    for k in range(args.steps):
        rays, secs, _, _ = oracle_sample(view, frames, k, parts, nthreads, seed=100)
        times.append(secs)
        rays_tot += rays
    total = sum(times)
    value = rays_tot / total / 1e9
    sample = (f"step k renders chunk k mod {parts} of a seeded split of each frame's 8x4 tiles into {parts} "
              f"(every {parts} steps cover every tile of the {len(frames)} frames once); C restatement of "
              f"raycast.comp.wgsl (oracle/), {nthreads} threads")
    line = {
        "impl": "reference", "metric": "primary_ray_grays_per_s", "value": value, "unit": "Grays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(wl_name, counts, active_voxels(view), frames),
        "arm": {"parallelism": f"cpu-threads x{nthreads}", "grid_build_s": round(t_view, 2),
                "grid_build": "oracle: restated generator + set_voxel, compute_sdf, masks(), atlas()",
                "rays_per_step": rays_tot // max(1, args.steps)},
        "cpu_baseline": {"value": value, "unit": "Grays/s", "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "woxel's own pass (Rust + wgpu 0.17 CPU adapter) cannot run here: no Rust toolchain, "
                "crates not vendored, no graphics stack; timed instead is the oracle's restatement",
    }
    print(json.dumps(line), flush=True)


def traffic_from_profile(kernel: str, workload: str):
    rec = NCU_TRAFFIC.get((kernel, workload))
    if rec is None:
        return None
    return {"bytes_per_launch": rec[0], "capture_commit": rec[1],
            "note": "ncu capture of one launch of this kernel on this workload (recorded, not this run)"}


def roofline_view(name: str, topo):
    """The view the oracle counts node-visit bytes on: built by the oracle alone (its
    generator, compute_sdf and atlas()) for the sphere workloads; for the 2.7M-leaf noise
    grid, whose single-threaded oracle SDF takes minutes, the product's masks and SDF
    (equal to the oracle's word for word on the grid's first octant, tests/test_sdf_fullsize.py)."""
    if name == "noise":
        return topo.view(), "product SDF (oracle-equal on the first octant)"
    return _oracle().workload_view(name), "oracle-built"


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def measure_mixed(ctx, grids, dev, flush, steps, warmup):
    """Mixed requests: 256 requests over the sphere and 2000-sphere grids with resolutions
    uniform over {256^2, 640x480, 1280x720, 1920x1080, 3840x2160}. Plain = one wx_render
    launch per request on one stream; batched = one persistent launch over all requests,
    replayed from a CUDA graph (wx_batch_launch). Both device-timed with CUDA events."""
    import torch

    from woxel_gb300 import workloads as W

    frames = W.mixed_frames()
    states = [f.state() for f in frames]
    outs = [torch.empty(f.width * f.height * 4, dtype=torch.uint8, device=dev) for f in frames]
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    rays = sum(f.rays for f in frames)

    def plain(events=None):
        for i, (f, st, o) in enumerate(zip(frames, states, outs)):
            if events is not None:
                events[i][0].record(stream)
            ctx.render(grids[f.grid], st, f.width, f.height, o, None, stream=sh)
            if events is not None:
                events[i][1].record(stream)

    plan = ctx.batch([(grids[f.grid], st, f.width, f.height, o, None) for f, st, o in zip(frames, states, outs)])
    for _ in range(warmup):
        plain()
        plan.launch(sh)
    torch.cuda.synchronize()
    p_ms, b_ms, lat = [], [], []
    for _ in range(steps):
        flush.zero_()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in frames]
        plain(ev)
        torch.cuda.synchronize()
        p_ms.append(ev[0][0].elapsed_time(ev[-1][1]))
        lat.extend(a.elapsed_time(b) for a, b in ev)
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch(sh)
        e1.record(stream)
        torch.cuda.synchronize()
        b_ms.append(e0.elapsed_time(e1))
    plan.close()
    # Per (grid, resolution) class: plain launch time (each launch between its own events).
    per_req = np.array(lat).reshape(len(p_ms), len(frames)).mean(axis=0)
    classes = {}
    for f, ms_f in zip(frames, per_req):
        c = classes.setdefault((f.grid, f"{f.width}x{f.height}"), {"requests": 0, "rays": 0, "ms": 0.0})
        c["requests"] += 1
        c["rays"] += f.rays
        c["ms"] += float(ms_f)
    for c in classes.values():
        c["grays_per_s"] = c["rays"] / (c["ms"] / 1e3) / 1e9
    # Upper bound of any batching: every ray of a grid at the best rate measured on that grid
    # (its largest frames, which fill the GPU alone).
    best = {}
    for (g, _), c in classes.items():
        best[g] = max(best.get(g, 0.0), c["grays_per_s"])
    grid_rays = {}
    for f in frames:
        grid_rays[f.grid] = grid_rays.get(f.grid, 0) + f.rays
    bound_s = sum(r / (best[g] * 1e9) for g, r in grid_rays.items())
    bound = rays / bound_s / 1e9
    lat.sort()
    pm, bm = statistics.mean(p_ms), statistics.mean(b_ms)
    return {
        "workload": "mixed: 256 requests over the sphere + 2000-sphere grids, resolutions "
                    "256x256..3840x2160 (seeded), mode 3",
        "rays_per_step": rays,
        "plain": {"value": rays / (pm / 1e3) / 1e9, "unit": "Grays/s", "ms_per_step": pm,
                  "request_latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[int(0.99 * (len(lat) - 1))]},
                  "launches_per_step": len(frames)},
        "batched": {"value": rays / (bm / 1e3) / 1e9, "unit": "Grays/s", "ms_per_step": bm,
                    "request_latency_ms": {"p50": bm, "p99": bm, "note": "every request completes with the batch"},
                    "launches_per_step": 1, "cuda_graph": True},
        "speedup": pm / bm,
        "classes": {f"{g} {res}": c for (g, res), c in sorted(classes.items())},
        "bound": {"value": bound, "unit": "Grays/s", "speedup_over_plain": bound / (rays / (pm / 1e3) / 1e9),
                  "best_grays_per_s": best,
                  "note": "every request's rays at the best per-grid rate of the plain launches (largest frames); "
                          "no batching can beat it, so the attainable speed-up over plain is bounded by it"},
        "batched_of_bound": (rays / (bm / 1e3) / 1e9) / bound,
    }


def serve_sweep(ctx, rates, duration, slice_tiles=262144, timeout=300.0, max_inflight=2):
    """Serving: open-loop Poisson arrivals over 8 resident grids (4 sphere-generator grids with
    distinct seeds, 4 2000-sphere grids with seeds 2..5, built on the GPU), the resolution mix
    of the mixed requests, HBM budget 150 GB. Each rate is replayed on the continuous-batching
    server and on the FIFO single-request server; reports p50/p99 request latency and served
    Grays/s."""
    import woxel_gb300 as wx
    from woxel_gb300 import workloads as W

    t0 = time.perf_counter()
    grids, kinds = [], []
    for s in range(4):
        grids.append(ctx.build_grid(W.sphere_topology(s), gpu=True))
        kinds.append("sphere")
    for s in range(2, 6):
        grids.append(ctx.build_grid(W.spheres_topology(s), gpu=True))
        kinds.append("spheres")
    grid_bytes = sum(g.info["device_bytes"] for g in grids)
    log(f"[serve] 8 grids, {grid_bytes / 1e9:.2f} GB of node pools, built in {time.perf_counter() - t0:.1f}s")
    budget = 150 * 10**9

    def trace(rate, seed):
        rng = np.random.default_rng(seed)
        n = max(1, int(rng.poisson(rate * duration)))
        arr = np.sort(rng.uniform(0, duration, size=n))
        reqs, rays = [], 0
        for i in range(n):
            gid = int(rng.integers(0, len(grids)))
            w, h = W.RESOLUTIONS[int(rng.integers(0, len(W.RESOLUTIONS)))]
            radius = 200.0 if kinds[gid] == "sphere" else 3000.0
            eye = wx.orbit_eyes(1, radius, int(rng.integers(0, 2**62)))[0]
            st = wx.state_build(eye=tuple(float(x) for x in eye), target=(0, 0, 0), aspect=w / h, fovy=60.0,
                                width=float(w), mode=3)
            reqs.append(wx.Server.request(gid, st, w, h, user=i))
            rays += (w // 8) * 8 * (h // 4) * 4
        return reqs, list(arr), rays

    out = []
    for mode in ("batched", "fifo"):
        srv = wx.Server(ctx, budget_bytes=budget, max_inflight=max_inflight, slice_tiles=slice_tiles,
                        fifo=(mode == "fifo"))
        for g in grids:
            srv.add_grid(g)
        wreqs, _, _ = trace(50.0, 1)  # warm-up: a few requests
        srv.replay(wreqs[:8], [0.0] * min(8, len(wreqs)), release=True)
        for k, rate in enumerate(rates):
            reqs, arr, rays = trace(rate, 1000 + k)
            t1 = time.perf_counter()
            res = srv.replay(reqs, arr, release=True, timeout_s=timeout)
            wall = time.perf_counter() - t1
            lat = np.array([r.t_done - r.t_submit for r in res]) * 1e3
            first = min(r.t_submit for r in res)
            last = max(r.t_done for r in res)
            out.append({"mode": mode, "rate_req_s": rate, "requests": len(reqs),
                        "offered_grays_per_s": rays / duration / 1e9,
                        "served_grays_per_s": rays / (last - first) / 1e9,
                        "latency_ms_p50": float(np.percentile(lat, 50)),
                        "latency_ms_p99": float(np.percentile(lat, 99)), "wall_s": wall})
            log(f"[serve] {mode} {rate:.0f} req/s: {out[-1]}")
        out[-1]["launches_total"] = srv.stats["launches"]
        srv.close()
    for g in grids:
        g.release()
    best = max((o for o in out if o["mode"] == "batched"), key=lambda o: o["served_grays_per_s"])
    fifo_best = max((o for o in out if o["mode"] == "fifo"), key=lambda o: o["served_grays_per_s"])
    return {"workload": "serving: Poisson arrivals over 8 resident grids (4 sphere, 4 2000-sphere), "
                        "resolutions 256x256..3840x2160, mode 3",
            "value": best["served_grays_per_s"], "fifo_value": fifo_best["served_grays_per_s"], "unit": "Grays/s",
            "speedup_over_fifo": best["served_grays_per_s"] / fifo_best["served_grays_per_s"],
            "budget_bytes": budget, "grid_bytes": grid_bytes, "duration_s_per_rate": duration,
            "slice_tiles": slice_tiles, "max_inflight": max_inflight, "sweep": out}


def run_serve(args):
    """--serve: the serving sweep alone, as its own JSON line."""
    import torch

    import woxel_gb300 as wx

    torch.cuda.set_device(0)
    ctx = wx.Context(0)
    r = serve_sweep(ctx, [float(x) for x in args.serve_rates.split(",")], args.serve_duration, args.serve_slice,
                    args.serve_timeout, args.serve_inflight)
    print(json.dumps({"metric": "served_primary_ray_grays_per_s", "value": r.pop("value"), "unit": "Grays/s",
                      "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": r.pop("workload")}, **r}), flush=True)


def extra_workload(ctx, name, dev, flush, steps, warmup):
    """A benchmark workload besides the main one (the r=64 sphere at 640x480, the 4096^3 noise
    grid at 3840x2160), measured like the main one: grid built on the GPU, autotuned on its
    frames, plain per-frame launches, L2 flushed between steps; the roofline from the oracle's
    node-visit bytes on a tile sample."""
    import torch

    from woxel_gb300 import workloads as W

    wl = W.workload(name)
    topo = wl.grids[wl.frames[0].grid]()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    grid = ctx.build_grid(topo, gpu=True)
    torch.cuda.synchronize(dev)
    t_build = time.perf_counter() - t0
    frames = wl.frames
    states = [f.state() for f in frames]
    outs = [torch.empty(f.width * f.height * 4, dtype=torch.uint8, device=dev) for f in frames]
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    saved = ctx.tuning
    tuned = ctx.autotune([(grid, st, f.width, f.height, o, None) for f, st, o in list(zip(frames, states, outs))[:4]],
                         reps=2)

    def step():
        for f, st, o in zip(frames, states, outs):
            ctx.render(grid, st, f.width, f.height, o, None, stream=sh)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize(dev)
    ms = []
    with ClockSampler(dev.index or 0) as clk:
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
    m = statistics.mean(ms)
    rays = wl.rays
    value = rays / (m / 1e3) / 1e9
    tn = ctx.tuning
    kernel = "k_persistent" if tn["kernel"] == 0 else ("k_wave" if tn["rays_per_lane"] > 1 else "k_pixel")
    ctx.set_tuning(**saved)
    info = grid.info
    grid.release()
    # Algorithmic bytes: the oracle's node-visit counts on a tile sample of the same frames.
    view, view_kind = roofline_view(name, topo)
    orc_frames = _oracle().workload_frames(name)
    assert all(wx_state_bytes(st) == o[2] for st, o in zip(states, orc_frames)), "uniforms differ from the oracle's"
    parts = {"sphere": 1, "noise": 32}[name]
    rays_s, _, bpr, grazing = oracle_sample(view, orc_frames, 0, parts, os.cpu_count() or 1, seed=5, stats=True)
    del view
    peak, peak_kind = hbm_peak()
    launch_ms = m / len(frames)
    achieved = bpr * frames[0].rays / (launch_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind, "kernel": kernel, "algorithmic_bytes_per_ray": bpr, "launch_ms": launch_ms,
            "view": view_kind, "oracle_sample_rays": rays_s}
    if name == "sphere":  # 2 MB of pools: L2-resident
        l2 = l2_copy_peak(dev)
        roof["l2"] = {"peak": l2, "frac": achieved / l2,
                      "peak_kind": "measured here: device copy between two L2-resident 32 MiB buffers"}
    return {"config": workload_config(name, (info["n5"], info["n4"], info["n3"]), info["active_voxels"],
                                      [(f.width, f.height) for f in frames]),
            "value": value, "unit": "Grays/s", "ms_per_step": m, "steps": steps, "warmup": warmup,
            "grid_build_gpu_s": round(t_build, 3), "device_bytes": info["device_bytes"], "tuning": tn,
            "autotune_best": tuned["best"], "roofline": roof, "grazing_fraction": grazing, "clocks": clk.summary()}


def wx_state_bytes(st) -> bytes:
    import woxel_gb300 as wx

    return wx.state_bytes(st)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spheres", choices=["sphere", "spheres", "noise"])
    ap.add_argument("--cpu-fraction", type=float, default=None,
                    help="fraction of each frame's tiles the CPU oracle renders per step (default: all of the "
                         "640x480 frame, 1/8 of the 1080p frames, 1/32 of the 4K frames)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the mixed-load batched comparison")
    ap.add_argument("--no-surface", action="store_true", help="skip the zero-crossing mode (render mode 5) figure")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch shape instead of autotuning on 4 frames")
    ap.add_argument("--serve", action="store_true", help="run the serving sweep (Poisson arrivals over 8 grids) instead")
    ap.add_argument("--serve-rates", default="100,200,500,1000,2000,5000")
    ap.add_argument("--serve-duration", type=float, default=5.0, help="seconds of arrivals per rate")
    ap.add_argument("--serve-slice", type=int, default=262144, help="tiles per launch")
    ap.add_argument("--serve-inflight", type=int, default=2, help="launches in flight (batched server)")
    ap.add_argument("--serve-timeout", type=float, default=300.0)
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the sphere, noise and serving figures of the default run")
    ap.add_argument("--extra-serve-rates", default="200,1000,5000")
    ap.add_argument("--extra-serve-duration", type=float, default=4.0)
    ap.add_argument("--kernel", default=None, choices=["persistent", "pixel"],
                    help="fix the kernel (default: the autotuner's choice)")
    ap.add_argument("--tile-width", type=int, default=None)
    ap.add_argument("--warps-per-block", type=int, default=None)
    ap.add_argument("--blocks-per-sm", type=int, default=None)
    ap.add_argument("--tile-order", type=int, default=None, choices=[0, 1],
                    help="0 tile rows top to bottom, 1 middle rows first")
    ap.add_argument("--rays-per-lane", type=int, default=None, choices=[1, 2, 4, 8],
                    help="tiles per warp of the per-frame kernel with lanes that refill (1: one pixel per lane)")
    args = ap.parse_args()
    if args.cpu_fraction is None:
        args.cpu_fraction = {"sphere": 1.0, "spheres": 1.0 / 8, "noise": 1.0 / 32}[args.workload]
    if args.impl == "reference":
        run_reference(args, args.workload)
        return
    if args.serve:
        run_serve(args)
        return

    import torch

    import woxel_gb300 as wx
    from woxel_gb300 import workloads as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    wl = W.workload(args.workload)
    t0 = time.perf_counter()
    topo = wl.grids[wl.frames[0].grid]()
    t_gen = time.perf_counter() - t0
    ctx = wx.Context(local)
    tune = {} if args.kernel is None else {"kernel": 0 if args.kernel == "persistent" else 1}
    for k in ("tile_width", "warps_per_block", "blocks_per_sm", "tile_order", "rays_per_lane"):
        if getattr(args, k) is not None:
            tune[k] = getattr(args, k)
    ctx.set_tuning(**tune)
    t0 = time.perf_counter()
    grid = ctx.build_grid(topo)
    t_build = time.perf_counter() - t0
    info = grid.info
    # The same pools built on the GPU (wx_grid_build_gpu), timed for the record and released.
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ctx.build_grid(topo, gpu=True).release()
    torch.cuda.synchronize(dev)
    t_build_gpu = time.perf_counter() - t0
    log(f"[bench] grid {args.workload}: {info} gen {t_gen:.1f}s sdf+upload {t_build:.1f}s (gpu {t_build_gpu:.2f}s)")
    frames = wl.frames
    states = [f.state() for f in frames]
    W_, H_ = frames[0].width, frames[0].height
    outs = [torch.empty(W_ * H_ * 4, dtype=torch.uint8, device=dev) for _ in frames]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step(events=None):
        for i, (st, o) in enumerate(zip(states, outs)):
            if events is not None:
                events[i][0].record(stream)
            ctx.render(grid, st, W_, H_, o, None, stream=sh)
            if events is not None:
                events[i][1].record(stream)

    tuned = None
    if (args.autotune and args.kernel is None and args.tile_width is None and args.warps_per_block is None
            and args.tile_order is None and args.rays_per_lane is None):
        t0 = time.perf_counter()
        tuned = ctx.autotune([(grid, st, W_, H_, o, None) for st, o in list(zip(states, outs))[:4]], reps=2)
        tuned["seconds"] = time.perf_counter() - t0
        tuned["table"] = [[c["kernel"], c["tile_width"], c["warps_per_block"], c["blocks_per_sm"], c["tile_order"],
                           c["rays_per_lane"], round(ms, 4)]
                          for c, ms in tuned["table"]]
        log(f"[bench] autotune -> {tuned['best']} in {tuned['seconds']:.1f}s")
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    # Timed steps: one pair of events around the step's launches, which follow each
    # other directly on the stream (back-to-back frames may overlap at their boundary).
    step_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed iterations (outside the step's events)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    # Per-frame latency and launch duration: events around every launch (they separate
    # the launches), on further steps of the same frames.
    launch_ms = []
    for _ in range(min(args.steps, 10)):
        flush.zero_()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in frames]
        step(ev)
        torch.cuda.synchronize()
        launch_ms.extend(a.elapsed_time(b) for a, b in ev)
    ms = max_over_ranks(statistics.mean(step_ms), dist, dev)
    rays_step = wl.rays
    value = replica_throughput(rays_step, world, ms)
    lat = sorted(launch_ms)
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]

    # e2e: through wx_render with pinned host output buffers (copies inside the timed region)
    e2e = None
    if not args.no_e2e:
        host = [torch.empty(W_ * H_ * 4, dtype=torch.uint8).pin_memory() for _ in frames]

        def step_host():
            for st, hb in zip(states, host):
                ctx.render(grid, st, W_, H_, hb, None, stream=sh)

        step_host()
        torch.cuda.synchronize()
        e_ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            step_host()
            torch.cuda.synchronize()
            e_ms.append(1e3 * (time.perf_counter() - t1))
        em = max_over_ranks(statistics.mean(e_ms), dist, dev)
        e2e = {"value": replica_throughput(rays_step, world, em), "unit": "Grays/s",
               "h2d_bytes_per_step": 256 * len(frames), "d2h_bytes_per_step": W_ * H_ * 4 * len(frames),
               "ms_per_step": em}

    # Batched vs plain on the same frames: all of them in one persistent launch (wx_render_batch),
    # which removes the per-frame launch tails. `value` stays the plain per-frame figure.
    same_batched = None
    if not args.no_batched:
        fr = [(grid, st, W_, H_, o, None) for st, o in zip(states, outs)]
        for _ in range(args.warmup):
            ctx.render_batch(fr, stream=sh)
        bm = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.render_batch(fr, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            bm.append(e0.elapsed_time(e1))
        b_ms = max_over_ranks(statistics.mean(bm), dist, dev)
        same_batched = {"value": replica_throughput(rays_step, world, b_ms), "unit": "Grays/s", "ms_per_step": b_ms,
                        "launches_per_step": 1, "speedup_over_plain": ms / b_ms,
                        "note": f"the same {len(frames)} frames in one persistent launch"}

    # Mode 3 traces one shadow ray per lit hit inside the same launches; they are not in `value`.
    # Counted from the hit records of one untimed render of each frame.
    shadow = None
    if frames[0].mode == 3:
        hb = torch.empty(W_ * H_ * 32, dtype=torch.uint8, device=dev)
        n_sh = 0
        for st, o in zip(states, outs):
            ctx.render(grid, st, W_, H_, o, hb, stream=sh)
            n_sh += int((hb.view(torch.int32).view(-1, 8)[:, 6] & 1).sum().item())
        del hb
        shadow = {"rays_per_step": n_sh, "value": world * n_sh / (ms / 1e3) / 1e9, "unit": "Grays/s",
                  "note": "shadow rays traced in the timed launches, rate over the same time; not part of value"}

    # Zero-crossing hit mode (render mode 5, an extension with no reference counterpart): the same
    # frames with level-set values attached; reported separately, not part of `value`.
    surface = None
    if args.workload in ("sphere", "spheres") and not args.no_surface:
        t0 = time.perf_counter()
        vals = W.spheres_values(topo) if args.workload == "spheres" else W.sphere_values(topo)
        grid.set_values(vals, 3.0)
        t_vals = time.perf_counter() - t0
        del vals
        st5 = []
        for st in states:
            c = wx.state_from_bytes(wx.state_bytes(st))
            c.render_mode[0] = 5
            st5.append(c)
        for c, o in zip(st5, outs):
            ctx.render(grid, c, W_, H_, o, None, stream=sh)
        sm = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for c, o in zip(st5, outs):
                ctx.render(grid, c, W_, H_, o, None, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            sm.append(e0.elapsed_time(e1))
        s_ms = max_over_ranks(statistics.mean(sm), dist, dev)
        surface = {"value": replica_throughput(rays_step, world, s_ms), "unit": "Grays/s", "ms_per_step": s_ms,
                   "render_mode": 5, "values_bytes": int(info["n3"]) * 512 * 4, "values_host_s": round(t_vals, 2),
                   "note": "zero-crossing hit mode (extension, no reference counterpart): primary HDDA, then "
                           "trilinear level-set search and secant; not part of value"}

    # Batched vs plain on the mixed-resolution load (needs the 2000-sphere grid)
    batched = None
    if not args.no_batched and args.workload == "spheres":
        sphere_grid = ctx.build_grid(W.sphere_topology())
        batched = measure_mixed(ctx, {"sphere": sphere_grid, "spheres": grid}, dev, flush, args.steps, args.warmup)
        sphere_grid.release()

    # roofline + CPU baseline from the oracle on a sample of the same tiles (rank 0)
    roof, cpu, graze = None, None, None
    tn = ctx.tuning  # after autotuning
    kernel_name = "k_persistent" if tn["kernel"] == 0 else ("k_wave" if tn["rays_per_lane"] > 1 else "k_pixel")
    if rank == 0:
        peak, peak_kind = hbm_peak()
        t0 = time.perf_counter()
        view, view_kind = roofline_view(args.workload, topo)
        t_view = time.perf_counter() - t0
        ofr = _oracle().workload_frames(args.workload)
        assert all(wx.state_bytes(st) == o[2] for st, o in zip(states, ofr)), "uniforms differ from the oracle's"
        nthreads = os.cpu_count() or 1
        parts = max(1, int(round(1.0 / args.cpu_fraction)))
        rays_s, secs, bpr, grazing = oracle_sample(view, ofr, 0, parts, nthreads, seed=5, stats=True)
        # Launches overlap on the stream: a launch's share of the timed region is
        # the step time over its launches; one launch timed alone is also kept.
        launch_avg_ms = ms / len(frames)
        launch_alone_ms = statistics.mean(launch_ms)
        bytes_launch = bpr * frames[0].rays
        achieved = bytes_launch / (launch_avg_ms / 1e3) / 1e9
        graze = {"fraction": grazing, "rays": rays_s,
                 "note": "primary rays of the CPU sample with a step whose winning tMax is within 1 ulp of "
                         "another or that lands within 1 ulp of a cell boundary; the kernels match the oracle "
                         "on them bit for bit (parity tests)"}
        l2 = l2_copy_peak(dev)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "traffic_from_profile": traffic_from_profile(kernel_name, args.workload),
                "peak_kind": peak_kind, "view": view_kind, "view_build_s": round(t_view, 1),
                "kernel": kernel_name, "algorithmic_bytes_per_ray": bpr,
                "algorithmic_bytes_per_launch": bytes_launch, "launch_ms": launch_avg_ms,
                "launch_alone": {"ms": launch_alone_ms, "achieved": bytes_launch / (launch_alone_ms / 1e3) / 1e9,
                                 "note": "one launch bracketed by its own events (separate pass)"},
                "l2": {"peak": l2, "frac": achieved / l2,
                       "peak_kind": "measured here: device copy between two L2-resident 32 MiB buffers"}}
        if not args.no_cpu:
            cpu = {"value": rays_s / secs / 1e9, "unit": "Grays/s", "cores": nthreads, "kind": "port",
                   "sample": f"1/{parts} of the 8x4 tiles of each of the {len(frames)} frames (seeded) "
                             f"({rays_s} rays), C restatement of raycast.comp.wgsl, {nthreads} threads"}
            r1, s1, _, _ = oracle_sample(view, ofr, 0, parts * 16, 1, seed=6)
            cpu["single_thread"] = {"value": r1 / s1 / 1e9, "unit": "Grays/s", "cores": 1,
                                    "sample": f"1/{parts * 16} of the tiles ({r1} rays)"}
        del view

    # The other benchmark configurations (the sphere, the noise grid, serving), one GPU only.
    extras = None
    if args.extras and world == 1 and args.workload == "spheres":
        extras = {}
        t0 = time.perf_counter()
        for name in ("sphere", "noise"):
            extras[name] = extra_workload(ctx, name, dev, flush, args.steps, args.warmup)
            log(f"[bench] {name}: {extras[name]['value']:.3f} Grays/s, roofline {extras[name]['roofline']['frac']:.3f}")
        extras["serving"] = serve_sweep(ctx, [float(x) for x in args.extra_serve_rates.split(",")],
                                        args.extra_serve_duration)
        extras["seconds"] = round(time.perf_counter() - t0, 1)

    if rank == 0:
        line = {
            "metric": "primary_ray_grays_per_s", "value": value, "unit": "Grays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.workload, (info["n5"], info["n4"], info["n3"]), info["active_voxels"],
                                      [(f.width, f.height) for f in frames]),
            "arm": {"parallelism": f"replicas x{world}", "l2": "flushed between steps (512 MB write)",
                    "device_bytes": info["device_bytes"],
                    "grid_build_s": {"host_sdf": round(t_build, 3), "gpu_sdf": round(t_build_gpu, 3)},
                    "tuning": ctx.tuning,
                    "autotune": tuned and {"table [kernel, tile_w, warps/block, blocks/SM (0 = all that fit), tile order (1 = middle rows first), rays per lane, ms for 4 frames]":
                                           tuned["table"],
                                           "seconds": tuned["seconds"]}},
            "frame_latency_ms": {"p50": p50, "p99": p99},
            "batched_same_frames": same_batched, "batched": batched, "shadow_rays": shadow, "surface": surface,
            "other_configs": extras,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "grazing_rays": graze,
            "gpu_launches": len(frames) * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
