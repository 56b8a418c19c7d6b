"""Benchmark of the GB300 software rasterizer (one JSON line on rank 0).

Workload (default ``c5``, the largest single-GPU configuration): the stress frame, 3840x2160
RGBA16F with 8x MSAA and float32 depth (LEQUAL), 10,035,200 triangles from 40 displaced geodesic
icospheres with random transforms (depth complexity ~8), a 4096x4096 RGBA8 texture with full
mips and 16x anisotropic filtering, 4 of the 40 instances alpha-blended back to front in one
ordered pass.  The same line carries the other configurations as sub-keys: ``plain_c2`` (1M
random triangles, 1920x1080 RGBA8 4x MSAA, 1024^2 texture, 8x anisotropic), ``batched_c3`` (256
views in one persistent pass replayed from a CUDA graph) and ``differentiable_c4`` (64 views at
256^2, forward + backward).  ``--workload c1|c2|c3|c4`` prints that configuration's own line.

A step is one render pass (binning, raster, shading, ordered stage, resolve) of the whole frame.
  value      shaded samples/s with geometry and texture resident in HBM (inputs larger than L2;
             C2 flushes L2 with a 256 MB write before every timed step); per-step device time
             from CUDA events on the renderer's stream.
  e2e        the same metric through the reference-style C-ABI with host buffers: each step
             uploads the pinned vertex + index buffers (marked rewritten), draws and reads the
             resolved colour back to pinned host memory; host wall time.
  roofline   the tile stage (raster + shade + ordered kernels, which produce every output byte)
             against measured HBM bandwidth.
  cpu_baseline  the CPU oracle (a restatement of the reference's CPU pipeline with this path's
             MSAA and texturing, one set-up per triangle, deferred shading of unblended passes)
             on a bounded sample of the same frame, rank 0 only.
  cpu_baseline_reference  the reference's own CPU renderer (TileRasterRenderer::drawElements,
             built by oracle/build_ref.py from the staged reference tree; AVX2 on x86, its scalar
             build elsewhere) on the plain 512x512 icosphere frame, the one configuration it
             supports (no MSAA, no texturing), with the core count it used.

``--impl reference`` times the reference-side CPU implementation on the host cores instead: the
oracle on a bounded sample of the same stress frame per step (the reference renderer has no
MSAA or texturing), plus the reference renderer's own plain-frame time.  Multi-GPU runs render
independent replicas of the single frame (it does not shard), report ``scaling: weak`` and take
the max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "ifrit-v2_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "shaded samples/s"
KERNELS_PER_PASS = 5  # counting binner, scan, scattering binner, raster, shade (one launch group)
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="c5", choices=["c1", "c2", "c3", "c4", "c5"])
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--no-extras", action="store_true", help="leave the c2/c3/c4 summaries out of the c5 line")
    p.add_argument("--reduced", action="store_true",
                   help="profiling case of the stress frame: 1920x1080, 40 instances of frequency 56 (2,508,800 "
                        "triangles), 2048^2 texture; not a bench configuration")
    return p.parse_args()


def workload(name):
    from ifrit_gb300 import scenes
    if name == "c1":
        v, f, mvp = scenes.c1_scene(1)
        return dict(name="c1", vertices=v, indices=f, mvp=mvp, W=512, H=512, S=1, attr=3, texture=None,
                    aniso=1, cull=2, shading=0, depth_func=3,
                    desc="plain frame: 20,480-triangle icosphere (subdivision 5, +-2% radial jitter, per-vertex "
                         "RGB), fov 60 at distance 3, 512x512 RGBA8 + D32 LEQUAL, 1x, back-face culling, Gouraud")
    v, f, mvp = scenes.c2_scene()
    tex = scenes.value_noise_texture(1024, 2)
    return dict(name="c2", vertices=v, indices=f, mvp=mvp, W=1920, H=1080, S=4, attr=2, texture=tex, aniso=8,
                cull=0, shading=1, depth_func=3,
                desc="1M random triangles (log-normal edges, median 4 px, sigma 1, depth complexity 5.9), "
                     "1920x1080 RGBA8 + D32 LEQUAL, 4x MSAA, 1024^2 RGBA8 value-noise texture with full mips, "
                     "trilinear + 8x anisotropic")


def algorithmic_bytes(w):
    """Compulsory bytes of one frame: vertices + indices read once, per-sample depth and
    resolved colour written once, the texture's full mip chain read once."""
    P = w["W"] * w["H"]
    tex = 0
    if w["texture"] is not None:
        th, tw = w["texture"].shape
        total, ww, hh = 0, tw, th
        while True:
            total += ww * hh
            if ww == 1 and hh == 1:
                break
            ww, hh = (ww + 1) >> 1, (hh + 1) >> 1
        tex = total * 4
    return int(w["vertices"].nbytes + w["indices"].nbytes + P * w["S"] * 4 + P * 4 + tex)


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name):
    """dram bytes per tile-kernel launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "tile_kernel_%s.txt" % name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None


def profiled_issue(name):
    """Fraction of issue slots each dominant tile kernel used (ncu sm__issue_active) in the committed
    summary, if present: the bound of these instruction-issue-bound kernels beside the DRAM roofline."""
    path = os.path.join(ROOT, "profiles", "tile_kernel_%s.txt" % name)
    try:
        for line in open(path):
            if line.startswith("issue_active_per_kernel:"):
                return {k: float(v) for k, v in (kv.split("=") for kv in line.split(":", 1)[1].split())}
    except (OSError, ValueError):
        pass
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "ifrit_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, device_index=0):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device_index):
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_frame(w, nthreads, frames=1):
    """Times the multithreaded CPU oracle on full frames; returns (seconds per frame, samples)."""
    from oracle import oracle as O
    tex_arg = None
    if w["texture"] is not None:
        chain, levels = O.build_mips(w["texture"])
        tex_arg = (chain, levels, w["texture"].shape[1], w["texture"].shape[0])
    d = O.make_draw(w["vertices"], w["indices"], w["mvp"], attr_offset=3, attr_count=w["attr"], cull_mode=w["cull"],
                    depth_func=w["depth_func"], shading=w["shading"], texture=tex_arg,
                    sampler={"max_aniso": w["aniso"]})
    times, shaded = [], 0
    for _ in range(frames):
        t0 = time.perf_counter()
        out = O.render([d], w["W"], w["H"], w["S"], nthreads=nthreads)
        times.append(time.perf_counter() - t0)
        shaded = int((out["vis"] >= 0).sum())
    return statistics.median(times), shaded


def spawn_ranks_if_needed(n):
    """`--gpus N` (N > 1) started without a launcher re-runs this script under
    torch.distributed.run with N ranks on 127.0.0.1 and exits with its status; started by a
    launcher with a different world size, it stops with an error."""
    world = int(os.environ.get("WORLD_SIZE", "0"))
    if n <= 1 and world <= 1:
        return
    if world == 0:
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
               "--master-addr", "127.0.0.1", "--master-port", str(port)] + sys.argv
        sys.exit(subprocess.call(cmd))
    if world != n:
        raise SystemExit("bench.py: --gpus %d but the launcher started %d ranks" % (n, world))


def dist_setup(n):
    if n <= 1 and int(os.environ.get("WORLD_SIZE", "1")) <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    if world != n:
        raise SystemExit("bench.py: --gpus %d but WORLD_SIZE is %d" % (n, world))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist.init_process_group("nccl")
    return rank, world, dist


def run_reference(args):
    """Reference arm: the CPU implementation of the path on the host cores, rank 0 only.  The
    stress frame (default) runs the oracle on a bounded sample per step (C5_SAMPLE); c1/c2 run
    one full frame of the oracle per step.  The reference renderer's own plain-frame time is
    added as cpu_baseline_reference."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    if args.workload == "c5":
        from ifrit_gb300 import scenes
        sc = scenes.c5_scene()
        step = lambda: c5_oracle_sample(sc, nthreads)  # noqa: E731
        cfg = {"workload": "stress: 3840x2160 RGBA16F + D32 LEQUAL, 8x MSAA, %d triangles from 40 displaced "
                           "geodesic icospheres (frequency 112) with random transforms, depth complexity ~8, "
                           "4096^2 RGBA8 texture with full mips, 16x anisotropic, 4 of 40 instances "
                           "alpha-blended back to front (one ordered pass)" % len(sc["indices"]),
               "width": sc["width"], "height": sc["height"], "samples": 8, "triangles": int(len(sc["indices"]))}
        sample = C5_SAMPLE
    else:
        w = workload(args.workload)
        step = lambda: cpu_oracle_frame(w, nthreads)  # noqa: E731
        cfg = {"workload": w["desc"], "width": w["W"], "height": w["H"], "samples": w["S"],
               "triangles": int(len(w["indices"]))}
        sample = "one full frame of the same workload per step"
    for _ in range(args.warmup):
        step()
    times, shaded = [], 0
    for _ in range(args.steps):
        t, shaded = step()
        times.append(t)
    ms = 1000.0 * statistics.mean(times)
    value = shaded / (ms / 1000.0)
    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (seeded)", "config": cfg,
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": nthreads, "kind": "port",
                         "sample": sample + " (the reference's CPU renderer has no MSAA or texturing, so the "
                                            "oracle, a restatement of its pipeline with this path's features, runs)"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_baseline_reference": reference_c1_baseline(),
    }
    print(json.dumps(line), flush=True)


def c3_algorithmic_bytes(views):
    """Compulsory bytes of the batch: per view, its vertices and indices read once, per-sample
    depth and resolved RGBA8 colour written once."""
    return int(sum(v["vertices"].nbytes + v["indices"].nbytes + v["width"] * v["height"] * (4 * v["samples"] + 4)
                   for v in views))


def run_c3(args, steps, warmup, e2e_steps, with_cpu=True, rank=0, world=1, dist=None):
    """Batched workload: 256 views (edges U{128,256,512,1024}, 1x/4x, 1k-200k triangles
    log-uniform, icospheres or soups, Gouraud).  With several ranks every rank renders its
    contiguous share of the views (ifrit_gb300.sharding.view_range; no exchange on the data path)
    and the result sums the ranks' samples over the slowest rank's time.  Returns a dict."""
    import torch
    import ifrit_gb300 as ig
    from ifrit_gb300 import scenes
    from ifrit_gb300.batch import BatchRenderer
    from ifrit_gb300.sharding import view_range

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    views = scenes.c3_batch()
    vb, ve = view_range(len(views), rank, world)
    views = views[vb:ve]
    T = sum(len(v["indices"]) for v in views)

    def build(subset, vis):
        br = BatchRenderer()
        for k, i in enumerate(subset):
            v = views[i]
            br.add_view(v["width"], v["height"], v["samples"], ig.FORMAT_RGBA8, visibility=vis)
            br.add_mesh(k, v["vertices"], v["indices"], v["mvp"], attr_count=v["vertices"].shape[1] - 3, cull=v["cull"])
        return br

    def time_batch(br, n, w):
        for _ in range(w):
            br.draw()
        br.finish()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n):
            br.draw()
        e1.record(stream)
        br.finish()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    everything = list(range(len(views)))
    small = [i for i, v in enumerate(views) if v["width"] == 128]
    # shaded samples per view, from one run with visibility output
    br = build(everything, True)
    br.draw()
    br.finish()
    shaded = [int((br.target(k)["vis"] >= 0).sum().item()) for k in range(len(views))]
    br.close()
    del br
    torch.cuda.empty_cache()
    clocks = ClockSampler()
    br = build(everything, False)
    br.draw()  # sizes, tunes, captures
    br.finish()
    clocks.start()
    if dist:
        dist.barrier()
    ms = time_batch(br, steps, warmup)
    clk = clocks.stop(torch.cuda.current_device())
    tuning = br.tuning()
    if world > 1:  # sharded batch: total samples over the slowest rank's time
        tot = torch.tensor([float(sum(shaded)), float(T)], dtype=torch.float64, device=dev)
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        mx = torch.tensor([ms], device=dev)
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        br.close()
        ms = float(mx.item())
        return {"value": float(tot[0]) / (ms / 1000.0), "ms_per_step": ms, "tris_per_s": float(tot[1]) / (ms / 1000.0),
                "kernels_per_step": 3 + 2 * len(set(v["samples"] for v in views)), "views": 256,
                "views_per_rank": len(views), "triangles": int(tot[1]), "tuning": {"tile_size": tuning[0],
                                                                                   "ctas_per_sm": tuning[1]},
                "clocks": clk, "sharding": "views %d-%d on rank %d of %d" % (vb, ve, rank, world)}
    # end to end: pinned host geometry uploaded every step, colours read back every step
    host_in = [(torch.from_numpy(v["vertices"]).pin_memory(), torch.from_numpy(v["indices"].reshape(-1)).pin_memory())
               for v in views]
    host_out = [torch.empty(br.target(k)["color"].shape, dtype=torch.int32, pin_memory=True) for k in everything]
    h2d = sum(a.numel() * 4 + b.numel() * 4 for a, b in host_in)
    d2h = sum(o.numel() * 4 for o in host_out)
    e2e = []
    for it in range(max(1, e2e_steps) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, (a, b) in enumerate(host_in):
            br.keep[k][0].copy_(a, non_blocking=True)
            br.keep[k][1].copy_(b, non_blocking=True)
        br.draw()
        for k in everything:
            host_out[k].copy_(br.target(k)["color"], non_blocking=True)
        br.finish()
        torch.cuda.synchronize()
        if it:
            e2e.append(time.perf_counter() - t0)
    br.close()
    del br
    torch.cuda.empty_cache()
    # small views: batched (only the 128^2 views) against the plain one-pass-per-frame path
    brs = build(small, False)
    brs.draw()
    brs.finish()
    ms_small = time_batch(brs, steps, warmup)
    brs.close()
    del brs
    plain = []
    for i in everything:
        v = views[i]
        r = ig.Renderer(v["width"], v["height"], v["samples"], ig.FORMAT_RGBA8, visibility=False)
        r.set_stream(stream.cuda_stream)
        r.set_state(cull=v["cull"], depth_func=ig.LESS_OR_EQUAL, shading=ig.FS_GOURAUD)
        r.set_mvp(v["mvp"])
        dv = torch.from_numpy(v["vertices"]).to(dev)
        di = torch.from_numpy(v["indices"].reshape(-1)).to(dev)
        stride = v["vertices"].shape[1]
        r.bind_device_geometry(dv.data_ptr(), stride, len(v["vertices"]), 3, stride - 3, di.data_ptr(), di.numel())
        r.draw_async()
        r.finish()  # settles scratch
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            r.draw_async()
            r.finish()
            ts.append(time.perf_counter() - t0)
        plain.append(statistics.median(ts))
        r.close()
    # overhead-bound small views: 256 views of 128^2 with ~1,000 triangles each, batched against
    # one pass per view (the regime where per-frame launch and synchronisation costs dominate)
    tiny = scenes.c3_batch(seed=7, num_views=256, sizes=(128,), tri_range=(900, 1100))
    views_saved = views
    views = tiny
    brt = build(list(range(len(tiny))), True)
    brt.draw()
    brt.finish()
    tiny_shaded = [int((brt.target(k)["vis"] >= 0).sum().item()) for k in range(len(tiny))]
    brt.close()
    del brt
    brt = build(list(range(len(tiny))), False)
    brt.draw()
    brt.finish()
    ms_tiny = time_batch(brt, steps, warmup)
    brt.close()
    del brt
    tiny_plain = []
    for v in tiny:
        r = ig.Renderer(v["width"], v["height"], v["samples"], ig.FORMAT_RGBA8, visibility=False)
        r.set_stream(stream.cuda_stream)
        r.set_state(cull=v["cull"], depth_func=ig.LESS_OR_EQUAL, shading=ig.FS_GOURAUD)
        r.set_mvp(v["mvp"])
        dv = torch.from_numpy(v["vertices"]).to(dev)
        di = torch.from_numpy(v["indices"].reshape(-1)).to(dev)
        stride = v["vertices"].shape[1]
        r.bind_device_geometry(dv.data_ptr(), stride, len(v["vertices"]), 3, stride - 3, di.data_ptr(), di.numel())
        r.draw_async()
        r.finish()
        t0 = time.perf_counter()
        for _ in range(3):
            r.draw_async()
            r.finish()
        tiny_plain.append((time.perf_counter() - t0) / 3)
        r.close()
    # the lean plain path: every view's renderer enqueues its pass (iftrDrawAsync) back to back on
    # one stream and the status is read once per renderer after the last one (no wait per frame)
    rs = []
    for v in tiny:
        r = ig.Renderer(v["width"], v["height"], v["samples"], ig.FORMAT_RGBA8, visibility=False)
        r.set_stream(stream.cuda_stream)
        r.set_state(cull=v["cull"], depth_func=ig.LESS_OR_EQUAL, shading=ig.FS_GOURAUD)
        r.set_mvp(v["mvp"])
        dv = torch.from_numpy(v["vertices"]).to(dev)
        di = torch.from_numpy(v["indices"].reshape(-1)).to(dev)
        stride = v["vertices"].shape[1]
        r.bind_device_geometry(dv.data_ptr(), stride, len(v["vertices"]), 3, stride - 3, di.data_ptr(), di.numel())
        r.draw_async()
        r.finish()
        rs.append((r, dv, di))
    lean = []
    for _ in range(3):
        t0 = time.perf_counter()
        for r, _, _ in rs:
            r.draw_async()
        for r, _, _ in rs:
            r.finish()
        lean.append(time.perf_counter() - t0)
    for r, _, _ in rs:
        r.close()
    del rs
    tiny_lean = statistics.median(lean)
    views = views_saved
    tiny_batched = sum(tiny_shaded) / (ms_tiny / 1000.0)
    tiny_plain_rate = sum(tiny_shaded) / sum(tiny_plain)
    plain_all = sum(shaded) / sum(plain)
    plain_small = sum(shaded[i] for i in small) / sum(plain[i] for i in small)
    batched_small = sum(shaded[i] for i in small) / (ms_small / 1000.0)
    B = c3_algorithmic_bytes(views)
    peak, peak_kind = peak_hbm()
    out = {
        "value": sum(shaded) / (ms / 1000.0), "ms_per_step": ms, "tris_per_s": T / (ms / 1000.0),
        # per pass: three binning kernels plus raster and shade per launch group (1x and 4x views)
        "kernels_per_step": 3 + 2 * len(set(v["samples"] for v in views)),
        "views": len(views), "triangles": T, "shaded_samples_per_step": sum(shaded),
        "pixels": int(sum(v["width"] * v["height"] for v in views)),
        "tuning": {"tile_size": tuning[0], "ctas_per_sm": tuning[1]},
        "plain": {"value": plain_all, "ms_per_step": 1000.0 * sum(plain),
                  "how": "one iftrDrawAsync + iftrFinish per view, device-resident geometry, host wall time"},
        "small_views": {"views": len(small), "size": 128, "batched": batched_small, "plain": plain_small,
                        "ratio": batched_small / plain_small,
                        "note": "the 128^2 views of the mix carry 1k-200k triangles each (triangle-bound)"},
        "overhead_bound_small_views": {"views": len(tiny), "size": 128, "triangles_per_view": "900-1100",
                                       "batched": tiny_batched, "plain": tiny_plain_rate,
                                       "ratio": tiny_batched / tiny_plain_rate, "ms_batched": ms_tiny,
                                       "ms_plain_per_view": 1000.0 * statistics.mean(tiny_plain),
                                       "plain_enqueued": sum(tiny_shaded) / tiny_lean,
                                       "ratio_to_enqueued": tiny_batched / (sum(tiny_shaded) / tiny_lean),
                                       "ms_plain_enqueued_per_view": 1000.0 * tiny_lean / len(tiny),
                                       "how_enqueued": "256 renderers, iftrDrawAsync each back to back on one stream, "
                                                       "then iftrFinish each (one status read per renderer, no wait "
                                                       "between frames), host wall time"},
        "roofline": {"bound": "hbm", "achieved": B / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": B / (ms / 1000.0) / 1e9 / peak, "traffic": None, "algorithmic_bytes": B,
                     "kernel": "whole batched pass", "peak_source": peak_kind},
        "e2e": {"value": sum(shaded) / statistics.mean(e2e), "unit": "samples/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * statistics.mean(e2e)},
        "clocks": clk,
    }
    if with_cpu:
        # bounded CPU sample: the oracle on views in order until ~10 s of CPU work
        from oracle import oracle as O
        nthreads = os.cpu_count() or 1
        spent, done = 0.0, 0
        for i in everything:
            v = views[i]
            d = O.make_draw(v["vertices"], v["indices"], v["mvp"], attr_offset=3, attr_count=v["vertices"].shape[1] - 3,
                            cull_mode=v["cull"], depth_func=3)
            t0 = time.perf_counter()
            res = O.render([d], v["width"], v["height"], v["samples"], nthreads=nthreads)
            spent += time.perf_counter() - t0
            done += int((res["vis"] >= 0).sum())
            if spent > 10.0:
                break
        out["cpu_baseline"] = {"value": done / spent, "unit": "samples/s", "cores": nthreads, "kind": "port",
                               "sample": "oracle on the batch's views in order until 10 s of work (%d samples)" % done}
    return out


def run_c4(steps, warmup, with_cpu=True, rank=0, world=1, dist=None):
    """Differentiable workload: 64 views at 256x256 float32 RGB of a 20,480-triangle icosphere
    (per-vertex colours, UVs, positions with noise std 0.05), 256x256 float32 texture, L2 loss
    against images of the clean positions.  Times the forward (visibility + shading +
    antialiasing) and forward + backward per step with CUDA events, L2 flushed before each.
    With several ranks every rank renders its contiguous share of the views and the step ends
    with the sum of the mesh gradients over the ranks (ifrit_gb300.sharding)."""
    import torch
    from ifrit_gb300 import scenes
    from ifrit_gb300.diff import DiffRenderer
    from ifrit_gb300.sharding import allreduce_gradients, view_range

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sc = scenes.c4_scene()
    vb, ve = view_range(len(sc["mvps"]), rank, world)
    dr = DiffRenderer(sc["faces"], len(sc["clean"]), sc["width"], sc["height"], sc["mvps"][vb:ve], sc["texture"])
    t = {k: torch.from_numpy(sc[k]).to(dev) for k in ("clean", "noisy", "colors", "uvs")}
    with torch.no_grad():
        target = dr.forward(t["clean"], t["colors"], t["uvs"])[0]
    pos = t["noisy"].clone().requires_grad_(True)
    col = t["colors"].clone().requires_grad_(True)
    uv = t["uvs"].clone().requires_grad_(True)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def fwd():
        with torch.no_grad():
            return dr.render(pos, col, uv)

    def fwd_bwd():
        pos.grad = col.grad = uv.grad = None
        loss = ((dr.render(pos, col, uv) - target) ** 2).sum()
        loss.backward()
        if world > 1:
            allreduce_gradients([pos.grad, col.grad, uv.grad])
        return loss

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for i in range(steps):
            flush.fill_(i & 255)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.mean(ms)

    clocks = ClockSampler()
    clocks.start()
    ms_f = timed(fwd)
    ms_fb = timed(fwd_bwd)
    clk = clocks.stop(torch.cuda.current_device())
    vis = dr.forward(t["noisy"], t["colors"], t["uvs"])[2]
    covered = int((vis >= 0).sum().item())
    N, H, W = dr.N, dr.H, dr.W
    if world > 1:  # all ranks' covered samples over the slowest rank's time
        tot = torch.tensor([float(covered), float(N)], dtype=torch.float64, device=dev)
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        mx = torch.tensor([ms_f, ms_fb], device=dev)
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        covered, N = int(tot[0]), int(tot[1])
        ms_f, ms_fb = float(mx[0]), float(mx[1])
        with_cpu = False
    out = {"views": N, "width": W, "height": H, "triangles": dr.T, "ms_forward": ms_f, "ms_forward_backward": ms_fb,
           "ratio": ms_fb / ms_f, "covered_pixels": covered, "value": covered / (ms_fb / 1000.0),
           "forward_samples_per_s": covered / (ms_f / 1000.0), "clocks": clk,
           # per step: rasterizer (3 binning + raster + shade), diff shade + antialias, adjoint
           "kernels_forward": 7, "kernels_forward_backward": 8}
    dr.close()
    if with_cpu:
        # the FP64 CPU restatement (forward + adjoint) on 4 of the views, and the GPU gradients
        # of the same 4 views against it
        from oracle import diff_oracle as D
        nv = 4
        sub = DiffRenderer(sc["faces"], len(sc["clean"]), W, H, sc["mvps"][:nv], sc["texture"])
        with torch.no_grad():
            tg = sub.forward(t["clean"], t["colors"], t["uvs"])[0]
        p2, c2, u2 = (x.clone().requires_grad_(True) for x in (t["noisy"], t["colors"], t["uvs"]))
        ((sub.render(p2, c2, u2) - tg) ** 2).sum().backward()
        _, _, vis4, codes4 = sub.forward(t["noisy"], t["colors"], t["uvs"])
        args = (sc["noisy"], sc["colors"], sc["uvs"], sc["texture"], sc["faces"], sc["mvps"][:nv], vis4.cpu().numpy(),
                codes4.cpu().numpy())
        t0 = time.perf_counter()
        _, gp, gc, gu, _ = D.loss_and_grads(*args, tg.cpu().numpy())
        cpu_s = time.perf_counter() - t0
        with torch.no_grad():
            upstream = (2 * (sub.forward(t["noisy"], t["colors"], t["uvs"])[0] - tg)).cpu().numpy()
        ap, ac, au = D.adjoint(*args, upstream)
        err = lambda g, r: float(np.abs(g.grad.cpu().numpy() - r).max() / max(np.abs(r).max(), 1e-30))
        out["grad_error_vs_fp64"] = {
            "adjoint": {"positions": err(p2, ap), "colors": err(c2, ac), "uvs": err(u2, au)},
            "end_to_end": {"positions": err(p2, gp), "colors": err(c2, gc), "uvs": err(u2, gu)},
            "views": nv, "metric": "max |g_gpu - g_fp64| / max |g_fp64|; adjoint: same dL/dimage on both sides, "
                                   "end_to_end: each side from its own forward"}
        cov4 = int((vis4 >= 0).sum().item())
        out["cpu_baseline"] = {"value": cov4 / cpu_s, "unit": "samples/s", "cores": torch.get_num_threads(),
                               "kind": "port", "sample": "FP64 forward + adjoint (torch CPU) of 4 of the 64 views"}
        sub.close()
    return out


def run_ours_c4(args):
    rank, world, dist = dist_setup(args.gpus)
    res = run_c4(args.steps, args.warmup, with_cpu=(world == 1), rank=rank, world=world, dist=dist)
    if rank != 0:
        return
    line = {"metric": "covered samples/s through forward + backward", "value": res["value"],
            "unit": "samples/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["ms_forward_backward"], "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "differentiable: %d views %dx%d float32 RGB, %d-triangle icosphere (colours, UVs, "
                                   "positions with noise std 0.05), 256^2 float32 texture, L2 loss; forward = visibility "
                                   "+ shading + silhouette antialiasing, backward = hand-written adjoint"
                                   % (res["views"], res["width"], res["height"], res["triangles"]),
                       "l2": "flushed before every timed step (256 MB write)",
                       "parallelism": "views sharded over %d ranks, gradient all-reduce" % world if world > 1
                       else "single"},
            "ms_forward": res["ms_forward"], "fwd_bwd_over_fwd": res["ratio"],
            "gpu_launches": res["kernels_forward_backward"] * args.steps, "clocks": res["clocks"],
            "e2e": None}
    for k in ("grad_error_vs_fp64", "cpu_baseline"):
        if k in res:
            line[k] = res[k]
    print(json.dumps(line), flush=True)


def c5_record(r, sc, ig):
    """Records the stress pass's draws (per-draw state calls on the host): opaque instances, then
    the blended ones back to front."""
    r.begin_pass(clear=True)
    for d in sc["draws"]:
        r.set_state(cull=ig.CULL_BACK, depth_func=ig.LESS_OR_EQUAL, depth_write=not d["blend"], shading=ig.FS_TEXTURED)
        r.set_blend(d["blend"], 6, 7, 1, 7)  # SRC_ALPHA, ONE_MINUS_SRC_ALPHA; alpha ONE, ONE_MINUS_SRC_ALPHA
        r.set_mvp(d["mvp"])
        r.pass_draw(d["first"], d["count"])


def c5_pass(r, sc, ig):
    """Records and runs the stress pass (iftrEndPass submits it and waits for it)."""
    c5_record(r, sc, ig)
    r.end_pass()


def c5_algorithmic_bytes(sc):
    """Vertices and indices read once, per-sample depth (8x) and resolved RGBA16F written once,
    the texture's mip chain read once, and the resolved colour of the blended instances' pixels
    read back once (counted as the whole target)."""
    P = sc["width"] * sc["height"]
    n, total = sc["texture"].shape[0], 0
    while True:
        total += n * n
        if n == 1:
            break
        n = (n + 1) >> 1
    return int(sc["vertices"].nbytes + sc["indices"].nbytes + P * 8 * 4 + P * 8 + total * 4 + P * 8)


C5_REDUCED = dict(width=1920, height=1080, frequency=56, tex_size=2048)


def c5_oracle_sample(sc, nthreads):
    """The CPU oracle on a bounded sample of the stress frame at full resolution: the first two
    (opaque) instances and the first blended one, in pass order.  Returns (seconds, shaded)."""
    from oracle import oracle as O
    chain, levels = O.build_mips(sc["texture"])
    tex = (chain, levels, sc["texture"].shape[1], sc["texture"].shape[0])
    picked = sc["draws"][:2] + [d for d in sc["draws"] if d["blend"]][:1]
    draws = []
    for d in picked:
        f = sc["indices"][d["first"] // 3:(d["first"] + d["count"]) // 3]
        draws.append(O.make_draw(sc["vertices"], f, d["mvp"], attr_offset=3, attr_count=2, cull_mode=2, depth_func=3,
                                 depth_write=int(not d["blend"]), blend=(6, 7, 1, 7) if d["blend"] else None,
                                 shading=O.SHADE_TEXTURED, texture=tex, sampler={"max_aniso": 16}))
    t0 = time.perf_counter()
    res = O.render(draws, sc["width"], sc["height"], 8, O.FMT_RGBA16F, nthreads=nthreads)
    return time.perf_counter() - t0, int((res["vis"] >= 0).sum())


C5_SAMPLE = ("oracle on 3 of the 40 instances (the first two opaque ones and the first blended one) at full "
             "3840x2160 8x resolution per step; samples/s of that sub-frame")


def reference_c1_baseline(frames=20, warm=3):
    """The reference's own CPU renderer (TileRasterRenderer::drawElements) on the plain 512x512
    icosphere frame: default (tag-buffer) path and in-order (deterministic) path, depth LESS."""
    from oracle import ref_renderer as R
    lib, kind = R.load()
    if lib is None:
        return {"unavailable": kind}
    w = workload("c1")
    _, depth, ms = R.render(lib, w["vertices"], w["indices"], w["mvp"], w["W"], w["H"], depth_func=1,
                            deterministic=False, warm=warm, timed=frames)
    covered = int((depth < 1e30).sum())
    _, _, ms_det = R.render(lib, w["vertices"], w["indices"], w["mvp"], w["W"], w["H"], depth_func=1,
                            deterministic=True, warm=warm, timed=frames)
    threads = R.num_threads(lib)
    return {"value": covered / (ms / 1000.0), "unit": "samples/s", "cores": threads + 1, "kind": "reference",
            "sample": "reference CPU renderer (%s, %d worker threads + the calling thread) on the plain 512x512 "
                      "Gouraud icosphere frame, 20,480 triangles, 1x, depth LESS: median of %d frames after %d "
                      "warm-up; its only supported configuration (no MSAA or texturing)" % (kind, threads, frames, warm),
            "workload": "c1", "ms_per_frame": ms, "tris_per_s": len(w["indices"]) / (ms / 1000.0),
            "ms_per_frame_in_order_path": ms_det, "covered_pixels": covered}


def run_ours_c5(args):
    import torch
    import ifrit_gb300 as ig
    from ifrit_gb300 import scenes

    rank, world, dist = dist_setup(args.gpus)
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sc = scenes.c5_scene(**C5_REDUCED) if args.reduced else scenes.c5_scene()
    W, H = sc["width"], sc["height"]
    r = ig.Renderer(W, H, 8, ig.FORMAT_RGBA16F, visibility=True)
    r.set_stream(stream.cuda_stream)
    r.set_geometry(sc["vertices"], sc["indices"], 2)
    r.set_texture(sc["texture"], max_aniso=16)
    c5_pass(r, sc, ig)
    shaded = int((r.visibility() >= 0).sum())
    r.lib.iftrSetVisibilityOutput(r.h, 0)
    r.set_stage_timing(True)
    for _ in range(args.warmup):
        c5_pass(r, sc, ig)
    clocks = ClockSampler()
    clocks.start()
    ms, stages = [], []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c5_record(r, sc, ig)  # host-side state calls of the 40 draws (inside the e2e figure)
        e0.record(stream)
        r.end_pass()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        stages.append(r.stage_times())
    clk = clocks.stop(torch.cuda.current_device())
    r.set_stage_timing(False)
    m = statistics.mean(ms)
    if dist:
        t = torch.tensor([m], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        m = float(t.item())
    out = torch.empty((H, W), dtype=torch.int64, pin_memory=True).numpy()
    e2e = []
    for i in range(max(1, args.e2e_steps) + 1):
        t0 = time.perf_counter()
        r.mark_geometry_dirty()
        c5_pass(r, sc, ig)
        r.color_into(out)
        if i:
            e2e.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e)
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    r.close()
    del r
    torch.cuda.empty_cache()
    if rank != 0:
        dist.barrier()
        return
    B = c5_algorithmic_bytes(sc)
    peak, peak_kind = peak_hbm()
    st = [statistics.mean(x[i] for x in stages) for i in range(6)]
    t_tile = (st[3] + st[4] + st[5]) / 1000.0
    T = len(sc["indices"])
    line = {"metric": METRIC, "value": world * shaded / (m / 1000.0), "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": m, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (seeded)",
            "config": {"workload": "stress: 3840x2160 RGBA16F + D32 LEQUAL, 8x MSAA, %d triangles from 40 displaced "
                                   "geodesic icospheres (frequency 112) with random transforms, depth complexity ~8, "
                                   "4096^2 RGBA8 texture with full mips, 16x anisotropic, 4 of 40 instances "
                                   "alpha-blended back to front (one ordered pass)" % T,
                       "width": W, "height": H, "samples": 8, "triangles": T, "shaded_samples_per_frame": shaded,
                       "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas" if world > 1 else "single",
                       "timed": "from the pass's submission (iftrEndPass: plan, descriptor upload, every kernel, "
                                "status read-back and wait); the 40 draws' state calls before it are in e2e"},
            "tris_per_s": world * T / (m / 1000.0),
            "stage_ms": {"binning": st[0] + st[1] + st[2], "raster": st[3], "shade": st[4], "ordered": st[5],
                         "binning_count_scan_scatter": st[:3]},
            "roofline": {"bound": "hbm", "achieved": B / t_tile / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": B / t_tile / 1e9 / peak, "traffic": profiled_traffic("c5"), "algorithmic_bytes": B,
                         "kernel": "tile stage (raster + shade + ordered kernels)", "peak_source": peak_kind,
                         "issue_active": profiled_issue("c5")},
            "pass_roofline_frac": B / (m / 1000.0) / 1e9 / peak,
            "e2e": {"value": world * shaded / e2e_s, "unit": "samples/s",
                    "h2d_bytes_per_step": int(sc["vertices"].nbytes + sc["indices"].nbytes),
                    "d2h_bytes_per_step": int(out.nbytes), "ms_per_step": 1000.0 * e2e_s},
            # count, scan, scatter, raster, shade, ordered (one launch group; 4K = 32,400 tiles,
            # one scan launch)
            "gpu_launches": 6 * args.steps, "clocks": clk}
    if args.reduced:
        line["config"]["workload"] = "profiling case (not the bench configuration): stress frame at %dx%d, %d " \
                                     "triangles, 2048^2 texture" % (W, H, T)
        print(json.dumps(line), flush=True)
        return
    nthreads = os.cpu_count() or 1
    dt, done = c5_oracle_sample(sc, nthreads)
    line["cpu_baseline"] = {"value": done / dt, "unit": "samples/s", "cores": nthreads, "kind": "port",
                            "sample": C5_SAMPLE}
    if not args.no_extras and world == 1:
        del sc
        res2 = measure_frame(workload("c2"), 10, 3, 3)
        line["plain_c2"] = {k: res2[k] for k in ("value", "ms_per_step", "tris_per_s", "stage_ms", "roofline",
                                                 "pass_roofline_frac", "e2e")}
        line["plain_c2"]["workload"] = workload("c2")["desc"]
        res1 = measure_frame(workload("c1"), 20, 3, 3, separate_breakdown=True)
        line["plain_c1"] = {k: res1[k] for k in ("value", "ms_per_step", "tris_per_s", "stage_ms", "e2e")}
        torch.cuda.empty_cache()
        res3 = run_c3(args, 5, 3, 3, with_cpu=False)
        line["batched_c3"] = {k: res3[k] for k in ("value", "ms_per_step", "tris_per_s", "views", "triangles", "tuning",
                                                    "plain", "small_views", "overhead_bound_small_views", "roofline",
                                                    "e2e")}
        torch.cuda.empty_cache()
        res4 = run_c4(5, 3, with_cpu=False)
        line["differentiable_c4"] = {k: res4[k] for k in ("views", "width", "height", "triangles", "ms_forward",
                                                          "ms_forward_backward", "ratio", "value")}
    line["cpu_baseline_reference"] = reference_c1_baseline()
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


def run_ours_c3(args):
    rank, world, dist = dist_setup(args.gpus)
    res = run_c3(args, args.steps, args.warmup, args.e2e_steps, with_cpu=(world == 1), rank=rank, world=world,
                 dist=dist)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": res["value"], "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32+i64",
            "data": "synthetic (seeded)",
            "config": {"workload": "batched: %d views (edges U{128,256,512,1024}, 1x/4x MSAA 50/50, RGBA8 + D32), "
                                   "%d triangles (1k-200k per view, log-uniform; geodesic icospheres or random soups), "
                                   "Gouraud, one persistent pass replayed from a CUDA graph" % (res["views"], res["triangles"]),
                       "l2": "inputs larger than L2 (no flush)",
                       "parallelism": "views sharded over %d ranks" % world if world > 1 else "single"},
            "tris_per_s": res["tris_per_s"], "gpu_launches": res["kernels_per_step"] * args.steps}
    line.update({k: res[k] for k in ("roofline", "e2e", "clocks", "plain", "small_views", "overhead_bound_small_views",
                                     "tuning", "cpu_baseline", "sharding") if k in res})
    if "e2e" not in line:
        line["e2e"] = None
    print(json.dumps(line), flush=True)


def measure_frame(w, steps, warmup, e2e_steps, dist=None, world=1, separate_breakdown=False):
    """Plain one-pass-per-frame measurement of a c1/c2 workload.  Returns a dict.  With
    separate_breakdown the timed steps record no per-stage events (they cost a few microseconds,
    which matters on a frame of 0.1 ms) and the stage breakdown comes from extra steps."""
    import torch
    import ifrit_gb300 as ig

    dev = torch.device("cuda", torch.cuda.current_device())
    r = ig.Renderer(w["W"], w["H"], w["S"], ig.FORMAT_RGBA8, visibility=True)
    stream = torch.cuda.current_stream(dev)
    r.set_stream(stream.cuda_stream)
    r.set_state(cull=w["cull"], depth_func=w["depth_func"], shading=w["shading"])
    r.set_mvp(w["mvp"])
    r.set_geometry(w["vertices"], w["indices"], w["attr"])
    if w["texture"] is not None:
        r.set_texture(w["texture"], max_aniso=w["aniso"])
    # settle scratch capacity and count the shaded samples of this frame
    r.draw(clear=True)
    shaded = int((r.visibility() >= 0).sum())
    r.lib.iftrSetVisibilityOutput(r.h, 0)
    r.set_stage_timing(not separate_breakdown)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    for _ in range(warmup):
        flush.fill_(1)
        r.draw_async(clear=True)
        r.finish()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    tile_ms, bin_ms, raster_ms, shade_ms, bin_parts = [], [], [], [], []
    clocks = ClockSampler()
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    def record_stages():
        st = r.stage_times()
        bin_parts.append(st[:3])
        bin_ms.append(st[0] + st[1] + st[2])
        raster_ms.append(st[3])
        shade_ms.append(st[4])
        tile_ms.append(st[3] + st[4])

    for i in range(steps):
        flush.fill_(i & 255)
        ev0[i].record(stream)
        r.draw_async(clear=True)
        ev1[i].record(stream)
        r.finish()
        if not separate_breakdown:
            record_stages()
    torch.cuda.synchronize()
    clk = clocks.stop(torch.cuda.current_device())
    if separate_breakdown:
        r.set_stage_timing(True)
        for i in range(min(steps, 5)):
            flush.fill_(i & 255)
            r.draw_async(clear=True)
            r.finish()
            record_stages()
    ms = statistics.mean(a.elapsed_time(b) for a, b in zip(ev0, ev1))
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    # end to end through the C-ABI with host buffers
    r.set_stage_timing(False)
    out = torch.empty(w["W"] * w["H"], dtype=torch.int32, pin_memory=True).numpy()
    e2e_times = []
    for i in range(max(1, e2e_steps) + 2):
        t0 = time.perf_counter()
        r.mark_geometry_dirty()
        r.draw(clear=True)
        r.color_into(out)
        if i >= 2:
            e2e_times.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e_times)
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    r.close()
    B = algorithmic_bytes(w)
    peak, peak_kind = peak_hbm()
    t_tile = statistics.mean(tile_ms) / 1000.0
    achieved = B / t_tile / 1e9
    return {
        "value": world * shaded / (ms / 1000.0), "ms_per_step": ms, "shaded": shaded,
        "tris_per_s": world * len(w["indices"]) / (ms / 1000.0),
        "stage_ms": {"binning": statistics.mean(bin_ms), "raster": statistics.mean(raster_ms),
                     "shade": statistics.mean(shade_ms),
                     "binning_count_scan_scatter": [statistics.mean(x[i] for x in bin_parts) for i in range(3)]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(w["name"]), "algorithmic_bytes": B,
                     "kernel": "tile stage (raster + shade kernels)", "peak_source": peak_kind,
                     "issue_active": profiled_issue(w["name"])},
        "pass_roofline_frac": B / (ms / 1000.0) / 1e9 / peak,
        "e2e": {"value": world * shaded / e2e_s, "unit": "samples/s",
                "h2d_bytes_per_step": int(w["vertices"].nbytes + w["indices"].nbytes),
                "d2h_bytes_per_step": int(out.nbytes), "ms_per_step": 1000.0 * e2e_s},
        "gpu_launches": KERNELS_PER_PASS * steps, "clocks": clk,
    }


def run_ours(args):
    rank, world, dist = dist_setup(args.gpus)
    w = workload(args.workload)
    res = measure_frame(w, args.steps, args.warmup, args.e2e_steps, dist, world)
    if rank != 0:
        dist.barrier()
        return
    line = {
        "metric": METRIC, "value": res["value"], "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "width": w["W"], "height": w["H"], "samples": w["S"],
                   "triangles": int(len(w["indices"])), "shaded_samples_per_frame": res["shaded"],
                   "l2": "flushed before every timed step (256 MB write)",
                   "parallelism": "replicas" if world > 1 else "single"},
    }
    for k in ("tris_per_s", "stage_ms", "roofline", "pass_roofline_frac", "e2e", "gpu_launches", "clocks"):
        line[k] = res[k]
    nthreads = os.cpu_count() or 1
    t_cpu, shaded_cpu = cpu_oracle_frame(w, nthreads, frames=2)
    line["cpu_baseline"] = {"value": shaded_cpu / t_cpu, "unit": "samples/s", "cores": nthreads, "kind": "port",
                            "sample": "one full frame of the same workload (median of 2)"}
    ref = reference_c1_baseline()
    if ref:
        line["cpu_baseline_reference"] = ref
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


def main():
    args = parse()
    spawn_ranks_if_needed(args.gpus)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c3":
        run_ours_c3(args)
    elif args.workload == "c4":
        run_ours_c4(args)
    elif args.workload == "c5":
        run_ours_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
