#!/usr/bin/env python
"""Benchmark of the GB300 tracing path on the mesh-stress workload.

One step = one full frame of the hot path: camera rays for every (pixel,
sample), the wavefront light-path loop (trace + LightPath::next) and the XYZ
accumulation, for a 1920x1080, 64 spp, max-6-bounce render of a seeded
noise-displaced level-8 icosphere (1,310,720 tris) on a 2-tri ground plane
lit by a sphere light and a 0.5-degree sun (GGX, roughness U(0.1, 0.8)).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--bounds fp32|fp16] [--workload mesh_stress|cornell|motion]

Prints one JSON line on rank 0.  --impl reference times the CPU oracle (a
restatement of the reference's CPU renderer; the Rust binary cannot be built
here) on all host threads, each step a bounded sample of the same frame.
Multi-GPU (one process per GPU under torchrun): by default every rank
renders its own full frame with its own seed (weak scaling, no collective on
the data path); with --split rows the ranks render interleaved rows of one
frame (rank r: rows r, r + N, ...) with the frame's seed and all-gather the
rows once per frame (strong scaling;
pixels identical to a 1-GPU render).  value = all ranks' samples / the
slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
# bytes of one wave descriptor (WaveDesc: 16-byte header + 16 segments of 64
# bytes), uploaded per wave by every render call
WAVE_DESC_BYTES = 16 + 16 * 64
# bytes one FP16 node test reads: anchor and meta 16, extents 8, six planes
# of four f16 48, child references 16 (the 8-byte pad is not read)
FP16_NODE_BYTES = 88
sys.path.insert(0, HERE)

L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--bounds", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--workload", default="mesh_stress",
                    choices=["mesh_stress", "cornell", "motion", "traversal", "serving", "parity", "compact"])
    ap.add_argument("--duration", type=float, default=60.0, help="serving: seconds of Poisson arrivals")
    ap.add_argument("--rate", type=float, default=40.0, help="serving: mean arrivals per second")
    ap.add_argument("--wave-paths", type=int, default=1 << 23, help="serving: paths per wave of each scene lane")
    ap.add_argument("--policy", default="shortest", choices=["fifo", "shortest"],
                    help="serving: admission / wave packing order (shortest remaining samples first, with aging)")
    ap.add_argument("--aging-ms", type=int, default=2000, help="serving: aging bound of the shortest-first policy")
    ap.add_argument("--plain-seconds", type=float, default=20.0,
                    help="serving: bound on the one-at-a-time plain-path baseline run")
    ap.add_argument("--rays", type=int, default=1 << 24, help="rays per set of the traversal microbenchmark")
    ap.add_argument("--elems", type=int, default=1 << 26, help="compact: triples per codec launch")
    ap.add_argument("--level", type=int, default=8, help="icosphere subdivision level of mesh_stress")
    ap.add_argument("--spp", type=int, default=0, help="override samples per pixel (profiling on smaller cases)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample duration")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true",
                    help="frame workloads: skip the bounded traversal and serving runs added to the line")
    ap.add_argument("--split", default="replicas", choices=["replicas", "rows"],
                    help="N>1 frame workloads: 'replicas' = every rank renders its own frame (weak scaling); "
                         "'rows' = the ranks render interleaved rows of one frame and all-gather them (strong scaling)")
    ap.add_argument("--form", default="both", choices=["both", "plain", "optimized"],
                    help="frame workloads: which forms to time (the headline is the optimized one)")
    ap.add_argument("--launch", default="",
                    help="optimized form: fixed launch configuration 'mode,minb[,queue binning bits[,wave paths"
                         "[,grid[,resident tail]]]]' (grid -1: each wavefront kernel's resident blocks; resident "
                         "tail n: the last n iterations of a wave on resident blocks) "
                         "instead of psy_autotune (profiling a known configuration)")
    return ap.parse_args()


def make_scene(args):
    from psychopath_gb300 import scenes
    if args.workload == "mesh_stress":
        sd = scenes.mesh_stress(level=args.level)
        desc = ("mesh_stress: level-%d noise-displaced icosphere (%d tris) + 2-tri ground, sphere light r=0.1 + "
                "0.5 deg sun disc, GGX roughness U(0.1,0.8); 1920x1080, 64 spp, max 6 bounces, seed 0"
                % (args.level, sd.num_tris))
    elif args.workload == "cornell":
        sd = scenes.cornell_box()
        desc = "cornell: 5 wall quads + 2 rotated boxes (34 tris), 0.25x0.25 rect light; 512x512, 16 spp, max 4 bounces"
    else:
        sd = scenes.motion_instances()
        desc = ("motion: 2000 motion-blurred instances of a 20480-tri displaced sphere + deforming mesh, 64 sphere "
                "lights; 1280x720, 32 spp")
    return sd, desc


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline
def cpu_render_sample(sd, target_seconds, threads):
    """Time the CPU oracle on a bounded sample of the frame: every k-th bucket
    of the reference's Hilbert bucket order, k chosen so the run takes about
    target_seconds on `threads` host threads."""
    from oracle.runner import OracleScene
    o = OracleScene(sd)
    stride = 4096
    t0 = time.perf_counter()
    _, st = o.render_sampled(stride, threads=threads)
    dt = time.perf_counter() - t0
    while dt < 0.5 and stride > 1:
        stride = max(1, stride // 4)
        t0 = time.perf_counter()
        _, st = o.render_sampled(stride, threads=threads)
        dt = time.perf_counter() - t0
    stride = max(1, int(round(stride * dt / target_seconds)))
    t0 = time.perf_counter()
    _, st = o.render_sampled(stride, threads=threads)
    dt = time.perf_counter() - t0
    o.close()
    return {"samples": st["samples"], "rays": st["ray_count"], "seconds": dt, "stride": stride}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sd, desc = make_scene(args)
    if args.spp:
        sd.spp = args.spp
    threads = os.cpu_count() or 1
    from oracle.runner import OracleScene
    o = OracleScene(sd)
    # calibrate the per-step sample: every stride-th bucket, ~target seconds
    stride = 4096
    t0 = time.perf_counter()
    o.render_sampled(stride, threads=threads)
    dt = time.perf_counter() - t0
    while dt < 0.3 and stride > 1:
        stride = max(1, stride // 4)
        t0 = time.perf_counter()
        o.render_sampled(stride, threads=threads)
        dt = time.perf_counter() - t0
    per_step_target = max(2.0, min(12.0, 100.0 / max(1, args.steps + args.warmup)))
    stride = max(1, int(round(stride * dt / per_step_target)))
    for _ in range(args.warmup):
        o.render_sampled(stride, threads=threads)
    samples, rays, secs = 0, 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, st = o.render_sampled(stride, threads=threads)
        secs += time.perf_counter() - t0
        samples += st["samples"]
        rays += st["ray_count"]
    value = samples / secs
    sample_desc = "every %d-th bucket (Hilbert order, 8x8 px x 64 spp) of the frame per step" % stride
    line = {
        "impl": "reference",
        "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": desc, "bounds": "f32 (CPU)"},
        "mrays_per_s": rays / secs / 1e6,
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                         "sample": sample_desc},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle (C++ restatement of the reference's CPU renderer); the Rust reference cannot be built here",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU
def time_frames(rend, xyz, flush, stream, steps, warmup, barrier, share=None, post=None):
    """W untimed frames, then K frames bracketed by CUDA events on the
    render stream (L2 flushed before each).  share: (first row, row step) of
    this rank's interleaved rows (None: the whole image); post: called after
    each frame inside the timed region (the all-gather of a row split).
    Returns (elapsed s, summed traversal-kernel s, rays, samples)."""
    import torch
    sp = stream.cuda_stream

    def frame(stats):
        if share is None:
            return rend.render_device(xyz.data_ptr(), stream=sp, stats=stats)
        return rend.render_rows_device(share[0], share[1], xyz.data_ptr(), stream=sp, stats=stats)

    for _ in range(warmup):
        frame(False)
        if post:
            post()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    trace_s, rays, samples = 0.0, 0, 0
    ev0.record(stream)
    for _ in range(steps):
        flush.zero_()
        st = frame(True)
        if post:
            post()
        trace_s += st["trace_time"]
        rays += st["ray_count"]
        samples += st["samples"]
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    return ev0.elapsed_time(ev1) / 1e3, trace_s, rays, samples


def run_ours(args):
    """Headline: the optimized form (f32 shading arithmetic, launch
    configuration picked by psy_autotune, CUDA-graph wave replay when the
    tuner keeps it).  Beside it: the plain form (f64 shading arithmetic as
    the reference, default launch configuration) on the same frame, and the
    relative RMSE between the two images."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from psychopath_gb300 import build, gpu
    build.build()
    sd, desc = make_scene(args)
    rows_split = world > 1 and args.split == "rows"
    if not rows_split:
        sd.seed = sd.seed + rank  # independent sample sets per replica
    if args.spp:
        sd.spp = args.spp
    W, H, spp = sd.width, sd.height, sd.spp
    share, gather = None, None
    if rows_split:
        from psychopath_gb300 import multi
        share = (rank, world)  # this rank's interleaved rows: rank, rank + world, ...

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # a dedicated stream: the library runs on the stream it is given, and the
    # L2 flush and the timing events must be ordered with its kernels (the
    # legacy default stream's handle is 0, which the ABI reads as "the
    # scene's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    xyz = torch.zeros(H * W * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    if rows_split:
        n_rows = len(multi.rows_of(H, world, rank))

        def gather():  # one all-gather of the ranks' rows per frame (NCCL)
            multi.gather_rows(xyz[: n_rows * W * 3].view(n_rows, W, 3), H, rank, world)

    # plain form
    t0 = time.perf_counter()
    plain = gpu.Scene(sd, bounds=args.bounds)
    build_s = time.perf_counter() - t0
    plain_img = None
    p_el, p_trace, p_rays, p_samples = 1.0, 0.0, 0, 0
    if args.form == "both":
        p_el, p_trace, p_rays, p_samples = time_frames(gpu.Renderer(plain), xyz, flush, stream, args.steps,
                                                       args.warmup, barrier, share, gather)
        plain_img = xyz.cpu().numpy().copy()
    if args.form == "plain":
        scene = plain  # report the plain form as the line's value
        tune = {"trace_mode": 0, "minb": 4, "wave_paths": 1 << 24, "sort_bits": 0, "use_graph": 0}
        tune_s = 0.0
    else:
        plain.close()
        # optimized form
        scene = gpu.Scene(sd, bounds=args.bounds, shading="f32")
        t0 = time.perf_counter()
        if args.launch:
            vals = [int(x) for x in args.launch.split(",")]
            mode, minb, bits = vals[0], vals[1], (vals[2] if len(vals) > 2 else 0)
            wave = vals[3] if len(vals) > 3 else 1 << 24
            grid = vals[4] if len(vals) > 4 else 0
            tail = vals[5] if len(vals) > 5 else 0
            scene.set_trace(mode, minb)
            scene.set_sort(bits)
            scene.set_launch(grid, wave)
            scene.set_resident_tail(tail)
            tune = {"trace_mode": mode, "minb": minb, "wave_paths": wave, "sort_bits": bits, "use_graph": 0,
                    "grid": grid, "resident_tail": tail, "fixed": True}
        else:
            tune = scene.autotune()
        tune_s = time.perf_counter() - t0
    rend = gpu.Renderer(scene)
    # traversal work counters for the roofline (one extra, untimed frame)
    scene.counters(True)
    rend.render_device(xyz.data_ptr(), stream=stream.cuda_stream, stats=True)  # counters run in stats mode
    torch.cuda.synchronize()
    n_nodes, n_tris, n_rays_c = scene.counters(False)
    clocks = ClockSampler(local)
    clocks.start()
    elapsed, trace_s, rays, samples = time_frames(rend, xyz, flush, stream, args.steps, args.warmup, barrier, share,
                                                  gather)
    clk = clocks.stop()
    opt_img = xyz.cpu().numpy()
    rmse = None
    nonfinite = {"optimized": int((~np.isfinite(opt_img)).reshape(-1, 3).any(axis=1).sum())}
    if plain_img is not None:
        # over pixels finite in both: the reference's own arithmetic turns a
        # rare sample into NaN (one sample of the motion frame), and both
        # forms reproduce it
        ok = np.isfinite(opt_img) & np.isfinite(plain_img)
        nonfinite["plain"] = int((~np.isfinite(plain_img)).reshape(-1, 3).any(axis=1).sum())
        a, b = opt_img[ok].astype(np.float64), plain_img[ok].astype(np.float64)
        rmse = float(np.sqrt(np.mean((a - b) ** 2)) / max(1e-30, np.sqrt(np.mean(b ** 2))))
    if args.form == "plain":
        p_el, p_samples = elapsed, samples
    t = torch.tensor([elapsed, p_el], device="cuda")
    tot = torch.tensor([samples, p_samples, rays, p_rays], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tot, op=torch.distributed.ReduceOp.SUM)
    elapsed, p_el = float(t[0].item()), float(t[1].item())
    samples_all, p_samples_all, rays_all, p_rays_all = (float(v) for v in tot.tolist())
    value = samples_all / elapsed
    plain_value = p_samples_all / p_el if p_samples else None

    # end to end through the public C ABI with a host image buffer (pinned,
    # as a caller streaming frames off the device would allocate it)
    img = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True).numpy()
    barrier()
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        if rows_split:  # rows on the device, all-gather, full image to the host
            rend.render_rows_device(rank, world, xyz.data_ptr(), stream=stream.cuda_stream)
            img = multi.gather_rows(xyz[: n_rows * W * 3].view(n_rows, W, 3), H, rank, world).cpu().numpy()
        else:
            img, _ = rend.render(out=img)
    e_el = time.perf_counter() - e0
    te = torch.tensor([e_el], device="cuda")
    if world > 1:
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
    frames_all = args.steps * (1 if rows_split else world)
    e2e_value = (W * H * spp * frames_all) / float(te.item())

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # roofline: algorithmic bytes of the traversal kernel (per ray: ray in
    # 32 B + hit out 16 B + 128 B per BVH4 node test + 36 B per triangle
    # test), over the measured traversal-kernel time of the timed frames
    node_bytes = FP16_NODE_BYTES if args.bounds == "fp16" else 128
    frames = args.steps
    alg_bytes_frame = 48.0 * n_rays_c + node_bytes * n_nodes + 36.0 * n_tris
    achieved = alg_bytes_frame * frames / max(trace_s, 1e-12) / 1e9
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        try:
            peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
        except Exception:
            pass
    # DRAM traffic of the frame's traversal launches: bytes per traced ray
    # from an ncu capture of the same launch form on a smaller frame of the
    # same scene (the committed summary), times this frame's rays
    traffic = frame_traffic(args.workload, tune, n_rays_c) if not rows_split else None  # bytes per frame
    rows = max(1, tune["wave_paths"] // (W * spp))
    waves = math.ceil(H / rows)
    iters = 2 * sd.max_bounces + 3
    # queue ordering between iterations: keys, scan, scatter (counting sort,
    # <= 16 bits) or keys + three kernels per 8-bit radix pass (wider keys)
    bits = tune["sort_bits"]
    per_binning = 0 if not bits else (3 if bits <= 16 else 1 + 3 * ((bits + 7) // 8))
    binning = per_binning * (iters - 1)
    # camera, (trace, shadow-result shade, hit shade) per iteration, accumulate
    launches_per_frame = waves * (2 + 3 * iters + binning) + waves  # + the ray-count kernel of stats frames
    line = {
        "metric": "samples/s", "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
        "scaling": "strong" if rows_split else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": desc, "bounds": args.bounds,
                   "form": ("plain: f64 shading, default launch" if args.form == "plain" else
                            "optimized: f32 shading, %s launch" % ("fixed" if args.launch else "autotuned")),
                   "graphs": "timed frames record per-stage events, so waves launch kernel by kernel even when the "
                             "tuner keeps graph replay (which saves launch gaps only)",
                   "l2": "256 MiB written between steps; path state per wave ~1.5-3 GB > L2",
                   "scene_build_s": round(build_s, 3), "scene_device_bytes": scene.device_bytes(),
                   "autotune": tune, "autotune_s": round(tune_s, 2)},
        "mrays_per_s": rays_all / elapsed / 1e6,
        "plain": ({"value": plain_value, "unit": "samples/s", "ms_per_step": p_el / args.steps * 1e3,
                   "mrays_per_s": p_rays_all / p_el / 1e6, "trace_kernel_s_per_frame": p_trace / frames,
                   "form": "f64 shading arithmetic (reference precision), default launch configuration"}
                  if plain_value else None),
        "speedup_vs_plain": value / plain_value if plain_value else None,
        "rel_rmse_vs_plain": rmse,
        "nonfinite_pixels": nonfinite,
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": waves * WAVE_DESC_BYTES,
                "d2h_bytes_per_step": W * H * 3 * 4 + 8,
                "note": "psy_render_image with a pinned host XYZ buffer and render statistics: per step the wave "
                        "descriptors go up (%d B each) and the image and the ray count (8 B) come back, inside the "
                        "timed loop; the scene is resident (uploaded once at psy_scene_create)" % WAVE_DESC_BYTES},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_per": "frame (all traversal launches of one frame)",
                     "peak_source": peak_src, "kernel": "k_trace_queue",
                     "per_frame": {"rays": n_rays_c, "node_tests": n_nodes, "tri_tests": n_tris,
                                   "alg_bytes": alg_bytes_frame, "trace_kernel_s": trace_s / frames}},
        "clocks": clk,
        "gpu_launches": launches_per_frame * args.steps,
    }
    if world == 1 and not args.no_sub:
        scene.close()  # the frame's wave buffers (up to ~27 GB) are not needed past this point
        del xyz, flush
        if args.form == "both" and plain_value:
            line["headline_form"] = served_fp16_frames(args, sd, plain_value, plain_img)
        # bounded runs of the traversal microbenchmark and of serving, so one
        # default run reports all three headline measurements
        sub_args = argparse.Namespace(**vars(args))
        sub_args.steps, sub_args.warmup = 3, 2
        line["sub"] = {
            "traversal_incoherent": run_traversal(sub_args, set_names=("incoherent",),
                                                  config_names=("plain", "static10+binned", "refill10+binned"),
                                                  with_gpu_bvh=False,
                                                  emit=False)}
        sub_args.duration, sub_args.rate, sub_args.plain_seconds = 20.0, 10.0, 10.0
        sub_args.bounds = "fp16"
        sv = run_serving(sub_args, emit=False)
        line["sub"]["serving"] = {k: sv[k] for k in ("value", "unit", "latency_ms", "offered_samples_per_s", "overloaded",
                                                     "plain_one_at_a_time", "tuned_one_at_a_time", "served_over_plain",
                                                     "served_over_tuned_one_at_a_time", "burst",
                                                     "requests_sharing_a_wave",
                                                     "hbm_peak_bytes", "clocks")}
        line["sub"]["serving"]["workload"] = sv["config"]["workload"]
        line["sub"]["serving"]["form"] = "fp16 bounds, f32 shading, autotuned; policy %s" % sv["config"]["policy"]
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cb = cpu_render_sample(sd, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": cb["samples"] / cb["seconds"], "unit": "samples/s", "cores": threads,
                                "kind": "port", "sample": "every %d-th bucket (Hilbert order) of the frame: %d samples, "
                                "%.1f s" % (cb["stride"], cb["samples"], cb["seconds"])}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def served_fp16_frames(args, sd, plain_value, plain_img):
    """The served, autotuned FP16-bounds form on this frame: a scene with FP16 child
    bounds and f32 shading, autotuned, served as a lane of the render server
    (waves of the tuned size, CUDA-graph replay); K frames submitted as K
    requests with host result buffers and timed from the first submit to the
    last result in host memory.  Against the plain form's samples/s on the
    same frame, and the image's relative RMSE against the plain image."""
    import numpy as np
    from psychopath_gb300 import gpu
    g = gpu.Scene(sd, bounds="fp16", shading="f32")
    t0 = time.perf_counter()
    tune = g.autotune()
    tune_s = time.perf_counter() - t0
    srv = gpu.Server(hbm_budget_bytes=120 * 10**9, wave_paths=tune["wave_paths"], use_graphs=True,
                     policy=args.policy, aging_ms=args.aging_ms)
    lane = srv.add_scene(g)
    W, H, spp = sd.width, sd.height, sd.spp
    for _ in range(max(1, args.warmup)):
        srv.wait(srv.submit(lane, W, H, spp, sd.seed), timeout=3600.0)
    t1 = time.perf_counter()
    ids = [srv.submit(lane, W, H, spp, sd.seed) for _ in range(args.steps)]
    sts = [srv.wait(i, timeout=3600.0) for i in ids]
    el = time.perf_counter() - t1
    if any(st["state"] != 2 for st in sts):
        raise RuntimeError("served frame failed")
    img = srv.result(ids[-1]).reshape(H, W, 3)
    srv.close()
    g.close()
    value = W * H * spp * args.steps / el
    rmse = None
    if plain_img is not None:
        p = plain_img.reshape(H, W, 3)
        ok = np.isfinite(img) & np.isfinite(p)
        a, b = img[ok].astype(np.float64), p[ok].astype(np.float64)
        rmse = float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))
    return {"form": "served + autotuned + FP16 child bounds (f32 shading); %d frames as requests with host results"
                    % args.steps,
            "value": value, "unit": "samples/s", "vs_plain": value / plain_value, "rel_rmse_vs_plain": rmse,
            "autotune": tune, "autotune_s": round(tune_s, 2)}


def frame_traffic(workload, tune, rays):
    """DRAM bytes (read + write) of a frame's traversal launches: the
    committed per-ray figure for this workload and launch form, times the
    rays traced; None without a matching summary."""
    path = os.path.join(HERE, "profiles", "frame_traffic.txt")
    if not os.path.exists(path):
        return None
    kv = dict(l.split(":", 1) for l in open(path) if ":" in l and not l.startswith("#"))
    launch = "%d,%d" % (tune.get("trace_mode", -1), tune.get("minb", -1))
    if kv.get("workload", "").strip() != workload or kv.get("launch", "").strip() != launch:
        return None
    return float(kv["dram_bytes_per_ray"]) * rays


# ---------------------------------------------------------------- traversal microbenchmark
def traversal_traffic(launch, rays):
    """DRAM bytes of one traversal launch of `rays` incoherent rays, scaled
    from the committed ncu summary (traffic grows with the ray count), or
    None when the summary is for another launch configuration."""
    path = os.path.join(HERE, "profiles", "traversal_traffic.txt")
    if not os.path.exists(path):
        return None
    kv = dict(l.split(":", 1) for l in open(path) if ":" in l and not l.startswith("#"))
    if kv.get("launch", "").strip() != launch:
        return None
    return float(kv["dram_bytes_per_ray"]) * rays


def run_traversal(args, set_names=("coherent", "incoherent"), config_names=None, with_gpu_bvh=True, emit=True):
    """16M coherent (pinhole) and 16M incoherent (cosine-hemisphere from random
    surface points, seed 7) rays against the 2048x1024-quad displaced grid
    (4,194,304 tris): Mrays/s, algorithmic GB/s, closest-hit agreement with the
    CPU oracle on a sample of each set.  Each set is traced under a few launch
    configurations (the plain one first: one thread per ray, default register
    budget, rays in the given order); every configuration returns identical
    hits (checked), and the line's value is the fastest on the incoherent set."""
    import numpy as np
    import torch
    from psychopath_gb300 import abi, gpu, scenes
    from oracle.runner import OracleScene
    torch.cuda.set_device(0)
    build_mod = __import__("psychopath_gb300.build", fromlist=["build"])
    build_mod.build()
    sd, P, F = scenes.grid_mesh(2048, 1024)
    n_side = int(round(math.sqrt(args.rays)))
    sets = {}
    if "coherent" in set_names:
        sets["coherent"] = scenes.coherent_rays(n_side)
    if "incoherent" in set_names:
        sets["incoherent"] = scenes.incoherent_rays(P, F, n_side * n_side, seed=7)
    t0 = time.perf_counter()
    g = gpu.Scene(sd, bounds=args.bounds)
    sah_build_s = time.perf_counter() - t0
    tr = gpu.Tracer(g)
    o = OracleScene(sd)
    sah_hits = {}
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak = float(json.load(open(peaks_path))["hbm_gbs"]) if os.path.exists(peaks_path) else 6800.0
    node_bytes = FP16_NODE_BYTES if args.bounds == "fp16" else 128
    stream = torch.cuda.Stream()  # non-null handle: kernels and events on one stream
    torch.cuda.set_stream(stream)
    configs = [("plain", 0, 4, False), ("minb8", 0, 8, False), ("minb8+binned", 0, 8, True),
               ("persistent8+binned", 1, 8, True), ("static8", 3, 8, False), ("static8+binned", 3, 8, True),
               ("static10+binned", 3, 10, True), ("static12+binned", 3, 12, True), ("static6+binned", 3, 6, True),
               ("spec8+binned", 4, 8, True), ("spec10+binned", 4, 10, True), ("refill10", 5, 10, False),
               ("refill10+binned", 5, 10, True)]
    if config_names is not None:
        configs = [c for c in configs if c[0] in config_names]
    out = {}
    for name, rays in sets.items():
        n = len(rays)
        d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
        d_hits = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
        g.set_trace(0, 4)
        g.set_ray_order(False)
        g.counters(True)
        tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        gn, gt, gr = g.counters(False)
        ref_hits = d_hits.cpu().numpy()
        sah_hits[name] = ref_hits
        # oracle on a sample: agreement and per-ray node / triangle tests
        idx = np.random.default_rng(11).choice(n, size=min(n, 200000), replace=False)
        ho, _, on, ot = o.trace(rays[idx], threads=os.cpu_count() or 1)
        hg = ref_hits.view(abi.hit_dtype())[idx]
        surf = ho["kind"] >= abi.PSY_HIT_SURFACE
        same = (hg["kind"] == ho["kind"]) & (~surf | ((hg["prim"] == ho["prim"]) & (hg["inst"] == ho["inst"])))
        bmin = np.minimum(np.minimum(ho["b0"], ho["b1"]), ho["b2"])
        near = surf & (np.abs(bmin) < 1e-4)
        n_node = on / len(idx)
        n_tri = ot / len(idx)
        alg = 32 + 16 + n_node * node_bytes + n_tri * 36
        res = {"rays": n, "alg_bytes_per_ray": alg, "oracle_node_tests_per_ray": n_node,
               "oracle_tri_tests_per_ray": n_tri, "gpu_node_tests_per_ray": gn / max(1, gr),
               "gpu_tri_tests_per_ray": gt / max(1, gr), "hit_agreement": float(same.mean()),
               "disagree_not_near_edge": int((~same & ~near).sum()), "sample": len(idx),
               "hit_fraction": float(surf.mean()), "configs": {}}
        for cname, mode, minb, binned in configs:
            g.set_trace(mode, minb)
            g.set_ray_order(binned)
            for _ in range(args.warmup):
                tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            sec = e0.elapsed_time(e1) / 1e3 / args.steps
            got = d_hits.cpu().numpy()
            identical = bool(np.array_equal(got, ref_hits))
            # forms that may break exact t ties differently (speculative
            # traversal): rays whose hit differs, and whether every such hit
            # has the same t
            hg_, hr_ = got.view(abi.hit_dtype()), ref_hits.view(abi.hit_dtype())
            ndiff = int((hg_ != hr_).sum())
            ties_only = bool(np.array_equal(hg_["t"], hr_["t"]) and np.array_equal(hg_["kind"], hr_["kind"]))
            # the traversal kernel alone: a binned call is the ray sort plus
            # the kernel over the sorted order; time the kernel on that same
            # order (rays gathered on the device, trace in the given order)
            ksec = sec
            if binned and n >= 65536:
                _, order = g.ray_order(rays)
                d_sorted = d_rays.view(n, -1)[torch.from_numpy(order.astype(np.int64)).cuda()].reshape(-1)
                g.set_ray_order(False)
                for _ in range(args.warmup):
                    tr.trace_device(d_sorted.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
                torch.cuda.synchronize()
                e0.record(stream)
                for _ in range(args.steps):
                    tr.trace_device(d_sorted.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize()
                ksec = e0.elapsed_time(e1) / 1e3 / args.steps
                del d_sorted
            gbs = alg * n / ksec / 1e9
            res["configs"][cname] = {"trace_mode": mode, "minb": minb, "binned": binned, "ms_per_call": sec * 1e3,
                                     "kernel_ms": ksec * 1e3, "mrays_per_s": n / sec / 1e6, "achieved_gbs": gbs,
                                     "frac": gbs / peak, "hits_identical_to_plain": identical,
                                     "hits_differing": ndiff, "differences_are_t_ties": ties_only}
        best = max(res["configs"].items(), key=lambda kv: kv[1]["mrays_per_s"])
        res["best"] = best[0]
        out[name] = res
        del d_rays, d_hits
    # the same rays against a GPU-built tree (PSY_BVH_GPU): creation time,
    # speed with the best launch configuration, hits against the SAH tree
    g.close()
    if not with_gpu_bvh:
        inc = out["incoherent"]
        bc = inc["configs"][inc["best"]]
        return {"rays": inc["rays"], "best": inc["best"], "mrays_per_s": bc["mrays_per_s"],
                "ms_per_call": bc["ms_per_call"], "kernel_ms": bc["kernel_ms"],
                "frac_kernel": bc["frac"], "frac_call": inc["alg_bytes_per_ray"] * inc["rays"] / (bc["ms_per_call"] * 1e-3)
                / 1e9 / peak, "alg_bytes_per_ray": inc["alg_bytes_per_ray"], "peak_gbs": peak,
                "hit_agreement": inc["hit_agreement"], "disagree_not_near_edge": inc["disagree_not_near_edge"],
                "sample": inc["sample"], "plain_mrays_per_s": inc["configs"]["plain"]["mrays_per_s"],
                "hits_identical_to_plain": bc["hits_identical_to_plain"], "bounds": args.bounds}
    t0 = time.perf_counter()
    gb = gpu.Scene(sd, bounds=args.bounds, bvh="gpu")
    gpu_build_s = time.perf_counter() - t0
    trb = gpu.Tracer(gb)
    gpu_bvh = {"create_s": round(gpu_build_s, 3), "sah_create_s": round(sah_build_s, 3), "sets": {}}
    for name, rays in sets.items():
        n = len(rays)
        best = out[name]["configs"][out[name]["best"]]
        gb.set_trace(best["trace_mode"], best["minb"])
        gb.set_ray_order(best["binned"])
        d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
        d_hits = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
        for _ in range(args.warmup):
            trb.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            trb.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3 / args.steps
        hb = d_hits.cpu().numpy().view(abi.hit_dtype())
        ref = sah_hits[name].view(abi.hit_dtype())
        surf = ref["kind"] >= abi.PSY_HIT_SURFACE
        same = (hb["kind"] == ref["kind"]) & (~surf | (hb["prim"] == ref["prim"]))
        gpu_bvh["sets"][name] = {"launch": out[name]["best"], "mrays_per_s": n / sec / 1e6,
                                 "hit_agreement_vs_sah": float(same.mean())}
        del d_rays, d_hits
    gb.close()
    inc = out["incoherent"]
    bc = inc["configs"][inc["best"]]
    line = {"metric": "Mrays/s (incoherent)", "value": bc["mrays_per_s"], "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": bc["ms_per_call"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded grid mesh and rays)",
            "config": {"workload": "traversal: 2048x1024-quad displaced grid (4,194,304 tris), %d rays per set"
                                   % len(sets["incoherent"]), "bounds": args.bounds, "launch": inc["best"],
                       "l2": "inputs (671 MB of rays per set) larger than L2"},
            "plain": inc["configs"]["plain"],
            "roofline": {"bound": "hbm", "achieved": bc["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": bc["frac"], "traffic": traversal_traffic(inc["best"], n_side * n_side),
                         "kernel": "k_trace_rays", "kernel_ms": bc["kernel_ms"],
                         "note": "algorithmic bytes from the oracle's node / triangle tests per ray over the "
                                 "kernel's own CUDA-event time (for a binned call: the kernel on the call's sorted "
                                 "order, without the sort)"},
            "sets": out, "gpu_bvh": gpu_bvh}
    if emit:
        print(json.dumps(line), flush=True)
    return line


# ---------------------------------------------------------------- compact codecs
COMPACT_CODECS = [("fluv32", "encode"), ("oct32", "encode"), ("oct32_precise", "encode"), ("unsigned32", "encode"),
                  ("unsigned40", "encode"), ("signed48", "encode"), ("fluv32", "decode"), ("oct32", "decode"),
                  ("unsigned32", "decode"), ("unsigned40", "decode"), ("signed48", "decode")]


def cpu_compact_sample(fmts, xyz, codes, target_seconds):
    """The oracle's codecs on a bounded sample: elements per second of each
    codec on one host thread (the crate's codecs are scalar functions)."""
    import numpy as np
    import oracle
    L = oracle.lib()
    out = {}
    per = max(0.05, target_seconds / len(COMPACT_CODECS))
    for name, op in COMPACT_CODECS:
        fmt, size = fmts[name]
        n, done, t0 = 1 << 16, 0, time.perf_counter()
        buf = np.zeros(n * max(size, 12), np.uint8)
        while time.perf_counter() - t0 < per:
            if op == "encode":
                L.psyo_compact_encode(fmt, xyz.ctypes.data, n, buf.ctypes.data, None)
            else:
                L.psyo_compact_decode(fmt, codes[name].ctypes.data, n, buf.ctypes.data)
            done += n
        out["%s_%s" % (name, op)] = done / (time.perf_counter() - t0)
    return out


def run_compact_reference(args):
    """The reference arm of the codec workload: the CPU oracle's fluv32 encode
    (the crate's `fluv32::encode`, restated) on all host threads, each
    thread encoding its share of a bounded batch of the same seeded triples
    (no GPU involved).  Rank 0 alone runs it under torchrun."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    from tests import compact_cases as cc
    rank, _, _ = dist_env()
    if rank != 0:
        return
    L = oracle.lib()
    threads = os.cpu_count() or 1
    n = min(args.elems, 1 << 24)  # a bounded sample of the workload
    host = np.abs(cc.random_triples(n, seed=2025))
    host[~np.isfinite(host)] = 0.0
    out = np.zeros(n * 4, np.uint8)
    fmt = cc.F["fluv32"]
    chunk = (n + threads - 1) // threads

    def part(i):
        lo, hi = i * chunk, min(n, (i + 1) * chunk)
        if hi > lo:
            L.psyo_compact_encode(fmt, host[lo:].ctypes.data, hi - lo, out[4 * lo:].ctypes.data, None)

    with ThreadPoolExecutor(threads) as pool:  # ctypes drops the GIL during the call
        def step():
            list(pool.map(part, range(threads)))
        for _ in range(max(3, args.warmup)):
            step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        secs = time.perf_counter() - t0
    whole = np.zeros(n * 4, np.uint8)  # the threaded split gives the one-call codes (untimed)
    L.psyo_compact_encode(fmt, host.ctypes.data, n, whole.ctypes.data, None)
    if not np.array_equal(out, whole):
        raise RuntimeError("threaded oracle encode differs from one call")
    value = n * args.steps / secs / 1e6
    line = {
        "impl": "reference", "metric": "fluv32 encode Melem/s", "value": value, "unit": "Melem/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/u8", "data": "synthetic (seeded f32 triples over the whole exponent range)",
        "config": {"workload": "compact codecs: %d triples per launch" % args.elems},
        "cpu_baseline": {"value": value, "unit": "Melem/s", "cores": threads, "kind": "port",
                         "sample": "%d triples per step, split over %d host threads" % (n, threads)},
        "e2e": {"value": value, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle (C++ restatement of the compact crate's fluv32); the Rust crate cannot be built here",
    }
    print(json.dumps(line), flush=True)
    return line


def run_compact(args):
    """The `compact` crate's codecs (sub_crates/compact) on the GPU: each
    codec launched on --elems seeded triples (or their codes) resident in HBM,
    larger than L2; per codec the CUDA-event time per launch, M elements/s and
    algorithmic GB/s (12-byte triple + code per element) against the
    measured HBM copy bandwidth.  Every launch's output is compared with the
    oracle on a 1M-element sample.  The headline is fluv32 encode (the codec
    the renderer itself uses for colours); e2e is the same codec through the
    C ABI with the triples in pinned host memory and the codes copied back."""
    import numpy as np
    import torch
    import oracle
    from psychopath_gb300 import abi, build, compact
    from tests import compact_cases as cc
    torch.cuda.set_device(0)
    build.build()
    L = oracle.lib()
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak = float(json.load(open(peaks_path))["hbm_gbs"]) if os.path.exists(peaks_path) else 6800.0
    n = args.elems
    fmts = {name: (cc.F[name], cc.SIZE[cc.F[name]]) for name in cc.F}
    # inputs in each format's domain (what the renderer stores: no NaN; XYZ
    # colours and the unsigned formats non-negative); the out-of-domain
    # paths are covered by the tests
    host = cc.random_triples(n, seed=2025)
    host[~np.isfinite(host)] = 0.0
    host_pos = np.abs(host)
    # unit-vector formats: directions uniform in [-1, 1)^3, as the crate's
    # oct32 property tests draw them (tests/proptest_tests.rs)
    host_dir = np.random.default_rng(2026).uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    unsigned = ("fluv32", "unsigned32", "unsigned40")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    d_xyz = torch.from_numpy(host.view(np.uint8).reshape(-1)).cuda()
    d_pos = torch.from_numpy(host_pos.view(np.uint8).reshape(-1)).cuda()
    d_dir = torch.from_numpy(host_dir.view(np.uint8).reshape(-1)).cuda()
    d_codes = {name: torch.empty(n * size, dtype=torch.uint8, device="cuda") for name, (_, size) in fmts.items()}
    d_out = torch.empty(n * 12, dtype=torch.uint8, device="cuda")
    d_bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    sample = min(n, 1 << 20)
    res, launches = {}, 0
    clocks = ClockSampler(0)
    clocks.start()
    for name, op in COMPACT_CODECS:
        fmt, size = fmts[name]

        src, src_host = ((d_pos, host_pos) if name in unsigned else
                         (d_dir, host_dir) if name.startswith("oct32") else (d_xyz, host))

        def launch():
            if op == "encode":
                compact.encode_device(fmt, src.data_ptr(), n, d_codes[name].data_ptr(), d_bad.data_ptr(),
                                      stream.cuda_stream)
            else:
                compact.decode_device(fmt, d_codes[name].data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)
        for _ in range(max(3, args.warmup)):
            launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            launch()
        e1.record(stream)
        torch.cuda.synchronize()
        launches += args.steps
        sec = e0.elapsed_time(e1) / 1e3 / args.steps
        # parity on the first `sample` elements against the oracle
        if op == "encode":
            got = d_codes[name][:sample * size].cpu().numpy()
            want = np.zeros(sample * size, np.uint8)
            L.psyo_compact_encode(fmt, src_host.ctypes.data, sample, want.ctypes.data, None)
            ok = bool(np.array_equal(got, want))
        else:
            codes = d_codes[name][:sample * size].cpu().numpy()
            got = d_out[:sample * 12].cpu().numpy().view(np.float32)
            want = np.zeros(sample * 3, np.float32)
            L.psyo_compact_decode(fmt, codes.ctypes.data, sample, want.ctypes.data)
            ok = bool(np.all((np.isnan(got) & np.isnan(want)) | (got.view(np.uint32) == want.view(np.uint32))))
        gbs = n * (12 + size) / sec / 1e9
        res["%s_%s" % (name, op)] = {"ms_per_launch": sec * 1e3, "melem_per_s": n / sec / 1e6, "achieved_gbs": gbs,
                                     "frac": gbs / peak, "bit_exact_vs_oracle": ok, "bytes_per_elem": 12 + size}
    # colour records (Color::write_compressed / from_compressed): XYZ,
    # blackbody and temperature colours in equal parts
    from psychopath_gb300.gpu import _check, lib as gpu_lib
    cols = np.zeros(n, abi.color_dtype())
    cols["kind"] = np.arange(n) % 3
    cols["v"] = host_pos
    cols["v"][cols["kind"] != 0, 0] = np.random.default_rng(2027).uniform(1000.0, 12000.0, int((cols["kind"] != 0).sum()))
    d_cols = torch.from_numpy(cols.view(np.uint8)).cuda()
    d_crec = torch.empty(n * 5, dtype=torch.uint8, device="cuda")
    d_cout = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    for op, bytes_per in (("compress", 21), ("decompress", 21)):
        def claunch():
            if op == "compress":
                _check(gpu_lib().psy_color_compress(d_cols.data_ptr(), n, d_crec.data_ptr(), d_bad.data_ptr(),
                                                    stream.cuda_stream))
            else:
                _check(gpu_lib().psy_color_decompress(d_crec.data_ptr(), n, d_cout.data_ptr(), d_bad.data_ptr(),
                                                      stream.cuda_stream))
        for _ in range(max(3, args.warmup)):
            claunch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            claunch()
        e1.record(stream)
        torch.cuda.synchronize()
        launches += args.steps
        sec = e0.elapsed_time(e1) / 1e3 / args.steps
        if op == "compress":
            want = np.zeros(sample * 5, np.uint8)
            L.psyo_color_compress(cols.ctypes.data, sample, want.ctypes.data, None)
            ok = bool(np.array_equal(d_crec[:sample * 5].cpu().numpy(), want))
        else:
            recs = d_crec[:sample * 5].cpu().numpy()
            want = np.zeros(sample, abi.color_dtype())
            L.psyo_color_decompress(recs.ctypes.data, sample, want.ctypes.data, None)
            got = d_cout[:sample * 16].cpu().numpy().view(abi.color_dtype())
            ok = bool(np.array_equal(got["kind"], want["kind"]) and np.array_equal(got["v"], want["v"]))
        gbs = n * bytes_per / sec / 1e9
        res["color_%s" % op] = {"ms_per_launch": sec * 1e3, "melem_per_s": n / sec / 1e6, "achieved_gbs": gbs,
                                "frac": gbs / peak, "bit_exact_vs_oracle": ok, "bytes_per_elem": bytes_per}
    del d_cols, d_crec, d_cout
    clk = clocks.stop()
    invalid_total = int(d_bad.item())
    # e2e: fluv32 encode through the C ABI from pinned host memory, codes back
    pinned_in = torch.from_numpy(host_pos.view(np.uint8).reshape(-1)).pin_memory()
    pinned_out = torch.empty(n * 4, dtype=torch.uint8).pin_memory()
    fmt = abi.PSY_COMPACT_FLUV32

    def e2e_step():
        d_pos.copy_(pinned_in, non_blocking=True)
        compact.encode_device(fmt, d_pos.data_ptr(), n, d_codes["fluv32"].data_ptr(), None, stream.cuda_stream)
        pinned_out.copy_(d_codes["fluv32"], non_blocking=True)
    for _ in range(max(3, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_sec = e0.elapsed_time(e1) / 1e3 / args.steps
    want = np.zeros(sample * 4, np.uint8)
    L.psyo_compact_encode(fmt, host_pos.ctypes.data, sample, want.ctypes.data, None)
    e2e_ok = bool(np.array_equal(pinned_out[:sample * 4].numpy(), want))
    cpu = None
    if not args.no_cpu_baseline:
        codes = {name: d_codes[name][:(1 << 16) * size].cpu().numpy() for name, (_, size) in fmts.items()}
        cpu = cpu_compact_sample(fmts, host_pos[:1 << 16].copy(), codes, min(args.cpu_seconds, 11.0))
    head = res["fluv32_encode"]
    line = {"metric": "fluv32 encode Melem/s", "value": head["melem_per_s"], "unit": "Melem/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": head["ms_per_launch"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/u8",
            "data": "synthetic (seeded f32 triples over the whole exponent range, special values mixed in)",
            "config": {"workload": "compact codecs: %d triples per launch" % n,
                       "l2": "inputs (%d MB of triples) larger than L2" % (n * 12 // 2 ** 20),
                       "inputs": "finite, seeded over the whole exponent range (non-negative for fluv32 and the "
                                 "unsigned formats); oct32: directions uniform in [-1, 1)^3",
                       "invalid_inputs_counted": invalid_total},
            "e2e": {"value": n / e2e_sec / 1e6, "unit": "Melem/s", "h2d_bytes_per_step": n * 12,
                    "d2h_bytes_per_step": n * 4, "bit_exact_vs_oracle": e2e_ok},
            "gpu_launches": launches, "clocks": clk,
            "roofline": {"bound": "hbm", "achieved": head["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": head["frac"], "traffic": None, "kernel": "k_compact<Encode<FLUV32>>",
                         "note": "16 algorithmic bytes per element (12-byte triple in, 4-byte code out) over the "
                                 "kernel's CUDA-event time"},
            "codecs": res}
    if cpu is not None:
        line["cpu_baseline"] = {"value": cpu["fluv32_encode"] / 1e6, "unit": "Melem/s", "cores": 1, "kind": "port",
                                "sample": "the oracle's codecs on 65,536 elements, repeated for about 1 s each",
                                "codecs_melem_per_s": {k: v / 1e6 for k, v in cpu.items()}}
    print(json.dumps(line), flush=True)
    return line


# ---------------------------------------------------------------- serving
def serving_requests(duration, rate, seed=2024):
    """Poisson arrivals: (t, scene, resolution, spp, seed) with the scene
    uniform over the three resident scenes, the resolution uniform over
    {256, 512, 1024} squared and spp uniform over {1, 4, 16, 64}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        out.append((t, int(rng.integers(0, 3)), (256, 512, 1024)[int(rng.integers(0, 3))],
                    (1, 4, 16, 64)[int(rng.integers(0, 4))], int(rng.integers(0, 1 << 30))))


def run_serving(args, emit=True):
    """Three resident scenes (cornell, mesh_stress, motion); requests arrive
    as a Poisson process and are served by psy_submit with host result
    buffers (so every latency includes the result's device-to-host copy).
    Reports p50/p99 latency, aggregate samples/s, and the same requests'
    samples/s when run one at a time on the plain render path."""
    import threading
    import numpy as np
    import torch
    from psychopath_gb300 import build, gpu, scenes
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    build.build()
    sds = [scenes.cornell_box(), scenes.mesh_stress(level=args.level), scenes.motion_instances()]
    names = ["cornell", "mesh_stress", "motion"]
    t0 = time.perf_counter()
    gs = [gpu.Scene(sd, bounds=args.bounds, shading="f32") for sd in sds]
    build_s = time.perf_counter() - t0
    tunes = [g.autotune() for g in gs]  # per-scene launch configuration, kept by the server's lanes
    plain_gs = [gpu.Scene(sd, bounds=args.bounds) for sd in sds]  # f64 shading, default launch
    reqs = serving_requests(args.duration, args.rate)
    offered = sum(r * r * spp for (_, _, r, spp, _) in reqs) / args.duration
    srv = gpu.Server(hbm_budget_bytes=120 * 10**9, wave_paths=args.wave_paths, use_graphs=True, policy=args.policy,
                     aging_ms=args.aging_ms)
    lanes = [srv.add_scene(g) for g in gs]
    # warm-up: capture each lane's graphs, touch the image pool
    for _ in range(max(1, args.warmup)):
        ids = [srv.submit(lanes[k], 256, 256, 4, 1) for k in range(3)]
        for i in ids:
            srv.wait(i)
    base = srv.stats()
    clocks = ClockSampler(local)
    clocks.start()
    ids = [None] * len(reqs)
    start = time.perf_counter()

    def submitter():
        for i, (t, k, res, spp, seed) in enumerate(reqs):
            delay = start + t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids[i] = srv.submit(lanes[k], res, res, spp, seed)

    th = threading.Thread(target=submitter)
    th.start()
    lat, qd, shared, waves = [], [], 0, 0
    for i in range(len(reqs)):
        while ids[i] is None:
            time.sleep(0.0005)
        st = srv.wait(ids[i], timeout=3600.0)
        if st["state"] != 2:
            raise RuntimeError("request %d ended in state %d (error %d)" % (i, st["state"], st["error"]))
        lat.append(st["latency_s"])
        qd.append(st["queued_s"])
        shared += st["shared_waves"] > 0
        waves += st["waves"]
        srv._bufs.pop(ids[i], None)  # release the host result
    end = time.perf_counter()
    th.join()
    clk = clocks.stop()
    stats = srv.stats()
    srv.close()
    samples = sum(r * r * spp for (_, _, r, spp, _) in reqs)
    served = samples / (end - start)
    lat = np.array(lat) * 1e3
    # the same requests one at a time (device image, then the result copied
    # to the host), over a bounded prefix of the list: first with the plain
    # path (f64 shading, default launch), then with the served scenes
    # themselves (f32 shading, the tuned launch) -- served / tuned isolates
    # the batching gain, served / plain adds the precision and launch gains
    dev = torch.empty(1024 * 1024 * 3, dtype=torch.float32, device="cuda")
    host = torch.empty(1024 * 1024 * 3, dtype=torch.float32, pin_memory=False)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def one_at_a_time(scenes_, n_max, seconds):
        samples_, secs_, n_ = 0, 0.0, 0
        for (_, k, res, spp, seed) in reqs[:n_max]:
            if secs_ >= seconds:
                break
            t1 = time.perf_counter()
            scenes_[k].render_sized(res, res, spp, seed, dev.data_ptr(), stream=stream.cuda_stream)
            host[: res * res * 3].copy_(dev[: res * res * 3])
            secs_ += time.perf_counter() - t1
            samples_ += res * res * spp
            n_ += 1
        return samples_, secs_, n_

    p_samples, p_secs, p_n = one_at_a_time(plain_gs, len(reqs), args.plain_seconds)
    t_samples, t_secs, t_n = one_at_a_time(gs, p_n, 1e30)
    plain = p_samples / p_secs
    tuned = t_samples / t_secs
    # the same prefix submitted at once to a fresh server (saturated: the
    # batching gain at full load, whatever the Poisson rate above)
    bsrv = gpu.Server(hbm_budget_bytes=120 * 10**9, wave_paths=args.wave_paths, use_graphs=True, policy=args.policy,
                      aging_ms=args.aging_ms)
    blanes = [bsrv.add_scene(g) for g in gs]
    for k in range(3):  # warm-up: graphs, image pool
        bsrv.wait(bsrv.submit(blanes[k], 256, 256, 4, 1))
    t1 = time.perf_counter()
    bids = [bsrv.submit(blanes[k], res, res, spp, seed) for (_, k, res, spp, seed) in reqs[:p_n]]
    bst = [bsrv.wait(i, timeout=3600.0) for i in bids]
    b_secs = time.perf_counter() - t1
    if any(st["state"] != 2 for st in bst):
        raise RuntimeError("burst request failed")
    blat = np.array([st["latency_s"] for st in bst]) * 1e3
    bsrv.close()
    burst = p_samples / b_secs
    line = {
        "metric": "samples/s (served)", "value": served, "unit": "samples/s", "n_gpus": 1, "steps": len(reqs),
        "warmup": args.warmup, "ms_per_step": (end - start) / max(1, len(reqs)) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes and arrivals)",
        "config": {"workload": "serving: 3 resident scenes (%s), Poisson %.0f req/s for %.0f s (%d requests), "
                               "resolution {256,512,1024}^2, spp {1,4,16,64}, HBM budget 120 GB" %
                               (", ".join(names), args.rate, args.duration, len(reqs)),
                   "bounds": args.bounds, "wave_paths": args.wave_paths, "graphs": True,
                   "policy": args.policy, "aging_ms": args.aging_ms,
                   "form": "served scenes: f32 shading, autotuned launch; plain: f64 shading, default launch",
                   "autotune": tunes, "scene_build_s": round(build_s, 2)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "mean": float(lat.mean()), "max": float(lat.max()),
                       "queued_p50": float(np.percentile(np.array(qd) * 1e3, 50))},
        "offered_samples_per_s": offered,
        "overloaded": offered > served * 1.02,
        "requests_sharing_a_wave": int(shared),
        "plain_one_at_a_time": {"value": plain, "unit": "samples/s", "requests": p_n,
                                "note": "each request alone on the plain path (f64 shading, default launch; "
                                        "render_sized + D2H), a prefix of the same request list"},
        "tuned_one_at_a_time": {"value": tuned, "unit": "samples/s", "requests": t_n,
                                "note": "each request alone on the served scenes themselves (f32 shading, tuned "
                                        "launch), the same prefix: served / this = the batching gain"},
        "served_over_plain": served / plain,
        "served_over_tuned_one_at_a_time": served / tuned,
        "burst": {"value": burst, "unit": "samples/s", "requests": p_n,
                  "over_tuned_one_at_a_time": burst / tuned, "over_plain_one_at_a_time": burst / plain,
                  "latency_ms_p50": float(np.percentile(blat, 50)), "latency_ms_p99": float(np.percentile(blat, 99)),
                  "note": "the same prefix submitted at once: served samples/s at saturation"},
        "e2e": {"value": served, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(r * r * 12 for (_, _, r, _, _) in reqs) / max(1, len(reqs))),
                "note": "psy_submit with host result buffers; latency ends when the image is in host memory"},
        "hbm_peak_bytes": stats["hbm_peak_bytes"],
        "waves": stats["waves"] - base["waves"],
        "gpu_launches": stats["kernel_launches"] - base["kernel_launches"],
        "clocks": clk,
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


# ---------------------------------------------------------------- image parity at full size
def image_errors(img, ref):
    """Relative image RMSE over pixels finite in both, the share of pixels
    with a channel beyond 1e-3 and 1e-2 relative difference, and the
    non-finite pixel counts."""
    import numpy as np
    fin_a, fin_b = np.isfinite(img).all(-1), np.isfinite(ref).all(-1)
    ok = fin_a & fin_b
    a, b = img[ok].astype(np.float64), ref[ok].astype(np.float64)
    rel = float(np.sqrt(np.mean((a - b) ** 2)) / max(1e-30, np.sqrt(np.mean(b ** 2))))
    d = (np.abs(a - b) / np.maximum(np.abs(b), 1e-3)).max(axis=-1)
    return {"rel_rmse": rel, "px_beyond_1e-3": float(np.mean(d > 1e-3)), "px_beyond_1e-2": float(np.mean(d > 1e-2)),
            "nonfinite": [int((~fin_a).sum()), int((~fin_b).sum())]}


def run_parity(args):
    """Image parity at the configurations' sizes: every GPU form of the
    renderer against the CPU oracle (f32, the reference's arithmetic) and the
    FP64 oracle (the same algorithm in f64), on the same scene, seed and
    samples.  Cornell 512x512x16 at 2 and 4 bounces and motion + instancing
    1280x720x32 in full; mesh stress 1920x1080x64 on its central 480x270 crop
    (1/16 of the frame, the icosphere's silhouette and its shadow).  Forms:
    plain (f64 shading, FP32 bounds), optimized (f32 shading, static-scene
    traversal where the scene allows it), fp16 (the optimized form with FP16
    child bounds), gpu_bvh (the optimized form on the GPU-built tree), served
    (the fp16 form through the render server, the frame as one request).
    The launch configuration does not change an image (tested bit for bit),
    so the forms run the default launch apart from the traversal kernel."""
    import numpy as np
    import torch
    from psychopath_gb300 import build, gpu, scenes
    from oracle.runner import OracleScene
    torch.cuda.set_device(0)
    build.build()
    threads = os.cpu_count() or 1
    cases = [("cornell_b2", scenes.cornell_box(max_bounces=2), None),
             ("cornell_b4", scenes.cornell_box(max_bounces=4), None),
             ("motion", scenes.motion_instances(), None),
             ("mesh_stress", scenes.mesh_stress(level=args.level), (720, 405, 1199, 674))]
    out = {}
    for name, sd, crop in cases:
        t0 = time.perf_counter()
        ref, _ = OracleScene(sd).render(threads=threads, crop=crop)
        t1 = time.perf_counter()
        ref64, _ = OracleScene(sd, f64=True).render(threads=threads, crop=crop)
        t2 = time.perf_counter()
        sl = (slice(None), slice(None)) if crop is None else (slice(crop[1], crop[3] + 1), slice(crop[0], crop[2] + 1))
        ref, ref64 = ref[sl], ref64[sl]
        res = {"size": [sd.width, sd.height, sd.spp], "max_bounces": sd.max_bounces,
               "region": "full frame" if crop is None else "crop x %d-%d, y %d-%d" % (crop[0], crop[2], crop[1], crop[3]),
               "oracle_s": round(t1 - t0, 2), "oracle64_s": round(t2 - t1, 2),
               "oracle_vs_oracle64": image_errors(ref, ref64), "forms": {}}
        forms = [("plain", dict(), None), ("optimized", dict(shading="f32"), 3),
                 ("fp16", dict(shading="f32", bounds="fp16"), 3), ("gpu_bvh", dict(shading="f32", bvh="gpu"), 3)]
        imgs = {}
        for fname, kw, mode in forms:
            g = gpu.Scene(sd, **kw)
            if mode is not None:
                g.set_trace(mode, 10)  # falls back to the general kernel where the scene needs it
            img, _ = gpu.Renderer(g).render(crop=crop)
            imgs[fname] = img[sl]
            res["forms"][fname] = {"vs_oracle": image_errors(img[sl], ref), "vs_oracle64": image_errors(img[sl], ref64)}
            if fname == "fp16":
                # the served form: the same scene as a lane of the render server
                srv = gpu.Server(hbm_budget_bytes=120 * 10**9, use_graphs=True)
                lane = srv.add_scene(g)
                rid = srv.submit(lane, sd.width, sd.height, sd.spp, sd.seed)
                st = srv.wait(rid, timeout=3600.0)
                simg = srv.result(rid).reshape(sd.height, sd.width, 3)
                srv.close()
                if st["state"] != 2:
                    raise RuntimeError("served render ended in state %d" % st["state"])
                res["forms"]["served"] = {"vs_oracle": image_errors(simg[sl], ref),
                                          "vs_oracle64": image_errors(simg[sl], ref64),
                                          "identical_to_fp16_form": bool(np.array_equal(simg[sl], img[sl],
                                                                                        equal_nan=True))}
            g.close()
        res["fp16_vs_optimized"] = image_errors(imgs["fp16"], imgs["optimized"])
        out[name] = res
        print(json.dumps({"parity": name, **res}), flush=True)
    worst = max(f["vs_oracle64"]["rel_rmse"] for r in out.values() for f in r["forms"].values())
    line = {"metric": "relative image RMSE vs the FP64 oracle (worst form and configuration)", "value": worst,
            "unit": "relative RMSE", "n_gpus": 1, "higher_is_better": False, "data": "synthetic (seeded scenes)",
            "configs": out}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.workload == "traversal":
        return run_traversal(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "parity":
        return run_parity(args)
    if args.workload == "compact":
        return run_compact_reference(args) if args.impl == "reference" else run_compact(args)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
