"""Throughput of the progressive path tracer: path samples/s at 1024^2 on the
512x512x400 head/neck phantom, one GB300.

A step is 16 accumulate-frames of one path per pixel over the 1024x1024 image in
one wavefront pass (vv_record_frames), then the a-trous denoiser and the display
passes once; `per_frame_record` times the reference's shape, one vv_record
(accumulate-frame, a-trous, display) per call. Inputs stay resident in HBM (the density,
mask, normal and label volumes, 1.2 GB, are larger than the 129 MB L2, so no
flush is needed between steps).

  value     device-timed throughput (CUDA events on the renderer's stream)
  e2e       the same through the C ABI with a host readback of the tone-mapped
            RGBA8 image every step (host wall clock)
  roofline  the path tracer: algorithmic bytes per frame (event counts x
            unique element bytes) / the timed region's time per frame,
            against measured HBM
  cpu_baseline  the CPU oracle timed on the host cores on a sample of rows

`--impl reference` times the reference's own shaders compiled as CPU code
(oracle/_ref; the CPU restatement where those were not built) on the same
workload. With torchrun and --gpus N > 1, each rank renders its own replica.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "path samples/s at 1024² on 512²×400 CT (1 GB300); time & p50/p99 latency to fixed RMSE"
UNIT = "path samples/s"
# Luminance RMSE (against the tracer's converged image) the default view of the
# 512x512x400 head/neck workload reaches after 1024 paths per pixel at 1024^2
# (estimated 0.003077; against a 16384-path render of the same view 0.003078).
RMSE_TARGET = 0.003077
RMSE_TARGET_SPP = 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="head_neck", choices=["head_neck", "torso"],
                    help="head_neck: 512x512x400 at 0.5x0.5x1 mm, 1024^2; torso: the precision workload, the "
                         "small phantom scaled to 512x512x800 1 mm voxels, 1920x1080")
    ap.add_argument("--size", type=int, default=0, help="square image side (default: the workload's)")
    ap.add_argument("--dims", default="", help="volume dims x,y,z (default: the workload's)")
    ap.add_argument("--density", default="unorm16", choices=list(DENSITY_FORMATS),
                    help="density storage (vv_precision): the reference's R16_UNORM, or FP16 / BF16 / FP32")
    ap.add_argument("--sums", default="fp32", choices=["fp32", "kahan"], help="running sums (vv_precision)")
    ap.add_argument("--fp64-after", type=int, default=0,
                    help="running sums continue in FP64 past this many paths/pixel (0: never)")
    ap.add_argument("--serve", type=int, default=0,
                    help="instead of the path-tracing bench, run this many render requests (Poisson arrivals "
                         "at --serve-rate per second) over 8 resident phantoms through the request loop")
    ap.add_argument("--serve-rate", type=float, default=40.0)
    ap.add_argument("--serve-modes", default="", help="comma-separated subset of the serving modes")
    ap.add_argument("--denoised-rmse", type=int, default=0,
                    help="instead of the path-tracing bench, train the learned denoiser for this many steps on "
                         "the head/neck workload at 1024^2 and time the fixed RMSE with it on held-out views")
    ap.add_argument("--denoised-train-views", type=int, default=12,
                    help="training views of --denoised-rmse (4 held-out views)")
    ap.add_argument("--bench-denoiser", type=int, default=1000,
                    help="Adam steps of the reduced time-to-RMSE run with the learned denoiser in the default line "
                         "(4 training views, 1 held out, the plain tracer's 256-path error; 0: skip)")
    ap.add_argument("--nn-timing", action="store_true",
                    help="time the learned denoiser's convolution shapes and U-Net forward pass at 1024^2")
    ap.add_argument("--denoiser-study", type=int, default=0,
                    help="instead of the path-tracing bench, train the learned denoiser for this many Adam steps "
                         "on pairs the tracer renders (4 vs 256 paths/pixel) and compare it with a-trous")
    ap.add_argument("--precision-study", type=int, default=0,
                    help="also render the default view to this many paths/pixel with each density storage "
                         "format and report each one's error against FP32 storage (same random streams)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--frames-per-step", type=int, default=16,
                    help="accumulate-frames per step; >1 batches them in one wavefront pass (vv_record_frames)")
    ap.add_argument("--record-steps", type=int, default=10,
                    help="also time this many single-frame vv_record calls (0: skip)")
    ap.add_argument("--ray-march-steps", type=int, default=10,
                    help="also time this many frames of the real-time ray marcher (path tracing off; 0: skip)")
    ap.add_argument("--light-map", action="store_true",
                    help="light with a seeded synthetic 2048x1024 light map (Environment::Map) instead of the studio")
    ap.add_argument("--rmse-requests", type=int, default=6,
                    help="views rendered to the fixed RMSE for the time-to-RMSE latencies (0: skip)")
    ap.add_argument("--rmse-reference-spp", type=int, default=0,
                    help="also render the default view to this many paths/pixel (e.g. 16384) and compare the "
                         "estimated RMSE at the target's paths/pixel with the error against that render")
    ap.add_argument("--rmse-target", type=float, default=RMSE_TARGET,
                    help="luminance RMSE to reach; 0 measures it on the default view at 1024 paths/pixel")
    return ap.parse_args()


DENSITY_FORMATS = {"unorm16": 0, "fp16": 1, "bf16": 2, "fp32": 3}
WORKLOADS = {"head_neck": ("512,512,400", (1024, 1024)), "torso": ("512,512,800", (1920, 1080))}


def dims_of(args):
    return args.dims or WORKLOADS[args.workload][0]


def image_size(args):
    """(width, height) of the workload's image, or args.size square."""
    return (args.size, args.size) if args.size else WORKLOADS[args.workload][1]


def precision_of(args, density=None):
    from volview_gb300 import abi
    fmt = DENSITY_FORMATS[density or args.density]
    return abi.precision(density_format=fmt, sums=abi.SUMS_KAHAN if args.sums == "kahan" else abi.SUMS_FP32,
                         fp64_after=args.fp64_after)


def dist_init(n):
    rank, world, local = 0, 1, 0
    if n > 1 or "WORLD_SIZE" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", 1))
        local = int(os.environ.get("LOCAL_RANK", 0))
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29533")
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def workload(args):
    from volview_gb300 import scene
    dims = tuple(int(v) for v in dims_of(args).split(","))
    W, H = image_size(args)
    if args.workload == "torso":
        return scene.torso_config(seed=1, dims=dims, width=W, height=H, spp=4096)
    return scene.head_neck_config(seed=2, dims=dims, spacing=(0.5, 0.5, 1.0), size=W, spp=1024)


def frame_params(cfg, center, diagonal, light_map=False):
    from volview_gb300 import abi, scene
    # CLI defaults (main.rs): hybrid labels, g = 0.6, a-trous; sagittal cut. The
    # CLI's light map (data/hdri/studio_small_09_2k.hdr) is not shipped, so the
    # reference falls back to the studio; --light-map stands a synthetic one in.
    p = scene.frame_params_for(cfg, center, diagonal, clip_sagittal=True, anisotropy=0.6, spf=1)
    if light_map:
        p.lighting.environment = abi.ENV_MAP
    return p


LIGHT_MAP_SIZE = (2048, 1024)


def light_map():
    from volview_gb300 import scene
    return scene.synthetic_light_map(*LIGHT_MAP_SIZE, seed=11)


def bench_config(args, F):
    W, H = image_size(args)
    volume = (f"head_neck {dims_of(args).replace(',', 'x')} int16 HU at 0.5x0.5x1 mm, 120 labels"
              if args.workload == "head_neck" else
              f"torso {dims_of(args).replace(',', 'x')} int16 HU at 1 mm (the 128^3 phantom's recipe scaled), "
              "10 labels")
    return {"workload": volume + ", soft labels, hybrid mode, sagittal clip, g=0.6, "
                        + ("synthetic 2048x1024 light map" if args.light_map else "studio light")
                        + f", {W}x{H}, "
                        f"1 path/pixel/frame",
            "precision": {"density": args.density, "sums": args.sums, "fp64_after": args.fp64_after},
            "frames_per_step": F,
            "step": ("vv_record_frames: %d accumulate-frames in one wavefront pass, then a-trous and the "
                     "tone-mapped display once" % F) if F > 1 else "vv_record",
            "l2": l2_note(args),
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


L2_BYTES = 129 * 10 ** 6


def volume_bytes(args):
    """Device bytes of the volumes every frame reads: per bricked voxel the
    density (2 bytes, 4 for FP32 storage), the normal (4), the label (1) and
    the label mask (4)."""
    bricked = 1
    for d in dims_of(args).split(","):
        bricked *= -(-int(d) // 8) * 8
    return bricked * ((4 if args.density == "fp32" else 2) + 4 + 1 + 4)


def l2_note(args):
    v = volume_bytes(args)
    if v > L2_BYTES:
        return "inputs larger than L2 (%.2f GB of volumes), no flush between steps" % (v / 1e9)
    return "inputs smaller than L2 (%.0f MB of volumes): steps re-read them from L2" % (v / 1e6)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes per frame of the path-tracing pass on the default workload
# (head/neck 512x512x400, 1024x1024, studio light, UNORM16 density), estimated
# from ncu: each stage kernel's DRAM read + write bytes per unit time, captured
# on the first eight stage launches of a 16-frame pass of the 256x256x200 /
# 512x512 case, times that kernel's time per frame in the full-size launch
# list (gpu__time_duration.sum only). The small case's volumes nearly fit in
# L2, so the volume traffic of the flight and shadow kernels is under-counted.
PASS_TRAFFIC_BYTES_PER_FRAME = 1.148e9


def ncu_traffic(args):
    """The estimate above for the default workload; None for any other."""
    if (args.workload, dims_of(args), image_size(args), args.light_map, args.density) != \
            ("head_neck", "512,512,400", (1024, 1024), False, "unorm16"):
        return None
    return PASS_TRAFFIC_BYTES_PER_FRAME


def cpu_sample(cpu, params, width, height, seconds, ref_lib=None):
    """Times the CPU path tracer on about `seconds` of work: rows spread over the
    frame, or whole frames at successive accumulation indices when one frame
    takes less. Returns (samples/s, paths, threads, seconds, description)."""
    import ctypes as C
    from oracle import oracle as O
    threads = O.threads()
    scene_c = cpu.scene() if ref_lib is None else None
    saved = cpu.accumulated

    def run(rows, accumulated):
        rows = np.ascontiguousarray(rows, np.int32)
        cpu.accumulated = accumulated
        u = cpu.uniforms(params, accumulated + 1, width, height)
        t = time.perf_counter()
        if ref_lib is None:
            O.lib().vvo_pt_rows(O.ptr(u), C.byref(scene_c), O.ptr(cpu.accum), O.ptr(cpu.albedo), O.ptr(cpu.normal),
                                O.ptr(cpu.hdr), O.ptr(rows), len(rows), threads)
        else:
            ref_lib.ref_set_uniforms(O.ptr(u), u.nbytes)
            ref_lib.ref_run_rows(0, width, C.c_void_p(rows.ctypes.data), len(rows), threads)
        return time.perf_counter() - t

    # Calibrate on a few rows spread over the frame, then size the sample.
    probe = np.linspace(0, height - 1, 8).astype(np.int32)
    per_row = max(run(probe, 0) / len(probe), 1e-5)
    n = int(min(height, max(8, seconds / per_row)))
    rows = np.unique(np.linspace(0, height - 1, n).astype(np.int32))
    frames, total, k = 0, 0.0, 0
    while True:
        total += run(rows, k)
        frames += 1
        k += max(int(params.path_tracing.samples_per_frame), 1)
        if len(rows) < height or total >= seconds:
            break
    cpu.accumulated = saved
    paths = frames * len(rows) * width
    what = (f"{frames} frames of {width}x{height}" if len(rows) == height else
            f"{len(rows)} rows spread over the {width}x{height} frame") + f", 1 path/pixel ({paths} paths, {total:.1f} s)"
    return paths / total, paths, threads, total, what


def time_to_rmse(r, params, args, frame, stream):
    """Latency to a fixed RMSE: views picked at random around the volume, each
    accumulated (batched frames, display once per chunk) until the RMSE
    estimated from its accumulation reaches the target; host wall clock from
    the view's first frame to the check that passes, readbacks included."""
    import copy
    from volview_gb300 import convergence as CV
    target = args.rmse_target
    if (args.light_map or args.workload != "head_neck") and target == RMSE_TARGET:
        target = 0.0  # the fixed target is the studio-lit head/neck workload's; measure this one's
    source = "fixed (default view, %d paths/pixel)" % RMSE_TARGET_SPP
    if target <= 0:
        # Measure the target: the default view at RMSE_TARGET_SPP paths per pixel,
        # from a fresh accumulation (resize restarts it).
        r.resize(r.width, r.height)
        done = 0
        while done < RMSE_TARGET_SPP:
            n = min(256, RMSE_TARGET_SPP - done)
            r.record_frames(frame[0], n, params)
            frame[0] += n
            done += n
        assert r.accumulated_samples() == RMSE_TARGET_SPP
        acc, alb, _ = r.read_accumulation()
        target = CV.rmse_estimate(acc, alb, RMSE_TARGET_SPP)
        source = "measured in this run (default view, %d paths/pixel)" % RMSE_TARGET_SPP
    rng = np.random.default_rng(7)
    latencies, spps = [], []
    for _ in range(args.rmse_requests):
        p = copy.deepcopy(params)
        p.camera.yaw = float(params.camera.yaw + rng.uniform(-0.6, 0.6))
        p.camera.pitch = float(params.camera.pitch + rng.uniform(-0.3, 0.3))
        r.synchronize()
        t0 = time.perf_counter()
        chunk = 64
        while True:
            r.record_frames(frame[0], chunk, p)
            frame[0] += chunk
            acc, alb, _ = r.read_accumulation(normal=False)
            n = r.accumulated_samples()
            e = CV.rmse_estimate(acc, alb, n)
            if e <= target:
                break
            chunk = int(min(max(CV.samples_for(e, n, target) - n, 8), 4096))
        latencies.append(time.perf_counter() - t0)
        spps.append(n)
    lat = np.array(latencies)
    return {"target_rmse": target, "target": source, "requests": len(lat),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "paths_per_pixel": spps,
            "views": "seeded random orbits around the default view: yaw +-0.6, pitch +-0.3 rad",
            "error": "luminance RMSE of the accumulation against the tracer's converged image, "
                     "estimated from per-pixel sums of luminance and squared luminance"}


def rmse_against_reference(r, params, args, frame):
    """The estimator checked at full size: the default view at RMSE_TARGET_SPP
    paths/pixel, its estimated RMSE, then the same accumulation continued to
    `args.rmse_reference_spp` and the error of the first image against it. The
    long render contains the short one, so the short image's expected squared
    error against it is s^2 (1/a - 1/N) per pixel; the measured RMSE is scaled by
    1 / sqrt(1 - a/N) to the error against the converged image."""
    from volview_gb300 import convergence as CV
    a, N = RMSE_TARGET_SPP, args.rmse_reference_spp
    p = params  # the time-to-RMSE views before this moved the camera: a new accumulation
    done = 0
    while done < N:
        n = min(1024, (a if done < a else N) - done)
        r.record_frames(frame[0], n, p)
        frame[0] += n
        done += n
        if done == a:
            assert r.accumulated_samples() == a
            acc, alb, _ = r.read_accumulation()
            est = CV.rmse_estimate(acc, alb, a)
            lum_a = acc[..., :3].astype(np.float64) @ CV.LUMA / a
    acc, _, _ = r.read_accumulation()
    lum_n = acc[..., :3].astype(np.float64) @ CV.LUMA / N
    measured = float(np.sqrt(np.mean((lum_a - lum_n) ** 2)) / np.sqrt(1.0 - a / N))
    return {"paths_per_pixel": a, "reference_paths_per_pixel": N, "estimated_rmse": est,
            "rmse_against_reference": measured, "ratio": est / measured}


def run_ours(args, rank, world, local):
    import torch
    from volview_gb300 import abi
    from volview_gb300 import renderer as R
    from volview_gb300.renderer import COUNT_BYTES, COUNT_NAMES
    torch.cuda.set_device(local)
    cfg = workload(args)
    W, H = image_size(args)
    stream = torch.cuda.Stream()
    ctx = R.Context(local, stream=stream.cuda_stream)
    r = R.Renderer(ctx, cfg["volume"], cfg["tf"], precision_of(args))
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    if args.light_map:
        r.set_environment_map(abi.env_struct(light_map()))
    params = frame_params(cfg, list(r.center), r.diagonal, args.light_map)
    r.resize(W, H)
    F = max(args.frames_per_step, 1)
    spf = int(params.path_tracing.samples_per_frame)
    frame = [1]

    def step():
        """One step: F accumulate-frames, then the denoiser and display passes."""
        if F == 1:
            r.record(frame[0], params)
        else:
            r.record_frames(frame[0], F, params)
        frame[0] += F

    def record():
        r.record(frame[0], params)
        frame[0] += 1

    record()  # masks, majorants and the first frame
    # Event counts of one frame (untimed) for the roofline's byte model.
    r.count_events(True)
    record()
    counts = r.count_events(False)
    for _ in range(args.warmup):
        step()
    r.synchronize()
    launches0 = r.kernel_launches()
    barrier(world)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clocks:
        torch.cuda.synchronize()
        r.time_pt(True)
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize()
        pt_ms, pt_launches = r.time_pt(False)
    barrier(world)
    launches = r.kernel_launches() - launches0
    ms = max_over_ranks(start.elapsed_time(end), world)
    samples = args.steps * F * W * H * spf * world
    value = samples / (ms / 1e3)
    # The reference's shape for comparison: one vv_record (one accumulate-frame
    # with the denoiser and display passes) per step.
    per_frame = None
    if args.record_steps > 0:
        for _ in range(2):
            record()
        r.synchronize()
        barrier(world)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s0.record(stream)
        for _ in range(args.record_steps):
            record()
        s1.record(stream)
        torch.cuda.synchronize()
        rms = max_over_ranks(s0.elapsed_time(s1), world)
        per_frame = {"value": args.record_steps * W * H * spf * world / (rms / 1e3), "unit": UNIT,
                     "ms_per_frame": rms / args.record_steps, "steps": args.record_steps,
                     "call": "vv_record (one accumulate-frame + a-trous + display per call)"}
    # e2e through the C ABI: a step plus the tone-mapped RGBA8 readback into
    # pinned host memory, every step (host wall clock).
    e2e = None
    if not args.no_e2e:
        host = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory()
        out = host.numpy()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
            r.read_output(out)
        t1 = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": samples / t1, "unit": UNIT, "h2d_bytes_per_step": 720,
               "d2h_bytes_per_step": W * H * 4,
               "call": "vv_record_frames + vv_read_output" if F > 1 else "vv_record + vv_read_output"}
    ray_march = None
    if args.ray_march_steps > 0:
        # The interactive mode on the same workload: the first frame builds the
        # occlusion and shadow volumes, later frames only march.
        q = __import__("copy").deepcopy(params)
        q.path_tracing.enabled = 0
        s0, s1, s2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        s0.record(stream)
        r.record(frame[0], q)
        s1.record(stream)
        for i in range(args.ray_march_steps):
            r.record(frame[0] + 1 + i, q)
        s2.record(stream)
        torch.cuda.synchronize()
        frame[0] += 1 + args.ray_march_steps
        rm_ms = s1.elapsed_time(s2) / args.ray_march_steps
        ray_march = {"ms_per_frame": rm_ms, "frames_per_s": 1e3 / rm_ms, "first_frame_ms": s0.elapsed_time(s1),
                     "call": "vv_record with path_tracing.enabled = 0 (dvr + display; the first frame also "
                             "builds the occlusion and shadow volumes)"}
    to_rmse = time_to_rmse(r, params, args, frame, stream) if args.rmse_requests > 0 else None
    if args.rmse_reference_spp > 0 and to_rmse is not None:
        to_rmse["check"] = rmse_against_reference(r, params, args, frame)
    # The same fixed error with the learned denoiser, at a reduced scale
    # (untimed by the step; its own wall times).
    denoised = None
    if args.bench_denoiser > 0 and rank == 0 and args.workload == "head_neck" and (W, H) == (1024, 1024):
        denoised = denoised_time_to_rmse(r, params, 4, 1, args.bench_denoiser, plain_spp=256)
    # Roofline of the path-tracing pass (the wavefront stage kernels of a frame).
    # Consecutive passes overlap (one pass's last waves beside the next one's
    # first), so the time per frame is the timed region's, display included.
    alg_bytes = float(sum(counts[n] * b for n, b in zip(COUNT_NAMES, COUNT_BYTES)))
    pt_frame_ms = ms / (args.steps * F)
    achieved = alg_bytes / (pt_frame_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = ncu_traffic(args)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded %s phantom; no CT data ships)" % args.workload.replace("_", "/"),
        "config": bench_config(args, F),
        "gpu_launches": int(launches),
        "path_vertices_per_s": counts["vertex"] / max(counts["pixel"], 1) * value,
        "per_frame_record": per_frame,
        "time_to_rmse": to_rmse,
        "denoised_time_to_rmse": denoised,
        "ray_march": ray_march,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "path-tracing pass (k_wf_* stage kernels), per frame of the timed steps",
                     "peak_source": peak_kind, "alg_bytes_per_frame": alg_bytes,
                     "ms_per_frame": pt_frame_ms, "pass_ms_per_frame": pt_ms / (args.steps * F),
                     "pt_launches": int(pt_launches), "events_per_frame": counts},
        "accumulated_samples": r.accumulated_samples(),
    }
    result["clocks"] = clocks.summary()
    if args.precision_study > 0 and rank == 0:
        result["precision_study"] = precision_study(args, cfg, ctx, stream)
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(cfg, r, params, args)
    r.destroy()
    ctx.destroy()
    if rank == 0:
        print(json.dumps(result))


def precision_study(args, cfg, ctx, stream):
    """The default view at args.precision_study paths/pixel with the density
    stored as FP32, R16_UNORM, FP16 and BF16, and once more as FP32 with Kahan
    running sums (FP64 past 65536): the same random streams in every render, so
    an image's luminance RMSE against the FP32-storage render is the storage
    error (plus the paths whose decisions it flips), set beside the Monte Carlo
    RMSE of the renders themselves."""
    import copy
    import torch
    from volview_gb300 import abi
    from volview_gb300 import convergence as CV
    from volview_gb300 import renderer as R
    W, H = image_size(args)
    spp = args.precision_study
    runs = [("fp32", "fp32", 0), ("unorm16", "fp32", 0), ("fp16", "fp32", 0), ("bf16", "fp32", 0),
            ("fp32", "kahan", 65536)]
    out, ref = {"paths_per_pixel": spp, "reference": "density stored as FP32, plain FP32 running sums"}, None
    for density, sums, fp64_after in runs:
        a = copy.copy(args)
        a.sums, a.fp64_after = sums, fp64_after
        r = R.Renderer(ctx, cfg["volume"], cfg["tf"], precision_of(a, density))
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
        if args.light_map:
            r.set_environment_map(abi.env_struct(light_map()))
        p = frame_params(cfg, list(r.center), r.diagonal, args.light_map)
        r.resize(W, H)
        r.record(1, p)  # masks and majorants
        r.resize(W, H)  # restarts the accumulation
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s0.record(stream)
        done, frame = 0, 2
        while done < spp:
            n = min(64, spp - done)
            r.record_frames(frame, n, p)
            frame, done = frame + n, done + n
        s1.record(stream)
        torch.cuda.synchronize()
        ms = s0.elapsed_time(s1)
        acc, alb, _ = r.read_accumulation(normal=False)
        r.destroy()
        lum = np.asarray(acc[..., :3], np.float64) @ CV.LUMA / spp
        key = density if sums == "fp32" else f"{density}+{sums}+fp64_after_{fp64_after}"
        entry = {"path_samples_per_s": W * H * spp / (ms / 1e3), "mc_rmse": CV.rmse_estimate(acc, alb, spp),
                 "mean_luminance": float(lum.mean())}
        if ref is None:
            ref = (lum, acc)
        else:
            entry["rmse_vs_fp32"] = float(np.sqrt(np.mean((lum - ref[0]) ** 2)))
            if sums != "fp32":
                d = np.abs(acc.astype(np.float64) - ref[1]) / np.maximum(np.abs(ref[1]), 1e-30)
                entry["sums_max_rel_diff"] = float(d[ref[1] != 0].max())
        out[key] = entry
    return out


SERVE_DIMS = [(256, 256, 256), (320, 320, 320), (384, 384, 300), (384, 384, 400), (448, 448, 400),
              (512, 512, 400), (512, 512, 600), (512, 512, 800)]
SERVE_SIZES = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
SERVE_SPP = [16, 64, 256, 1024]


def serve_requests(volumes, n, rate, seed=5):
    """n requests with Poisson arrivals: a resident phantom, an image size and
    paths per pixel drawn uniformly, a random orbit, a sagittal clip plane at a
    random depth (or none) and each label hidden with probability 0.2."""
    from oracle import oracle as O  # geometry of the volumes (host math only)
    from volview_gb300 import abi, scene
    from volview_gb300 import serving as S
    rng = np.random.default_rng(seed)
    names = sorted(volumes)
    t, out = 0.0, []
    for _ in range(n):
        t += rng.exponential(1.0 / rate)
        name = names[rng.integers(len(names))]
        cfg = volumes[name]
        g = O.geometry(cfg["volume"])
        clip = bool(rng.random() < 0.5)
        p = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=clip, anisotropy=0.6, spf=1)
        p.camera.yaw = abi.f32(p.camera.yaw + rng.uniform(-np.pi, np.pi))
        p.camera.pitch = abi.f32(p.camera.pitch + rng.uniform(-0.4, 0.4))
        if clip:
            lo, hi = g.bounds_lo[0], g.bounds_hi[0]
            p.clipping.planes[0].position = abi.f32(lo + (hi - lo) * rng.uniform(0.3, 0.7))
        for label in range(1, 11):
            if rng.random() < 0.2:
                p.labels.colors[label][3] = 0.0
        w, h = SERVE_SIZES[rng.integers(len(SERVE_SIZES))]
        spp = SERVE_SPP[rng.integers(len(SERVE_SPP))]
        out.append(S.Request(name, w, h, spp, p, arrival=t))
    return out


def run_serve(args):
    """The serving workload: 8 resident phantoms (256^3 to 512x512x800), one
    renderer each, requests admitted by device memory and overlapping on the
    device, shortest first with aging (`value`) and in arrival order; the same
    requests one at a time in arrival order for comparison."""
    import copy
    import torch
    from volview_gb300 import scene
    from volview_gb300 import serving as S
    t0 = time.perf_counter()
    volumes = {f"v{i}_{d[0]}x{d[1]}x{d[2]}": scene.torso_config(seed=1 + i, dims=d, soft=False)
               for i, d in enumerate(SERVE_DIMS)}
    gen_s = time.perf_counter() - t0
    free, total = torch.cuda.mem_get_info(0)
    budget = int(free * 0.85)
    result = {"metric": "serving: requests/s and p50/p99 latency, 8 resident phantoms, Poisson arrivals",
              "unit": "requests/s", "higher_is_better": True, "n_gpus": 1, "dtype": "f32",
              "data": "synthetic (seeded phantoms)",
              "config": {"workload": "8 resident phantoms %s, 1 mm voxels; requests: image uniform in %s, "
                                     "paths/pixel uniform in %s, random orbit, sagittal clip at random depth "
                                     "half the time, each label hidden with probability 0.2; Poisson arrivals "
                                     "at %.0f/s" % (SERVE_DIMS, SERVE_SIZES, SERVE_SPP, args.serve_rate),
                         "requests": args.serve, "budget_bytes": budget, "phantom_generation_s": gen_s}}
    modes = (("continuous_shortest_first", dict(order="shortest", aging_s=2.0, max_per_volume=1)),
             ("batched_shortest_first", dict(batched=True, order="shortest", aging_s=2.0)),
             ("continuous_shortest_first_lean", dict(order="shortest", aging_s=2.0, max_per_volume=1, passes=2,
                                                     slot_frames=8)),
             ("continuous_fifo", dict(order="fifo", max_per_volume=1)),
             ("one_at_a_time", dict(order="fifo", max_active=1)))
    if args.serve_modes:
        modes = tuple(m for m in modes if m[0] in args.serve_modes.split(","))
    for mode, kw in modes:
        kw = dict(kw)
        if kw.pop("batched", False):
            # One resident copy of each volume, a view per concurrent request,
            # batched passes of up to 8 requests of a volume (vv_batch_record).
            make_base, make_view, engine, base, view, reserve = S.batched_factory(volumes)
            srv = S.BatchedServer(make_base, make_view, engine, budget, base, view, reserve, **kw)
            for name in volumes:
                srv.preload(name).synchronize()
        else:
            make, base = S.renderer_factory(volumes)
            srv = S.Server(make, base, budget, **kw)
            for name in volumes:
                srv.preload(name)  # resident before the requests come
            for r in list(srv.owned):
                r.synchronize()
        reqs = [copy.copy(q) for q in serve_requests(volumes, args.serve, args.serve_rate)]
        with Clocks(0) as clocks:
            t0 = time.perf_counter()
            done = srv.run(reqs)
            wall = time.perf_counter() - t0
        stats = S.summary(done, wall)
        stats.update({"renderers_created": srv.created, "peak_device_bytes": srv.peak_bytes,
                      "clocks": clocks.summary()})
        if isinstance(srv, S.BatchedServer):
            stats.update({"batched_passes": srv.passes,
                          "mean_requests_per_pass": float(np.mean(srv.batch_sizes)) if srv.batch_sizes else 0.0,
                          "engine_device_bytes": srv.engine.device_bytes()})
        result[mode] = stats
        srv.close()
    first = "continuous_shortest_first" if "continuous_shortest_first" in result else modes[0][0]
    result["value"] = result[first]["requests_per_s"]
    print(json.dumps(result))


NN_SHAPES = [(16, 32), (32, 32), (32, 16), (48, 48), (64, 64), (80, 32), (64, 80)]


def run_nn_timing(args):
    """The learned denoiser's 3x3 convolution at 1024^2 for the shapes the
    U-Net's full-resolution and deeper levels use (vv_nn_conv3x3: tcgen05
    where it takes the shape, mma.sync otherwise), each timed over 20 launches
    after 3 warm-up ones with CUDA events, and the whole U-Net forward pass at
    1024^2 (random weights; the time does not depend on them)."""
    import torch
    from volview_gb300 import learned_denoiser as LD
    from volview_gb300 import renderer as R
    lib = R.load()
    n, h, w = 1, 1024, 1024
    out = {}

    def timed(fn, reps=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for cin, cout in NN_SHAPES:
        X = torch.randn((n, h, w, cin), device="cuda").half()
        W = (torch.randn((cout, 3, 3, cin), device="cuda") * 0.1).half()
        B = torch.zeros(cout, device="cuda")
        Y = torch.empty((n, h, w, cout), device="cuda", dtype=torch.float16)
        ms = timed(lambda: lib.vv_nn_conv3x3(X.data_ptr(), n, h, w, cin, W.data_ptr(), B.data_ptr(), cout, 1,
                                             Y.data_ptr(), None))
        tc = lib.vv_nn_conv3x3_tc(X.data_ptr(), n, h, w, cin, W.data_ptr(), B.data_ptr(), cout, 1, Y.data_ptr(),
                                  None) == 0
        flops = 2.0 * n * h * w * cout * 9 * cin
        out[f"{cin}->{cout}"] = {"us": ms * 1e3, "tflops": flops / ms / 1e9, "path": "tcgen05" if tc else "mma.sync"}
    net = LD.UNet()
    x = torch.zeros((1, 1024, 1024, LD.IN_CHANNELS), dtype=torch.float16, device="cuda")
    unet_ms = timed(lambda: net.forward(x), reps=10)
    flops = sum(2 * 9 * net.shapes[op[1]][0] * net.shapes[op[1]][1] *
                (1024 >> (0 if op[1] == "head" else int(op[1][1]))) ** 2 for op in net.plan if op[0] == "conv")
    print(json.dumps({"metric": "learned denoiser: 3x3 convolution and U-Net forward at 1024^2", "unit": "ms",
                      "higher_is_better": False, "value": unet_ms, "unet_gflop": flops / 1e9,
                      "unet_tflops": flops / (unet_ms / 1e3) / 1e12, "convolutions": out}))


def run_denoiser_study(args):
    """The learned denoiser at a reduced scale of its configuration: the
    head/neck recipe at 256x256x200 (1 x 1 x 2 mm), 256x256 images, 128
    training views (4 paths/pixel in, 256 as target) and 16 held-out views
    (1024 paths/pixel as reference); the U-Net's luminance RMSE beside the raw
    4-path image's and the a-trous filter's, and inference time at 1024^2."""
    import torch
    from volview_gb300 import abi, scene
    from volview_gb300 import learned_denoiser as LD
    from volview_gb300 import renderer as R
    t0 = time.perf_counter()
    cfg = scene.head_neck_config(seed=4, dims=(256, 256, 200), spacing=(1.0, 1.0, 2.0), size=256)
    gen_s = time.perf_counter() - t0
    ctx = R.Context(0)
    r = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    r.resize(256, 256)
    center, diag = list(r.center), r.diagonal
    train_views = LD.random_views(cfg, center, diag, 128, seed=11)
    test_views = LD.random_views(cfg, center, diag, 16, seed=12)
    res = LD.study(r, cfg, train_views, test_views, low_spp=4, train_spp=256, test_spp=1024,
                   steps=args.denoiser_study, batch=4)
    net = res.pop("net")
    # Inference at 1024^2 (features and network), and the a-trous passes there.
    x = torch.zeros((1, 1024, 1024, LD.IN_CHANNELS), dtype=torch.float16, device="cuda")
    for _ in range(3):
        net.forward(x)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        net.forward(x)
    e1.record()
    torch.cuda.synchronize()
    unet_ms = e0.elapsed_time(e1) / 10
    flops = 0
    h = w = 1024
    for op in net.plan:
        if op[0] == "conv":
            cin, cout = net.shapes[op[1]]
            lv = 0 if op[1] == "head" else int(op[1][1])
            flops += 2 * 9 * cin * cout * (h >> lv) * (w >> lv)
    r.destroy()
    ctx.destroy()
    losses = res.pop("losses")
    res.update({"loss_first": losses[0], "loss_last": float(np.mean(losses[-20:])),
                "unet_forward_ms_1024": unet_ms, "unet_gflop_1024": flops / 1e9,
                "unet_tflops_1024": flops / (unet_ms / 1e3) / 1e12, "phantom_generation_s": gen_s})
    print(json.dumps({"metric": "learned denoiser: luminance RMSE at 4 paths/pixel against 1024",
                      "unit": "RMSE", "higher_is_better": False, "value": res["mean_rmse"]["unet"],
                      "config": {"workload": "head/neck recipe 256x256x200 at 1x1x2 mm, 256x256, 128 training "
                                             "views (4 vs 256 paths/pixel), 16 held-out views (1024), %d Adam "
                                             "steps of 4 images" % args.denoiser_study},
                      "study": res}))


def denoised_time_to_rmse(r, base, train_n, test_n, steps, plain_spp=1024):
    """Time to the plain tracer's error at plain_spp paths/pixel with the
    learned denoiser on renderer r (head/neck): the U-Net trained on 256^2
    crops of `train_n` full-size views (4, 16, 64 and 256 paths/pixel in, 1024
    as target); on `test_n` held-out views the plain image at plain_spp
    paths/pixel and the network's output blended per pixel with the raw mean
    by inverse variance, at 4 paths/pixel up to half of plain_spp, against a
    reference of 4096 further, independent paths: the fewest paths/pixel at
    which the blend is as close as the plain image, and the wall times of
    both (render, readback, network). A view the blend does not bring to the
    plain error falls back to plain rendering (1x)."""
    import copy
    from volview_gb300 import abi
    from volview_gb300 import learned_denoiser as LD

    def views(n, seed):
        out = []
        g = np.random.default_rng(seed)
        for _ in range(n):
            p = copy.deepcopy(base)
            p.path_tracing.denoiser = abi.DENOISE_OFF
            p.camera.yaw = abi.f32(base.camera.yaw + g.uniform(-0.6, 0.6))
            p.camera.pitch = abi.f32(base.camera.pitch + g.uniform(-0.3, 0.3))
            out.append(p)
        return out

    t0 = time.perf_counter()
    levels = tuple(k for k in (4, 8, 16, 32, 64, 128, 256, 512) if k <= plain_spp // 2)
    res = LD.time_to_rmse_study(r, views(train_n, 31), views(test_n, 32), levels=levels, plain_spp=plain_spp,
                                steps=steps)
    res.pop("net")
    losses = res.pop("losses")
    res["loss_first"], res["loss_last"] = losses[0], float(np.mean(losses[-20:]))
    spp = [v["spp_to_target"] for v in res["views"]]
    speedup = [v["plain_ms"] / v["denoised_ms"] if v["denoised_ms"] else 1.0 for v in res["views"]]
    return {"metric": "time to the plain tracer's %d-path error with the learned denoiser" % plain_spp,
            "unit": "x faster (wall)", "higher_is_better": True, "value": float(np.median(speedup)),
            "speedup_per_view": speedup, "paths_per_pixel_to_target": spp, "training_views": train_n,
            "held_out_views": test_n, "adam_steps": steps, "seconds": time.perf_counter() - t0,
            "views": "yaw +-0.6, pitch +-0.3 around the default view (training and held-out from different seeds)",
            "study": res}


def run_denoised_rmse(args):
    """denoised_time_to_rmse at full scale: --denoised-train-views training
    views (12 by default), 4 held out."""
    from volview_gb300 import abi
    from volview_gb300 import renderer as R
    cfg = workload(args)
    W, H = image_size(args)
    ctx = R.Context(0)
    r = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    r.resize(W, H)
    base = frame_params(cfg, list(r.center), r.diagonal, args.light_map)
    res = denoised_time_to_rmse(r, base, args.denoised_train_views, 4, args.denoised_rmse)
    r.destroy()
    ctx.destroy()
    res["config"] = {"workload": bench_config(args, 1)["workload"]}
    print(json.dumps(res))


def cpu_renderer_from_device(cfg, r, params):
    """The oracle's CPU renderer with the device's pre-pass volumes (bit-exact or
    within one quantum of the oracle's own, see tests) so only the path tracer
    is timed."""
    from oracle import oracle as O
    from volview_gb300 import abi
    cpu = O.CpuRenderer.__new__(O.CpuRenderer)
    cpu.volume = cfg["volume"]
    cpu.hu = cfg["hu"]
    cpu.dims = tuple(cfg["volume"].dims)
    cpu.geo = O.geometry(cfg["volume"])
    cpu.density = r.read_volume(abi.VOLUME_DENSITY)
    cpu.density_format = r.precision.density_format
    cpu.mask_format = r.precision.mask_format
    cpu.majorants = r.precision.majorants
    cpu.set_transfer_function(cfg["tf"])
    cpu.normals = r.read_volume(abi.VOLUME_NORMALS)
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    cpu.mask = r.read_volume(abi.VOLUME_MASK)
    cpu.majorant = r.read_volume(abi.VOLUME_MAJORANT)
    cpu.env_rad = cpu.env_table = None
    cpu.env_peak_u = 0.0
    if params.lighting.environment == abi.ENV_MAP:
        cpu.set_environment_map(light_map())
    cpu.accumulated = 0
    cpu.accum_key = None
    cpu.resize(r.width, r.height)
    cpu.mask_key = "device"
    return cpu


def cpu_baseline(cfg, r, params, args):
    cpu = cpu_renderer_from_device(cfg, r, params)
    rate, paths, threads, secs, what = cpu_sample(cpu, params, r.width, r.height, args.cpu_seconds)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what}; CPU restatement of pt.comp, pre-pass volumes from the device"}


def run_reference(args, rank, world):
    """The reference's shaders compiled as CPU code on the same workload."""
    if rank != 0:
        return
    from oracle import oracle as O
    from oracle import ref as REF
    cfg = workload(args)
    W, H = image_size(args)
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    if args.light_map:
        cpu.set_environment_map(light_map())
    g = cpu.geo
    params = frame_params(cfg, list(g.center), g.diagonal, args.light_map)
    cpu.resize(W, H)
    kind = "port"
    ref_lib = None
    if REF.available():
        kind = "reference"
        cpu.normals = REF.normals(cpu, cpu._uniforms_geometry_only())
        u = cpu.uniforms(params, 1, W, H)
        cpu.mask = REF.mask(cpu, u, O.mask_margin(cfg["volume"], params.labels), int(params.labels.smoothing))
        cpu.majorant = REF.majorant(cpu, u)
        cpu.mask_key = "reference"
        ref_lib = REF.shader("pt")
        ref_lib.ref_set_uniforms(REF._p(u), 21200)
        REF.bind_common(ref_lib, cpu, np.zeros(16, np.uint8))
        for name, img, fmt in ((b"accum_image", cpu.accum, REF.RGBA32F), (b"guide_albedo_image", cpu.albedo, REF.RGBA32F),
                               (b"guide_normal_image", cpu.normal, REF.RGBA32F), (b"hdr_image", cpu.hdr, REF.RGBA16F)):
            ref_lib.ref_bind_image(name, REF._p(img), fmt, W, H, 1)
        ref_lib.ref_run_rows.argtypes = [__import__("ctypes").c_int, __import__("ctypes").c_int,
                                         __import__("ctypes").c_void_p, __import__("ctypes").c_int,
                                         __import__("ctypes").c_int]
    else:
        cpu.prepare(params, W, H)
    rates = []
    per_step = args.cpu_seconds / max(args.steps, 1) * 4
    for i in range(args.warmup + args.steps):
        rate, paths, threads, secs, what = cpu_sample(cpu, params, W, H, max(per_step, 1.0), ref_lib)
        if i >= args.warmup:
            rates.append((paths, secs, what))
    total_paths = sum(p for p, _, _ in rates)
    total_s = sum(s for _, s, _ in rates)
    value = total_paths / total_s
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / len(rates) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded head/neck phantom)",
        "config": bench_config(args, max(args.frames_per_step, 1)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": O.threads(), "kind": kind,
                         "sample": f"per step {rates[0][2]}; "
                                   + ("shaders/pt.comp compiled as CPU code" if kind == "reference"
                                      else "the port: the oracle's CPU restatement of pt.comp, not the "
                                           "reference's shaders compiled as CPU code (their generated sources "
                                           "are not on this machine); the two agree bit for bit on the "
                                           "committed golden frames")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    args = parse()
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.serve > 0:
        if rank == 0:
            run_serve(args)
    elif args.nn_timing:
        if rank == 0:
            run_nn_timing(args)
    elif args.denoiser_study > 0:
        if rank == 0:
            run_denoiser_study(args)
    elif args.denoised_rmse > 0:
        if rank == 0:
            run_denoised_rmse(args)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
