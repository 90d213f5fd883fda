"""Benchmark: NEE spectral path tracing of the random-shapes scene on GB300.

Workload (one "step"): the NEE integrator over 500 icospheres (subdivision 2) on a
40 x 40 ground quad with 3 blackbody quad lights, 1024 x 1024 pixels, 64 samples
per pixel, path depth 12, spectral range 380..780 nm, seeded synthetic scene.
Metric: Msamples/s (one sample = one camera path carrying 4 hero wavelengths).
The GPU and the CPU baseline trace the identical samples (same Sobol index and
pixel seed give the same radiance within 1e-4), so at equal spp their images have
equal relMSE. That is measured, not assumed: both arms render the 128 x 128 centre
crop at the step's 64 spp with sample indices 4096..4159 and report the crop's
relMSE against the FP64 oracle fixture (4096 spp, indices 0..4095,
tests/golden/nee_random_shapes_crop128_fp64_4096spp.npz).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload nee|bdpt|serve|denoise] [--no-cpu] [--size S --spp P]

--impl reference times the CPU restatement of the reference integrator (the
oracle library alone, its own tables, all host threads) on a strided subsample of
the same step: every 4th pixel in x and y of the 1024 x 1024 frame with all 64
sample indices.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="nee_random_shapes_500_icospheres", width=1024, height=1024, spp=64, max_depth=12,
                integrator="nee", lambda_nm=[380, 780], scene_seed=0)
METRIC = "Msamples/s (NEE, random-shapes scene, 1024x1024, 64 spp, depth 12, equal relMSE)"
# --workload bdpt: the bidirectional integrator on the caustic box (box layout, 150 icospheres of
# which 60% dispersive dielectrics, 10 sphere lights; ~196k triangles), 512 x 512, 32 spp,
# camera and light subpath depth 10. Its CPU baseline is the oracle's BDPT on a centre crop (BDPT
# couples the pixels of a camera group through their shared light path, so it is not strided).
BDPT_WORKLOAD = dict(workload="bdpt_caustic_box_150_spheres_10_sphere_lights", width=512, height=512, spp=32,
                     max_depth=10, light_vertices=10, integrator="bdpt", lambda_nm=[380, 780], scene_seed=0)
BDPT_METRIC = "Msamples/s (BDPT with MIS, caustic box scene, 512x512, 32 spp, depth 10)"
# --workload serve: the serving loop. 8 resident scene variants of the box layout (about 10k to
# 2M triangles), one trace of requests (resolution from {128,256,512,1024}^2, spp from
# {1,4,16,64}, integrator from {uni, NEE, BDPT}, scene uniform) replayed with Poisson arrivals at
# each rate; every request is also run alone to give its isolated latency.
SERVE_WORKLOAD = dict(workload="serve_poisson_8_box_variants_10k_to_2M_triangles", resolutions=[128, 256, 512, 1024],
                      spp=[1, 4, 16, 64], integrators=["uni", "nee", "bdpt"], rates_per_s=[50, 100, 200, 400, 800],
                      loads=[0.5, 0.8, 1.0], requests=200, max_depth=8, light_vertices=8, lambda_nm=[380, 780], seed=0)
SERVE_METRIC = "serve: Msamples/s at full load with p50/p99 latency (Poisson arrivals, mixed sizes/spp/integrators)"
# --workload denoise: the learned denoiser. Training pairs are rendered by the tracer from 48 seeded
# box scenes (384x216, inputs at 2-32 spp with first-hit features -> 8192-spp targets), the U-Net
# is trained on the GPU with Adam (lr 1e-3 decayed to 1e-5), and a held-out 1920x1080 box scene
# compares the wall time to reach relMSE 1e-3: plain accumulation vs few-spp renders + the
# network, with a per-tile fallback to plain accumulation where the two-half error estimate
# exceeds a threshold; three more held-out scenes (960x544) report the network's relMSE.
DENOISE_WORKLOAD = dict(workload="denoise_unet_box_scenes_1080p", train_scenes=48, train_width=384, train_height=216,
                        train_input_spp=[2, 4, 8, 16, 32], train_target_spp=8192, train_steps=12000, batch=8, crop=128, lr=1e-3,
                        lr_final=1e-5,
                        eval_width=1920, eval_height=1080, eval_reference_spp=65536, eval_seed=100000, integrator="uni",
                        extra_eval_seeds=[100001, 100002, 100003], extra_reference_spp=16384,
                        max_depth=8, tile=64, target_relmse=1e-3, lambda_nm=[380, 780])
DENOISE_METRIC = "denoise: wall-time speed-up to relMSE 1e-3 at 1920x1080 (plain accumulation time / denoised time)"
UNET_FLOP_PER_PIXEL = 2 * 9 * (16 * 32 + 32 * 32 + (32 * 64 + 64 * 64) / 4 + (64 * 128 + 128 * 128) / 16 +
                               (128 * 256 + 256 * 256) / 64 + (384 * 128 + 128 * 128) / 16 + (192 * 64 + 64 * 64) / 4 +
                               (96 * 32 + 32 * 32)) + 2 * 3 * 32
CPU_STRIDE = 4  # bounded CPU sample: every 4th pixel in x and y of the frame, all of the step's spp
BDPT_CPU_CROP = 64  # bounded CPU sample of the BDPT step: a 64 x 64 centre crop, all of the step's spp
GOLDEN = os.path.join(ROOT, "tests", "golden")
FP64_FIXTURE = os.path.join(GOLDEN, "nee_random_shapes_crop128_fp64_4096spp.npz")
RELMSE_EPS = 1e-2  # relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + eps), XYZ


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6699.5), "measured"
    except Exception:
        return 6800.0, "fallback"


def l2_copy_gbs(local):
    """Bandwidth of a copy whose 48 MB (24 MB read, 24 MB written) stay in L2: the
    denominator of the traversal kernel's L2 fraction (its node and triangle bytes hit L1/L2)."""
    import torch
    a = torch.empty(6 << 20, dtype=torch.float32, device="cuda:%d" % local).uniform_()
    b = torch.empty_like(a)
    for _ in range(20):
        b.copy_(a)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        torch.cuda.synchronize()
        e0.record()
        for _ in range(50):
            b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 50 * 2 * a.numel() * 4 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import statistics
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


E2E_MAX_STEPS = 3  # end-to-end steps after the timed ones (at most)


def rank_sample_base(rank, spp, warmup, steps):
    """First sample index of a rank's block: every render a rank makes (warm-up, timed and
    end-to-end steps) takes its own spp indices from the block, so the ranks' samples are
    disjoint and together form one image of (ranks x steps x spp) samples."""
    return rank * spp * (warmup + steps + E2E_MAX_STEPS)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def oracle_handle(scene, params):
    """The oracle (FP32 CPU restatement of the reference integrator) on `scene` with the
    oracle library's own tables: no GPU library is loaded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    return pyoracle.OracleSceneHandle(scene, pyoracle.own_luts()).ensure_rgb_table(params)


def workload_params(spp_start=0, spp=None, crop=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    return pyoracle.render_params(WORKLOAD["integrator"], WORKLOAD["width"], WORKLOAD["height"], spp_start=spp_start,
                                  spp=spp or WORKLOAD["spp"], max_depth=WORKLOAD["max_depth"],
                                  lambda_range=WORKLOAD["lambda_nm"], crop=crop,
                                  light_vertices=WORKLOAD.get("light_vertices", 0))


def cpu_port_rate(handle, threads=None, spp=None):
    """The oracle on a bounded sample of one step: uni/NEE every CPU_STRIDE-th pixel of the
    frame in x and y; BDPT a centre crop. All of the step's sample indices."""
    threads = threads or os.cpu_count() or 1
    spp = spp or WORKLOAD["spp"]
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    if WORKLOAD["integrator"] == "bdpt":
        side = min(BDPT_CPU_CROP, W, H)
        crop = ((W - side) // 2, (H - side) // 2, side, side)
        r = handle.render(workload_params(spp=spp, crop=crop), precision=32, threads=threads, records=False, film=False)
        n = side * side * spp
        what = "%dx%d centre crop x %d spp of the step (%d samples, %.1f s)" % (side, side, spp, n, r["seconds"])
    else:
        r = handle.render_strided(workload_params(spp=spp), CPU_STRIDE, precision=32, threads=threads)
        n = ((W + CPU_STRIDE - 1) // CPU_STRIDE) * ((H + CPU_STRIDE - 1) // CPU_STRIDE) * spp
        what = ("every %dth pixel in x and y of the %dx%d frame x all %d spp of the step (%d samples, %.1f s)"
                % (CPU_STRIDE, W, H, spp, n, r["seconds"]))
    return n / r["seconds"] / 1e6, threads, what


def fixture_name(integrator=None):
    """The FP64 fixture of the current workload rendered with `integrator` (default: the
    workload's own), or None."""
    integrator = integrator or WORKLOAD["integrator"]
    if WORKLOAD["workload"] == BDPT_WORKLOAD["workload"] and (WORKLOAD["width"], WORKLOAD["height"]) == (512, 512):
        return "%s_caustic_box" % integrator
    if WORKLOAD["workload"] == "nee_random_shapes_500_icospheres" and (WORKLOAD["width"], WORKLOAD["height"]) == (1024, 1024):
        return "nee_random_shapes" if integrator == "nee" else None
    return None


def load_fp64_fixture(integrator=None):
    """(mean XYZ, variance of that mean, spec, path) of the FP64 oracle crop of the workload,
    or None when there is none for it."""
    import numpy as np
    name = fixture_name(integrator)
    if name is None:
        return None
    path = os.path.join(GOLDEN, "%s_crop128_fp64_4096spp.npz" % name)
    try:
        z = np.load(path)
    except OSError:
        return None
    return z["mean"].astype(np.float64), z["var_of_mean"].astype(np.float64), json.loads(str(z["spec"])), path


def relmse(img, ref, eps=RELMSE_EPS):
    import numpy as np
    img = np.asarray(img, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref * ref + eps)))


def fp64_judge_params(spec):
    """The judged render: the fixture's crop at the step's spp, with sample indices just past
    the fixture's (so the two estimates are independent)."""
    import copy
    p = workload_params(spp_start=spec["spp_start"] + spec["spp"], spp=WORKLOAD["spp"], crop=spec["crop"])
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    p.integrator = pyoracle.N.INTEGRATORS[spec["integrator"]]
    p.max_depth = spec["max_depth"]
    return p


def cpu_relmse_vs_fp64(handle, threads=None):
    fx = load_fp64_fixture()
    if fx is None:
        return None
    mean, var, spec, _ = fx
    img = handle.render(fp64_judge_params(spec), precision=32, threads=threads or os.cpu_count() or 1, records=False,
                        film=True)["film"]
    return relmse(img, mean)


def gpu_relmse_vs_fp64(ctx, integrator=None):
    """The GPU's render of the fixture's crop at the step's spp against the fixture."""
    import numpy as np
    fx = load_fp64_fixture(integrator)
    if fx is None:
        return None
    mean, var, spec, path = fx
    jp = fp64_judge_params(spec)
    W, H = spec["width"], spec["height"]
    ctx.film_clear(W, H)
    ctx.render(ctx.params(spec["integrator"], W, H, spp_start=jp.spp_start, spp=jp.spp_count, max_depth=spec["max_depth"],
                          lambda_range=spec["lambda_nm"], crop=spec["crop"], light_vertices=spec.get("light_vertices", 0)))
    xyz, _ = ctx.film()
    cx, cy, cw, ch = spec["crop"]
    return {"gpu": relmse(xyz[cy:cy + ch, cx:cx + cw, :3], mean), "cpu": None, "eps": RELMSE_EPS,
            "integrator": spec["integrator"],
            "fixture_noise_term": float(np.mean(var / (mean * mean + RELMSE_EPS))), "crop": spec["crop"],
            "spp": int(jp.spp_count), "sample_indices": [int(jp.spp_start), int(jp.spp_start + jp.spp_count)],
            "fixture": os.path.relpath(path, ROOT), "fixture_spp": spec["spp"]}


def run_reference(args, world, rank):
    from yapt_gb300 import configs
    if rank != 0:
        return
    bdpt = WORKLOAD["integrator"] == "bdpt"
    scene = configs.caustic_box_scene(WORKLOAD["scene_seed"]) if bdpt else configs.random_shapes_scene(WORKLOAD["scene_seed"])
    h = oracle_handle(scene, workload_params())
    for _ in range(args.warmup):
        cpu_port_rate(h, spp=1)
    rates = []
    t0 = time.time()
    for _ in range(args.steps):
        r, threads, sample = cpu_port_rate(h)
        rates.append(r)
    value = sum(rates) / len(rates)
    ms_per_step = (time.time() - t0) * 1e3 / args.steps
    line = {"impl": "reference", "metric": BDPT_METRIC if bdpt else METRIC, "value": value, "unit": "Msamples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(WORKLOAD),
            "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": threads, "kind": "port", "sample": sample,
                             "cpu_model": cpu_model(), "threads": threads},
            "relmse_vs_fp64": cpu_relmse_vs_fp64(h),
            "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import numpy as np
    from yapt_gb300 import configs
    from yapt_gb300 import _native as N
    from yapt_gb300.runtime import Context
    import torch

    torch.cuda.set_device(local)
    bdpt = WORKLOAD["integrator"] == "bdpt"
    scene = configs.caustic_box_scene(WORKLOAD["scene_seed"]) if bdpt else configs.random_shapes_scene(WORKLOAD["scene_seed"])
    ctx = Context(local)
    ctx.upload_scene(scene)
    info = ctx.scene_info()
    W, H, spp = WORKLOAD["width"], WORKLOAD["height"], WORKLOAD["spp"]
    ctx.film_clear(W, H)
    # each rank renders its own block of sample indices of the same image (weak scaling)
    base = rank_sample_base(rank, spp, args.warmup, args.steps)

    def params(step, flags=0):
        return ctx.params(WORKLOAD["integrator"], W, H, spp_start=base + step * spp, spp=spp,
                          max_depth=WORKLOAD["max_depth"], lambda_range=WORKLOAD["lambda_nm"], flags=flags,
                          light_vertices=WORKLOAD.get("light_vertices", 0))

    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    for w in range(args.warmup):
        ctx.render(params(w))
    ctx.synchronize()
    # timed region: device time of each render (CUDA events on the render stream), L2 flushed between steps
    kernel_ms = []
    launches = 0
    rays = 0
    kinds = {}
    time_flag = N.YG_FLAG_TIME_KERNELS
    timed_kinds = list(N.KERNEL_KINDS) + (["connect"] if bdpt else [])
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.time()
        for s in range(args.steps):
            flush.fill_(float(s))
            torch.cuda.synchronize()
            ctx.render(params(args.warmup + s, flags=time_flag))
            st = ctx.last_stats()
            kernel_ms.append(st["ms"])
            launches += st["launches"]
            rays += st["rays"]
            if time_flag:
                kp = ctx.kernel_profile()
                for k in timed_kinds:
                    acc = kinds.setdefault(k, {"ms": 0.0, "launches": 0})
                    acc["ms"] += kp[k]["ms"]
                    acc["launches"] += kp[k]["launches"]
        ctx.synchronize()
        torch.cuda.synchronize()
        wall = time.time() - t0
    barrier(world)
    dev_s = allmax(world, sum(kernel_ms) / 1e3)
    samples_total = allsum(world, float(W * H * spp * args.steps))
    value = samples_total / dev_s / 1e6

    # end to end through the C ABI with host buffers: request in, film out, every step
    xyz = np.zeros((H, W, 3), np.float32)
    barrier(world)
    t1 = time.time()
    e2e_steps = max(1, min(args.steps, E2E_MAX_STEPS))
    for s in range(e2e_steps):
        p = params(args.warmup + args.steps + s)
        ctx.render(p)
        xyz, cnt = ctx.film()
    e2e_s = allmax(world, time.time() - t1)
    e2e_value = allsum(world, float(W * H * spp * e2e_steps)) / e2e_s / 1e6
    h2d = 128 + spp * 256 * 4  # request struct + its Sobol points
    d2h = W * H * 16  # film sums

    peak, peak_kind = read_peaks()
    traffic = None
    if bdpt:
        # per-kind device time of the camera-side kernels from the timed steps; the connection
        # records from one counting render of the same workload. Algorithmic bytes of wbConnect,
        # per record: its (camera slot, light vertex) pair, the camera vertex's surface, context
        # and state, the prepared light vertex (read once per record, as the kernel does; L1/L2
        # serve the repeats), and the record written (origin, direction, target, contribution).
        ctx.render(params(0, flags=N.YG_FLAG_COUNT_TRAVERSAL | N.YG_FLAG_NO_FILM | N.YG_FLAG_TIME_KERNELS))
        kp = ctx.kernel_profile()
        tc = {"nodes": 0, "triangles": 0}
        names = {"trace": "wbTrace", "regroup": "wfClassify+wfRegroup", "shade": "wbShade", "connect": "wbConnect",
                 "shadow": "wbVisibility+wbAccumulate"}
        total_ms = sum(v["ms"] for v in kinds.values())
        records = kp["shadow_rays"] / max(1, kp["connect"]["launches"])
        per_launch_bytes = records * kp["connection_record_bytes"]
        avg_ms = kinds["connect"]["ms"] / max(1, kinds["connect"]["launches"])
        shares = {names[k]: v["ms"] / total_ms for k, v in kinds.items()}
        dominant = {"kernel": "wbConnect", "largest_share": max(shares, key=shares.get), "timed_share_by_kind": shares,
                    "kernels": {"wbConnect": {"records_per_launch": records,
                                              "bytes_per_record": kp["connection_record_bytes"],
                                              "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_ms": avg_ms,
                                              "achieved_gbs": per_launch_bytes / (avg_ms / 1e3) / 1e9,
                                              "share_of_timed_kernels": kinds["connect"]["ms"] / total_ms}}}
    else:
        # per-kind device time from the timed steps; algorithmic bytes from one counting step
        # of the same workload (same kernels, traversal counters on), per bounce:
        #  wfTrace:  rays read (origin and direction of the queued record, 32 B), hits and their
        #            shading-class keys written (20 B + 1 B), wide BVH nodes (80 B) and
        #            triangles (48 B) its rays visit;
        #  regroup:  the move of every record with its hit (key 1 B + record 84 B + hit 20 B read,
        #            104 B written);
        #  wfShade:  (the four class-group launches of a bounce together) per shaded path the
        #            regrouped record and hit read (104 B), the record of every continuing path
        #            written (84 B), the radiance and hero wavelength of every ended path (20 B),
        #            a shadow-queue entry (56 B) per light sample; volume stacks not counted.
        ctx.render(params(0, flags=N.YG_FLAG_COUNT_TRAVERSAL | N.YG_FLAG_NO_FILM | N.YG_FLAG_TIME_KERNELS))
        kp = ctx.kernel_profile()
        tc = {"nodes": kp["closest_nodes"] + kp["shadow_nodes"], "triangles": kp["closest_triangles"] + kp["shadow_triangles"]}
        samples_step = W * H * spp
        R = kp["closest_rays"]
        algo = {
            "trace": (R * (32 + 20 + 1) + kp["closest_nodes"] * 80 + kp["closest_triangles"] * 48),
            "regroup": R * (1 + 104 + 104),
            "shade": (R * 104 + (R - samples_step) * 84 + samples_step * 20 + kp["shadow_rays"] * 56),
        }
        names = {"trace": "wfTrace", "regroup": "wfRegroupQ", "shade": "wfShade"}
        total_ms = sum(v["ms"] for v in kinds.values())
        kernels = {}
        for k in ("trace", "regroup", "shade"):
            nl = max(1, kp[k]["launches"])
            avg = kinds[k]["ms"] / max(1, kinds[k]["launches"])
            kernels[names[k]] = {"algorithmic_bytes_per_launch": algo[k] / nl, "avg_launch_ms": avg,
                                 "achieved_gbs": algo[k] / nl / (avg / 1e3) / 1e9,
                                 "share_of_timed_kernels": kinds[k]["ms"] / total_ms}
        # the traversal's node and triangle bytes come from L1/L2: its fraction of an L2-resident copy
        l2 = l2_copy_gbs(local)
        kernels["wfTrace"]["l2_copy_gbs_measured"] = l2
        kernels["wfTrace"]["l2_frac"] = kernels["wfTrace"]["achieved_gbs"] / l2
        dom = max(kernels, key=lambda n: kernels[n]["share_of_timed_kernels"])
        per_launch_bytes = kernels[dom]["algorithmic_bytes_per_launch"]
        avg_ms = kernels[dom]["avg_launch_ms"]
        dominant = {"kernel": dom, "rays_per_launch": kp["closest_rays"] / max(1, kp["trace"]["launches"]),
                    "timed_share_by_kind": {k: v["ms"] / total_ms for k, v in kinds.items()}, "kernels": kernels}
        try:
            with open(os.path.join(ROOT, "profiles", "path_kernel_traffic.json")) as f:
                tj = json.load(f)
            traffic = tj[dom]["dram_bytes_per_launch"]
            for n in kernels:
                if n in tj:
                    kernels[n]["traffic"] = tj[n]["dram_bytes_per_launch"]
        except (OSError, KeyError, ValueError):
            pass
    achieved = per_launch_bytes / (avg_ms / 1e3) / 1e9
    # equal relMSE, measured: the GPU's and the CPU baseline's render of the FP64 fixture's crop
    # at the step's spp (same sample indices, disjoint from the fixture's), each against the fixture
    judged = gpu_relmse_vs_fp64(ctx) if rank == 0 else None
    versus = None
    if bdpt and rank == 0 and judged is not None:
        # BDPT against NEE at equal relMSE on the caustic box: each integrator's crop at the
        # step's spp against its own FP64 image (the two use different multiple-scattering models
        # on rough dielectrics), and each integrator's device time per sample of the full frame;
        # with relMSE proportional to 1/spp, the time to any common relMSE scales as
        # (time per spp) x relMSE at the step's spp
        nee_j = gpu_relmse_vs_fp64(ctx, "nee")
        ctx.film_clear(W, H)
        nee_ms = []
        for k in range(3):
            ctx.render(ctx.params("nee", W, H, spp_start=base + k * spp, spp=spp, max_depth=WORKLOAD["max_depth"],
                                  lambda_range=WORKLOAD["lambda_nm"]))
            nee_ms.append(ctx.last_stats()["ms"])
        ms_bdpt = sum(kernel_ms) / len(kernel_ms)
        ms_nee = sorted(nee_ms)[1]
        if nee_j is not None:
            versus = {"relmse_bdpt": judged["gpu"], "relmse_nee": nee_j["gpu"], "spp": spp,
                      "ms_per_frame_bdpt": ms_bdpt, "ms_per_frame_nee": ms_nee,
                      "nee_fixture": nee_j["fixture"],
                      "time_to_equal_relmse_bdpt_over_nee": (ms_bdpt * judged["gpu"]) / (ms_nee * nee_j["gpu"])}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        h = oracle_handle(scene, workload_params())
        r, threads, sample = cpu_port_rate(h)
        cpu = {"value": r, "unit": "Msamples/s", "cores": threads, "kind": "port", "sample": sample,
               "cpu_model": cpu_model(), "threads": threads}
        if judged is not None:
            judged["cpu"] = cpu_relmse_vs_fp64(h)
    if rank == 0:
        line = {"metric": BDPT_METRIC if bdpt else METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": sum(kernel_ms) / len(kernel_ms), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(WORKLOAD, triangles=info["triangles"], bvh_nodes=info["nodes"], lights=info["lights"],
                               l2="flushed between steps (256 MB write)",
                               parallelism="replicas: each GPU renders its own sample indices"),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": per_launch_bytes, "dominant": dominant,
                             "nodes_per_sample": tc["nodes"] / (W * H * spp),
                             "triangles_per_sample": tc["triangles"] / (W * H * spp)},
                "cpu_baseline": cpu, "relmse_vs_fp64": judged, "bdpt_vs_nee": versus,
                "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "rays_per_sample": rays / (W * H * spp * args.steps),
                "mrays_per_s": value * rays / (W * H * spp * args.steps),
                "wall_s_timed": wall, "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    ctx.close()


def run_serve(args, world, rank, local):
    import numpy as np
    from yapt_gb300 import configs
    from yapt_gb300.runtime import Context, Server
    if rank != 0:
        return
    W = dict(SERVE_WORKLOAD)
    if args.serve_requests:
        W["requests"] = args.serve_requests
    W["round"] = args.serve_round
    t0 = time.time()
    scenes = [configs.serve_scene(v) for v in range(8)]
    ctxs = []
    for sc in scenes:
        c = Context(local)
        c.upload_scene(sc)
        ctxs.append(c)
    setup_s = time.time() - t0
    rng = np.random.Generator(np.random.PCG64(W["seed"]))
    trace = []
    for i in range(W["requests"]):
        res = int(rng.choice(W["resolutions"]))
        spp = int(rng.choice(W["spp"]))
        integ = str(rng.choice(W["integrators"]))
        scene = int(rng.integers(8))
        p = Context.params(integ, res, res, spp_start=0, spp=spp, max_depth=W["max_depth"],
                           lambda_range=W["lambda_nm"], seed=i, light_vertices=W["light_vertices"])
        trace.append((scene, p, integ, res, spp))
    total_samples = sum(res * res * spp for (_, _, _, res, spp) in trace)
    srv = Server(ctxs, lambda_range=W["lambda_nm"], max_depth=W["max_depth"], memory_budget_bytes=64 << 30,
                 persistent=W["round"] == "persistent")
    # warm-up: compile the merged round's graph and touch every scene
    for s in range(8):
        srv.wait(srv.submit(s, Context.params("nee", 64, 64, spp=1, max_depth=W["max_depth"], lambda_range=W["lambda_nm"])))
    srv.wait(srv.submit(0, Context.params("bdpt", 64, 64, spp=1, max_depth=W["max_depth"], lambda_range=W["lambda_nm"],
                                          light_vertices=W["light_vertices"])))
    # isolated latency of every request (alone on the server)
    iso, iso_res = [], []
    for (scene, p, _, _, _) in trace:
        rid = srv.submit(scene, p)
        info = srv.wait(rid)
        iso.append(info["t_done"] - info["t_submit"])
        iso_res.append(srv.result(rid)[0])
        srv.release(rid)
    per_rate = []
    identical = 0
    compared = 0
    # offered load rho = rate x mean isolated latency: rates at rho 0.5, 0.8 and 1 (full load: the
    # trace's work equals the GPU's capacity), then the configuration's rates (beyond capacity for
    # this trace, whose BDPT requests dominate the work)
    full_load_rate = len(trace) / float(np.sum(iso))
    for rate in [full_load_rate * rho for rho in W["loads"]] + list(W["rates_per_s"]):
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(trace)))
        start = time.time()
        ids = []
        for k, (scene, p, _, _, _) in enumerate(trace):
            delay = arrivals[k] - (time.time() - start)
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(scene, p))
        infos = [srv.wait(r) for r in ids]
        makespan = max(i["t_done"] for i in infos) - min(i["t_submit"] for i in infos)
        lat = np.array([i["t_done"] - i["t_submit"] for i in infos])
        slow = lat / np.array(iso)
        for k, r in enumerate(ids):
            compared += 1
            identical += int(np.array_equal(srv.result(r)[0], iso_res[k]))
            srv.release(r)
        per_rate.append({"rate_per_s": rate, "offered_load": rate / full_load_rate,
                         "p50_latency_s": float(np.percentile(lat, 50)),
                         "p99_latency_s": float(np.percentile(lat, 99)),
                         "p99_latency_over_isolated_p99": float(np.percentile(lat, 99) / np.percentile(iso, 99)),
                         "p50_slowdown": float(np.percentile(slow, 50)), "p99_slowdown": float(np.percentile(slow, 99)),
                         "makespan_s": makespan, "msamples_per_s": total_samples / makespan / 1e6})
    st = srv.stats()
    srv.close()
    for c in ctxs:
        c.close()
    best = per_rate[len(W["loads"]) - 1]  # full load
    line = {"metric": SERVE_METRIC, "value": best["msamples_per_s"], "unit": "Msamples/s", "n_gpus": 1,
            "steps": len(per_rate), "warmup": 9, "full_load_rate_per_s": full_load_rate, "ms_per_step": best["makespan_s"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(W, triangles=[s.triangle_count() for s in scenes], scene_setup_s=setup_s,
                           trace_samples=total_samples),
            "serve": per_rate, "isolated_latency_s": {"p50": float(np.percentile(iso, 50)), "p99": float(np.percentile(iso, 99)),
                                                      "sum": float(np.sum(iso))},
            "results_identical_alone_and_in_mix": "%d/%d" % (identical, compared),
            "server": {k: st[k] for k in ("rounds", "graph_replays", "persistent_rounds", "bdpt_slices", "failed",
                                          "peak_bytes_in_use")}}
    print(json.dumps(line), flush=True)


def run_denoise(args, world, rank, local):
    import numpy as np
    import torch
    from yapt_gb300 import configs
    from yapt_gb300 import denoise as D
    from yapt_gb300.runtime import Context
    if rank != 0:
        return
    W = DENOISE_WORKLOAD
    torch.cuda.set_device(local)
    lam = tuple(W["lambda_nm"])
    ctx = Context(local)
    # -- training data: tracer renders of seeded box scenes
    t0 = time.time()
    pairs = []
    TW, TH = W["train_width"], W["train_height"]
    for seed in range(W["train_scenes"]):
        ctx.upload_scene(configs.box_scene(seed, aspect=TW / TH))
        ref = D.render_reference(ctx, TW, TH, W["train_target_spp"], spp_start=100000, integrator=W["integrator"],
                                 max_depth=W["max_depth"], lambda_range=lam)
        for k, spp in enumerate(W["train_input_spp"]):
            inp = D.render_features(ctx, TW, TH, spp, spp_start=1000 * k, integrator=W["integrator"],
                                    max_depth=W["max_depth"], lambda_range=lam)
            pairs.append((inp, ref))
    data_s = time.time() - t0
    net = D.UNet(seed=0)
    dev = [(D.to_device_input(net, *inp, depth_scale=4.0), torch.from_numpy(np.ascontiguousarray(ref, np.float32).reshape(-1)).cuda(),
            TH, TW) for (inp, ref) in pairs]
    torch.cuda.synchronize()
    t1 = time.time()
    hist = D.train(net, dev, steps=W["train_steps"], batch=W["batch"], crop=W["crop"], lr=W["lr"], seed=1,
                   lr_final=W["lr_final"])
    torch.cuda.synchronize()
    train_s = time.time() - t1
    # -- held-out evaluation scene at 1920x1080
    EW, EH = W["eval_width"], W["eval_height"]
    ctx.upload_scene(configs.box_scene(W["eval_seed"], aspect=EW / EH))
    kw = dict(integrator=W["integrator"], max_depth=W["max_depth"], lambda_range=lam)
    ref = D.render_reference(ctx, EW, EH, W["eval_reference_spp"], spp_start=1 << 20, **kw)

    def plain(spp, start=0):
        torch.cuda.synchronize()
        t = time.time()
        ctx.film_clear(EW, EH)
        ctx.render(ctx.params(W["integrator"], EW, EH, spp_start=start, spp=spp, max_depth=W["max_depth"], lambda_range=lam))
        xyz, _ = ctx.film()
        return xyz @ D.SRGB_FROM_XYZ.T, time.time() - t

    plain_curve = []
    for spp in (4, 16, 64, 256, 1024):
        img, dt = plain(spp)
        plain_curve.append((spp, D.relmse(img, ref), dt))
    # relMSE of plain accumulation ~ c / spp: fit c on the measured points (reference error included)
    c_fit = float(np.median([r * s for (s, r, _) in plain_curve]))
    spp_plain = int(np.ceil(c_fit / W["target_relmse"]))
    img, t_plain = plain(spp_plain)
    r_plain = D.relmse(img, ref)
    tile = W["tile"]

    pipe = D.DenoisePipeline(net, ctx, EH, EW, tile=W["tile"], depth_scale=4.0)

    def denoised(spp):
        # device pipeline: half render A and the full render, the network on both, the per-tile
        # error estimate, plain accumulation of the flagged tiles; the image is read back
        torch.cuda.synchronize()
        t = time.time()
        out, fb = pipe.run(spp, spp_plain, W["target_relmse"], integrator=W["integrator"], max_depth=W["max_depth"],
                           lambda_range=lam)
        dt = time.time() - t
        return out, dt, fb, pipe.tiles

    den_curve = []
    best = None
    denoised(8)  # warm-up (buffers, first launches)
    for spp in (4, 8, 16, 32, 64, 128):
        out, dt, fb, tiles = denoised(spp)
        r = D.relmse(out, ref)
        den_curve.append({"spp": spp, "relmse": r, "seconds": dt, "fallback_tiles": fb, "tiles": tiles})
        # time to the target: the fastest operating point (samples per pixel) that reaches it
        if r <= W["target_relmse"] and (best is None or dt < best["seconds"]):
            best = den_curve[-1]
    # generalisation: further held-out scenes at 960x544 (sides multiples of 8, as the network's
    # three pooling levels need) against 16,384-spp references, the denoised image at 8 and 32
    # spp beside plain accumulation at the same spp
    seeds_eval = []
    SW, SH = 960, 544
    for sd in W["extra_eval_seeds"]:
        ctx.upload_scene(configs.box_scene(sd, aspect=SW / SH))
        sref = D.render_reference(ctx, SW, SH, W["extra_reference_spp"], spp_start=1 << 20, **kw)
        spipe = D.DenoisePipeline(net, ctx, SH, SW, tile=W["tile"], depth_scale=4.0)
        row = {"seed": sd, "width": SW, "height": SH, "reference_spp": W["extra_reference_spp"]}
        for spp in (8, 32):
            out, _ = spipe.run(spp, spp_plain, W["target_relmse"], integrator=W["integrator"], max_depth=W["max_depth"],
                               lambda_range=lam)
            ctx.film_clear(SW, SH)
            ctx.render(ctx.params(W["integrator"], SW, SH, spp=spp, max_depth=W["max_depth"], lambda_range=lam))
            xyz, _ = ctx.film()
            row["denoised_relmse_%dspp" % spp] = D.relmse(out, sref)
            row["plain_relmse_%dspp" % spp] = D.relmse(xyz @ D.SRGB_FROM_XYZ.T, sref)
        seeds_eval.append(row)
    ctx.upload_scene(configs.box_scene(W["eval_seed"], aspect=EW / EH))
    # the reference's own denoiser (edge-stopping a-trous, 5 passes) on the same renders: the
    # render gathers its features, the filter runs on the device, the image is read back
    from yapt_gb300 import _native as N
    from yapt_gb300.runtime import atrous_params
    ap_ = atrous_params()

    def atrous(spp):
        torch.cuda.synchronize()
        t = time.time()
        ctx.film_clear(EW, EH)
        ctx.render(ctx.params(W["integrator"], EW, EH, spp_start=0, spp=spp, max_depth=W["max_depth"], lambda_range=lam,
                              flags=N.YG_FLAG_ATROUS_FEATURES))
        out, _ = ctx.atrous_denoise(ap_)
        return out[..., :3] @ D.SRGB_FROM_XYZ.T, time.time() - t

    atrous(8)  # warm-up
    at_curve, at_best = [], None
    for spp in (4, 8, 16, 32, 64, 128, 256):  # the denoised pipeline's grid, and beyond
        img, dt = atrous(spp)
        r = D.relmse(img, ref)
        at_curve.append({"spp": spp, "relmse": r, "seconds": dt})
        if r <= W["target_relmse"] and (at_best is None or dt < at_best["seconds"]):
            at_best = at_curve[-1]
    # filter time alone at 1080p (prefilter + 5 passes), device events
    ctx.film_clear(EW, EH)
    ctx.render(ctx.params(W["integrator"], EW, EH, spp=4, max_depth=W["max_depth"], lambda_range=lam,
                          flags=N.YG_FLAG_ATROUS_FEATURES))
    a_out = torch.empty((EH, EW, 4), dtype=torch.float32, device="cuda")
    a_var = torch.empty((EH, EW), dtype=torch.float32, device="cuda")
    for _ in range(3):
        N.check(ctx.lib.yg_atrous_denoise(ctx.h, ap_, a_out.data_ptr(), a_var.data_ptr()))
    torch.cuda.synchronize()
    t = time.time()
    for _ in range(10):
        N.check(ctx.lib.yg_atrous_denoise(ctx.h, ap_, a_out.data_ptr(), a_var.data_ptr()))
    atrous_ms = (time.time() - t) * 1e2
    # network throughput at 1080p (3 forward passes measured above; time one more with events)
    packed = D.to_device_input(net, *D.render_features(ctx, EW, EH, 4, **kw), depth_scale=4.0)
    for _ in range(3):
        net.forward(packed, 1, EH, EW)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 10
    for _ in range(reps):
        net.forward(packed, 1, EH, EW)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / reps
    flops = UNET_FLOP_PER_PIXEL * EW * EH
    tflops = flops / (fwd_ms / 1e3) / 1e12
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("bf16_tflops", 1900.0)
        peak_kind = "measured"
    except Exception:
        peak, peak_kind = 1900.0, "fallback"
    speedup = (t_plain / best["seconds"]) if best else None
    line = {"metric": DENOISE_METRIC, "value": speedup, "unit": "x", "n_gpus": 1, "steps": W["train_steps"],
            "warmup": 3, "ms_per_step": train_s * 1e3 / W["train_steps"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": dict(W, plain_spp_for_target=spp_plain, relmse_constant_c=c_fit),
            "plain": {"spp": spp_plain, "seconds": t_plain, "relmse": r_plain,
                      "curve": [{"spp": s_, "relmse": r_, "seconds": d_} for (s_, r_, d_) in plain_curve]},
            "denoised": {"best": best, "curve": den_curve, "held_out_seeds": seeds_eval},
            "atrous_baseline": {"best": at_best, "curve": at_curve, "filter_ms_1080p": atrous_ms,
                                "speedup_to_target": (t_plain / at_best["seconds"]) if at_best else None,
                                "unet_speedup_over_atrous": (at_best["seconds"] / best["seconds"]) if (at_best and best) else None},
            "training": {"data_seconds": data_s, "train_seconds": train_s, "first_loss": float(np.mean(hist[:20])),
                         "last_loss": float(np.mean(hist[-20:]))},
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                         "traffic": None, "peak_source": peak_kind, "kernel": "U-Net forward at 1920x1080 (all layers)",
                         "flop_per_pixel": UNET_FLOP_PER_PIXEL, "forward_ms": fwd_ms}}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--size", type=int, default=0, help="image side for a smaller profiling case")
    ap.add_argument("--spp", type=int, default=0, help="samples per pixel for a smaller profiling case")
    ap.add_argument("--workload", default="nee", choices=["nee", "bdpt", "serve", "denoise"])
    ap.add_argument("--serve-round", default="graph", choices=["graph", "persistent"],
                    help="serve: merged rounds as a captured graph of launches or as one persistent kernel")
    ap.add_argument("--serve-requests", type=int, default=0, help="serve: requests in the trace (0: the workload's)")
    args = ap.parse_args()
    if args.workload == "bdpt":
        WORKLOAD.clear()
        WORKLOAD.update(BDPT_WORKLOAD)
    if args.size:
        WORKLOAD["width"] = WORKLOAD["height"] = args.size
    if args.spp:
        WORKLOAD["spp"] = args.spp
    world, rank, local = dist_setup()
    if args.workload == "denoise":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned denoiser"}), flush=True)
            return
        run_denoise(args, world, rank, local)
        return
    if args.workload == "serve":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop"}), flush=True)
            return
        run_serve(args, world, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
