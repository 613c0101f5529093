"""Benchmark: ms/frame at 1080p at equal MSE against the converged render, learned
candidate proposal vs plain uniform-source RIS, on one GB300.

Workload (config 3 of the benchmark set): 1024^3 fBm terrain (seed 4), 65,536 emitter
voxels (70% in 32 Gaussian blobs, sigma 24) grouped in 256 clusters, 1920x1080, area
lights with solid-angle side sampling, temporal reuse (20x M clamp) and 5-tap / 30-px
spatial reuse, camera on a seeded 300-frame Catmull-Rom path. A step is one frame:
albedo -> candidates (+ proposal inference) + temporal -> spatial -> shading+accumulate.

Quality protocol (untimed setup, --quality full): a converged render (FP64 mean of
--conv-frames frames of the unbiased estimator: spatial and temporal reuse off) at path
frame 150; the proposal's warm start, trained for --train-frames frames along the path on
the plain method's reservoirs; then the plain method at 32 candidates (the reference's
NUMBEROFCANDIDATES) and the learned method at every count in CANDS (and, as "learned2" /
"learned4", at CANDS2 / CANDS4 with one network evaluation per run of up to two / four
consecutive hit pixels on the same voxel side within 2 voxels), the learned views
running --online training steps (65,536 samples each) inside every frame on their own
final reservoirs: per point --mse-seeds views x --mse-frames frames at the static pose,
device ms/frame and per-frame MSE against the converged render. Intervals are 95%
percentile-bootstrap intervals over seeds. The timed configuration is the fastest learned
configuration whose intervals of mean-MSE(learned) / mean-MSE(plain 32) and of
median-MSE(learned) / median-MSE(plain 32) both lie at or below 1 (equal MSE), else plain
at 32; `value` is its device ms/frame over the timed steps along the camera path,
training steps included.

Arms:
  --impl ours       the CUDA path (libvxr.so) - the JSON line's `value` is device time
                    per frame with all inputs resident in HBM; `e2e` goes through the
                    C ABI calls that return each frame's image in page-locked host
                    memory, pipelined (vxr_view_render_to_host_async: frame f + 1 renders
                    while the host waits for image f), and synchronously
                    (vxr_view_render_to_host, `e2e.synchronous`).
  --impl reference  the reference's own render-path kernel source compiled for the
                    host CPU (oracle/_ref, OpenMP over all host threads), else the C
                    restatement; each step renders one whole frame of the same
                    workload (scene and frame constants from host-only code: the
                    CUDA library is not loaded).
Multi-GPU (torchrun): replicas only - every rank renders its own copy of the view.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# clock samples and the autotuner's cache (VXR_BENCH_OUT overrides the folder)
OUT_DIR = os.environ.get("VXR_BENCH_OUT", os.path.join(ROOT, "_build"))
sys.path.insert(0, ROOT)

METRIC = "ms/frame @1080p at equal MSE vs converged: learned proposal vs plain, 1 GB300"
# algorithmic bytes per pixel per stage (each buffer counted once per stage)
BYTES_PER_PX = {
    "albedo": 12,        # W G-buffer 8 + seed 4
    "candidates": 88,    # R G 8 + seed 4 + prev G 8 + prev reservoir 32; W reservoir 32 + seed 4
    "spatial": 80,       # R G 8 + seed 4 + reservoir 32; W reservoir 32 + seed 4
    "shade": 72,         # R G 8 + reservoir 32; W frame 16 + accumulator 16
}
STAGES = ["albedo", "candidates", "spatial", "shade", "accumulate"]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    """dense BF16 TFLOP/s for a kernel timed inside a long step (the sustained figure)"""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if "bf16_tflops_sustained" in d:
            return float(d["bf16_tflops_sustained"]), "measured (sustained)"
    return 1700.0, "fallback (sustained)"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.p = None
        self.path = os.path.join(OUT_DIR, f"clocks_bench_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
        return dist, rank, ws
    return None, 0, 1


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_scene(config):
    import smallproject_gb300 as vx
    desc = vx.scene_preset(config)
    world = vx.World()
    world.generate(desc)
    return vx, desc, world


def cpu_model():
    """The host CPU's model name (lscpu / /proc/cpuinfo), or None."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def probe_cpu_opencl():
    """Whether a CPU OpenCL runtime exists on this host (the reference's own kernels could
    then run unmodified on the host cores): ICD vendor files, an OpenCL loader, and the
    CPU devices of every platform it lists. Enumerates only; creates no context."""
    import ctypes
    import ctypes.util
    import glob
    vendors = sorted(glob.glob("/etc/OpenCL/vendors/*.icd"))
    names = [ctypes.util.find_library("OpenCL")] + sorted(glob.glob("/usr/lib/*/libOpenCL.so*")) + sorted(
        glob.glob("/usr/local/cuda/targets/*/lib/libOpenCL.so*"))
    out = {"icd_vendor_files": vendors, "loader": None, "platforms": [], "cpu_devices": 0}
    for n in names:
        if not n:
            continue
        try:
            lib = ctypes.CDLL(n)
        except OSError:
            continue
        out["loader"] = n
        cnt = ctypes.c_uint(0)
        rc = lib.clGetPlatformIDs(0, None, ctypes.byref(cnt))
        if rc != 0 or cnt.value == 0:
            out["platform_query"] = f"clGetPlatformIDs returned {rc}, {cnt.value} platforms"
            break
        ids = (ctypes.c_void_p * cnt.value)()
        lib.clGetPlatformIDs(cnt.value, ids, None)
        for pid in ids:
            buf = ctypes.create_string_buffer(256)
            lib.clGetPlatformInfo(ctypes.c_void_p(pid), 0x0902, 256, buf, None)   # CL_PLATFORM_NAME
            nd = ctypes.c_uint(0)
            lib.clGetDeviceIDs(ctypes.c_void_p(pid), ctypes.c_ulonglong(2), 0, None, ctypes.byref(nd))  # CPU
            out["platforms"].append({"name": buf.value.decode(errors="replace"), "cpu_devices": nd.value})
            out["cpu_devices"] += nd.value
        break
    out["status"] = ("present" if out["cpu_devices"] else
                     "absent: " + ("no OpenCL loader" if not out["loader"] else "no platform with a CPU device") +
                     ("" if vendors else ", no ICD vendor files"))
    return out


def workload_camera(config, path, f):
    """Camera of frame f of a configuration's workload: config 0 a static camera at
    (128, 160, 0) looking at the world centre; config 1 a 120-frame Catmull-Rom spline;
    config 3 the 300-frame spline. path(seed, f, n) -> (pos, target) is the scene's."""
    if config == 0:
        return (128.0, 160.0, 0.0), (128.0, 128.0, 128.0)
    n = 120 if config == 1 else NFR
    return path(1, f % n, n)


def cpu_arm(config, steps, warmup, W, H):
    """Time the reference's CPU implementation on whole frames of the workload: the
    reference's own kernel source compiled for the host (oracle/_ref, OpenMP over every
    host thread), else the C restatement. The scene, camera path and frame constants come
    from host-only code (oracle/scene_host.cpp with the project's scene generator, the
    oracle's camera restatement): the CUDA library is not loaded. Each step is one frame
    (albedo, candidates + temporal, spatial, shading, accumulation), timed with
    time.perf_counter around the five stage calls, like World::Render's per-stage timers
    (template/world.cpp:2439-2471)."""
    from oracle import binding as ob
    scene = ob.HostScene(config)
    arrays = ob.WorldArrays(scene.grid, scene.bricks, scene.lights)
    kind = "reference" if ob.load_ref() is not None else "port"
    point = config == 0
    r = ob.Renderer("ref" if kind == "reference" else "port", arrays, W, H, point)
    cam = ob.CameraPath(W, H)
    times, stage_s = [], [0.0] * 5
    for f in range(warmup + steps):
        pos, tgt = workload_camera(config, scene.camera_path, f)
        cam.lookat(pos, tgt)
        k = cam.begin(numberOfLights=len(scene.lights), numberOfCandidates=32, numberOfMaxTemporalImportance=20,
                      spatialRadius=30, spatialTaps=5, spatial=1, temporal=1, accumulate=0)
        r.frame_start()
        t0 = time.perf_counter()
        for s in range(1, 6):
            ts = time.perf_counter()
            r.stage(k, s)
            if f >= warmup:
                stage_s[s - 1] += time.perf_counter() - ts
        dt = time.perf_counter() - t0
        cam.end()
        if f >= warmup:
            times.append(dt)
    r.close()
    ms = 1000.0 * sum(times) / len(times)
    info = {"frames": steps, "warmup": warmup, "width": W, "height": H,
            "median_ms": 1000.0 * statistics.median(times),
            "stage_ms": {n: 1000.0 * t / steps for n, t in zip(STAGES, stage_s)},
            "threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())), "cpu_model": cpu_model(),
            "desc": f"{steps} whole {W}x{H} frames of config {config} (after {warmup} untimed), "
                    f"{'point' if point else 'area'} lights, 32 candidates, temporal and spatial reuse"}
    return ms, kind, info


CANDS = (2, 3, 4, 8, 12)
CANDS2 = (2, 3, 4, 8, 12)
# runs of four are the fastest family: 10 and 12 candidates land near plain's frame time,
# where the equal-time comparison is made
CANDS4 = (1, 2, 3, 4, 8, 10, 12)
# hit pixels per network evaluation of each learned family (pixels_per_eval; runs of up to
# eight measured no faster than runs of up to four at config 3)
FAMILY_PPE = {"learned": 1, "learned2": 2, "learned4": 4}
# Compulsory HBM bytes of the temporal kernel per hit pixel: own G-buffer 8, candidate
# reservoir 32 and seed 4 always; the reprojected pixel's previous G-buffer 8 and history
# reservoir 32 when it is on screen (99 % on the camera path); the combined reservoir 32
# and seed 4 written when the history is accepted (58 %) - fractions measured with the
# oracle on four consecutive frames of the path at 480 x 270.
TEMPORAL_BYTES_PER_HIT = 44.0 + 0.99 * 40.0 + 0.58 * 36.0
POSE = 150
KERNEL_PASS_FRAMES = 30   # frames of the per-kernel timing pass (each waited for)
NFR = 300
# DRAM bytes per launch of the dominant kernel from the ncu capture of the 960x540 case
# (profiles/), scaled by 4 to 1920x1080 (the ray count grows with the pixel count)
NCU_TRAFFIC_1080P = {"shadow_candidates": 4 * (71.57e6 + 2.96e6), "shadow_shading": 4 * (62.44e6 + 1.91e6),
                     "ris_candidates": 4 * (10.33e6 + 0.01e6), "albedo": 4 * (33.93e6 + 0.47e6)}


def boot_ci(groups, stat, n=2000, seed=0):
    """Percentile-bootstrap 95% interval of stat over the frames of resampled seeds (each
    group holds one seed's per-frame MSEs: frames of one seed are not independent)."""
    rng = np.random.default_rng(seed)
    k = len(groups)
    vals = [stat(np.concatenate([groups[i] for i in rng.integers(0, k, k)])) for _ in range(n)]
    return [float(np.percentile(vals, 2.5)), float(np.percentile(vals, 97.5))]


def boot_ratio(ga, gb, stat, n=2000, seed=1):
    """95% interval of stat(a) / stat(b), the seeds of each arm resampled independently."""
    rng = np.random.default_rng(seed)
    ka, kb = len(ga), len(gb)
    vals = [stat(np.concatenate([ga[i] for i in rng.integers(0, ka, ka)])) /
            stat(np.concatenate([gb[i] for i in rng.integers(0, kb, kb)])) for _ in range(n)]
    return [float(np.percentile(vals, 2.5)), float(np.percentile(vals, 97.5))]


def decide(table, groups):
    """The quality protocol's decisions over table[key] = {"ms", "mse", "mse_ci95",
    "mse_median", ...} (key "plain_32" or "<family>_<K>") and groups[key] = per-seed arrays
    of per-frame MSEs. Adds each learned point's bootstrap ratio intervals against plain 32
    and returns (equal MSE pick, pick by the mean alone, pick by the median alone, learned
    MSE monotone within the intervals, equal-time point per family, equal-time pick)."""
    p32 = table["plain_32"]
    learned = [k for k in table if k != "plain_32"]
    for k in learned:
        r = table[k]
        r["mse_ratio_ci95"] = boot_ratio(groups[k], groups["plain_32"], np.mean)
        r["median_mse_ratio_ci95"] = boot_ratio(groups[k], groups["plain_32"], np.median)
    # equal MSE: among the learned configurations whose mean-MSE and median-MSE ratios to
    # plain-32 are both at most 1 with 95 % confidence (upper ends of the bootstrap
    # intervals <= 1), the fastest; also the fastest by each criterion alone
    ok_mean = [table[k] for k in learned if table[k]["mse_ratio_ci95"][1] <= 1.0]
    ok_med = [table[k] for k in learned if table[k]["median_mse_ratio_ci95"][1] <= 1.0]
    ok = [r for r in ok_mean if r in ok_med]
    eq = min(ok, key=lambda r: r["ms"]) if ok else None
    eq_mean = min(ok_mean, key=lambda r: r["ms"]) if ok_mean else None
    eq_med = min(ok_med, key=lambda r: r["ms"]) if ok_med else None
    # monotone within the intervals: a larger count is never significantly worse
    cands = sorted(int(k.split("_")[1]) for k in learned if k.startswith("learned_"))
    mono = all(table[f"learned_{b}"]["mse_ci95"][0] <= table[f"learned_{a}"]["mse_ci95"][1]
               for i, a in enumerate(cands) for b in cands[i + 1:])

    # equal time: per family, the learned configuration with the largest ms/frame not above
    # plain's; the headline one is the family whose point is closest to plain's time
    def at_time(fam):
        at = [table[k] for k in learned if k.rsplit("_", 1)[0] == fam and table[k]["ms"] <= p32["ms"]]
        return max(at, key=lambda r: r["ms"]) if at else None

    fams = {f: at_time(f) for f in sorted({k.rsplit("_", 1)[0] for k in learned})}
    ets = [r for r in fams.values() if r is not None]
    et = max(ets, key=lambda r: r["ms"]) if ets else None
    return eq, eq_mean, eq_med, mono, fams, et


def pretrain(vx, world, W, H, tuning, args, desc):
    """The proposal's warm start: trained online along the camera path on the plain
    method's reservoirs (the uniform source is the fallback until the network exists)."""
    trainer = vx.View(world, vx.view_desc(W, H, vx.LIGHTS_AREA, rng_seed=5))
    trainer.set_tuning(tuning)
    trainer.proposal_enable(seed=2, batch=65536, epsilon=args.epsilon)
    t0 = time.perf_counter()
    losses = []
    for f in range(args.train_frames):
        p, t = vx.camera_path(desc, 1, f % NFR, NFR)
        trainer.lookat(p, t)
        trainer.render()
        losses.append(trainer.proposal_train(1))
    trainer.wait()
    train_s = time.perf_counter() - t0
    # device time of one training step (gather, forward, backward, Adam) on its own
    trainer.timer_begin()
    for _ in range(10):
        trainer.proposal_train(1)
    train_step_ms = trainer.timer_end() / 10
    params = trainer.proposal_params()
    trainer.close()
    return params, {"train_frames": args.train_frames, "train_s": train_s, "train_batch": 65536,
                    "train_step_ms": train_step_ms, "loss_first": float(np.mean(losses[:5])),
                    "loss_last": float(np.mean(losses[-5:]))}


def quality_eval(vx, world, desc, W, H, tuning, args, params, online):
    """Converged render, then the MSE / ms table: plain at 32 candidates, learned at every
    count in CANDS with `online` training steps inside each of its frames. Per point
    args.mse_seeds views (seeds) x args.mse_frames frames at the static pose; decisions on
    bootstrap intervals over seeds."""
    pos, tgt = vx.camera_path(desc, 1, POSE, NFR)
    ref = vx.View(world, vx.view_desc(W, H, vx.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=77))
    ref.set_tuning(tuning)
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    t0 = time.perf_counter()
    for _ in range(args.conv_frames):
        ref.render()
        ref.sum64_add()
    ref.wait()
    conv_s = time.perf_counter() - t0
    # learned: one network evaluation per hit pixel; learned2 / 4: per run of up to two /
    # four consecutive hit pixels on the same voxel side within 2 voxels of the run's first
    # (pixels_per_eval: faster inference, the run shares one distribution)
    points = ([("plain", 32)] + [("learned", c) for c in CANDS] + [("learned2", c) for c in CANDS2] +
              [("learned4", c) for c in CANDS4])
    groups, table = {}, {}
    for method, c in points:
        ms_l, per_seed, kms_l = [], [], {}
        for seed in range(args.mse_seeds):
            v = vx.View(world, vx.view_desc(W, H, vx.LIGHTS_AREA, num_candidates=c, rng_seed=1000 + seed))
            v.set_tuning(tuning)
            v.lookat(pos, tgt)
            if method != "plain":
                v.proposal_enable(seed=2, batch=65536, epsilon=args.epsilon,
                                  pixels_per_eval=FAMILY_PPE[method], training_lag=args.training_lag)
                v.proposal_set_params(params)
                v.proposal_use(True)
                v.proposal_online(online)
            for _ in range(8):
                v.render()
            v.wait()
            v.timer_begin()
            for _ in range(8):
                v.render()
            ms_l.append(v.timer_end() / 8)
            v.wait()
            # kernel times over the MSE frames (each waited for by its error read)
            v.kernel_timing(True)
            v.kernel_stats(reset=True)
            e = []
            for _ in range(args.mse_frames):
                v.render()
                e.append(v.error_vs(ref, 0)[0])
            per_seed.append(np.array(e))
            v.kernel_timing(False)
            ks = v.kernel_stats(reset=True)
            for k in ("proposal_infer", "ris_candidates", "proposal_train"):
                if ks[k][1]:
                    kms_l.setdefault(k, []).append(ks[k][0] / ks[k][1])
            v.close()
        key = f"{method}_{c}"
        groups[key] = per_seed
        allf = np.concatenate(per_seed)
        table[key] = {"method": method, "candidates": c, "ms": float(np.median(ms_l)),
                      "mse": float(allf.mean()), "mse_ci95": boot_ci(per_seed, np.mean),
                      "mse_median": float(np.median(allf)), "mse_median_ci95": boot_ci(per_seed, np.median),
                      "frames": int(allf.size), "seeds": len(per_seed),
                      "kernel_ms": {k: float(np.median(x)) for k, x in kms_l.items()}}
    ref.close()
    p32 = table["plain_32"]
    eq, eq_mean, eq_med, mono, fams, et = decide(table, groups)
    return {"pose_frame": POSE, "converged_frames": args.conv_frames, "converged_s": conv_s,
            "epsilon": args.epsilon, "online_steps_per_frame": online,
            "frames_per_point": args.mse_seeds * args.mse_frames, "seeds_per_point": args.mse_seeds,
            "table": table, "plain_reference": p32, "learned_at_equal_mse": eq,
            "learned_at_equal_mean_mse": eq_mean, "learned_at_equal_median_mse": eq_med,
            "learned_mse_monotone_within_ci": mono,
            "decision_rule": "equal MSE: the fastest learned configuration whose bootstrap 95% intervals of "
                             "mean-MSE(learned) / mean-MSE(plain 32) and of median-MSE(learned) / median-MSE(plain 32) "
                             "both lie at or below 1; equal time: per family (learned, learned2 / 4 = one network "
                             "evaluation per run of up to two / four compatible hit pixels) the largest learned "
                             "ms/frame not above plain's, the family whose point is closest to plain's ms/frame",
            "equal_time_per_family": fams,
            "equal_time": None if et is None else {
                "learned": et, "mse_ratio": et["mse"] / p32["mse"], "mse_ratio_ci95": et["mse_ratio_ci95"],
                "median_mse_ratio": et["mse_median"] / p32["mse_median"],
                "median_mse_ratio_ci95": et["median_mse_ratio_ci95"]}}


def config4_learned(vx, world, cams, tuning, args, warmup, W, H):
    """Config 4 with the learned proposal built here (256 emitter clusters, hidden width
    64: config 4 names 4,096 clusters and width 128, which are not built), each 3840x2160
    view on its own stream: a warm start along the views' paths at 960x540 (the network's
    hash grid is in world space), an equal-MSE check at 960x540 on view 0's pose (plain at
    32 against one evaluation per run of up to four at 2, 4 and 8 candidates; 32 seeds x 8
    frames against a 2048-frame converged render; the decision of the config-3 protocol),
    then the four views' frame time at the chosen count (4 when none qualifies, marked so)
    beside plain at 32 on the same per-view streams (host wall time per frame, every view
    waited for)."""
    world.cluster_lights(256, seed=1, iters=6)
    QW, QH = 960, 540
    trainer = vx.View(world, vx.view_desc(QW, QH, vx.LIGHTS_AREA, rng_seed=5))
    trainer.set_tuning(tuning)
    trainer.proposal_enable(seed=2, batch=65536, epsilon=args.epsilon)
    t0 = time.perf_counter()
    for f in range(args.train_frames):
        pos, tgt = cams[f % len(cams)](f // len(cams))
        trainer.lookat(pos, tgt)
        trainer.render()
        trainer.proposal_train(1)
    trainer.wait()
    params = trainer.proposal_params()
    train_s = time.perf_counter() - t0
    trainer.close()

    def learned_view(w_, h_, k, seed):
        v = vx.View(world, vx.view_desc(w_, h_, vx.LIGHTS_AREA, num_candidates=k, rng_seed=seed))
        v.set_tuning(tuning)
        v.proposal_enable(seed=2, batch=65536, epsilon=args.epsilon, pixels_per_eval=4, training_lag=1)
        v.proposal_set_params(params)
        v.proposal_use(True)
        v.proposal_online(1)
        return v

    pos, tgt = cams[0](60)
    ref = vx.View(world, vx.view_desc(QW, QH, vx.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=77))
    ref.set_tuning(tuning)
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    for _ in range(2048):
        ref.render()
        ref.sum64_add()
    ref.wait()
    groups, table = {}, {}
    for method, k in [("plain", 32), ("learned4", 2), ("learned4", 4), ("learned4", 8)]:
        per_seed = []
        for seed in range(32):
            if method == "plain":
                v = vx.View(world, vx.view_desc(QW, QH, vx.LIGHTS_AREA, num_candidates=k, rng_seed=3000 + seed))
                v.set_tuning(tuning)
            else:
                v = learned_view(QW, QH, k, 3000 + seed)
            v.lookat(pos, tgt)
            for _ in range(8):
                v.render()
            e = []
            for _ in range(8):
                v.render()
                e.append(v.error_vs(ref, 0)[0])
            per_seed.append(np.array(e))
            v.close()
        key = f"{method}_{k}"
        groups[key] = per_seed
        allf = np.concatenate(per_seed)
        table[key] = {"method": method, "candidates": k, "ms": float(k), "mse": float(allf.mean()),
                      "mse_ci95": boot_ci(per_seed, np.mean), "mse_median": float(np.median(allf)),
                      "mse_median_ci95": boot_ci(per_seed, np.median), "frames": int(allf.size),
                      "seeds": len(per_seed)}
    ref.close()
    # the fewest candidates that qualify ("ms" holds the count here: fewer is faster)
    eq, _, _, _, _, _ = decide(table, groups)
    for r in table.values():
        r.pop("ms")
    out = {"clusters": 256, "hidden": 64, "train_frames": args.train_frames, "train_s": train_s,
           "quality_960x540": table, "equal_mse_candidates": eq["candidates"] if eq else None}
    k_timed = eq["candidates"] if eq else 4
    out["timed_candidates"] = k_timed
    out["timed_at_equal_mse"] = eq is not None

    def timed(vs):
        """host ms per frame of the views; per-kernel mean ms of view 0 (CUDA events)"""
        step = 20000
        for _ in range(warmup):
            for v, c in zip(vs, cams):
                v.lookat(*c(step))
                v.render()
            step += 1
        for v in vs:
            v.wait()
        vs[0].kernel_timing(True)
        vs[0].kernel_stats(reset=True)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for v, c in zip(vs, cams):
                v.lookat(*c(step))
                v.render()
            step += 1
            for v in vs:
                v.wait()
        ms = (time.perf_counter() - t0) * 1000.0 / args.steps
        vs[0].kernel_timing(False)
        ks = {k: (a / n if n else 0.0) for k, (a, n) in vs[0].kernel_stats(reset=True).items()}
        return ms, ks

    lviews = [learned_view(W, H, k_timed, 5000 + i) for i in range(len(cams))]
    out["learned_views_host_ms_per_frame"], out["learned_view0_kernel_ms"] = timed(lviews)
    for v in lviews:
        v.close()
    pviews = [vx.View(world, vx.view_desc(W, H, vx.LIGHTS_AREA, rng_seed=5000 + i)) for i in range(len(cams))]
    for v in pviews:
        v.set_tuning(tuning)
    out["plain_views_host_ms_per_frame"], out["plain_view0_kernel_ms"] = timed(pviews)
    for v in pviews:
        v.close()
    return out


def run_batch(args, dist, rank, ws, warmup):
    """Configs 2 and 4: several views rendered as one batch per frame (CUDA graph), autotuned."""
    import smallproject_gb300 as vx
    from smallproject_gb300 import autotune as at
    from smallproject_gb300 import workloads as wl
    if args.config == 2:
        worlds, views, descs, specs = wl.build_config2(seed=3)
        cams = wl.config2_cameras(descs, specs, frames=60)
        metric = "ms/frame, 8-view batch (config 2)"
        workload = ("config2: 8 views, worlds {256,512,1024}^3, emitters log-uniform [16, 65536], resolutions "
                    "{360p, 720p, 1080p}, point/area at random, seed 3, one CUDA graph per frame (views in 1, 2 or 4 "
                    "chains of parallel branches: the fastest)")
    else:
        world, views, desc, seeds = wl.build_config4()
        worlds = [world]
        specs = [{"width": v.desc.width, "height": v.desc.height, "light_model": "area", "path_seed": sd}
                 for v, sd in zip(views, seeds)]
        cams = [lambda f, sd=sd: vx.camera_path(desc, sd, f % 120, 120) for sd in seeds]
        metric = "ms/frame, 4 x 3840x2160 batch (config 4, plain method)"
        workload = ("config4: 4 views at 3840x2160, 1024^3 fBm 6 octaves + caves seed 5, 1,048,576 emitters "
                    "(layer + 10% scattered), area lights, plain method, one CUDA graph per frame (views in 1, 2 or 4 "
                    "chains of parallel branches: the fastest)")
    batch = vx.Batch(views, graph=True)
    t, rep = at.autotune_batch(batch, cams, frames=2, rounds=1)
    step = [10000]

    def timed_batch(b):
        """(GPU ms, host ms) per frame of batch b over the timed steps, after warm-up"""
        def frame():
            for v, c in zip(views, cams):
                pos, tgt = c(step[0])
                v.lookat(pos, tgt)
            step[0] += 1
            b.render()

        for _ in range(warmup):
            frame()
        b.wait()
        barrier(dist)
        t0 = time.perf_counter()
        gpu = 0.0
        for _ in range(args.steps):
            frame()
            gpu += b.wait()
        host = (time.perf_counter() - t0) * 1000.0 / args.steps
        barrier(dist)
        return max_over_ranks(dist, gpu / args.steps), host

    # one chain (every stage one launch over all views), then the views split into 2 and 4
    # chains on parallel graph branches, with the tuning found for one chain
    per_chains = {}
    for nc in (1, 2, 4):
        if nc > len(views):
            continue
        b = batch if nc == 1 else vx.Batch(views, graph=True, chains=nc)
        if nc > 1:
            b.set_tuning(t)
        gpu_ms, host_ms = timed_batch(b)
        per_chains[nc] = {"ms": gpu_ms, "host_ms": host_ms}
        if nc > 1:
            b.close()
    best_chains = min(per_chains, key=lambda c: per_chains[c]["ms"])
    ms, wall_ms = per_chains[best_chains]["ms"], per_chains[best_chains]["host_ms"]
    # the same views rendered individually (each on its own stream, all enqueued, then waited)
    for v in views:
        v.set_tuning(t)
    for _ in range(warmup):
        for v, c in zip(views, cams):
            pos, tgt = c(step[0])
            v.lookat(pos, tgt)
            v.render()
        step[0] += 1
    for v in views:
        v.wait()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for v, c in zip(views, cams):
            pos, tgt = c(step[0])
            v.lookat(pos, tgt)
            v.render()
        step[0] += 1
        for v in views:
            v.wait()
    single_wall_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    learned4 = None
    if args.config == 4 and not args.no_learned and rank == 0:
        for v in views:
            v.close()
        batch.close()
        views, batch = [], None
        learned4 = config4_learned(vx, world, cams, t, args, warmup, specs[0]["width"], specs[0]["height"])
    if rank != 0:
        return
    npx = sum(s["width"] * s["height"] for s in specs)
    line = {"metric": metric, "value": ms, "unit": "ms/frame", "n_gpus": ws,
            "steps": args.steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
            "config": {"workload": workload, "views": specs, "pixels": npx},
            "pixels_per_s": npx / (ms * 1e-3), "host_ms_per_frame": wall_ms,
            "chains": best_chains, "per_chains": per_chains,
            "individual_views_host_ms_per_frame": single_wall_ms,
            "tuning": rep["tuning"], "tuning_search": rep}
    if learned4 is not None:
        line["learned"] = learned4
    print(json.dumps(line))
    if batch is not None:
        batch.close()
    for v in views:
        v.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=250)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-steps", type=int, default=10, help="whole frames of the CPU baseline leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="library default launch tuning instead of the autotuner")
    ap.add_argument("--no-small-configs", action="store_true", help="skip the config 0 / config 1 measurements")
    ap.add_argument("--no-learned", action="store_true", help="config 4: skip the learned-proposal measurement")
    ap.add_argument("--quality", choices=["full", "train", "off"], default="full",
                    help="train: train the proposal and time the learned method at --candidates (no converged "
                         "render, no sweep); off: time the plain method at 32 candidates")
    ap.add_argument("--candidates", type=int, default=8, help="candidate count of the learned method (--quality train)")
    ap.add_argument("--conv-frames", type=int, default=4096)
    ap.add_argument("--train-frames", type=int, default=800)
    ap.add_argument("--mse-seeds", type=int, default=96)
    ap.add_argument("--mse-frames", type=int, default=16)
    ap.add_argument("--epsilon", type=float, default=0.1, help="defensive (uniform emitter) share of the proposal")
    ap.add_argument("--online", type=int, default=1, help="proposal training steps inside every learned frame")
    ap.add_argument("--training-lag", type=int, default=1, choices=[0, 1],
                    help="1 (default): a frame's inference uses the weights of the training step two frames back, "
                         "each step overlapping the whole next frame; 0: of the previous frame's step")
    ap.add_argument("--pixels-per-eval", type=int, default=1, choices=[1, 2, 4, 8],
                    help="learned method with --quality train: hit pixels per network evaluation")
    args = ap.parse_args()
    W, H = args.width, args.height
    warmup = max(args.warmup, 3)

    dist, rank, ws = dist_init(args)
    config = {"workload": f"config{args.config}: Voxel ReSTIR {W}x{H}, area lights, temporal 20x clamp, 5 taps / "
                          "30 px spatial, 1024^3 fBm terrain seed 4, 65,536 emitters (70% in 32 blobs) in 256 "
                          "clusters, Catmull-Rom camera path",
              "resolution": [W, H], "scene_config": args.config,
              "l2": "per-frame working set (G-buffers, reservoirs, frame, accumulator: 237 MB at 1080p) exceeds "
                    "the 129 MB L2; no flush between frames"}

    if args.impl == "reference":
        if rank != 0:
            return
        if args.config not in (0, 1, 3):
            print(json.dumps({"impl": "reference", "unavailable": f"config {args.config} is a batch of views: the "
                              "reference renders one view per World"}))
            return
        # whole frames of ~0.85 s each at config 3: at most 30 of them, so the arm stays
        # within a minute whatever --steps the GPU arm times
        ref_steps = min(args.steps, 30)
        ms, kind, sample = cpu_arm(args.config, ref_steps, args.warmup, W, H)
        config["method"] = "plain uniform-source RIS, 32 candidates"
        line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms/frame", "n_gpus": args.gpus,
                "steps": ref_steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
                "config": config,
                "cpu_baseline": {"value": ms, "unit": "ms/frame", "cores": sample["threads"], "kind": kind,
                                 "sample": sample["desc"], "cpu_model": sample["cpu_model"]},
                "stage_ms": sample["stage_ms"], "median_ms": sample["median_ms"],
                "opencl_cpu_runtime": probe_cpu_opencl(),
                "e2e": {"value": ms, "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from smallproject_gb300 import build as B
    B.build()
    if args.config in (2, 4):
        run_batch(args, dist, rank, ws, warmup)
        return
    vx, desc, world = make_scene(args.config)
    world.cluster_lights(256, seed=1, iters=8)
    vdesc = vx.view_desc(W, H, vx.LIGHTS_AREA, accumulate=0)

    def cams(f):
        return vx.camera_path(desc, 1, f % NFR, NFR)

    tuning, tuning_report = vx.tuning(), None
    if not args.no_tune:
        # launch parameters only (results are identical for every tuning); untimed setup
        from smallproject_gb300 import autotune as at
        cache = os.path.join(OUT_DIR, "vxr_tuning.json")
        tuning, tuning_report = at.autotune(world, vdesc, lambda f: cams(1000 + f), frames=4, rounds=2,
                                            cache_path=cache)

    quality, params = None, None
    if args.quality in ("full", "train") and rank == 0:
        params, train_info = pretrain(vx, world, W, H, tuning, args, desc)
        if args.quality == "full":
            quality = quality_eval(vx, world, desc, W, H, tuning, args, params, args.online)
            quality.update(train_info)
        else:
            quality = train_info
    if dist is not None:
        obj = [quality, params]
        dist.broadcast_object_list(obj, src=0)
        quality, params = obj
    share = args.pixels_per_eval
    if args.quality == "train":
        learned, cand = True, args.candidates
        config["method"] = (f"learned proposal, {cand} candidates, {args.online} training step(s) per frame "
                            f"(warm start: {args.train_frames} frames)")
    else:
        eq = quality["learned_at_equal_mse"] if quality else None
        learned = eq is not None
        cand = eq["candidates"] if learned else 32
        share = FAMILY_PPE[eq["method"]] if learned else 1
        config["method"] = (f"learned proposal, {cand} candidates (equal MSE to plain at 32), "
                            f"{f'one network evaluation per run of up to {share} compatible hit pixels, ' if share > 1 else ''}{args.online} "
                            "training step(s) of 65,536 samples inside every frame"
                            f"{' (each used two frames later, overlapping the next frame)' if args.training_lag else ''}"
                            if learned
                            else "plain uniform-source RIS, 32 candidates")

    def make_view(learned_view, c):
        v = vx.View(world, vx.view_desc(W, H, vx.LIGHTS_AREA, accumulate=0, num_candidates=c))
        v.set_tuning(tuning)
        if learned_view:
            v.proposal_enable(seed=2, batch=65536, epsilon=args.epsilon, pixels_per_eval=share,
                              training_lag=args.training_lag)
            v.proposal_set_params(params)
            v.proposal_use(True)
            v.proposal_online(args.online)
        return v

    def timed(view, steps, start):
        for f in range(warmup):
            pos, tgt = cams(start + f)
            view.lookat(pos, tgt)
            view.render()
        view.wait()
        view.stage_stats(reset=True)
        view.kernel_timing(True)
        view.kernel_stats(reset=True)
        barrier(dist)
        view.timer_begin()
        for f in range(steps):
            pos, tgt = cams(start + warmup + f)
            view.lookat(pos, tgt)
            view.render()
        ms = view.timer_end()
        view.wait()
        barrier(dist)
        view.kernel_timing(False)
        return ms

    # the plain method at 32 candidates for context (same path, same tuning)
    plain_ms = None
    if learned:
        pv = make_view(False, 32)
        plain_ms = max_over_ranks(dist, timed(pv, args.steps, 0)) / args.steps
        pv.close()

    view = make_view(learned, cand)
    clocks = None
    for f in range(warmup):
        pos, tgt = cams(f)
        view.lookat(pos, tgt)
        view.render()
    view.wait()
    view.stage_stats(reset=True)
    view.kernel_timing(True)
    view.kernel_stats(reset=True)
    barrier(dist)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if rank == 0 else None
    view.timer_begin()
    for f in range(args.steps):
        pos, tgt = cams(warmup + f)
        view.lookat(pos, tgt)
        view.render()
    ms_total = view.timer_end()
    view.wait()
    barrier(dist)
    clk = clocks.stop() if clocks else None
    view.kernel_timing(False)
    ms_total = max_over_ranks(dist, ms_total)
    ms_frame = ms_total / args.steps
    launches = sum(v[1] for v in view.kernel_stats(reset=True).values())   # in the timed region
    # per-stage and per-kernel times from a separate pass of frames each waited for:
    # back to back, a frame's front half runs beside the previous frame's shading and the
    # training step beside the next frame, so their events would bracket shared time
    view.stage_stats(reset=True)
    view.kernel_timing(True)
    for f in range(KERNEL_PASS_FRAMES):
        pos, tgt = cams(warmup + args.steps + f)
        view.lookat(pos, tgt)
        view.render()
        view.wait()
    view.kernel_timing(False)
    sums, counts = view.stage_stats(reset=True)
    stage_ms = {STAGES[i]: (sums[i] / counts[i] if counts[i] else 0.0) for i in range(5)}
    kstats = view.kernel_stats(reset=True)
    kernel_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in kstats.items()}
    hits, rays_c, rays_s = view.work_counts()
    # the proposal MLP on the tensor cores: its multiply-adds per network evaluation
    # (32 -> H -> H -> H -> K) times the frame's evaluations, over the inference kernel's
    # mean time (which also builds the sampling tables and draws every pixel's candidates)
    mlp = None
    if learned:
        _, K_, H_ = view.proposal_shape()
        rows = view.proposal_rows()
        flop = 2.0 * (32 * H_ + 2 * H_ * H_ + H_ * K_) * rows
        peak_tf, peak_tf_kind = bf16_peak()
        infer_ms = kernel_ms.get("proposal_infer", 0.0)
        if infer_ms > 0:
            tf = flop / (infer_ms * 1e-3) / 1e12
            mlp = {"kernel": "proposal_infer", "bound": "tensor", "evaluations_per_frame": rows,
                   "hit_pixels": hits, "flop_per_launch": flop, "achieved": tf, "peak": peak_tf,
                   "peak_kind": peak_tf_kind, "unit": "TFLOP/s", "frac": tf / peak_tf,
                   "note": "MLP multiply-adds only; the kernel's time also covers the sampling tables and draws "
                           "(ncu: tensor pipe 4.6 - 5.4 % active)"}

    # end to end through the C ABI with page-locked host images: pipelined (frame f + 1
    # renders while the host waits for image f; two host buffers) and synchronous
    # (vxr_view_render_to_host: each frame waits for its own image)
    pinned = [vx.PinnedBuffer(W * H * 4), vx.PinnedBuffer(W * H * 4)]
    e2e_steps = max(5, min(args.steps, 30))

    def e2e_of(v):
        for f in range(3):
            pos, tgt = cams(f)
            v.render_to_host(pos, tgt, pinned[0].array)
        t0 = time.perf_counter()
        prev = None
        for f in range(e2e_steps):
            pos, tgt = cams(f)
            t = v.render_to_host_async(pos, tgt, pinned[f % 2].array)
            if prev is not None:
                v.image_wait(prev)
            prev = t
        v.image_wait(prev)
        piped = (time.perf_counter() - t0) * 1000.0 / e2e_steps
        t0 = time.perf_counter()
        for f in range(e2e_steps):
            pos, tgt = cams(f)
            v.render_to_host(pos, tgt, pinned[0].array)
        sync = (time.perf_counter() - t0) * 1000.0 / e2e_steps
        return max_over_ranks(dist, piped), max_over_ranks(dist, sync)

    e2e_ms, e2e_sync_ms = e2e_of(view)
    img_ok = all(bool(np.isfinite(p.array).all() and p.array.max() > 0) for p in pinned)
    e2e_plain_ms = e2e_plain_sync_ms = None
    if learned:
        pv = make_view(False, 32)
        e2e_plain_ms, e2e_plain_sync_ms = e2e_of(pv)
        pv.close()
    for p in pinned:
        p.close()
    modes = other_modes(make_view, cams, min(args.steps, 30), warmup) if rank == 0 else None
    configs01 = None
    if rank == 0 and not args.no_small_configs:
        def tune_small(w, d):
            if args.no_tune:
                return None
            from smallproject_gb300 import autotune as at
            cam = lambda f: ((128.0 + f, 160.0, 0.0), (128.0, 128.0, 128.0))
            t, _ = at.autotune(w, d, cam, frames=3, rounds=1, cache_path=os.path.join(OUT_DIR, "vxr_tuning.json"))
            return t
        configs01 = small_configs(vx, tune_small, min(args.steps, 30), warmup)

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    npx = W * H
    stage_rooflines = {s: {"ms": stage_ms[s], "GB/s": BYTES_PER_PX[s] * npx / (stage_ms[s] * 1e-3) / 1e9
                           if stage_ms[s] > 0 else 0.0, "frac": (BYTES_PER_PX[s] * npx / (stage_ms[s] * 1e-3) / 1e9)
                           / hbm if stage_ms[s] > 0 else 0.0}
                       for s in ("albedo", "candidates", "spatial", "shade")}
    # dominant kernel (largest share of the timed frames); algorithmic bytes per launch:
    # shadow tracers read the 32-byte request and write at most a 4-byte flag per ray.
    # The training step is left out: in the timed frames it runs on a low-priority side
    # stream in the SM slots the next frame leaves free, off the frame's critical path
    dom = max((k for k in kernel_ms if k != "proposal_train"), key=lambda k: kernel_ms[k] * (kstats[k][1] or 0))
    per_launch_bytes = {"shadow_candidates": 36.0 * rays_c, "shadow_shading": 36.0 * rays_s,
                        "ris_candidates": 80.0 * hits, "albedo": 12.0 * npx, "spatial": 80.0 * npx,
                        "proposal_infer": 8.0 * hits + 8.0 * cand * hits, "temporal": TEMPORAL_BYTES_PER_HIT * hits,
                        "shade_finish": 72.0 * npx, "shade_request": 72.0 * hits, "compact_hits": 12.0 * npx,
                        "accumulate": 48.0 * npx}
    ab = per_launch_bytes.get(dom, 0.0)
    achieved = ab / (kernel_ms[dom] * 1e-3) / 1e9 if kernel_ms[dom] > 0 else 0.0
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": f"of {peak_kind}",
                "traffic": NCU_TRAFFIC_1080P.get(dom) if (W, H) == (1920, 1080) else None,
                "bytes_per_launch": ab,
                "note": "the DDA is latency / ALU bound (L2-resident bricks), not HBM bound: see rays_per_s"}
    rays = hits + rays_c + rays_s
    # the reservoir passes against the HBM roofline (bytes per unit: see TEMPORAL_BYTES_PER_HIT
    # and the kernels' docstrings in DESIGN)
    reservoir_roofline = {}
    for k in ("temporal", "spatial", "shade_finish", "shade_request"):
        if kernel_ms.get(k, 0.0) > 0:
            gbs = per_launch_bytes[k] / (kernel_ms[k] * 1e-3) / 1e9
            reservoir_roofline[k] = {"ms": kernel_ms[k], "bytes_per_launch": per_launch_bytes[k], "GB/s": gbs,
                                     "frac": gbs / hbm}
    cpu = None
    if not args.no_cpu_baseline:
        cms, kind, sample = cpu_arm(args.config, args.cpu_steps, 1, W, H)
        cpu = {"value": cms, "unit": "ms/frame", "cores": sample["threads"], "kind": kind, "sample": sample["desc"],
               "cpu_model": sample["cpu_model"]}
    # replicas: every rank renders its own view; the job's frame time is the slowest
    # rank's, and the job delivers ws frames per frame time
    value = ms_frame
    line = {"metric": METRIC, "value": value, "unit": "ms/frame", "n_gpus": ws, "steps": args.steps,
            "warmup": warmup, "ms_per_step": ms_frame, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": config, "plain_ms_per_frame": plain_ms if learned else ms_frame,
            "stage_ms": stage_ms, "kernel_ms": kernel_ms, "stage_roofline": stage_rooflines,
            "rays_per_frame": rays, "rays_per_s": rays / (ms_frame * 1e-3),
            "roofline": roofline, "reservoir_roofline": reservoir_roofline, "mlp_roofline": mlp,
            "cpu_baseline": cpu, "quality": quality,
            "frames_per_s_job": ws * 1000.0 / ms_frame,
            "e2e": {"value": e2e_ms, "unit": "ms/frame", "h2d_bytes_per_step": 4 * 176,
                    "d2h_bytes_per_step": npx * 16, "image_ok": img_ok, "pipelined": True,
                    "synchronous": e2e_sync_ms,
                    "plain_32": e2e_plain_ms if learned else e2e_ms,
                    "plain_32_synchronous": e2e_plain_sync_ms if learned else e2e_sync_ms},
            "gpu_launches": launches, "clocks": clk,
            "tuning": view.get_tuning().as_dict(), "tuning_search": tuning_report,
            "modes": modes, "configs_0_1": configs01, "world_commit": world_commit_times(world, args)}
    print(json.dumps(line))
    view.close()


def small_configs(vx, tuning_fn, steps, warmup):
    """Configs 0 and 1 of the benchmark set on the GPU (plain method, 32 candidates):
    config 0 - 256^3 fBm terrain (seed 1), 64 emitters, point lights, 640x360, static
    camera; config 1 - 1024^3 terrain (seed 2), 4,096 emitters in the air, area lights,
    1280x720, 120-frame spline. ms/frame and per-kernel ms over `steps` frames; config 0
    also the reference's kernels on the host cores (16 frames, the reference arm's code)."""
    out = {}
    for c, (W, H, lm) in ((0, (640, 360, vx.LIGHTS_POINT)), (1, (1280, 720, vx.LIGHTS_AREA))):
        d = vx.scene_preset(c)
        w = vx.World()
        w.generate(d)
        v = vx.View(w, vx.view_desc(W, H, lm, accumulate=0))
        t = tuning_fn(w, v.desc)
        if t is not None:
            v.set_tuning(t)
        cam = lambda f, d=d, c=c: workload_camera(c, lambda sd, ff, n: vx.camera_path(d, sd, ff, n), f)
        for f in range(warmup):
            v.lookat(*cam(f))
            v.render()
        v.wait()
        v.timer_begin()
        for f in range(steps):
            v.lookat(*cam(warmup + f))
            v.render()
        ms = v.timer_end() / steps
        v.wait()
        # stage and kernel times from frames each waited for (no overlap between frames)
        v.kernel_timing(True)
        v.kernel_stats(reset=True)
        v.stage_stats(reset=True)
        for f in range(min(steps, KERNEL_PASS_FRAMES)):
            v.lookat(*cam(warmup + steps + f))
            v.render()
            v.wait()
        v.kernel_timing(False)
        ks = v.kernel_stats(reset=True)
        sums, counts = v.stage_stats(reset=True)
        hits, rc, rs = v.work_counts()
        out[f"config{c}"] = {"resolution": [W, H], "light_model": "point" if lm == vx.LIGHTS_POINT else "area",
                             "emitters": int(d.emitters), "ms_per_frame": ms, "frames": steps,
                             "stage_ms": {STAGES[i]: (sums[i] / counts[i] if counts[i] else 0.0) for i in range(5)},
                             "kernel_ms": {k: a / n for k, (a, n) in ks.items() if n},
                             "rays_per_s": (hits + rc + rs) / (ms * 1e-3)}
        v.close()
        w.close()
    cms, kind, sample = cpu_arm(0, 16, 1, 640, 360)
    out["config0"]["cpu_reference"] = {"ms_per_frame": cms, "median_ms": sample["median_ms"], "kind": kind,
                                       "threads": sample["threads"], "cpu_model": sample["cpu_model"],
                                       "stage_ms": sample["stage_ms"], "sample": sample["desc"]}
    return out


def other_modes(make_view, cams, steps, warmup):
    """Frame time of the renderer's two other modes on the bench's scene, resolution and
    camera path (plain method, 32 candidates): the sky dome on (a synthetic 1024 x 512
    sky: a horizon gradient with hashed noise and LoadSky's artificial sun, its sky
    lights from vxr_sky_lights, random blue-noise tables), and the path tracer (one
    renderPathTracer sample per pixel and frame, then the accumulator)."""
    import smallproject_gb300 as vx
    from smallproject_gb300 import scene_io
    rng = np.random.default_rng(23)
    h, w = 512, 1024
    rows = np.linspace(1.0, 0.05, h, dtype=np.float32)[:, None, None]
    rgb = (rows * np.array([0.6, 0.8, 1.2], np.float32) * (0.9 + 0.2 * rng.random((h, w, 1), dtype=np.float32)))
    tex = scene_io.sky_texture(rgb.astype(np.float32), scale=1.5)
    bn = rng.integers(0, 256, vx.BLUE_NOISE_WORDS, dtype=np.uint32)
    out = {}
    view = make_view(False, 32)

    def run(frame):
        for f in range(warmup):
            frame(f)
        view.wait()
        view.timer_begin()
        for f in range(steps):
            frame(warmup + f)
        ms = view.timer_end() / steps
        view.wait()
        # kernel times from frames each waited for (back to back, a frame's front half
        # runs beside the previous frame's shading)
        view.kernel_timing(True)
        view.kernel_stats(reset=True)
        for f in range(min(steps, KERNEL_PASS_FRAMES)):
            frame(warmup + steps + f)
            view.wait()
        view.kernel_timing(False)
        ks = view.kernel_stats(reset=True)
        return ms, {k: v[0] / v[1] for k, v in ks.items() if v[1]}

    def render(f):
        pos, tgt = cams(f)
        view.lookat(pos, tgt)
        view.render()

    ms, ks = run(render)
    out["plain_ms_per_frame"] = ms
    out["plain_shade_finish_ms"] = ks.get("shade_finish")
    view.set_sky(tex, vx.sky_lights(tex), 0.5, bn)
    ms, ks = run(render)
    out["sky"] = {"ms_per_frame": ms, "shade_finish_ms": ks.get("shade_finish"),
                  "sky_texels": [w, h], "light_scale": 0.5}
    view.set_sky(None)

    def path_trace(f):
        pos, tgt = cams(f)
        view.lookat(pos, tgt)
        view.begin_frame()
        view.stage(vx.STAGE_PATH_TRACE)
        view.stage(vx.STAGE_ACCUMULATE)
        view.end_frame()

    ms, _ = run(path_trace)
    out["path_trace"] = {"ms_per_frame": ms, "samples_per_pixel": 1}
    view.close()
    return out


def world_commit_times(world, args):
    """Host wall time of sending the world to the device: everything (vxr_world_upload)
    against incremental commits after editing 1 and 1,000 random voxels (after every other
    measurement: it changes the world)."""
    rng = np.random.default_rng(17)
    out = {}
    t0 = time.perf_counter()
    world.upload()
    out["full_upload_ms"] = (time.perf_counter() - t0) * 1e3
    out["bricks"] = world.brick_count()
    for n in (1, 1000):
        for _ in range(n):
            x, y, z = (int(v) for v in rng.integers(0, 1024, 3))
            world.set(x, y, z, 0xF5A5)
        t0 = time.perf_counter()
        sent, full = world.commit()
        out[f"edit_{n}_voxels"] = {"ms": (time.perf_counter() - t0) * 1e3, "bricks_sent": sent, "full": full}
    return out


if __name__ == "__main__":
    main()
