"""Benchmark: ms/frame of the Voxel ReSTIR render path on one GB300.

Workload (config 3 of the benchmark set, plain uniform-source method): 1024^3 fBm
terrain (seed 4), 65,536 emitter voxels (70% in 32 Gaussian blobs, sigma 24),
1920x1080, area lights with solid-angle side sampling, 32 candidates, temporal reuse
(20x M clamp) and 5-tap / 30-px spatial reuse, camera on a seeded Catmull-Rom path.
A step is one frame: albedo -> candidates+temporal -> spatial -> shading+accumulate.

Arms:
  --impl ours       the CUDA path (libvxr.so) - the JSON line's `value` is device time
                    per frame with all inputs resident in HBM; `e2e` goes through the
                    C ABI call that returns the image in page-locked host memory.
  --impl reference  the reference's own render-path kernel source compiled for the
                    host CPU (oracle/_ref, OpenMP over all host threads), else the C
                    restatement; each step renders a bounded strip of the same frame
                    and is scaled to a full frame.
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


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.p = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")
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


def cpu_arm(args, desc, world, steps, warmup, W, H):
    """Time the reference's CPU implementation on a strip of rows of the frame."""
    import smallproject_gb300 as vx
    from oracle import binding as ob
    g, b, l = world.arrays()
    arrays = ob.WorldArrays(g, b, l)
    kind = "reference" if ob.load_ref() is not None else "port"
    r = ob.Renderer("ref" if kind == "reference" else "port", arrays, W, H, False)
    rows = args.cpu_rows
    y0 = H // 2 - rows // 2
    cam = vx.Camera()
    times = []
    for f in range(warmup + steps):
        pos, tgt = vx.camera_path(desc, 1, f, 300)
        cam.lookat(pos, tgt)
        k = cam.begin_frame(W, H)
        k.numberOfLights, k.numberOfCandidates, k.numberOfMaxTemporalImportance = len(l), 32, 20
        k.spatialRadius, k.spatialTaps, k.spatial, k.temporal, k.accumulate = 30, 5, 1, 1, 0
        r.frame_start()
        t0 = time.perf_counter()
        for s in range(1, 6):
            r.stage(k, s, y0, y0 + rows)
        dt = time.perf_counter() - t0
        cam.end_frame()
        if f >= warmup:
            times.append(dt)
    r.close()
    per_frame_ms = statistics.median(times) * 1000.0 * (H / rows)
    return per_frame_ms, kind, {"rows": rows, "y0": y0, "width": W, "frames": steps,
                                "desc": f"{rows} rows x {W} px of each {W}x{H} frame, scaled by {H}/{rows}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-rows", type=int, default=96, help="rows of the frame timed on the CPU per step")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tile", type=str, default="", help="threads per block, e.g. 16x8")
    ap.add_argument("--no-tune", action="store_true", help="library default launch tuning instead of the autotuner")
    args = ap.parse_args()
    W, H = args.width, args.height
    warmup = max(args.warmup, 3)

    dist, rank, ws = dist_init(args)
    config = {"workload": f"config{args.config}: plain Voxel ReSTIR, {W}x{H}, area lights, 32 candidates, "
                          "temporal 20x clamp, 5 taps / 30 px spatial, 1024^3 fBm terrain seed 4, "
                          "65,536 emitters (70% in 32 blobs), Catmull-Rom camera path",
              "resolution": [W, H], "scene_config": args.config, "method": "plain uniform-source RIS",
              "l2": "per-frame working set (G-buffers, reservoirs, frame, accumulator: 237 MB at 1080p) exceeds "
                    "the 129 MB L2; no flush between frames"}

    if args.impl == "reference":
        if rank != 0:
            return
        from smallproject_gb300 import build as B
        B.build()
        vx, desc, world = make_scene(args.config)
        ms, kind, sample = cpu_arm(args, desc, world, args.steps, min(args.warmup, 1), W, H)
        line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms/frame", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": min(args.warmup, 1), "ms_per_step": ms, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
                "config": config,
                "cpu_baseline": {"value": ms, "unit": "ms/frame", "cores": os.cpu_count(), "kind": kind,
                                 "sample": sample["desc"]},
                "e2e": {"value": ms, "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from smallproject_gb300 import build as B
    B.build()
    vx, desc, world = make_scene(args.config)
    tile = {}
    if args.tile:
        tx, ty = args.tile.split("x")
        tile = dict(tile_x=int(tx), tile_y=int(ty))
    vdesc = vx.view_desc(W, H, vx.LIGHTS_AREA, accumulate=0, **tile)
    nfr = 300
    tuning_report = None
    if not args.no_tune and not tile:
        # launch parameters only (results are identical for every tuning); untimed setup
        from smallproject_gb300 import autotune as at
        cache = os.path.join(ROOT, "gpurun_out" if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else "_build",
                             "vxr_tuning.json")
        t, tuning_report = at.autotune(world, vdesc, lambda f: vx.camera_path(desc, 1, (1000 + f) % nfr, nfr),
                                       frames=4, rounds=2, cache_path=cache)
    view = vx.View(world, vdesc)
    if tuning_report is not None:
        view.set_tuning(t)

    def frame(f):
        pos, tgt = vx.camera_path(desc, 1, f % nfr, nfr)
        view.lookat(pos, tgt)
        view.render()

    for f in range(warmup):
        frame(f)
    view.wait()
    view.stage_stats(reset=True)

    barrier(dist)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if rank == 0 else None
    view.timer_begin()
    for f in range(args.steps):
        frame(warmup + f)
    ms_total = view.timer_end()
    view.wait()
    barrier(dist)
    clk = clocks.stop() if clocks else None
    ms_total = max_over_ranks(dist, ms_total)
    ms_frame = ms_total / args.steps
    sums, counts = view.stage_stats(reset=True)
    stage_ms = {STAGES[i]: (sums[i] / counts[i] if counts[i] else 0.0) for i in range(5)}

    # end to end through the C ABI with a page-locked host image
    pinned = vx.PinnedBuffer(W * H * 4)
    e2e_steps = max(5, min(args.steps, 30))
    for f in range(3):
        pos, tgt = vx.camera_path(desc, 1, f, nfr)
        view.render_to_host(pos, tgt, pinned.array)
    t0 = time.perf_counter()
    for f in range(e2e_steps):
        pos, tgt = vx.camera_path(desc, 1, f, nfr)
        view.render_to_host(pos, tgt, pinned.array)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / e2e_steps
    e2e_ms = max_over_ranks(dist, e2e_ms)
    img_ok = bool(np.isfinite(pinned.array).all() and pinned.array.max() > 0)
    pinned.close()

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    npx = W * H
    # dominant kernel = the slowest stage
    dom = max(("albedo", "candidates", "spatial", "shade"), key=lambda s: stage_ms[s])
    achieved = BYTES_PER_PX[dom] * npx / (stage_ms[dom] * 1e-3) / 1e9 if stage_ms[dom] > 0 else 0.0
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": f"of {peak_kind}", "traffic": None,
                "bytes_per_launch": BYTES_PER_PX[dom] * npx}
    stage_rooflines = {s: {"ms": stage_ms[s], "GB/s": BYTES_PER_PX[s] * npx / (stage_ms[s] * 1e-3) / 1e9
                           if stage_ms[s] > 0 else 0.0, "frac": (BYTES_PER_PX[s] * npx / (stage_ms[s] * 1e-3) / 1e9)
                           / hbm if stage_ms[s] > 0 else 0.0}
                       for s in ("albedo", "candidates", "spatial", "shade")}
    rays_per_s = 3.0 * npx / (ms_frame * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:
        cms, kind, sample = cpu_arm(args, desc, world, args.cpu_steps, 1, W, H)
        cpu = {"value": cms, "unit": "ms/frame", "cores": os.cpu_count(), "kind": kind, "sample": sample["desc"]}
    value = ms_frame / ws   # replicas: ws frames per ms_frame across the job
    line = {"metric": METRIC, "value": value, "unit": "ms/frame", "n_gpus": ws, "steps": args.steps,
            "warmup": warmup, "ms_per_step": ms_frame, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": config, "stage_ms": stage_ms, "stage_roofline": stage_rooflines, "rays_per_s": rays_per_s,
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": e2e_ms, "unit": "ms/frame", "h2d_bytes_per_step": 4 * 176,
                    "d2h_bytes_per_step": npx * 16, "image_ok": img_ok},
            "gpu_launches": 4 * args.steps, "clocks": clk,
            "tuning": view.get_tuning().as_dict(), "tuning_search": tuning_report}
    print(json.dumps(line))
    view.close()


if __name__ == "__main__":
    main()
