"""Benchmark of the dense RGB-D tracking step (frames/s at 640x480):
warm-started batched tracking against the plain tracker.

Headline (value): warm-started batched tracking.  A step = one batch of
--batch-pairs held-out 640x480 frame pairs (6x4x3 m rooms with 20 spheres,
fx = fy = 525, depth noise 0.0012 z^2, 5 % dropout, relative motion <= 10 deg /
10 cm) tracked by one odo_batch_track_warm call: the warm-start network's
proposal for every pair, 3 pyramid levels with 2/2/2 ICP+RGB iterations and
no SO3 stage, and a fall-back to the reference's schedule (SO3 + 10/5/4) for
the pairs whose residual or proposal disagreement fails the test.  The
network is trained first, on the GPU, by the library's own kernels, on
150,000 GPU-rendered pairs labelled by the plain tracker (setup, about 2.5
minutes, not timed).  Two
batches (> L2) are resident in HBM and alternate.  Beside it, on the same
pairs: the plain batched tracker (odo_batch_track), and the plain
single-pair drop-in path (one frame per call through the reference's call
order initICPModel -> initRGBModel -> initICP -> initRGB ->
getIncrementalTransformation, on the 300-frame synthetic trajectory).

Arms:
  ours (default)  the CUDA library; value = warm-started frames/s with inputs
                  in HBM; e2e = the same with every step's inputs copied from
                  pinned host memory (on copy streams, overlapping the
                  previous step's tracking) and the results read back;
  --impl reference  the reference's tracking math (plain schedule) on the host
                  cores (the CPU oracle, a restatement of src/odom/*; the
                  reference itself cannot be built here), all host threads, on
                  pairs of the same distribution.
Studies (--study): batch (mixed-resolution verification), precision
(corridor pairs against the FP64 oracle), warm (the warm start in detail),
phases (where the time of a warm-started batched step goes).
Multi-GPU: replicas (a tracking call does not shard); each rank tracks its own
copy of the workload; value = frames of all ranks / max time over ranks.
"""
import argparse
import contextlib
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ICP+RGB tracking frames/s @640x480: warm-started vs plain, equal pose error"
BYTES_PER_PX_ITER = 62  # ICP 48 B (4 maps x 12 B) + photometric 14 B per pixel-iteration
# the association kernel's algorithmic bytes are the 62 B of its inputs; the
# correspondence record it writes for the photometric pass (an artefact of
# the two-pass structure, as the reference's DataTerm is) is reported apart
RECORD_BYTES_PER_PX = 16
# one-kernel ncu captures of this build whose `dram_bytes_per_px:` lines give
# the measured traffic per pixel (traffic grows with the pixels processed)
TRAFFIC_PROFILE_BATCH = "k_icp_rgbres_b_L0_24pairs_640x480.md"
TRAFFIC_PROFILE_SINGLE = "k_icp_rgbres_L0_single_640x480.md"
PREPROC_BYTES_PER_PX = 140  # per-frame map/pyramid building, per level-0 pixel (x 4/3 over the pyramid)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pool", type=int, default=64)
    ap.add_argument("--mode", default="graph", choices=["graph", "stream", "persistent"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--study", default=None, choices=[None, "batch", "precision", "warm", "phases"],
                    help="batch: 512 mixed-resolution pairs per launch (batched verification); "
                         "precision: 1000 corridor pairs, FP32 vs compensated FP32 vs the FP64 oracle; "
                         "phases: the time split of a warm-started batched step")
    ap.add_argument("--nvtx-steps", action="store_true",
                    help="phases study: only one warm-started and one plain step, inside the NVTX ranges "
                         "warm_step / plain_step (for a profiler's launch list)")
    ap.add_argument("--pairs", type=int, default=None)
    ap.add_argument("--pairs-out", default=None, help="precision study: per-pair CSV path")
    ap.add_argument("--corridor", default="tapered", choices=["tapered", "clutter"],
                    help="precision study: clutter-free corridors with tapered walls (cond(JtJ) mostly 1e6-1e9) "
                         "or straight corridors with 24 clutter spheres")
    ap.add_argument("--no-autotune", action="store_true", help="batch study: keep the default launch shape")
    ap.add_argument("--launch", default=None, help="batch study: fixed launch shape THREADSxPIXELS (e.g. 128x8)")
    ap.add_argument("--sizes", default="mixed", choices=["mixed", "640x480"],
                    help="batch study: resolutions drawn uniformly from 160x120/320x240/640x480, or 640x480 only")
    ap.add_argument("--train-pairs", type=int, default=150000, help="warm study: rendered training pairs")
    ap.add_argument("--epochs", type=int, default=50)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-pairs", type=int, default=2000)
    ap.add_argument("--warm-levels", type=int, default=3)
    ap.add_argument("--warm-iters", default="2,2,2")
    ap.add_argument("--max-disagree", type=float, default=5.0, help="warm study: fall-back angle (deg)")
    ap.add_argument("--oracle-pairs", type=int, default=24, help="warm study: pairs also tracked by the FP64 oracle")
    ap.add_argument("--save-params", default=None)
    ap.add_argument("--load-params", default=None, help="warm study: skip training, use these parameters")
    ap.add_argument("--sweep", action="store_true", help="warm study: also evaluate other warm schedules")
    ap.add_argument("--batch-pairs", type=int, default=1000, help="pairs per warm-started batched step")
    ap.add_argument("--verify-pairs", type=int, default=512,
                    help="pairs per launch of the batched-verification line (0: skip it)")
    ap.add_argument("--residual-ratio", type=float, default=16.0)
    ap.add_argument("--front-end", type=int, default=1,
                    help="also time the producers of the tracker's inputs (depth pre-filter, model prediction, "
                         "fill-in) at 640x480")
    a = ap.parse_args()
    if a.pairs is None:
        a.pairs = 1000 if a.study == "precision" else 512
    return a


@contextlib.contextmanager
def no_gc():
    """Python's cyclic garbage collector paused over a timed region (as
    timeit does): a full collection of the held-out set's Python objects
    takes tens to hundreds of milliseconds and would be charged to whichever
    step it falls in.  The library itself allocates nothing per call."""
    gc.collect()
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_pool(n, seed):
    from slam_gb300 import synth
    cam = synth.Camera()
    scene = synth.make_room(seed, 20)
    T = synth.trajectory(seed, 300)
    frames = [synth.trajectory_frame(scene, T, k, cam, seed) for k in range(1, n + 1)]
    return cam, frames


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def frame_bytes(cam, iters):
    n0 = cam.width * cam.height
    b = 0
    for l, it in enumerate(iters):
        b += it * (n0 >> (2 * l)) * BYTES_PER_PX_ITER
    return b + PREPROC_BYTES_PER_PX * n0 * 4 // 3


# ----------------------------------------------------------------------------
# CPU arm (the oracle port of the reference's tracking math)
# ----------------------------------------------------------------------------
def cpu_track(frames, cam, nframes=None, seconds=None):
    from oracle import oracle
    from slam_gb300 import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    o = oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DEFAULT_DIST_THRESH,
                        DEFAULT_ANGLE_THRESH, prec=32)
    o.initFirstRGB(frames[0]["model_rgba"])
    done = 0
    t0 = time.perf_counter()
    while True:
        f = frames[done % len(frames)]
        T1 = f["T1"].astype(np.float32)
        o.initICPModel(f["model_vert"], f["model_norm"], 20.0, T1)
        o.initRGBModel(f["model_rgba"])
        o.initICP(f["depth"], 20.0)
        o.initRGB(f["rgba"])
        o.getIncrementalTransformation(T1[:3, 3], T1[:3, :3], False, 10.0, True, False, True)
        done += 1
        el = time.perf_counter() - t0
        if nframes is not None and done >= nframes:
            break
        if seconds is not None and el >= seconds and done >= 3:
            break
    return done, time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    ncores = os.cpu_count() or 1
    oracle.set_threads(ncores)
    from slam_gb300 import synth
    cam = synth.Camera()
    frames = [synth.make_pair(args.seed * 31 + 7000 + k, cam=cam, max_deg=10.0, max_m=0.10) for k in range(8)]
    cpu_track(frames, cam, nframes=max(1, args.warmup))
    with no_gc():
        n, el = cpu_track(frames, cam, nframes=args.steps)
    fps = n / el
    out = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / n, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "640x480 room pairs (6x4x3 m rooms, 20 spheres, motion <= 10 deg / 10 cm), "
                                  "plain tracking (the reference has no warm start)",
                      "iterations": [10, 5, 4], "icpWeight": 10, "so3": True},
           "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": oracle.get_threads(), "kind": "port",
                            "sample": f"{n} pair trackings (8 distinct pairs cycled) on the host cores"},
           "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from slam_gb300 import _build
    _build.build()
    from slam_gb300 import MODE_GRAPH, MODE_PERSISTENT, MODE_STREAM, RGBDOdometry, _native, synth

    cam, frames = make_pool(args.pool, args.seed)
    stream = torch.cuda.current_stream()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    devd = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)
    dframes = [{"v": dev(f["model_vert"]), "n": dev(f["model_norm"]), "mc": dev(f["model_rgba"]),
                "d": devd(f["depth"]), "c": dev(f["rgba"]), "T1": f["T1"].astype(np.float32)} for f in frames]
    in_bytes = sum(dframes[0][k].numel() * dframes[0][k].element_size() for k in ("v", "n", "mc", "d", "c"))
    odo = RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, stream=stream.cuda_stream)
    odo.set_mode({"graph": MODE_GRAPH, "stream": MODE_STREAM, "persistent": MODE_PERSISTENT}[args.mode])
    odo.initFirstRGB(dframes[0]["mc"])

    def step(f):
        odo.initICPModel(f["v"], f["n"], 20.0, f["T1"])
        odo.initRGBModel(f["mc"])
        odo.initICP(f["d"], 20.0)
        odo.initRGB(f["c"])
        return odo.getIncrementalTransformation(f["T1"][:3, 3], f["T1"][:3, :3], False, 10.0, True, False, True)

    for k in range(max(args.warmup, 3)):
        step(dframes[k % len(dframes)])
    iters = odo.iterations()
    torch.cuda.synchronize()

    # ---- device-resident inputs -------------------------------------------
    n_single = max(args.steps, 300)  # side measurement: a fixed sample of frames
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    poses = []
    with no_gc():
        e0.record(stream)
        for k in range(n_single):
            poses.append(step(dframes[k % len(dframes)]))
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    fps = world * n_single / (ms / 1000.0)
    errs = [synth.pose_error(synth.pose(np.float64(R), np.float64(t)), frames[k]["T2"])
            for k, (t, R) in enumerate(poses[:len(frames)])]

    # ---- the same frames in the other execution modes (persistent: one
    # cooperative kernel per pyramid level; stream: the graph's kernels
    # launched one by one) ----
    mode_fps = {}
    for name, m in (("persistent", MODE_PERSISTENT), ("stream", MODE_STREAM)):
        if name == args.mode:
            continue
        odo.set_mode(m)
        for k in range(3):
            step(dframes[k % len(dframes)])
        with no_gc():
            torch.cuda.synchronize()
            e0.record(stream)
            for k in range(n_single):
                step(dframes[k % len(dframes)])
            e1.record(stream)
            torch.cuda.synchronize()
        mode_fps[name] = n_single / (e0.elapsed_time(e1) / 1000.0)
    odo.set_mode({"graph": MODE_GRAPH, "stream": MODE_STREAM, "persistent": MODE_PERSISTENT}[args.mode])
    for k in range(3):
        step(dframes[k % len(dframes)])

    # ---- end to end: host inputs copied per step ------------------------
    hframes = [{k: (v.cpu().pin_memory() if isinstance(v, torch.Tensor) else v) for k, v in f.items()}
               for f in dframes[:8]]
    stage = {k: torch.empty_like(dframes[0][k]) for k in ("v", "n", "mc", "d", "c")}
    ekeys = ("v", "n", "mc", "d", "c")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with no_gc():
        e2.record(stream)
        for k in range(n_single):
            h = hframes[k % len(hframes)]
            for key in ekeys:
                stage[key].copy_(h[key], non_blocking=True)
            step({**stage, "T1": h["T1"]})
        e3.record(stream)
        torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3)
    if world > 1:
        tt = torch.tensor([ms_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_e2e = float(tt.item())
    fps_e2e = world * n_single / (ms_e2e / 1000.0)

    # ---- roofline of the dominant kernel (association + residual pass) ----
    odo.profile(reset=True)
    step(dframes[0])
    phases = odo.profile(reset=True)
    level_ms = {f"L{l}": odo.time_iteration(l, reps=50) for l in (2, 1)}
    k_ms, s_ms, it_ms = odo.time_iteration(0, reps=100)
    level_ms["L0"] = [k_ms, s_ms, it_ms]
    n0 = cam.width * cam.height
    alg_bytes = BYTES_PER_PX_ITER * n0
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    # per frame: the init calls (model maps; model depth + intensity and two
    # pyramid steps; two depth pyramid steps and the maps; live depth +
    # intensity and two pyramid steps = 10), then the tracking call (state
    # copy in, derivatives, SO3, begin, end, state copy out = 6) and two
    # kernels per iteration of 10/5/4
    launches_per_frame = 10 + 6 + 2 * (10 + 5 + 4)

    out = None
    if rank == 0:
        cpu = None
        try:
            if args.cpu_seconds <= 0:
                raise RuntimeError("skipped (--cpu-seconds 0)")
            from oracle import oracle
            oracle.set_threads(os.cpu_count() or 1)
            n, el = cpu_track(frames[:8], cam, seconds=args.cpu_seconds)
            cpu = {"value": n / el, "unit": "frames/s", "cores": oracle.get_threads(), "kind": "port",
                   "sample": f"{n} frames (640x480, full tracking call) of the same trajectory, "
                             f"{el:.1f} s on the host cores"}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "frames/s", "cores": 0, "kind": "port", "sample": f"failed: {exc}"}
        rot = [e[0] for e in errs]
        tr = [e[1] for e in errs]
        plain = {"frames_per_s": fps, "ms_per_frame": ms / n_single, "steps": n_single,
                 "workload": "640x480 frame-to-model tracking, one frame per call (the drop-in path), synthetic "
                             f"300-frame room trajectory, first {len(frames)} frames cycled",
                 "levels": ["640x480", "320x240", "160x120"], "iterations": [10, 5, 4], "icpWeight": 10,
                 "so3": True, "mode": args.mode,
                 "l2": f"inputs larger than L2: {len(frames)} frames x {in_bytes / 1e6:.1f} MB resident in HBM, "
                       "a different frame every step",
                 "e2e": {"value": fps_e2e, "unit": "frames/s", "h2d_bytes_per_step": int(in_bytes),
                         "d2h_bytes_per_step": int(_native.load().odo_state_bytes())},
                 "roofline": {"bound": "hbm", "kernel": "k_icp_rgbres (level 0)", "achieved": achieved,
                              "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                              "traffic": (profile_traffic(TRAFFIC_PROFILE_SINGLE) or 0) * n0 or None,
                              "kernel_ms": k_ms, "photometric_kernel_ms": s_ms, "iteration_ms": it_ms,
                              "alg_bytes_per_launch": alg_bytes,
                              "note": "level-0 maps (~20 MB) are L2-resident within a frame"},
                 "frame_bytes": frame_bytes(cam, iters[1:]),
                 "frame_roofline_gbs": frame_bytes(cam, iters[1:]) / (ms / n_single * 1e-3) / 1e9,
                 "pose_error_vs_gt": {"rot_rad_mean": float(np.mean(rot)), "trans_m_mean": float(np.mean(tr)),
                                      "rot_rad_max": float(np.max(rot)), "trans_m_max": float(np.max(tr))},
                 "iterations": iters, "clocks": clk, "iteration_ms_by_level": level_ms,
                 "frames_per_s_other_modes": mode_fps,
                 "device_phases_us": phases, "gpu_launches": launches_per_frame * n_single}
    warm = measure_warm_batched(args, stream, local, world)
    verif = measure_batched_verification(args, stream, world) if args.verify_pairs > 0 else None
    front = measure_front_end(args, stream) if rank == 0 and args.front_end else None
    if rank == 0:
        W = warm
        out = {"metric": METRIC, "value": W["fps"], "unit": "frames/s", "n_gpus": world, "steps": W["steps"],
               "warmup": W["warmup"], "ms_per_step": W["ms_per_step"], "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": f"warm-started batched tracking: {W['batch_pairs']} held-out 640x480 room pairs "
                                      f"per step, {W['eval_pairs']} held-out pairs cycled (6x4x3 m rooms, "
                                      "20 spheres, motion <= 10 deg / 10 cm), network proposal + "
                                      f"{args.warm_levels} levels {args.warm_iters} without SO3, fall-back to the "
                                      "plain schedule",
                          "batch_pairs": W["batch_pairs"], "eval_pairs": W["eval_pairs"],
                          "warm_schedule": W["schedule"], "fallback": W["fallback_cfg"], "train": W["train"],
                          "launch": W["launch"],
                          "l2": f"inputs larger than L2: {W['pool_batches']} batches x {W['batch_bytes'] / 1e9:.1f} GB "
                                "resident in HBM, cycled",
                          "parallelism": "replicas" if world > 1 else "single GPU"},
               "e2e": W["e2e"], "roofline": W["roofline"],
               "plain_batched": W["plain_batched"], "plain_single_pair": plain,
               "speedup": {"vs_plain_single_pair": W["fps"] / plain["frames_per_s"],
                           "vs_plain_batched": W["fps"] / W["plain_batched"]["frames_per_s"],
                           "eval_thresholds_vs_plain_batched": W["eval_thresholds"]["speedup_vs_plain_batched"]},
               "eval_thresholds": W["eval_thresholds"], "accuracy": W["accuracy"],
               "batched_verification": verif, "front_end": front, "clocks": W["clocks"],
               "gpu_launches": W["gpu_launches"], "cpu_baseline": cpu}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def measure_front_end(args, stream, reps=20):
    """The producers of the tracker's inputs at 640x480, one frame per launch
    as the reference runs them: depth_bilateral.frag / depth_metric.frag,
    IndexMap::combinedPredict (surfel splatting) and FillIn, each timed with
    CUDA events per launch with L2 flushed (a 256 MB write) between launches,
    against its algorithmic bytes; the oracle's CPU restatement of the same
    kernel is timed beside it."""
    import torch
    from oracle import oracle
    from slam_gb300 import model, odometry, synth
    cam = synth.Camera()
    rng = np.random.default_rng(args.seed + 77)
    scene = synth.make_room(args.seed + 77)
    T0 = synth.room_camera(rng)
    views = []
    for _ in range(6):
        T = T0 @ synth.random_motion(rng, 15.0, 0.3)
        m = synth.render(scene, T, cam, depth=False, rgba=True, model=True)
        S = model.surfels_from_view(m["vert"], m["norm"], m["rgba"], T, cam)
        S[:, 3] = rng.uniform(5.0, 20.0, size=len(S)).astype(np.float32)
        views.append(S)
    S = np.concatenate(views)
    fr = synth.render(scene, T0, cam, depth=True, rgba=True, model=False)
    raw = fr["depth"]                      # sensor-like noise and dropout from the renderer
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda().view(torch.uint16)
    d_rgba = dev(fr["rgba"])
    d_S = dev(S)
    params = model.predict_params(cam, conf_threshold=10.0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    scratch = torch.empty(_native_load().odo_model_predict_scratch_bytes(cam.width, cam.height) // 8,
                          dtype=torch.int64, device="cuda")
    peak, peak_kind = measured_peaks()
    npx = cam.width * cam.height

    def timed(fn):
        for _ in range(3):
            fn()
        ts = []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(reps):
            flush.fill_(1)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    def cpu_timed(fn, budget_s=2.0):
        n, t0 = 0, time.perf_counter()
        while True:
            fn()
            n += 1
            if time.perf_counter() - t0 > budget_s:
                return (time.perf_counter() - t0) * 1e3 / n

    out = {}
    pred = model.predict(d_S, T0, params, scratch=scratch)
    hp = [p.cpu().numpy() for p in pred[:3]]
    rows = [
        ("depth_bilateral", lambda: odometry.filter_depth(d_raw, 20.0), 4 * npx,
         "2 B read + 2 B written per pixel (13x13 window from a shared-memory tile)",
         lambda: oracle.depth_bilateral(raw, 20.0)),
        ("depth_metric", lambda: odometry.depth_metric(d_raw, 20.0), 6 * npx, "2 B read + 4 B written per pixel",
         lambda: oracle.depth_metric(raw, 20.0)),
        ("model_predict", lambda: model.predict(d_S, T0, params, scratch=scratch), 48 * len(S) + (8 + 38) * npx,
         "48 B per surfel read, 8 B per pixel depth-index word, 38 B per pixel of maps written",
         lambda: oracle.model_predict(S, model.t_inv_of(T0), cam, max_depth=20.0, conf_threshold=10.0, time=1,
                                      max_time=2 ** 30, time_delta=2 ** 30)),
        ("fill_in", lambda: model.fill_in(pred[1], pred[2], pred[0], d_raw, d_rgba, cam), (42 + 36) * npx,
         "42 B read (predicted maps, raw depth and colour) + 36 B written per pixel",
         lambda: oracle.fill_in(hp[1], hp[2], hp[0], raw, fr["rgba"], cam)),
    ]
    for name, fn, alg, what, cpu_fn in rows:
        ms = timed(fn)
        gbs = alg / (ms * 1e-3) / 1e9
        row = {"ms": ms, "alg_bytes": int(alg), "alg_bytes_def": what, "achieved_gbs": gbs,
               "frac_of_peak": gbs / peak, "peak_kind": peak_kind}
        if cpu_fn is not None:
            try:
                row["cpu_oracle_ms"] = cpu_timed(cpu_fn)
            except Exception as exc:
                row["cpu_oracle_ms"] = f"failed: {exc}"
        out[name] = row
    out["workload"] = (f"640x480, one frame per launch; surfel map of {len(S)} surfels from 6 views of one room; "
                       "L2 flushed between launches")
    return out


def _native_load():
    from slam_gb300 import _native
    return _native.load()


def profile_traffic(name):
    """DRAM bytes (read + write) per pixel of a kernel, from the
    `dram_bytes_per_px:` line of the committed ncu summary profiles/<name>
    (a one-kernel capture of this build); None when absent."""
    import re
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                m = re.match(r"\s*[-*]?\s*`?dram_bytes_per_px:\s*([0-9.]+)", line)
                if m:
                    return float(m.group(1))
    except OSError:
        pass
    return None


def oracle_distance(pool, res_sets, npairs):
    """FP64 oracle (plain schedule, the reference's call order) on the first
    `npairs` pairs of pool[0]: the distance of each result set's poses from
    it.  res_sets: {name: results of pool[0]}."""
    import torch
    from oracle import oracle
    from slam_gb300 import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH, synth
    from slam_gb300.batch import result_pose
    ps = pool[0]
    cam = ps.cam
    oracle.set_threads(os.cpu_count() or 1)
    d = {k: [] for k in res_sets}
    for i in range(min(npairs, ps.n)):
        h = {k: getattr(ps, k)[i].cpu().numpy() for k in ("model_vert", "model_norm", "model_rgba", "rgba")}
        depth = ps.depth[i].cpu().view(torch.int16).numpy().view(np.uint16)
        o = oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DEFAULT_DIST_THRESH,
                            DEFAULT_ANGLE_THRESH, prec=64)
        T1 = ps.T1[i].astype(np.float32)
        o.initFirstRGB(h["model_rgba"])
        o.initICPModel(h["model_vert"], h["model_norm"], 20.0, T1)
        o.initRGBModel(h["model_rgba"])
        o.initICP(depth, 20.0)
        o.initRGB(h["rgba"])
        t, R = o.getIncrementalTransformation(T1[:3, 3], T1[:3, :3], False, 10.0, True, False, True)
        o.close()
        T64 = synth.pose(np.asarray(R, np.float64), np.asarray(t, np.float64))
        for k, res in res_sets.items():
            d[k].append(synth.pose_error(result_pose(res[i]), T64))
    out = {"pairs": min(npairs, ps.n), "reference": "FP64 oracle, plain schedule (SO3 + 10/5/4)"}
    for k, v in d.items():
        v = np.array(v)
        out[k] = {"within_1e-5": float(np.mean((v[:, 0] <= 1e-5) & (v[:, 1] <= 1e-5))),
                  "rot_rad_p50": float(np.median(v[:, 0])), "trans_m_p50": float(np.median(v[:, 1])),
                  "rot_rad_max": float(v[:, 0].max()), "trans_m_max": float(v[:, 1].max())}
    return out


def measure_warm_batched(args, stream, local, world):
    """The headline: warm-started batched tracking of 640x480 pairs (the
    network trained here first, on the GPU, by the library's own kernels) over
    the held-out evaluation set, with the plain batched tracker timed on the
    same pairs and the evaluation's fall-back thresholds reported beside the
    tuned ones."""
    import torch
    from slam_gb300 import synth, warmstart as ws
    from slam_gb300.batch import BatchOdometry, result_pose
    cam = synth.Camera()
    nb = args.batch_pairs
    b = BatchOdometry(nb, stream=stream.cuda_stream)
    # the whole step's proposals in one forward pass (training uses 256)
    net = ws.WarmStartNet(max_batch=max(256, nb), stream=stream.cuda_stream)
    t0 = time.time()
    ts = ws.make_training_set(net, b, args.seed * 17 + 3, args.train_pairs)
    net.set_loss_metric(ts["metric"])
    gen_s = time.time() - t0
    t0 = time.time()
    hist = ws.train(net, ts["inputs"], ts["labels"], epochs=args.epochs, batch=256, lr=args.lr, lr_final=args.lr / 30)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    plain_res = float(np.median(ts["residuals"]))
    n_train = int(ts["labels"].shape[0])
    del ts
    its = tuple(int(v) for v in args.warm_iters.split(","))
    tuned = dict(levels=args.warm_levels, iterations=its, residual_limit=args.residual_ratio * plain_res,
                 max_disagree_deg=args.max_disagree)
    spec = dict(levels=args.warm_levels, iterations=its, residual_limit=1.5 * plain_res, max_disagree_deg=0.5)
    # held-out evaluation set: eval_pairs pairs in batches of nb, all resident
    nbatch = max(1, -(-args.eval_pairs // nb))
    pool = [ws.make_room_pairs(args.seed * 31 + 1000 + k, nb, cam, 10.0, 0.10) for k in range(nbatch)]
    fps = [p.frame_pairs() for p in pool]
    descs = [b._descs(f) for f in fps]
    batch_bytes = sum(t[0].numel() * t[0].element_size() * nb for t in
                      (pool[0].model_vert, pool[0].model_norm, pool[0].model_rgba, pool[0].depth, pool[0].rgba))
    threads, ppt, _ = b.autotune(fps[0])
    W = max(args.warmup, 3)
    K = args.steps
    for k in range(W):
        b.track(fps[k % nbatch], descs=descs[k % nbatch])
        b.track_warm(net, fps[k % nbatch], descs=descs[k % nbatch], **tuned)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, steps):
        with no_gc():
            torch.cuda.synchronize()
            e0.record(stream)
            for k in range(steps):
                fn(k)
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # ---- warm-started, inputs resident in HBM: exactly K steps ----
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    ms_w = timed(lambda k: b.track_warm(net, fps[k % nbatch], descs=descs[k % nbatch], **tuned), K)
    clk = clocks.stop()
    # ---- plain batched on the same pairs ----
    ms_p = timed(lambda k: b.track(fps[k % nbatch], descs=descs[k % nbatch]), K)
    # ---- the evaluation's fall-back thresholds (residual > 1.5x plain, pose
    # disagreement > 0.5 deg), one timed pass over the held-out set ----
    spec_res = []
    ms_s = timed(lambda k: spec_res.append(b.track_warm(net, fps[k], descs=descs[k], **spec)), nbatch)
    if world > 1:
        tt = torch.tensor([ms_w, ms_p, ms_s], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_w, ms_p, ms_s = (float(v) for v in tt.tolist())
    # ---- accuracy over the whole held-out set (untimed) ----
    tuned_res = [b.track_warm(net, fps[k], descs=descs[k], **tuned) for k in range(nbatch)]
    plain_res_all = [list(b.track(fps[k], descs=descs[k])) for k in range(nbatch)]

    def errs(res_list):
        return np.array([synth.pose_error(result_pose(r), pool[k].T2[i])
                         for k, res in enumerate(res_list) for i, r in enumerate(res)])

    pct = lambda v: {"p50": float(np.percentile(v, 50)), "p90": float(np.percentile(v, 90))}
    fail = lambda e: float(np.mean((e[:, 0] > np.radians(2.0)) | (e[:, 1] > 0.05)))
    iters = lambda res_list: np.array([list(r.iterations) for res in res_list for r in res], np.float64)

    def summary(res_list, fb_list=None):
        e = errs(res_list)
        out = {"rot_rad": pct(e[:, 0]), "trans_m": pct(e[:, 1]), "fail": fail(e),
               "iterations_mean": iters(res_list).mean(axis=0).tolist()}
        if fb_list is not None:
            out["fallback_rate"] = float(np.mean(np.concatenate(fb_list)))
        return out

    acc_tuned = summary([r for r, _ in tuned_res], [f for _, f in tuned_res])
    acc_spec = summary([r for r, _ in spec_res], [f for _, f in spec_res])
    acc_plain = summary(plain_res_all)
    it_plain = np.array(acc_plain["iterations_mean"])
    saved = lambda a: float((it_plain[1:].sum() - np.array(a["iterations_mean"])[1:].sum()) / it_plain[1:].sum())
    # distance from the FP64 oracle's plain tracking, on a sample of pairs
    dist = oracle_distance(pool, {"warm_tuned": tuned_res[0][0], "warm_eval_thresholds": spec_res[0][0],
                                  "plain_batched": plain_res_all[0]}, args.oracle_pairs)
    # ---- end to end: each step's inputs copied from pinned host memory ----
    # (double-buffered: step k+1's copies, split over N_COPY copy streams,
    # run while step k is tracked; the timed region holds every step's
    # copies and the read-back of its results)
    # (two of the held-out batches in pinned host memory; step k copies
    # batch k % 2 into its device buffer and tracks it)
    keys = ("model_vert", "model_norm", "model_rgba", "depth", "rgba")
    nh = min(2, nbatch)
    host = [{k: getattr(pool[h], k).cpu().pin_memory() for k in keys} for h in range(nh)]
    N_COPY = 4
    css = [torch.cuda.Stream() for _ in range(N_COPY)]
    ev_copy = [[torch.cuda.Event() for _ in css] for _ in range(2)]
    ev_used = [torch.cuda.Event(), torch.cuda.Event()]
    chunk = -(-nb // N_COPY)

    def issue_copy(k, wait=True):
        buf = k % nh
        for j, c in enumerate(css):
            if wait:
                c.wait_event(ev_used[buf])  # the step that last read this buffer is done
            with torch.cuda.stream(c):
                for key in keys:
                    getattr(pool[buf], key)[j * chunk:(j + 1) * chunk].copy_(host[buf][key][j * chunk:(j + 1) * chunk],
                                                                               non_blocking=True)
            ev_copy[buf][j].record(c)

    # H2D bandwidth of one step's copies alone (after one untimed round)
    for rnd in range(2):
        torch.cuda.synchronize()
        t_h2d = time.perf_counter()
        issue_copy(0, wait=False)
        torch.cuda.synchronize()
        t_h2d = time.perf_counter() - t_h2d
    h2d_gbs = batch_bytes / t_h2d / 1e9
    for ev in ev_used:
        ev.record(stream)
    step_host = []
    with no_gc():
        torch.cuda.synchronize()
        e0.record(stream)
        for c in css:
            c.wait_event(e0)
        issue_copy(0)
        ev_in = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        ev_out = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        for k in range(K):
            th = time.perf_counter()
            if k + 1 < K:
                issue_copy(k + 1)
            for ev in ev_copy[k % nh]:
                stream.wait_event(ev)
            ev_in[k].record(stream)
            th2 = time.perf_counter()
            _, fb_k = b.track_warm(net, fps[k % nh], descs=descs[k % nh], **tuned)
            ev_out[k].record(stream)
            ev_used[k % nh].record(stream)
            step_host.append([round((time.perf_counter() - th) * 1e3, 2), round((time.perf_counter() - th2) * 1e3, 2),
                              int(fb_k.sum())])
        e1.record(stream)
        torch.cuda.synchronize()
        for k in range(K):  # device time from the step's inputs being in place to the end of its tracking
            step_host[k].append(round(ev_in[k].elapsed_time(ev_out[k]), 2))
    ms_e2e = e0.elapsed_time(e1)
    if world > 1:
        tt = torch.tensor([ms_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_e2e = float(tt.item())
    # ---- roofline: the batched association kernel at level 0 ----
    b.track(fps[0], descs=descs[0])
    k_ms, s_ms, it_ms = b.time_iteration(0, reps=10)
    px = nb * cam.width * cam.height
    alg = BYTES_PER_PX_ITER * px
    peak, peak_kind = measured_peaks()
    achieved = alg / (k_ms * 1e-3) / 1e9
    traffic_px = profile_traffic(TRAFFIC_PROFILE_BATCH)
    # kernels per warm step: the network (per 256 pairs: argument copy,
    # packing, 8 GEMMs; then the time-out flag copy), the warm graph
    # (argument and state copies in, stamp, model maps, 2 photometric inputs,
    # 4 pyramid steps, 2 depth pyramid steps, maps, derivatives, begin, seed,
    # 3 per iteration, end, state copy out), the proposals' copy out, and the
    # fall-back batch (copies in, stamp, its photometric input and 2 pyramid
    # steps for the SO3 stage, SO3, begin, 3 per iteration of 10/5/4, end,
    # copy out)
    fbr = acc_tuned["fallback_rate"]
    net_k = -(-nb // max(256, nb)) * 10 + 1
    warm_graph = 18 + 3 * sum(its[:args.warm_levels])
    fallback = 10 + 3 * 19
    launches = K * (net_k + warm_graph + 1 + (fallback if fbr > 0 else 0))
    return {"fps": world * K * nb / (ms_w * 1e-3), "ms_per_step": ms_w / K, "steps": K, "warmup": W, "batch_pairs": nb,
            "eval_pairs": nbatch * nb, "pool_batches": nbatch, "batch_bytes": batch_bytes,
            "schedule": {"levels": args.warm_levels, "iterations": list(its), "so3": False},
            "fallback_cfg": {"residual_limit": tuned["residual_limit"], "residual_ratio": args.residual_ratio,
                             "plain_residual_median": plain_res, "max_disagree_deg": args.max_disagree},
            "eval_thresholds": {"residual_ratio": 1.5, "max_disagree_deg": 0.5,
                                "frames_per_s": world * nbatch * nb / (ms_s * 1e-3), "ms_per_step": ms_s / nbatch,
                                "speedup_vs_plain_batched": (nbatch * nb / (ms_s * 1e-3)) / (K * nb / (ms_p * 1e-3)),
                                "iterations_saved": saved(acc_spec), **acc_spec},
            "train": {"pairs_rendered": args.train_pairs, "pairs_kept": n_train, "epochs": args.epochs,
                      "generation_s": gen_s, "train_s": train_s, "last_epoch_loss": hist[-1]},
            "launch": {"threads": threads, "pixels_per_thread": ppt},
            "e2e": {"value": world * K * nb / (ms_e2e * 1e-3), "unit": "frames/s", "h2d_bytes_per_step": int(batch_bytes),
                    "median_step_frames_per_s": world * nb / (float(np.median([s[0] for s in step_host])) * 1e-3),
                    "d2h_bytes_per_step": int(nb * ctypes_sizeof_result()), "h2d_gbs_alone": h2d_gbs,
                    "note": "copies of step k+1 (4 copy streams) overlap the tracking of step k (two input buffers)",
                    "steps_host_ms_track_host_ms_fallbacks_track_device_ms": step_host,
                    "step_note": "the tracking of every step takes the same device time; the host time of a step "
                                 "is longer when that step's input copy from host memory is slower (some copies of "
                                 "the 6.45 GB run at a fraction of the usual ~210 GB/s)"},
            "roofline": {"bound": "hbm", "kernel": "k_icp_rgbres_b (level 0, all pairs of a step)",
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "alg_bytes_per_px": BYTES_PER_PX_ITER,
                         "alg_bytes_per_launch": alg,
                         "traffic": traffic_px * px if traffic_px else None,
                         "traffic_source": "profiles/" + TRAFFIC_PROFILE_BATCH +
                                           " (one-kernel ncu capture, DRAM bytes per pixel x the launch's pixels)",
                         "record_bytes_per_px": RECORD_BYTES_PER_PX,
                         "record_note": "the correspondence record the kernel writes for the photometric pass "
                                        "is not algorithmic traffic; it is inside `traffic`",
                         "kernel_ms": k_ms, "photometric_kernel_ms": s_ms, "iteration_ms": it_ms,
                         "iteration_frac": alg / (it_ms * 1e-3) / 1e9 / peak},
            "plain_batched": {"frames_per_s": world * K * nb / (ms_p * 1e-3), "ms_per_step": ms_p / K,
                              "schedule": "SO3 + 10/5/4, the reference's"},
            "accuracy": {"held_out_pairs": nbatch * nb, "warm_tuned": acc_tuned, "plain_batched": acc_plain,
                         "iterations_saved_tuned": saved(acc_tuned),
                         "fail_definition": "error > 2 deg or > 5 cm vs ground truth",
                         "vs_fp64_oracle": dist},
            "clocks": clk, "gpu_launches": int(launches)}


def measure_batched_verification(args, stream, world):
    """Batched verification: args.verify_pairs pairs per launch at sizes drawn
    uniformly from {160x120, 320x240, 640x480} (fx scaled), seeded rooms,
    motion <= 8 deg / 15 cm, 2-3 pyramid levels, the reference's schedule with
    SO3, one CUDA graph with the autotuned launch shape; pairs/s and the
    per-pair device latency (p50 / p99)."""
    import torch
    from slam_gb300 import synth, warmstart as ws
    from slam_gb300.batch import BatchOdometry, FramePair, result_pose
    n = args.verify_pairs
    rng = np.random.default_rng(args.seed * 7 + 5)
    size_of = rng.integers(0, 3, size=n)
    levels = rng.integers(2, 4, size=n)
    sizes = [(160, 120), (320, 240), (640, 480)]
    sets = {}
    for si, (w, h) in enumerate(sizes):
        cnt = int((size_of == si).sum())
        if cnt:
            sets[si] = ws.make_room_pairs(args.seed * 131 + si, cnt, synth.Camera().scaled(w, h), 8.0, 0.15)
    fps, T2, next_of = [], [], {si: 0 for si in sets}
    for i in range(n):
        si = int(size_of[i])
        ps, j = sets[si], next_of[si]
        next_of[si] += 1
        fps.append(FramePair(ps.cam, ps.model_vert[j], ps.model_norm[j], ps.model_rgba[j], ps.depth[j], ps.rgba[j],
                             ps.model_rgba[j], ps.T1[j], levels=int(levels[i])))
        T2.append(ps.T2[j])
    b = BatchOdometry(n, stream=stream.cuda_stream)
    threads, ppt, tune_ms = b.autotune(fps)
    descs = b._descs(fps)
    for _ in range(max(args.warmup, 3)):
        b.track(fps, descs=descs)
    K = max(args.steps, 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with no_gc():
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(K):
            res = b.track(fps, descs=descs)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    done = np.array([r.done_us for r in res])
    err = np.array([synth.pose_error(result_pose(r), T) for r, T in zip(res, T2)])
    return {"metric": "batched verification pairs/s", "value": world * n / (ms * 1e-3), "unit": "pairs/s",
            "steps": K, "ms_per_step": ms,
            "workload": f"{n} pairs per launch, sizes uniform over 160x120/320x240/640x480 "
                        f"({', '.join('%dx%d: %d' % (sizes[k] + (int((size_of == k).sum()),)) for k in range(3))}), "
                        "motion <= 8 deg / 15 cm, 2-3 levels, ICP+RGB with SO3, one CUDA graph",
            "launch": {"threads": threads, "pixels_per_thread": ppt, "autotune_best_ms": tune_ms},
            "latency_us": {"p50": float(np.percentile(done, 50)), "p99": float(np.percentile(done, 99)),
                           "note": "device time from the batch's first kernel to the end of the pair's last solve; "
                                   "all pairs advance level by level together"},
            "pose_error_vs_gt": {"rot_rad_p50": float(np.median(err[:, 0])),
                                 "trans_m_p50": float(np.median(err[:, 1]))}}


def ctypes_sizeof_result():
    import ctypes
    from slam_gb300 import _native
    return ctypes.sizeof(_native.OdoPairResult)


def make_batch_pairs(n, seed, sizes="mixed"):
    """Mixed-resolution verification pairs: sizes uniform over
    {160x120, 320x240, 640x480} (fx scaled; or 640x480 only), seeded rooms,
    motion <= 8 deg / 15 cm, 2-3 pyramid levels."""
    from slam_gb300 import synth
    rng = np.random.default_rng(seed)
    sizes = [(160, 120), (320, 240), (640, 480)] if sizes == "mixed" else [(640, 480)] * 3
    rooms = [synth.make_room(seed * 1000 + r, 20) for r in range(16)]
    pairs = []
    for i in range(n):
        w, h = sizes[int(rng.integers(0, 3))]
        p = synth.make_pair(seed * 100000 + i, cam=synth.Camera().scaled(w, h), max_deg=8.0, max_m=0.15,
                            scene=rooms[i % 16])
        p["levels"] = int(rng.integers(2, 4))
        pairs.append(p)
    return pairs


def run_batch_study(args):
    import torch
    from slam_gb300 import synth
    from slam_gb300.batch import BatchOdometry, FramePair, result_pose
    torch.cuda.set_device(0)
    t0 = time.time()
    pairs = make_batch_pairs(args.pairs, args.seed, args.sizes)
    gen_s = time.time() - t0
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    devd = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)
    fps = [FramePair(p["cam"], dev(p["model_vert"]), dev(p["model_norm"]), dev(p["model_rgba"]), devd(p["depth"]),
                     dev(p["rgba"]), dev(p["prev_rgba"]), p["T1"], levels=p["levels"]) for p in pairs]
    stream = torch.cuda.current_stream()
    b = BatchOdometry(len(fps), stream=stream.cuda_stream)
    default_res = b.track(fps)
    for _ in range(2):
        b.track(fps)
    torch.cuda.synchronize()
    t = time.perf_counter()
    b.track(fps)
    default_ms = (time.perf_counter() - t) * 1e3
    default_poses = [result_pose(r) for r in default_res]
    if args.launch:
        threads, ppt = (int(v) for v in args.launch.split("x"))
        b.set_launch(threads, ppt)
        tune_ms = None
    elif args.no_autotune:
        threads, ppt, tune_ms = 256, 2, default_ms
    else:
        threads, ppt, tune_ms = b.autotune(fps)
    descs = b._descs(fps)
    for _ in range(max(args.warmup, 3)):
        b.track(fps, descs=descs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        res = b.track(fps, descs=descs)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    done = np.array([r.done_us for r in res])
    err = [synth.pose_error(result_pose(r), p["T2"]) for r, p in zip(res, pairs)]
    d_default = [synth.pose_error(result_pose(r), T) for r, T in zip(res, default_poses)]
    differs = [k for k, d in enumerate(d_default) if d[0] > 1e-5 or d[1] > 1e-5]
    # a pair "fails" when its tracked pose is off the ground truth by > 2 deg or 10 cm
    failed = [k for k, e in enumerate(err) if e[0] > math.radians(2.0) or e[1] > 0.10]
    px_iters = 0
    for p in pairs:
        n0 = p["cam"].width * p["cam"].height
        px_iters += sum(it * (n0 >> (2 * l)) for l, it in enumerate([10, 5, 4][:p["levels"]]))
    out = {"metric": "batched verification pairs/s (mixed 160x120-640x480, one CUDA graph)",
           "value": len(pairs) / (ms * 1e-3), "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "data": "synthetic",
           "config": {"workload": f"{len(pairs)} pairs per launch, sizes " +
                                  ("uniform over 160x120/320x240/640x480" if args.sizes == "mixed" else "640x480") +
                                  ", motion <= 8 deg / 15 cm, 2-3 levels, ICP+RGB, SO3 on",
                      "autotuned_launch": {"threads": threads, "pixels_per_thread": ppt, "ms": tune_ms},
                      "default_launch": {"threads": 256, "pixels_per_thread": 2, "ms_host_timed": default_ms},
                      "generation_s": gen_s},
           "pixel_iterations_per_step": px_iters,
           "gpix_iter_per_s": px_iters / (ms * 1e-3) / 1e9,
           "latency_us": {"p50": float(np.percentile(done, 50)), "p99": float(np.percentile(done, 99)),
                          "batch_ms": ms,
                          "note": "per pair: device time from the batch's first kernel to the end of the pair's "
                                  "last Gauss-Newton solve; results reach the host with the whole batch"},
           "pose_error_vs_gt": {"rot_rad_median": float(np.median([e[0] for e in err])),
                                "trans_m_median": float(np.median([e[1] for e in err])),
                                "failed_pairs": len(failed)},
           "autotuned_vs_default_launch": {
               "pairs_differing_over_1e-5": len(differs),
               "of_which_failed": len(set(differs) & set(failed)),
               "max_diff_converged_pairs": [max([d_default[k][0] for k in differs if k not in failed] + [0.0]),
                                            max([d_default[k][1] for k in differs if k not in failed] + [0.0])]}}
    print(json.dumps(out), flush=True)


def _unpack29(v):
    A = np.zeros((6, 6))
    b = np.zeros(6)
    k = 0
    for i in range(6):
        for j in range(i, 7):
            if j == 6:
                b[i] = v[k]
            else:
                A[i, j] = A[j, i] = v[k]
            k += 1
    return A, b


PRECISION_FIELDS = ["pair", "cond", "inliers", "point", "relA_fp32", "relA_comp", "relb_fp32", "relb_comp",
                    "inc_rot_fp32", "inc_rot_comp", "inc_trans_fp32", "inc_trans_comp", "count_diff_fp32",
                    "count_diff_comp"]


def precision_corridor(i, seed, cam, kind):
    """Pair i of the precision study.  'tapered': no clutter, side walls
    tapered by |taper| log-uniform in [2e-4, 4e-3] (random sign), which puts
    cond(JtJ) of the level-0 ICP normal equations mostly in 1e6-1e9;
    'clutter': straight walls and 24 clutter spheres (cond mostly 1e3-1e5,
    or singular when no sphere is in view)."""
    from slam_gb300 import synth
    s = seed * 100000 + i
    if kind == "clutter":
        return synth.make_corridor_pair(s, cam=cam)
    rng = np.random.default_rng(s ^ 0x7a9e)
    taper = float(np.exp(rng.uniform(np.log(2e-4), np.log(4e-3)))) * (1.0 if rng.uniform() < 0.5 else -1.0)
    return synth.make_corridor_pair(s, cam=cam, nclutter=0, taper=taper)


def precision_pair(i, seed, g32, gcomp, k64, cam, dist, angle, kind="tapered"):
    """One corridor pair of the precision study: the ICP normal equations at
    level 0 (at the start pose and at the FP64 oracle's converged pose) as the
    tracker's FP32 and compensated-FP32 reductions deliver them, against the
    FP64 oracle's on the same FP32 maps; the increments A^-1 b of each (one
    FP64 LDLT, as the tracker's solve); the tracked poses against the FP64
    oracle's tracking of the same raw frames."""
    import torch
    from slam_gb300 import synth
    from oracle import oracle
    p = precision_corridor(i, seed, cam, kind)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    devd = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)
    T1 = p["T1"]
    poses = {}
    for name, g in (("fp32", g32), ("comp", gcomp)):
        g.initFirstRGB(dev(p["prev_rgba"]))
        g.initICPModel(dev(p["model_vert"]), dev(p["model_norm"]), 20.0, T1.astype(np.float32))
        g.initRGBModel(dev(p["model_rgba"]))
        g.initICP(devd(p["depth"]), 20.0)
        g.initRGB(dev(p["rgba"]))
        t, R = g.getIncrementalTransformation(T1[:3, 3].astype(np.float32), T1[:3, :3].astype(np.float32),
                                              rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False, so3=True)
        poses[name] = synth.pose(np.asarray(R, np.float64), np.asarray(t, np.float64))
    o = oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, dist, angle, prec=64)
    o.initFirstRGB(p["prev_rgba"])
    o.initICPModel(p["model_vert"], p["model_norm"], 20.0, T1.astype(np.float32))
    o.initRGBModel(p["model_rgba"])
    o.initICP(p["depth"], 20.0)
    o.initRGB(p["rgba"])
    t64, R64 = o.getIncrementalTransformation(T1[:3, 3], T1[:3, :3], rgbOnly=False, icpWeight=10.0, pyramid=True,
                                              fastOdom=False, so3=True)
    T64 = synth.pose(np.asarray(R64, np.float64), np.asarray(t64, np.float64))
    o.close()
    maps = [g32.download(w, 0) for w in (1, 2, 3, 4)]
    rows = []
    Rp, tp = T1[:3, :3].astype(np.float32), T1[:3, 3].astype(np.float32)
    Rpi = np.linalg.inv(Rp.astype(np.float64)).astype(np.float32)
    for point, Tc in (("start", T1), ("converged", T64)):
        Rc, tc = Tc[:3, :3].astype(np.float32), Tc[:3, 3].astype(np.float32)
        s64, _, _ = k64.icp_step(Rc, tc, maps[0], maps[1], Rpi, tp, cam.fx, cam.fy, cam.cx, cam.cy, maps[2], maps[3],
                                 dist, angle)
        A64, b64 = _unpack29(s64)
        x64 = oracle.ldlt_solve6(A64, b64)
        row = {"pair": i, "cond": float(np.linalg.cond(A64)), "inliers": int(s64[28]), "point": point}
        for name, g in (("fp32", g32), ("comp", gcomp)):
            s = g.debug_icp_sums(0, Rc, tc, Rpi, tp)
            A, b = _unpack29(s)
            x = oracle.ldlt_solve6(A, b)
            row["relA_" + name] = float(np.linalg.norm(A - A64) / np.linalg.norm(A64))
            row["relb_" + name] = float(np.linalg.norm(b - b64) / max(np.linalg.norm(b64), 1e-300))
            row["inc_trans_" + name] = float(np.linalg.norm(x[:3] - x64[:3]))
            row["inc_rot_" + name] = float(np.linalg.norm(x[3:] - x64[3:]))
            row["count_diff_" + name] = int(s[28] - s64[28])
        rows.append(row)
    pose_rows = {}
    for name in ("fp32", "comp"):
        pose_rows[name] = synth.pose_error(poses[name], T64)
    pose_rows["fp64_vs_gt"] = synth.pose_error(T64, p["T2"])
    pose_rows["fp32_vs_comp"] = synth.pose_error(poses["fp32"], poses["comp"])
    return rows, pose_rows


def run_precision_study(args):
    """Precision study on low-texture corridor pairs (2 m x 20 m, floor-dominated
    views, ~3 % of pixels on clutter): FP32 and compensated-FP32 JtJ/Jtr,
    increments and tracked poses against the FP64 oracle (the oracle is the
    checker here; nothing measured runs on it)."""
    import csv
    import torch
    from slam_gb300 import synth, RGBDOdometry, PREC_COMPENSATED
    from oracle import oracle
    torch.cuda.set_device(0)
    cam = synth.Camera()
    from slam_gb300.odometry import DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    dist, angle = DEFAULT_DIST_THRESH, DEFAULT_ANGLE_THRESH
    g32 = RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, dist, angle)
    gcomp = RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, dist, angle)
    gcomp.set_precision(PREC_COMPENSATED)
    k64 = oracle.Kernels(64)
    t0 = time.time()
    rows, poses = [], []
    for i in range(args.pairs):
        r, pr = precision_pair(i, args.seed, g32, gcomp, k64, cam, dist, angle, args.corridor)
        rows += r
        poses.append(pr)
    elapsed = time.time() - t0
    if args.pairs_out:
        with open(args.pairs_out, "w", newline="") as f:
            w = csv.writer(f)
            w.writerow(PRECISION_FIELDS + ["pose_rot_fp32", "pose_trans_fp32", "pose_rot_comp", "pose_trans_comp",
                                           "fp64_rot_vs_gt", "fp64_trans_vs_gt"])
            for r in rows:
                pr = poses[r["pair"]]
                w.writerow([r[k] for k in PRECISION_FIELDS] + list(pr["fp32"]) + list(pr["comp"]) +
                           list(pr["fp64_vs_gt"]))
    pct = lambda v: {"p50": float(np.percentile(v, 50)), "p90": float(np.percentile(v, 90)),
                     "p99": float(np.percentile(v, 99)), "max": float(np.max(v))}
    summary = {}
    for point in ("start", "converged"):
        sel = [r for r in rows if r["point"] == point]
        d = {"cond": {"p5": float(np.percentile([r["cond"] for r in sel], 5)),
                      "p50": float(np.percentile([r["cond"] for r in sel], 50)),
                      "p95": float(np.percentile([r["cond"] for r in sel], 95))},
             "pairs_with_inlier_count_diff": int(sum(1 for r in sel if r["count_diff_fp32"] != 0))}
        for name in ("fp32", "comp"):
            d[name] = {k: pct([r[k + "_" + name] for r in sel]) for k in ("relA", "relb", "inc_rot", "inc_trans")}
        summary[point] = d
    pose = {}
    for name in ("fp32", "comp"):
        rot = np.array([p[name][0] for p in poses])
        tr = np.array([p[name][1] for p in poses])
        pose[name] = {"rot_rad": pct(rot), "trans_m": pct(tr),
                      "frac_within_1e-5": float(np.mean((rot <= 1e-5) & (tr <= 1e-5)))}
    # by the condition number of the FP64 JtJ at the start pose
    bins = {}
    start = {r["pair"]: r for r in rows if r["point"] == "start"}
    for lo, hi, name in ((0, 1e4, "<1e4"), (1e4, 1e6, "1e4-1e6"), (1e6, 1e9, "1e6-1e9"), (1e9, np.inf, ">1e9")):
        idx = [k for k, r in start.items() if lo <= r["cond"] < hi]
        if not idx:
            bins[name] = {"pairs": 0}
            continue
        b = {"pairs": len(idx)}
        for name_ in ("fp32", "comp"):
            med = lambda key: float(np.median([start[k][key + "_" + name_] for k in idx]))
            rot = np.array([poses[k][name_][0] for k in idx])
            tr = np.array([poses[k][name_][1] for k in idx])
            b[name_] = {"relA_p50": med("relA"), "relb_p50": med("relb"), "inc_rot_p50": med("inc_rot"),
                        "inc_trans_p50": med("inc_trans"), "pose_rot_p50": float(np.median(rot)),
                        "pose_trans_p50": float(np.median(tr)),
                        "frac_within_1e-5": float(np.mean((rot <= 1e-5) & (tr <= 1e-5)))}
        bins[name] = b
    pose["fp64_oracle_vs_ground_truth"] = {"rot_rad": pct([p["fp64_vs_gt"][0] for p in poses]),
                                           "trans_m": pct([p["fp64_vs_gt"][1] for p in poses])}
    pose["fp32_vs_comp"] = {"rot_rad": pct([p["fp32_vs_comp"][0] for p in poses]),
                            "trans_m": pct([p["fp32_vs_comp"][1] for p in poses])}
    corridor = ("no clutter, side walls tapered by 2e-4..4e-3 (log-uniform)" if args.corridor == "tapered"
                else "24 clutter spheres, straight walls")
    out = {"study": "precision", "pairs": args.pairs, "data": "synthetic",
           "config": {"workload": "low-texture corridor 2 m x 20 m (" + corridor + "), camera 1.5 m above the "
                                  "floor pitched down 25-40 deg, <= 3 deg / 5 cm relative motion, 640x480, 3 levels "
                                  "10/5/4, ICP+RGB (icpWeight 10), SO3 on",
                      "jtj": "level-0 ICP sums at the start pose and at the FP64 oracle's converged pose; "
                             "FP64 reference = oracle on the same FP32 maps"},
           "jtj_increment": summary, "pose_vs_fp64_oracle": pose, "by_start_cond": bins, "elapsed_s": elapsed}
    print(json.dumps(out), flush=True)


def _res_array(res):
    """Poses [n,4,4], lastICPError [n], iterations [n,4] of a result array."""
    n = len(res)
    P = np.array([np.array(r.pose, np.float64).reshape(4, 4) for r in res]).reshape(n, 4, 4)
    e = np.array([r.lastICPError for r in res], np.float64)
    it = np.array([list(r.iterations) for r in res], np.int64).reshape(n, 4)
    return P, e, it


def _errs(P, T):
    from slam_gb300 import synth
    return np.array([synth.pose_error(P[i], T[i]) for i in range(len(P))]).reshape(len(P), 2)


def run_warm_study(args):
    """Learned warm start (batched) against the plain tracker on held-out
    640x480 room pairs (motion <= 10 deg / 10 cm): the network is trained
    here, on the GPU, by the library's own kernels, on pairs rendered on the
    GPU and labelled by the plain tracker."""
    import torch
    from slam_gb300 import synth, warmstart as ws, RGBDOdometry, DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH
    from slam_gb300.batch import BatchOdometry
    torch.cuda.set_device(0)
    cam = synth.Camera()
    b = BatchOdometry(512)
    net = ws.WarmStartNet(max_batch=256)
    if args.load_params:
        d = np.load(args.load_params)
        net.set_params(d["params"])
        plain_res, n_train, gen_s, train_s, hist = float(d["plain_residual"]), int(d["n_train"]), 0.0, 0.0, [None]
    else:
        t0 = time.time()
        ts = ws.make_training_set(net, b, args.seed * 17 + 3, args.train_pairs)
        torch.cuda.synchronize()
        gen_s = time.time() - t0
        net.set_loss_metric(ts["metric"])
        t0 = time.time()
        hist = ws.train(net, ts["inputs"], ts["labels"], epochs=args.epochs, batch=256, lr=args.lr,
                        lr_final=args.lr / 30)
        torch.cuda.synchronize()
        train_s = time.time() - t0
        plain_res = float(np.median(ts["residuals"]))
        n_train = int(ts["labels"].shape[0])
        del ts
        if args.save_params:
            np.savez(args.save_params, params=net.get_params(), plain_residual=plain_res, n_train=n_train)
    its = tuple(int(v) for v in args.warm_iters.split(","))
    wkw = dict(levels=args.warm_levels, iterations=its, residual_limit=args.residual_ratio * plain_res,
               max_disagree_deg=args.max_disagree)
    chunk, reps = 500, 3
    t_plain = t_warm = 0.0
    rows = {"plain": [], "warm": []}
    T2, fbs, props_err = [], [], []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    oracle_sets, single_fps = [], None
    for c, s in enumerate(range(0, args.eval_pairs, chunk)):
        m = min(chunk, args.eval_pairs - s)
        ps = ws.make_room_pairs(args.seed * 31 + 1000 + c, m, cam, 10.0, 0.10)
        fps = ps.frame_pairs()
        descs = b._descs(fps)
        if c == 0:
            tuned = b.autotune(fps)                          # launch shape of both paths
            prop = net.propose(fps).cpu().numpy().astype(np.float64)
            gt = np.stack([ws.motion_vec(np.linalg.inv(ps.T1[i]) @ ps.T2[i]) for i in range(m)])
            prop_err = (np.linalg.norm(prop[:, :3] - gt[:, :3], axis=1), np.linalg.norm(prop[:, 3:] - gt[:, 3:], axis=1))
            sweep = []
            if args.sweep:
                rp0 = b.track(fps, descs=descs)
                Pp0 = _res_array(rp0)[0]
                for lv, it_ in ((3, (1, 2, 2)), (3, (2, 2, 1)), (3, (2, 2, 2)), (3, (3, 2, 2))):
                    for ratio in (6.0, 8.0, 12.0, 16.0):
                        kw = dict(wkw, levels=lv, iterations=it_, residual_limit=ratio * plain_res)
                        b.track_warm(net, fps, descs=descs, **kw)
                        torch.cuda.synchronize()
                        tt = time.perf_counter()
                        rw0, fb0 = b.track_warm(net, fps, descs=descs, **kw)
                        torch.cuda.synchronize()
                        tt = time.perf_counter() - tt
                        Pw0, ew0, _ = _res_array(rw0)
                        ee = _errs(Pw0, ps.T2)
                        sweep.append({"levels": lv, "iterations": list(it_), "residual_ratio": ratio,
                                      "fps": m / tt, "fallback": float(fb0.mean()),
                                      "rot_p50": float(np.median(ee[:, 0])), "trans_p50": float(np.median(ee[:, 1])),
                                      "rot_p90": float(np.percentile(ee[:, 0], 90)),
                                      "trans_p90": float(np.percentile(ee[:, 1], 90)),
                                      "fail": float(np.mean((ee[:, 0] > np.radians(2)) | (ee[:, 1] > 0.05)))})
        rp = b.track(fps, descs=descs)                      # warm-up (graph instantiation)
        rw, fb = b.track_warm(net, fps, descs=descs, **wkw)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            rp = b.track(fps, descs=descs)
        e1.record(stream)
        torch.cuda.synchronize()
        t_plain += e0.elapsed_time(e1) / reps
        e0.record(stream)
        for _ in range(reps):
            rw, fb = b.track_warm(net, fps, descs=descs, **wkw)
        e1.record(stream)
        torch.cuda.synchronize()
        t_warm += e0.elapsed_time(e1) / reps
        if c == 0:
            # one more step of each, bracketed by NVTX ranges, for a profiler's
            # launch list (ncu --nvtx --nvtx-include "warm_step/" ...)
            for name, fn in (("plain_step", lambda: b.track(fps, descs=descs)),
                             ("warm_step", lambda: b.track_warm(net, fps, descs=descs, **wkw))):
                _nvtx(name, fn)
        rows["plain"].append(_res_array(rp))
        rows["warm"].append(_res_array(rw))
        fbs.append(fb)
        T2.append(ps.T2)
        if c == 0 and args.oracle_pairs > 0:
            k = min(args.oracle_pairs, m)
            oracle_sets = [(ps.cam, ps.T1[i], ps.model_vert[i].cpu().numpy(), ps.model_norm[i].cpu().numpy(),
                            ps.model_rgba[i].cpu().numpy(), ps.depth[i].view(torch.int16).cpu().numpy().view(np.uint16),
                            ps.rgba[i].cpu().numpy()) for i in range(k)]
            # the drop-in single-pair path on the same pairs
            h = RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy)
            torch.cuda.synchronize()
            t = time.perf_counter()
            for i in range(k):
                h.initFirstRGB(ps.model_rgba[i])
                h.initICPModel(ps.model_vert[i], ps.model_norm[i], 20.0, ps.T1[i])
                h.initRGBModel(ps.model_rgba[i])
                h.initICP(ps.depth[i], 20.0)
                h.initRGB(ps.rgba[i])
                h.getIncrementalTransformation(ps.T1[i][:3, 3].astype(np.float32), ps.T1[i][:3, :3].astype(np.float32))
            torch.cuda.synchronize()
            single_fps = k / (time.perf_counter() - t)
        del ps, fps
    Pp, ep, itp = (np.concatenate([r[j] for r in rows["plain"]]) for j in range(3))
    Pw, ew, itw = (np.concatenate([r[j] for r in rows["warm"]]) for j in range(3))
    T2 = np.concatenate(T2)
    fb = np.concatenate(fbs)
    n = len(Pp)
    err_p, err_w = _errs(Pp, T2), _errs(Pw, T2)
    d = _errs(Pw, Pp)
    fail = lambda e: float(np.mean((e[:, 0] > np.radians(2.0)) | (e[:, 1] > 0.05)))
    pct = lambda v: {"p50": float(np.percentile(v, 50)), "p90": float(np.percentile(v, 90))}
    disagree = (ew > 1.5 * ep) | (d[:, 0] > np.radians(0.5))
    # FP64 oracle on the first pairs (plain tracking of the same frames)
    from oracle import oracle
    orc = []
    for i, (c_, T1, mv, mn, mc, dep, rgba) in enumerate(oracle_sets):
        o = oracle.Odometry(c_.width, c_.height, c_.cx, c_.cy, c_.fx, c_.fy, DEFAULT_DIST_THRESH,
                            DEFAULT_ANGLE_THRESH, prec=64)
        o.initFirstRGB(mc)
        o.initICPModel(mv, mn, 20.0, T1.astype(np.float32))
        o.initRGBModel(mc)
        o.initICP(dep, 20.0)
        o.initRGB(rgba)
        t, R = o.getIncrementalTransformation(T1[:3, 3], T1[:3, :3])
        To = synth.pose(np.asarray(R, np.float64), np.asarray(t, np.float64))
        o.close()
        orc.append((synth.pose_error(Pp[i], To), synth.pose_error(Pw[i], To), synth.pose_error(To, T2[i])))
    within = lambda k: float(np.mean([(x[k][0] <= 1e-5 and x[k][1] <= 1e-5) for x in orc])) if orc else None
    out = {"study": "warm", "metric": "warm-started batched vs plain tracking frames/s @640x480, equal pose error",
           "unit": "frames/s", "data": "synthetic",
           "config": {"workload": f"{n} held-out room pairs 640x480 (6x4x3 m rooms, 20 spheres), motion <= 10 deg / "
                                  "10 cm, batches of 500",
                      "train": {"pairs_rendered": args.train_pairs, "pairs_kept": n_train, "epochs": args.epochs,
                                "generation_s": gen_s, "train_s": train_s, "last_epoch_loss": hist[-1]},
                      "warm_schedule": {"levels": args.warm_levels, "iterations": list(its), "so3": False},
                      "fallback": {"residual_limit": args.residual_ratio * plain_res, "residual_ratio": args.residual_ratio,
                                   "max_disagree_deg": args.max_disagree}},
           "plain_batched_fps": n / (t_plain * 1e-3), "warm_batched_fps": n / (t_warm * 1e-3),
           "plain_single_pair_fps": single_fps,
           "speedup_vs_plain_batched": t_plain / t_warm,
           "speedup_vs_plain_single": n / (t_warm * 1e-3) / single_fps if single_fps else None,
           "pose_error_vs_gt": {"plain": {"rot_rad": pct(err_p[:, 0]), "trans_m": pct(err_p[:, 1]), "fail": fail(err_p)},
                                "warm": {"rot_rad": pct(err_w[:, 0]), "trans_m": pct(err_w[:, 1]), "fail": fail(err_w)}},
           "warm_vs_plain": {"within_1e-5": float(np.mean((d[:, 0] <= 1e-5) & (d[:, 1] <= 1e-5))),
                             "within_1e-4": float(np.mean((d[:, 0] <= 1e-4) & (d[:, 1] <= 1e-4))),
                             "disagreement_rate": float(np.mean(disagree))},
           "runtime_fallback_rate": float(np.mean(fb)),
           "iterations_mean": {"plain": itp.mean(axis=0).tolist(), "warm": itw.mean(axis=0).tolist()},
           "proposal_error_vs_gt": {"trans_m": pct(prop_err[0]), "rot_rad": pct(prop_err[1])},
           "launch": {"threads": tuned[0], "pixels_per_thread": tuned[1]},
           "loss_history": [h for h in hist if h is not None][-5:], "sweep": sweep,
           "fp64_oracle": {"pairs": len(orc), "plain_within_1e-5": within(0), "warm_within_1e-5": within(1),
                           "oracle_vs_gt_rot_p50": float(np.median([x[2][0] for x in orc])) if orc else None}}
    print(json.dumps(out), flush=True)


def _nvtx(name, fn):
    """fn() inside an NVTX push/pop range (when torch has NVTX)."""
    import torch
    torch.cuda.synchronize()
    try:
        torch.cuda.nvtx.range_push(name)
        pushed = True
    except Exception:
        pushed = False
    try:
        out = fn()
        torch.cuda.synchronize()
    finally:
        if pushed:
            torch.cuda.nvtx.range_pop()
    return out


def run_phases_study(args):
    """The time split of a warm-started batched step of --batch-pairs 640x480
    pairs (CUDA events around whole calls, no profiler): the step without
    fall-backs; the same tracking from precomputed proposals (no network in
    the step); the network alone; 1/1/1 iterations and one level-0
    iteration (so the preprocessing and one iteration set separate); the
    plain step; per-level iteration kernels.  The network is untrained
    (its proposals only feed the 2/2/2 schedule, whose cost does not depend
    on them)."""
    import ctypes
    import torch
    from slam_gb300 import synth, warmstart as ws, _native
    from slam_gb300.batch import BatchOdometry
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    nb = args.batch_pairs
    b = BatchOdometry(nb, stream=stream.cuda_stream)
    net = ws.WarmStartNet(max_batch=nb, stream=stream.cuda_stream)
    pool = ws.make_room_pairs(args.seed * 31 + 1000, nb, synth.Camera(), 10.0, 0.10)
    fps = pool.frame_pairs()
    descs = b._descs(fps)
    b.set_launch(256, 64)
    L = _native.load()
    nofb = dict(levels=3, iterations=(2, 2, 2), residual_limit=0.0, max_disagree_deg=0.0)
    if args.nvtx_steps:
        for _ in range(max(args.warmup, 3)):
            b.track_warm(net, fps, descs=descs, **nofb)
            b.track(fps, descs=descs)
        _nvtx("warm_step", lambda: b.track_warm(net, fps, descs=descs, **nofb))
        _nvtx("plain_step", lambda: b.track(fps, descs=descs))
        print(json.dumps({"study": "phases", "nvtx_steps": ["warm_step", "plain_step"], "pairs": nb}), flush=True)
        return
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, r

    def descs_with(levels, its):
        d = b._descs(fps)
        for i in range(nb):
            d[i].levels = levels
            for l in range(3):
                d[i].iterations[l] = its[l]
        return d

    prop = torch.empty((nb, 6), dtype=torch.float32, device="cuda")

    def net_only():
        assert L.odo_cnn_propose(net._h, descs, nb, ctypes.c_void_p(prop.data_ptr())) == 0
        assert L.odo_cnn_wait(net._h) == 0

    out = {"study": "phases", "pairs": nb, "steps": args.steps, "unit": "ms per step",
           "config": {"workload": f"{nb} held-out 640x480 room pairs, warm schedule 3 levels 2/2/2 without SO3, "
                                  "no fall-backs; untrained network"}}
    out["warm_step_no_fallback"] = timed(lambda: b.track_warm(net, fps, descs=descs, **nofb))[0]
    out["network_alone"] = timed(net_only)[0]
    for key, levels, its in (("from_proposals_2_2_2", 3, (2, 2, 2)), ("from_proposals_1_1_1", 3, (1, 1, 1)),
                             ("from_proposals_level0_once", 1, (1, 0, 0))):
        d = descs_with(levels, its)
        ms, res = timed(lambda: b.track_init(fps, prop, descs=d))
        out[key] = {"ms": ms, "device_ms_first_kernel_to_last_solve": max(r.done_us for r in res) * 1e-3}
    out["plain_step"] = timed(lambda: b.track(fps, descs=descs))[0]
    out["iteration_kernels_ms"] = {"level%d" % l: dict(zip(("association", "photometric_and_solve", "whole"),
                                                           b.time_iteration(l, 20))) for l in range(3)}
    a, c, d = (out[k]["ms"] for k in ("from_proposals_2_2_2", "from_proposals_1_1_1", "from_proposals_level0_once"))
    out["derived"] = {"network_on_the_critical_path": out["warm_step_no_fallback"] - a,
                      "one_iteration_set_2_2_2_minus_1_1_1": a - c,
                      "preprocessing_and_fixed_costs": c - (a - c)}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.study == "phases":
        run_phases_study(args)
        return
    if args.study == "warm":
        run_warm_study(args)
        return
    if args.study == "batch":
        run_batch_study(args)
        return
    if args.study == "precision":
        run_precision_study(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
