"""Benchmark: ray casting on the 1,045,506-triangle heightfield at 1920x1080.

One step = one RAY frame: a closest-hit primary ray for every pixel and, for
every pixel that hits, one any-hit shadow ray toward the directional light
(the RAY tracer's ray set, Raytracer.cpp:27-97 + 497-522). Metric: Mrays/s =
BVH queries (primary + shadow) per second.

  value     device time of the frame (CUDA events on the tracer's stream, the
            scene resident in HBM, L2 flushed by a 512 MB write before every
            step, outside the timed events)
  e2e       the same frame through the C ABI with host buffers:
            rc_cast_with_shadow(pinned host rays -> pinned host results), the
            host-link traffic inside the timed region (the kernel reads the
            rays and writes the records in place)
  roofline  the frame's kernel (primary and shadow rays in one kernel; with
            RC_TRACE_FUSED=0 the primary kernel of the two) against the roof
            that binds it, instruction issue: warp instructions per launch
            (ncu) / its average event time, over 4 warp instructions per
            cycle per SM at the sampled SM clock. Beside it the HBM fraction
            (ncu DRAM bytes per launch / event time / measured copy
            bandwidth), ncu's L1 / L2 throughput fractions and the
            algorithmic bytes per launch (64 B per inner-node fetch + 48 B
            per triangle test, counted by a counting render that equals the
            float32 oracle's count, + 16 B record per pixel; + 8 B queue
            entry per hit pixel in the two-kernel form)

At N = 1 the line also carries the rest of the headline (unless
--headline-only):
  path_1m   plain path tracing of the same heightfield (+ an emissive panel
            overhead) at 1080p, 1 path per pixel, depth 4: device and e2e
            Mrays/s and the float64 port of the reference's path tracer on
            this host's cores (Tracer.cpp:58, PathTracer.cpp:25)
  path_room the same measures on the room (2,012 triangles, 320x240, 16 spp
            CMJ, depth 4)
  nrc       time to display RMSE 0.01 of the radiance-cache tracer and of
            the plain tracer against a float64 4096-spp ground truth on the
            heightfield + 200 blobs scene at 1080p, closed in a box lit by an
            emissive ceiling panel (the scene has no emitter of its own)
  nrc_sky   the same under a uniform sky instead of the box
  batch     64 rooms of uneven size in one CUDA-graph launch per frame
            (1 warm-up + 2 timed frames): aggregate Mrays/s, per-scene
            latency p50 / p99, and the float64 port's rate on every 8th
            scene of the batch (one after another, as the reference renders)

`--impl reference` times the reference's CPU ray casting on this host's cores
(the reference's own code where it was compiled, else the float64 port) on
the same workload, one full frame per step.

Multi-GPU: replicas only (every rank renders the full frame on its own GPU).
"""

from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s"
WORKLOAD = "heightfield ray cast 1920x1080: primary closest hit + directional shadow any-hit, 1,045,506 tris, SAH leaf<=4"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200; batch: 5, each step one 64-scene frame of about 4 s)")
    ap.add_argument("--warmup", type=int, default=None, help="untimed warm-up steps (default 10; batch: 3)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--order", choices=["nearest", "reference"], default="nearest")
    ap.add_argument("--workload", choices=["raycast", "batch", "nrc", "build", "large", "path", "cpu"], default="raycast",
                    help="raycast: the 1080p heightfield frame (default); batch: 64 rooms in one graph launch; "
                         "nrc: time to display RMSE 0.01, radiance cache vs plain path tracing")
    ap.add_argument("--enclosed", action="store_true",
                    help="nrc / large workloads: the geometry inside a closed box lit by an emissive panel, no sky")
    ap.add_argument("--gt-spp", type=int, default=4096, help="nrc / large: ground-truth samples per pixel")
    ap.add_argument("--scale", type=float, default=1.0, help="nrc: film scale (1 = 1920x1080)")
    ap.add_argument("--terminate-segment", type=int, default=2,
                    help="nrc: paths end into the cache at the hit of this segment")
    ap.add_argument("--headline-only", action="store_true",
                    help="raycast: the RAY frame only, without the path-tracing and radiance-cache records")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.workload == "batch" else 200
    if args.warmup is None:
        args.warmup = 3 if args.workload == "batch" else 10
    return args


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clock / throttle samples every 20 ms from before the warm-up
    to the end of the timed region. The summary uses the samples taken inside
    the timed region; when that region is shorter than a few sampling periods
    it widens the window backwards into the warm-up frames just before it (the
    same kernels at the same load) and says so."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.samples = []   # (host time, line)
        self.thread = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), line.strip()))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()
        time.sleep(0.05)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        parsed = []
        for ts, ln in self.samples:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                parsed.append((ts, float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        if not parsed or self.t0 is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        window = "timed region"
        inside = [p for p in parsed if self.t0 <= p[0] <= self.t1]
        if len(inside) < 3:
            before = [p for p in parsed if p[0] <= self.t1]
            inside = before[-5:]
            window = "timed region + the warm-up frames before it (region shorter than the sampling period)"
        reasons = set()
        for _, _, _, flags in inside:
            for name, val in zip(names, flags):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(p[1] for p in inside), "sm_max_mhz": inside[-1][2],
                "reasons": sorted(reasons), "samples": len(inside), "window": window}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_metrics(fused=False):
    """Figures of one launch of the frame's dominant kernel (the one-kernel
    frame of primary + shadow rays, or the two-kernel frame's primary kernel)
    from the committed ncu summary: DRAM bytes, warp instructions executed and
    the issue / L1 / L2 / DRAM throughput fractions ncu reported. Empty when
    the summary is missing."""
    f = ROOT / "profiles" / ("raycast_frame_fused_heightfield_1080p.md" if fused
                             else "raycast_primary_heightfield_1080p.md")
    if not f.exists():
        return {}
    text = f.read_text()
    out = {}
    for key in ("dram_bytes_per_launch", "warp_instructions_per_launch", "issue_active_frac", "l1_throughput_frac",
                "l2_throughput_frac", "dram_throughput_frac"):
        m = re.search(rf"^{key}:\s*([0-9.eE+]+)", text, re.M)
        if m:
            out[key] = float(m.group(1))
    return out


def profiled_traffic(fused=False):
    """DRAM bytes per launch of the frame's dominant kernel from the committed
    ncu summary, or None."""
    return profiled_metrics(fused).get("dram_bytes_per_launch")


def issue_roofline(prof, launch_s, sm_mhz, num_sms, alg_bytes, traffic, hbm_peak, peak_kind):
    """The frame kernel against the roof that binds it: instruction issue.

    The node array (17.6 MB) and the triangles the rays touch stay in L1/L2,
    so DRAM moves a fraction of a percent of the algorithmic bytes and HBM is
    not the bound; ncu shows the schedulers issuing in about three cycles of
    four (ALU pipe: the slab tests' min/max and compares). So:
      achieved = warp instructions of one launch (ncu; the count is fixed by
                 the frame's work) / the launch's CUDA-event time
      peak     = 4 warp instructions per cycle per SM (one per scheduler)
                 x SMs x the median SM clock sampled in the timed region
    The HBM fraction (ncu DRAM bytes of one launch / event time / the
    measured copy bandwidth) and ncu's L1 / L2 throughput fractions are
    reported beside it, with the algorithmic bytes per second."""
    out = {"bound": "issue", "unit": "G warp-instructions/s", "achieved": None, "peak": None, "frac": None,
           "avg_launch_ms": round(launch_s * 1e3, 4), "traffic": traffic,
           "algorithmic_bytes_per_launch": int(alg_bytes),
           "algorithmic_gbs": round(alg_bytes / launch_s / 1e9, 1)}
    inst = prof.get("warp_instructions_per_launch")
    if inst and sm_mhz:
        achieved = inst / launch_s / 1e9
        peak = 4.0 * num_sms * sm_mhz / 1e3
        out.update(achieved=round(achieved, 1), peak=round(peak, 1), frac=round(achieved / peak, 4),
                   peak_kind=f"4 warp-instructions/cycle/SM x {num_sms} SMs x {sm_mhz:.0f} MHz (median sampled)",
                   warp_instructions_per_launch=inst)
    hbm = {"peak_gbs": hbm_peak, "peak_kind": peak_kind, "achieved_gbs": None, "frac": None}
    if traffic:
        hbm["achieved_gbs"] = round(traffic / launch_s / 1e9, 1)
        hbm["frac"] = round(traffic / launch_s / 1e9 / hbm_peak, 5)
    out["hbm"] = hbm
    out["ncu_fracs"] = {k: prof[k] for k in ("issue_active_frac", "l1_throughput_frac", "l2_throughput_frac",
                                             "dram_throughput_frac") if k in prof}
    return out


def reduce_replicas(times, counts, world, device):
    """Whole-job figures of N replicas: each timed region is the maximum over
    the ranks, each count (rays) the sum. `device` holds the reduction's
    tensors (the rank's GPU under NCCL, the CPU under gloo). Returns the
    times then the counts, as floats."""
    import torch

    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device=device)
    c = torch.tensor([float(x) for x in counts], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
    return (*t.tolist(), *c.tolist())


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# CPU reference / port timing (one full frame per step)

def cpu_raycast(sc, steps, warmup, bvh):
    """The reference's ray casting of the frame on this host's cores: its own
    code where oracle/_ref was built, else the float64 port (the oracle's
    own BVH unless `bvh` is given, its float64 camera). Loads no part of the
    product library."""
    import oracle

    threads = cpu_threads()
    build_s = 0.0
    if oracle.ref_available(fast=True):
        kind = "reference"
        t_build = time.perf_counter()
        ref = oracle.RefScene(sc, fast=True)
        build_s = time.perf_counter() - t_build
        ref.set_general(0, 3, 1, 1)

        def frame():
            _, _, rays, sec = ref.render(sc.width, sc.height, threads=threads)
            return rays, sec
    else:
        kind = "port"
        t_build = time.perf_counter()
        orc = oracle.Oracle(sc, prebuilt=bvh)
        build_s = time.perf_counter() - t_build
        cam64 = oracle.camera64_of(sc)
        L = -np.array(sc.light_direction, np.float64)
        n = sc.width * sc.height

        def frame():
            _, _, _, rays, sec = orc.raycast64(cam64, sc.width, n, L, 1e-5, threads=threads)
            return rays, sec
    for _ in range(warmup):
        frame()
    tot_rays, tot_sec, best = 0, 0.0, 0.0
    for _ in range(steps):
        rays, sec = frame()
        tot_rays += rays
        tot_sec += sec
        best = max(best, rays / sec / 1e6)
    return {"kind": kind, "cores": threads, "value": tot_rays / tot_sec / 1e6, "best": best, "bvh_build_s": build_s,
            "rays_per_frame": tot_rays // max(steps, 1), "sec_per_frame": tot_sec / max(steps, 1)}


# ---------------------------------------------------------------------------

def bench_config():
    """The workload both arms time, by the same keys (how each arm runs it
    goes elsewhere in its line)."""
    return {"workload": WORKLOAD, "pixels": 1920 * 1080, "triangles": 1_045_506, "spp": 1,
            "rays": "1 primary closest hit per pixel + 1 directional-light shadow any-hit per primary hit"}


def run_reference(args, rank, world):
    """The reference's CPU ray casting of the same frame on this host's cores:
    the reference's own code where it was compiled here (oracle/_ref), else
    the float64 port, which builds its BVH itself with its restatement of
    FlatBVH::build (FlatBVH.cpp:89-204) outside the timed region. Nothing of
    the product library is loaded."""
    if rank != 0:
        return 0
    from raycer_gb300 import scenes
    sc = scenes.heightfield_scene()
    try:
        res = cpu_raycast(sc, args.steps, args.warmup, None)
    except ImportError as e:
        print(json.dumps({"impl": "reference", "unavailable": f"oracle not built: {e}"}))
        return 0
    line = {
        "impl": "reference", "metric": METRIC, "value": round(res["value"], 3), "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(res["sec_per_frame"] * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded fBm heightfield, value noise seed 2)",
        "config": bench_config(),
        "rays_per_step": int(res["rays_per_frame"]),
        "cpu_baseline": {"value": round(res["value"], 3), "unit": METRIC, "cores": res["cores"], "kind": res["kind"],
                         "sample": "full 1920x1080 frame per step (all pixels, primary + shadow rays)",
                         "bvh_build_s": round(res["bvh_build_s"], 2)},
        "e2e": {"value": round(res["value"], 3), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args, rank, local_rank, world):
    import ctypes as C

    import torch

    from raycer_gb300 import _native as N
    from raycer_gb300 import scenes
    from raycer_gb300.tracer import CAST_DTYPE, RAY_DTYPE, CudaTracer, TracerState, camera_record

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    sc = scenes.heightfield_scene()
    n_pix = sc.width * sc.height
    tracer = CudaTracer(local_rank)
    num_sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    tracer.initializeBuffers(sc)
    tracer.initializeImageBuffers(sc.width, sc.height)
    tracer.set_traversal_order(N.RC_ORDER_NEAREST if args.order == "nearest" else N.RC_ORDER_REFERENCE)
    state = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n_pix)

    # Traversal counts of one frame (deterministic; equal to the float32
    # oracle's counters) for the roofline's algorithmic bytes.
    tracer.set_counting(True)
    tracer.run(state)
    counted = tracer.stats()
    tracer.set_counting(False)

    stream = torch.cuda.ExternalStream(N.lib().rc_stream(tracer.handle), device=torch.device("cuda", local_rank))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=torch.device("cuda", local_rank))

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    clocks = ClockSampler(local_rank).start()
    time.sleep(0.3)   # the sampler's first reading
    for _ in range(args.warmup):
        flush_l2()
        tracer.run(state)

    frame_ms, prim_ms, shadow_ms, rays = [], [], [], []
    barrier()
    clocks.mark_start()
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush_l2()
        tracer.run(state)
        s = tracer.stats()
        frame_ms.append(s["last_ms"])
        prim_ms.append(s["stage_ms"][0])
        shadow_ms.append(s["stage_ms"][1])
        rays.append(s["rays_traced"])
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clocks.mark_end()
    clocks.stop()
    dev_sec = sum(frame_ms) / 1e3
    total_rays = sum(rays)

    # e2e: host rays in, host results out, through rc_cast_with_shadow.
    cam = camera_record(sc)
    pos = np.array(cam.position, np.float32)
    ys, xs = np.divmod(np.arange(n_pix), sc.width)
    dx = xs.astype(np.float32) / np.float32(cam.image_plane_width) - np.float32(0.5)
    dy = ys.astype(np.float32) / np.float32(cam.image_plane_height) - np.float32(0.5)
    p = (np.array(cam.image_plane_center, np.float32)[None, :] + dx[:, None] * np.array(cam.right, np.float32) +
         (dy * np.float32(cam.aspect_ratio))[:, None] * np.array(cam.up, np.float32))
    d = p - pos[None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays_pinned = torch.empty((n_pix, 8), dtype=torch.float32, pin_memory=True)
    rays_np = rays_pinned.numpy()
    rays_np[:, 0:3] = pos
    rays_np[:, 3] = 0.0
    rays_np[:, 4:7] = d
    rays_np[:, 7] = np.float32(3.4028234663852886e38)
    out_pinned = torch.empty((n_pix, 4), dtype=torch.int32, pin_memory=True)
    rp = C.c_void_p(rays_pinned.data_ptr())
    op = C.c_void_p(out_pinned.data_ptr())
    order = N.RC_ORDER_NEAREST if args.order == "nearest" else N.RC_ORDER_REFERENCE
    for _ in range(max(1, args.warmup)):
        assert N.lib().rc_cast_with_shadow(tracer.handle, rp, n_pix, order, op) == N.RC_OK
    # the same rays every step: primary + shadow rays counted once, outside the timed loop
    rays_per_call = tracer.stats()["rays_traced"]
    cast_with_shadow = N.lib().rc_cast_with_shadow
    handle = tracer.handle
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = cast_with_shadow(handle, rp, n_pix, order, op)
        if st != N.RC_OK:
            raise RuntimeError(N.lib().rc_last_error(tracer.handle).decode())
    barrier()
    e2e_sec = time.perf_counter() - t0
    e2e_rays = rays_per_call * args.steps


    dev_sec, e2e_sec, t_wall, total_rays, e2e_rays = reduce_replicas(
        (dev_sec, e2e_sec, t_wall), (total_rays, e2e_rays), world, torch.device("cuda", local_rank))

    line = None
    if rank == 0:
        peak, peak_kind = measured_peaks()
        s0_nodes, s0_tris = counted["stage_nodes"][0], counted["stage_tris"][0]
        hits = counted["stage_rays"][1]
        # One kernel per frame (shadow rays traced where the primary hit was
        # found; the shadow stage's time is then 0): its bytes are both
        # stages' node and triangle fetches + the records, written once.
        fused = statistics.mean(shadow_ms) == 0.0
        if fused:
            k_nodes = s0_nodes + counted["stage_nodes"][1]
            k_tris = s0_tris + counted["stage_tris"][1]
            prim_bytes = 64 * k_nodes + 48 * k_tris + 16 * n_pix
        else:
            k_nodes, k_tris = s0_nodes, s0_tris
            prim_bytes = 64 * s0_nodes + 48 * s0_tris + 16 * n_pix + 8 * hits
        prim_avg = statistics.mean(prim_ms) / 1e3
        achieved = prim_bytes / prim_avg / 1e9
        prof = profiled_metrics(fused)
        traffic = prof.get("dram_bytes_per_launch")
        clk = clocks.summary()
        roofline = issue_roofline(prof, prim_avg, clk.get("sm_mhz"), num_sms, prim_bytes, traffic, peak, peak_kind)
        line = {
            "metric": METRIC, "value": round(total_rays / dev_sec / 1e6, 2), "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dev_sec / args.steps * 1e3, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm heightfield, value noise seed 2)",
            "config": bench_config(),
            "rays_per_step": int(rays[0]),
            "setup": {"traversal_order": args.order, "l2": "flushed (512 MB write) before every step",
                      "parallelism": f"replicas x{world}"},
            "e2e": {"value": round(e2e_rays / e2e_sec / 1e6, 2), "unit": METRIC,
                    "h2d_bytes_per_step": n_pix * 32, "d2h_bytes_per_step": n_pix * 16},
            "gpu_launches": (1 if fused else 2) * args.steps,
            "roofline": dict(roofline,
                             kernel="k_raycast_primary (closest hit + shadow any-hit, one kernel)" if fused
                             else "k_raycast_primary (closest hit)",
                             node_fetches=int(k_nodes), triangle_tests=int(k_tris),
                             # BVH-node bytes (64 B per inner-node fetch) per second of the kernel
                             bvh_node_gbs=round(k_nodes * 64 / prim_avg / 1e9, 1)),
            "stages_ms": {"primary": round(statistics.mean(prim_ms), 4), "shadow": round(statistics.mean(shadow_ms), 4)},
            "wall_s": round(t_wall, 3),
            "clocks": clk,
        }
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    tracer.close()
    if rank == 0:
        if world == 1 and not args.headline_only:
            # the rest of the headline: plain path tracing on the 1M-triangle
            # scene, and the radiance cache's time to RMSE 0.01
            line["path_1m"] = path_1m_record(max(3, min(args.steps, 20)), max(3, min(args.warmup, 5)), local_rank)
            line["path_room"] = path_room_record(max(3, min(args.steps, 20)), max(3, min(args.warmup, 5)), local_rank)
            line["nrc"] = nrc_record(args.gt_spp, local_rank, enclosed=True)
            line["nrc_sky"] = nrc_record(args.gt_spp, local_rank, enclosed=False)
            line["batch"] = batch_record(2, 1, local_rank)
        if world == 1:
            try:
                res = cpu_raycast(sc, 2, 1, None)
                line["cpu_baseline"] = {"value": round(res["value"], 3), "unit": METRIC, "cores": res["cores"],
                                        "kind": res["kind"],
                                        "sample": "full 1920x1080 frame (primary + shadow rays), 1 warm-up + 2 "
                                                  "timed frames"}
            except ImportError as e:
                line["cpu_baseline"] = {"value": None, "unit": METRIC, "cores": cpu_threads(), "kind": "port",
                                        "sample": f"unavailable: {e}"}
        print(json.dumps(line))
    return 0


def path_1m_record(steps, warmup, device):
    """Plain path tracing of the 1,045,506-triangle heightfield at 1920x1080
    (Tracer::run Tracer.cpp:58 -> PathTracer::traceRecursive PathTracer.cpp:25:
    one camera ray per pixel, 4 segments, the 2 rho |cos| estimator; an
    emissive panel overhead is the light, see scenes.heightfield_path_scene)."""
    from raycer_gb300 import scenes

    return path_record(scenes.heightfield_path_scene(), "path tracing 1920x1080, 1 camera ray per pixel, depth 4, "
                       "heightfield 1,045,506 tris + 2-triangle emissive panel", steps, warmup, device)


def path_room_record(steps, warmup, device):
    """Plain path tracing of the room (2,012 triangles, emissive ceiling quad)
    at 320x240, 4x4 CMJ samples per pixel, 4 segments, box filter."""
    from raycer_gb300 import scenes

    return path_record(scenes.room_scene(), "path tracing 320x240, 16 spp (4x4 CMJ), depth 4, room 2,012 tris",
                       steps, warmup, device)


def path_record(sc, workload, steps, warmup, device):
    """One step = one frame (rc_render of every pixel). Device Mrays/s from the
    renders' CUDA events with the L2 flushed before every frame; e2e through
    the public API: the render and the tone-mapped image read back to the
    host (rc_render + rc_resolve), wall clock. CPU: the float64 port of the
    reference's path tracer (its own BVH build, outside the timing) on all
    host cores, full frames, the same samples per pixel and depth."""
    import torch

    import oracle
    from raycer_gb300 import _native as N
    from raycer_gb300.tracer import CudaTracer, TracerState

    n = sc.width * sc.height
    depth = int(sc.settings.get("max_path_length", 4))
    ms_sqrt = int(sc.settings.get("multi_sample_count_sqrt", 1))
    dev = torch.device("cuda", device)
    out = {"workload": workload, "triangles": sc.triangle_count}
    with CudaTracer(device) as t:
        t.initializeBuffers(sc, seed=1)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
        stream = torch.cuda.ExternalStream(N.lib().rc_stream(t.handle), device=dev)
        flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
        for _ in range(warmup):
            with torch.cuda.stream(stream):
                flush.zero_()
            t.run(st)
        ms, rays, ext = [], [], []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            t.run(st)
            s = t.stats()
            ms.append(s["last_ms"])
            rays.append(s["rays_traced"])
            ext.append(s["stage_ms"][0])
        # untimed warm-up of the end-to-end loop: the first images land in
        # fresh host pages
        for _ in range(warmup):
            t.run(st)
            img = t.downloadImage()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(steps):
            t.run(st)
            img = t.downloadImage()
        e2e_s = time.perf_counter() - t0
        e2e_rays = t.stats()["rays_traced"] * steps
    dev_mrays = sum(rays) / (sum(ms) / 1e3) / 1e6
    out.update({"steps": steps, "warmup": warmup, "mrays_per_s": round(dev_mrays, 1),
                "ms_per_frame": round(statistics.mean(ms), 4), "rays_per_frame": int(statistics.mean(rays)),
                "extend_share": round(sum(ext) / sum(ms), 3),
                "e2e": {"value": round(e2e_rays / e2e_s / 1e6, 1), "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": n * 16,
                        "note": "rc_render + rc_resolve (tone-mapped RGBA float image to the host) per frame"},
                "image_mean": round(float(img[..., :3].mean()), 4)})
    try:
        threads = cpu_threads()
        t0 = time.perf_counter()
        orc = oracle.Oracle(sc)
        build_s = time.perf_counter() - t0
        cam64 = oracle.camera64_of(sc)
        orc.render_path64(cam64, sc.width, n, depth, 1, ms_sqrt, seed=1, threads=threads)   # warm-up
        c_rays = c_sec = 0
        for k in range(2):
            _, r, sec = orc.render_path64(cam64, sc.width, n, depth, 1, ms_sqrt, seed=2 + k, threads=threads)
            c_rays += r
            c_sec += sec
        cpu = c_rays / c_sec / 1e6
        out["cpu_baseline"] = {"value": round(cpu, 3), "unit": METRIC, "cores": threads, "kind": "port",
                               "sample": f"full {sc.width}x{sc.height} frame, 1 warm-up + 2 timed frames",
                               "bvh_build_s": round(build_s, 2)}
        out["device_over_cpu"] = round(dev_mrays / cpu, 1)
        out["e2e_over_cpu"] = round(out["e2e"]["value"] / cpu, 1)
    except ImportError as e:
        out["cpu_baseline"] = {"value": None, "sample": f"unavailable: {e}"}
    return out


def nrc_record(gt_spp, device, enclosed=False, max_seconds=60.0):
    """Time to display RMSE 0.01 at 1080p: the radiance-cache tracer against
    the plain path tracer, both against a float64 ground truth of `gt_spp`
    plain frames (raycer_gb300.nrc_eval.time_to_rmse)."""
    from raycer_gb300 import scenes
    from raycer_gb300.nrc_eval import time_to_rmse

    t0 = time.perf_counter()
    sc = scenes.heightfield_blobs_scene(enclosed=enclosed)
    build_s = time.perf_counter() - t0
    res = time_to_rmse(sc, target=0.01, gt_spp=gt_spp, max_frames=4096, max_seconds=max_seconds, device=device)

    def run_dict(r):
        return {"frames": r.frames, "seconds": round(r.seconds, 3), "gpu_ms": round(r.gpu_ms, 1),
                "rmse": round(r.rmse, 5), "reached": r.reached,
                "mrays_per_s": round(r.rays / max(r.seconds, 1e-9) / 1e6, 1)}

    return {"workload": f"radiance cache vs plain path tracing: heightfield + 200 blobs, {sc.triangle_count} tris, "
                        f"{sc.width}x{sc.height}, 1 spp/frame, depth 12, "
                        + ("closed box lit by a 20 x 11 emissive ceiling panel of radiance 3" if enclosed
                           else "sky-lit"),
            "target_rmse": 0.01, "gt_spp": res.gt_spp, "gt_seconds": round(res.gt_seconds, 1),
            "scene_build_s": round(build_s, 1), "plain": run_dict(res.plain), "cache": run_dict(res.cache),
            "time_ratio_cache_over_plain": (round(res.cache.seconds / res.plain.seconds, 3)
                                            if res.plain.reached and res.cache.reached else None),
            "cache_stats": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in res.cache_stats.items()}}


def batch_record(steps, warmup, device=0, cpu=True):
    """64 independent rooms (extra triangles log-uniform in [1e3, 2e6], film
    256..1024 square, 1..64 spp, depth 8 with Russian roulette from segment 3)
    rendered as one CUDA-graph launch per frame after autotuning; device time
    of the graph launch (CUDA events). With `cpu`, the port's rate on a
    sample of the scenes (batch_cpu_baseline) and the frame's estimated time
    on the host cores at that rate."""
    from raycer_gb300 import scenes
    from raycer_gb300.batch import Batch

    scs = scenes.batch_scenes(seed=3)
    t0 = time.perf_counter()
    b = Batch(device)
    for i, sc in enumerate(scs):
        b.add_scene(sc, seed=3000 + i)
    setup_s = time.perf_counter() - t0
    tuning = b.autotune(budget_ms=4000.0)
    for _ in range(warmup):
        b.render()
    ms, rays, done = [], [], []
    for _ in range(steps):
        d = b.render()
        s = b.stats()
        ms.append(s["last_ms"])
        rays.append(s["rays_traced"])
        done.append(d)
    done = np.concatenate(done)
    out = {
        "workload": "batched path tracing: 64 rooms + log-uniform[1e3, 2e6] extra tris, 256^2..1024^2, "
                    "1..64 spp, depth 8, Russian roulette from segment 3, one CUDA-graph launch per frame",
        "steps": steps, "warmup": warmup, "mrays_per_s": round(sum(rays) / (sum(ms) / 1e3) / 1e6, 2),
        "ms_per_frame": round(statistics.mean(ms), 3),
        "triangles": int(sum(sc.triangle_count for sc in scs)), "paths_per_frame": int(s["paths"]),
        "rays_per_frame": int(statistics.mean(rays)), "passes": s["passes"], "graph_nodes": s["graph_nodes"],
        "setup_s": round(setup_s, 1),
        "per_scene_latency_ms": {"p50": round(float(np.percentile(done, 50)), 3),
                                 "p99": round(float(np.percentile(done, 99)), 3)},
        "tuning": {k: tuning[k] for k in ("slots", "extend_block", "measured_paths_per_ms")},
    }
    b.close()
    if cpu:
        try:
            res = batch_cpu_baseline(scs)
            res["frame_seconds_estimate"] = round(out["rays_per_frame"] / (res["value"] * 1e6), 1)
            out["cpu_baseline"] = res
            out["device_over_cpu"] = round(out["mrays_per_s"] / res["value"], 1)
        except ImportError as e:
            out["cpu_baseline"] = {"value": None, "sample": f"unavailable: {e}"}
    return out


def batch_cpu_baseline(scs, stride=8, pixels_per_scene=1 << 14):
    """The batch on the host cores: the float64 port of the reference's path
    tracer, one scene after another (as the reference renders them), on one
    scene from each `stride`-scene band of the batch sorted by triangle count
    (the middle one of the band: a sample with the batch's spread of sizes),
    each from its own BVH (the port's restatement of FlatBVH::build, outside
    the timing), over a band of
    `pixels_per_scene` pixels (at least one of the port's 1000-pixel chunks
    per thread: the reference's schedule(dynamic, 1000)) across the film's
    middle rows, one sample per pixel, with the scene's maximum path length.
    The rate is rays per second, which the samples per pixel do not change;
    the reference's path tracer has no Russian roulette, so its paths run to
    the maximum length."""
    import oracle

    threads = cpu_threads()
    rays = sec = build_s = 0.0
    pixels = 0
    picked = sorted(scs, key=lambda sc: sc.triangle_count)[stride // 2::stride]
    for i, sc in enumerate(picked):
        depth = int(sc.settings.get("max_path_length", 8))
        n = sc.width * sc.height
        count = max(1, min(n, max(1000 * threads, pixels_per_scene)))
        start = max(0, min(n - count, (sc.height // 2) * sc.width - count // 2))
        t0 = time.perf_counter()
        orc = oracle.Oracle(sc)
        build_s += time.perf_counter() - t0
        try:
            _, r, s = orc.render_path64(oracle.camera64_of(sc), sc.width, count, depth, 1, 1, seed=7 + i,
                                        threads=threads, pixel_start=start)
        finally:
            orc.close()
        rays += r
        sec += s
        pixels += count
    return {"value": round(rays / sec / 1e6, 3), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(picked)} of the {len(scs)} scenes (the middle one of every {stride} by triangle count: "
                      f"{', '.join(str(sc.triangle_count) for sc in picked)} tris), one after another, a band of "
                      f"{pixels // len(picked)} pixels across each film's middle rows at 1 sample per pixel; "
                      f"no Russian roulette", "rays": int(rays), "seconds": round(sec, 2),
            "bvh_build_s": round(build_s, 1)}


def run_batch(args, rank, world):
    """The batch workload on its own (batch_record), one JSON line."""
    if rank != 0:
        return 0
    r = batch_record(args.steps, args.warmup)
    line = {"metric": METRIC, "value": r["mrays_per_s"], "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_frame"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (64 seeded rooms)",
            "config": {k: r[k] for k in ("workload", "triangles", "paths_per_frame", "rays_per_frame", "passes",
                                         "graph_nodes", "setup_s")},
            "per_scene_latency_ms": r["per_scene_latency_ms"], "tuning": r["tuning"]}
    if "cpu_baseline" in r:
        line["cpu_baseline"] = r["cpu_baseline"]
    print(json.dumps(line))
    return 0


def run_nrc(args, rank, world):
    """Heightfield + 200 blob instances (5.1M tris), 1080p, 1 spp per frame,
    depth 12, sky-lit: wall time until the display RMSE against a float64
    4096-spp plain-tracer ground truth reaches 0.01, plain tracer vs the
    radiance-cache tracer (paths end into the cache at the hit of segment 2;
    1 slot in 16 trains; 4 Adam steps of 16384 samples per frame)."""
    if rank != 0:
        return 0
    from raycer_gb300 import scenes
    from raycer_gb300.nrc_eval import time_to_rmse

    w, h = int(round(1920 * args.scale)), int(round(1080 * args.scale))
    t0 = time.perf_counter()
    sc = scenes.heightfield_blobs_scene(width=w, height=h, enclosed=args.enclosed)
    build_s = time.perf_counter() - t0
    res = time_to_rmse(sc, target=0.01, gt_spp=args.gt_spp, max_frames=4096, max_seconds=90.0,
                       cache_config=dict(terminate_segment=args.terminate_segment),
                       progress=lambda m: print(m, file=sys.stderr, flush=True))

    def run_dict(r):
        return {"frames": r.frames, "seconds": round(r.seconds, 3), "gpu_ms": round(r.gpu_ms, 1),
                "rmse": round(r.rmse, 5), "reached": r.reached,
                "mrays_per_s": round(r.rays / max(r.seconds, 1e-9) / 1e6, 1)}

    line = {
        "metric": "time-to-RMSE 0.01 (s), radiance cache", "value": round(res.cache.seconds, 3), "unit": "s",
        "n_gpus": 1, "steps": res.cache.frames, "warmup": 0,
        "ms_per_step": round(1e3 * res.cache.seconds / max(res.cache.frames, 1), 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (MLP) / f32 (paths)",
        "data": "synthetic (seeded heightfield + blob instances)",
        "config": {"workload": f"radiance cache: heightfield + 200 blobs, {sc.triangle_count} tris, {w}x{h}, "
                               "1 spp/frame, depth 12, " + ("inside a closed box lit by an emissive panel, no sky"
                                                            if args.enclosed else "sky-lit"),
                   "gt_spp": res.gt_spp, "gt_seconds": round(res.gt_seconds, 1), "scene_build_s": round(build_s, 1),
                   "terminate_segment": args.terminate_segment},
        "plain": run_dict(res.plain), "cache": run_dict(res.cache),
        "time_ratio_cache_over_plain": (round(res.cache.seconds / res.plain.seconds, 3)
                                        if res.plain.reached and res.cache.reached else None),
        "cache_stats": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in res.cache_stats.items()},
        "curves": {"plain": res.plain.curve[::max(1, len(res.plain.curve) // 24)],
                   "cache": res.cache.curve[::max(1, len(res.cache.curve) // 24)]},
    }
    print(json.dumps(line))
    return 0


def run_cpu(args, rank, world):
    """CPU path-tracing throughput on this host's cores (the float64 port of
    the reference's path tracer, all threads, its own BVH and camera): the
    room at 320x240, 16 spp, depth 4, a full frame (best of 3); and the
    64-scene batch on its size-sampled eighth (batch_cpu_baseline)."""
    if rank != 0:
        return 0
    import oracle
    from raycer_gb300 import scenes

    threads = cpu_threads()
    sc = scenes.room_scene()
    orc = oracle.Oracle(sc)
    best = None
    for _ in range(3):
        _, rays, sec = orc.render_path64(oracle.camera64_of(sc), sc.width, sc.width * sc.height, 4, 1, 4, seed=1,
                                         threads=threads)
        if best is None or sec < best[1]:
            best = (rays, sec)
    orc.close()
    batch = batch_cpu_baseline(scenes.batch_scenes(seed=3))
    print(json.dumps({"metric": "Mrays/s", "workload": "cpu", "unit": "Mrays/s", "higher_is_better": True,
                      "kind": "port", "cores": threads,
                      "config0_room": {"rays": int(best[0]), "seconds": round(best[1], 4),
                                       "mrays_per_s": round(best[0] / best[1] / 1e6, 2)},
                      "config2_batch": batch}))
    return 0


def run_build(args, rank, world):
    """BVH build + upload time of the reference SAH builder (host) and the
    GPU linear-BVH builder on the 1,045,506-triangle heightfield and the
    5,141,506-triangle heightfield + blobs scene, with the RAY frame's
    device time (1080p primary + shadow) on each tree."""
    if rank != 0:
        return 0
    from raycer_gb300 import _native as N
    from raycer_gb300 import scenes
    from raycer_gb300.tracer import CudaTracer, TracerState

    out = {}
    for name, make in (("heightfield_1M", scenes.heightfield_scene), ("heightfield_blobs_5M",
                                                                     scenes.heightfield_blobs_scene)):
        sc = make()
        sc.settings["tracer"] = "ray"
        if sc.light_direction is None:
            sc.light_direction = (-0.3, -1.0, -0.2)
        row = {"triangles": sc.triangle_count}
        for label, b in (("sah_host", N.RC_BUILDER_REFERENCE_SAH), ("lbvh_gpu", N.RC_BUILDER_GPU_LBVH)):
            with CudaTracer(0) as t:
                assert N.lib().rc_set_bvh_builder(t.handle, b) == N.RC_OK
                builds = []
                for _ in range(max(1, min(args.steps, 3))):
                    t.initializeBuffers(sc)
                    builds.append(t.stats()["build_ms"])
                st = t.stats()
                t.initializeImageBuffers(sc.width, sc.height)
                state = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height,
                                    pixelCount=sc.width * sc.height)
                t.set_counting(True)
                t.run(state)
                counted = t.stats()
                t.set_counting(False)
                for _ in range(3):
                    t.run(state)
                ms, rays = [], []
                for _ in range(10):
                    t.run(state)
                    s2 = t.stats()
                    ms.append(s2["last_ms"])
                    rays.append(s2["rays_traced"])
                row[label] = {"build_ms": round(min(builds), 1), "bvh_inner_nodes": st["bvh_inner_nodes"],
                              "bvh_depth": st["bvh_depth"],
                              "frame_mrays_per_s": round(sum(rays) / (sum(ms) / 1e3) / 1e6, 1),
                              "node_visits_per_ray": round(counted["node_visits"] / max(counted["rays_traced"], 1), 2),
                              "tri_tests_per_ray": round(counted["tri_tests"] / max(counted["rays_traced"], 1), 2)}
        out[name] = row
    print(json.dumps({"metric": "BVH build ms", "workload": "build", "unit": "ms", "higher_is_better": False,
                      "n_gpus": 1, "results": out}))
    return 0


def run_large(args, rank, world):
    """The combined run: 3840x2160, depth 16, a 4,188,162-triangle fBm
    heightfield (seed 5) + 800 instances of a 20,480-triangle blob (30 %
    dielectric, IOR U(1.3, 1.7)), lit by a uniform sky or (--enclosed) by the
    radiance-cache workload's closed box and ceiling panel. Plain path tracing
    for 256 frames of 1 spp, then the radiance-cache tracer until its display
    RMSE against a float64 ground truth of --gt-spp samples per pixel
    (rendered 16 per frame) reaches the plain run's; times are the renders'
    wall clock.

    CPU arm: the reference's path tracer has no dielectrics, so the float64
    port traces the same geometry with every material Lambertian (the
    dielectric blobs take their albedo), flattened, from its own BVH, at a
    reduced 480x270 sample of the frame on all host cores; its Mrays/s times
    the rays the plain GPU tracer traced to reach its RMSE estimate the CPU's
    time to the same error (linear in pixels x samples, as the Mrays/s of the
    sample)."""
    if rank != 0:
        return 0
    import dataclasses

    import oracle
    from raycer_gb300 import scenes
    from raycer_gb300.nrc import GroundTruth, RadianceCache
    from raycer_gb300.nrc_eval import _run
    from raycer_gb300.tracer import CudaTracer, TracerState, general_record

    w, h = int(round(3840 * args.scale)), int(round(2160 * args.scale))
    t0 = time.perf_counter()
    sc = scenes.heightfield_blobs_instanced(instances=800, blob_level=5, seed=5, hf_nx=2048, hf_nz=1024, width=w,
                                            height=h, dielectric_fraction=0.3, hf_seed=5, enclosed=args.enclosed)
    sc.settings.update(max_path_length=16)
    gen_s = time.perf_counter() - t0
    log = lambda m: print(m, file=sys.stderr, flush=True)
    with CudaTracer(0) as t:
        t.initializeInstanced(sc, seed=5)
        upload_ms = t.stats()["build_ms"]
        t.initializeImageBuffers(w, h)
        st = TracerState(scene=sc, filmWidth=w, filmHeight=h, pixelCount=w * h)
        gt_settings = dict(sc.settings, path_sample_count=16)
        gt_scene = scenes.InstancedScene(**{**sc.__dict__, "settings": gt_settings})
        t.set_general(general_record(gt_scene, seed=5))
        gt = GroundTruth(t)
        t1 = time.perf_counter()
        for i in range(args.gt_spp // 16):
            t.run(st)
            gt.add_film(clear_film=True)
        gt_s = time.perf_counter() - t1
        log(f"ground truth {args.gt_spp} spp in {gt_s:.1f} s")
        t.set_general(general_record(sc, seed=5 + 7919))
        plain = _run(t, st, gt, 0.0, 256, 1e9, 256)
        log(f"plain 256 frames: {plain.seconds:.2f} s, rmse {plain.rmse:.4f}")
        cache = RadianceCache(t)
        cached = _run(t, st, gt, plain.rmse, 1024, 180.0, 4)
        log(f"cache: {cached.frames} frames, {cached.seconds:.2f} s, rmse {cached.rmse:.4f}")
        stats = cache.stats()
    lighting = "closed box, 20 x 11 ceiling panel of radiance 3" if args.enclosed else "sky-lit"
    line = {
        "metric": "Mrays/s", "value": round(plain.rays / plain.seconds / 1e6, 1), "unit": "Mrays/s",
        "n_gpus": 1, "steps": plain.frames, "warmup": 0,
        "ms_per_step": round(1e3 * plain.seconds / plain.frames, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (paths) / bf16 (cache MLP)",
        "data": "synthetic (seeded heightfield + blob instances)",
        "config": {"workload": f"combined run: {w}x{h}, depth 16, heightfield 4,188,162 tris + 800 x 20,480-tri "
                               f"blob instances ({sc.triangle_count} flattened), 30 % dielectric, {lighting}",
                   "scene_generation_s": round(gen_s, 1), "upload_and_build_ms": round(upload_ms, 1),
                   "gt_spp": args.gt_spp, "gt_seconds": round(gt_s, 1)},
        "plain_256spp": {"seconds": round(plain.seconds, 3), "rmse": round(plain.rmse, 5),
                         "mrays_per_s": round(plain.rays / plain.seconds / 1e6, 1), "rays": int(plain.rays)},
        "cache_equal_rmse": {"frames": cached.frames, "seconds": round(cached.seconds, 3),
                             "rmse": round(cached.rmse, 5), "reached": cached.reached,
                             "mrays_per_s": round(cached.rays / max(cached.seconds, 1e-9) / 1e6, 1)},
        "time_ratio_cache_over_plain": round(cached.seconds / plain.seconds, 3) if cached.reached else None,
        "cache_stats": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in stats.items()},
    }
    # CPU arm (see the docstring): the Lambertian version, flattened, 480x270 sample
    try:
        flat = sc.flatten()
        flat.materials = [dataclasses.replace(m, dielectric=False, ior=0.0) for m in flat.materials]
        cw, ch = 480, 270
        flat.width, flat.height = cw, ch
        threads = cpu_threads()
        tb = time.perf_counter()
        orc = oracle.Oracle(flat)
        build_s = time.perf_counter() - tb
        _, rays, sec = orc.render_path64(oracle.camera64_of(flat), cw, cw * ch, 16, 1, 1, seed=1, threads=threads)
        cpu = rays / sec / 1e6
        line["cpu_baseline"] = {
            "value": round(cpu, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{cw}x{ch}, 1 spp, depth 16, every material Lambertian ({rays} rays in {sec:.1f} s; "
                      f"BVH build of {flat.triangle_count} flattened triangles {build_s:.0f} s, untimed)",
            "equal_rmse_seconds_estimate": round(plain.rays / (cpu * 1e6), 1),
            "note": "the reference's path tracer has no dielectrics; its time to the plain GPU tracer's RMSE "
                    "is estimated as the rays the plain GPU tracer traced / the CPU's Mrays/s"}
        line["time_ratio_cache_over_cpu"] = round(cached.seconds / line["cpu_baseline"]["equal_rmse_seconds_estimate"],
                                                  5) if cached.reached else None
    except (ImportError, MemoryError) as e:
        line["cpu_baseline"] = {"value": None, "sample": f"unavailable: {e}"}
    print(json.dumps(line))
    return 0


def run_path(args, rank, world):
    """Plain path-tracing throughput (PATH renders, device time of rc_render):
    the room (2,012 triangles, 320x240, 16 spp CMJ, depth 4, box filter) and
    the 5,141,506-triangle heightfield + blobs at 1920x1080, 1 spp, depth 12,
    sky-lit."""
    if rank != 0:
        return 0
    from raycer_gb300 import scenes
    from raycer_gb300.tracer import CudaTracer, TracerState

    out = {}
    cases = (("room_320x240_16spp_depth4", lambda: scenes.room_scene()),
             ("heightfield_blobs_1080p_1spp_depth12", lambda: scenes.heightfield_blobs_scene()))
    for name, make in cases:
        sc = make()
        with CudaTracer(0) as t:
            t.initializeBuffers(sc, seed=1)
            t.initializeImageBuffers(sc.width, sc.height)
            st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
            for _ in range(args.warmup):
                t.run(st)
            ms, rays = [], []
            for _ in range(args.steps):
                t.run(st)
                s2 = t.stats()
                ms.append(s2["last_ms"])
                rays.append(s2["rays_traced"])
            out[name] = {"triangles": sc.triangle_count, "ms_per_frame": round(statistics.mean(ms), 3),
                         "mrays_per_s": round(sum(rays) / (sum(ms) / 1e3) / 1e6, 1),
                         "rays_per_frame": int(statistics.mean(rays)),
                         "extend_ms": round(s2["stage_ms"][0], 3)}
    print(json.dumps({"metric": "Mrays/s", "workload": "path", "unit": "Mrays/s", "higher_is_better": True,
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "results": out}))
    return 0


def main():
    args = parse_args()
    rank, local_rank, world = dist_env()
    if args.workload == "batch":
        return run_batch(args, rank, world)
    if args.workload == "nrc":
        return run_nrc(args, rank, world)
    if args.workload == "build":
        return run_build(args, rank, world)
    if args.workload == "large":
        return run_large(args, rank, world)
    if args.workload == "cpu":
        return run_cpu(args, rank, world)
    if args.workload == "path":
        return run_path(args, rank, world)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, local_rank, world)


if __name__ == "__main__":
    sys.exit(main())
