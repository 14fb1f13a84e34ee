"""Equal-error timing of the radiance cache against the plain path tracer.

``time_to_rmse`` renders a float64 ground truth (``gt_spp`` frames of the
plain tracer at 1 sample per pixel, each added to a float64 film on the
device), then runs the plain tracer and the cache-terminated tracer frame by
frame from a cleared film until the display-space RMSE against the ground
truth (``GroundTruth.rmse``) falls to ``target``. Each frame is one
``rc_render`` call (the cache's lookups and training run inside it); its time
is the render's wall-clock time, host to host. The error checks between
frames are not timed.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

from .nrc import GroundTruth, RadianceCache
from .tracer import CudaTracer, TracerState, general_record


@dataclass
class Run:
    frames: int = 0
    seconds: float = 0.0        # wall-clock of the rendered frames
    gpu_ms: float = 0.0         # sum of the renders' device time (rc_stats.last_ms)
    rays: int = 0
    rmse: float = float("inf")
    reached: bool = False
    curve: list = field(default_factory=list)  # (frames, seconds, rmse)


@dataclass
class Result:
    target: float
    gt_spp: int
    gt_seconds: float
    plain: Run
    cache: Run
    cache_stats: dict


def _run(t: CudaTracer, st: TracerState, gt: GroundTruth, target: float, max_frames: int, max_seconds: float,
         check_every: int) -> Run:
    r = Run()
    t.clear()
    while r.frames < max_frames and r.seconds < max_seconds:
        t0 = time.perf_counter()
        t.run(st)
        r.seconds += time.perf_counter() - t0
        s = t.stats()
        r.gpu_ms += s["last_ms"]
        r.rays += s["rays_traced"]
        r.frames += 1
        if r.frames % check_every == 0 or r.frames == max_frames:
            r.rmse = gt.rmse()
            r.curve.append((r.frames, r.seconds, r.rmse))
            if r.rmse <= target:
                r.reached = True
                break
    return r


def time_to_rmse(scene, target: float = 0.01, gt_spp: int = 4096, max_frames: int = 4096,
                 max_seconds: float = 120.0, check_every: int = 1, cache_config: dict | None = None,
                 seed: int = 1, device: int = 0, progress=None) -> Result:
    with CudaTracer(device) as t:
        t.initializeBuffers(scene, seed=seed)
        t.initializeImageBuffers(scene.width, scene.height)
        st = TracerState(scene=scene, filmWidth=scene.width, filmHeight=scene.height,
                         pixelCount=scene.width * scene.height)
        gt = GroundTruth(t)
        t0 = time.perf_counter()
        for i in range(gt_spp):
            t.run(st)
            gt.add_film(clear_film=True)
            if progress and (i + 1) % 256 == 0:
                progress(f"ground truth {i + 1}/{gt_spp}")
        gt_seconds = time.perf_counter() - t0
        # independent samples for the timed runs
        t.set_general(general_record(scene, seed=seed + 7919))
        plain = _run(t, st, gt, target, max_frames, max_seconds, check_every)
        if progress:
            progress(f"plain: {plain.frames} frames, {plain.seconds:.2f} s, rmse {plain.rmse:.4f}")
        cache = RadianceCache(t, **(cache_config or {}))
        cached = _run(t, st, gt, target, max_frames, max_seconds, check_every)
        stats = cache.stats()
        if progress:
            progress(f"cache: {cached.frames} frames, {cached.seconds:.2f} s, rmse {cached.rmse:.4f}")
        return Result(target, gt_spp, gt_seconds, plain, cached, stats)


def render_frames(scene, frames: int, cache_config: dict | None = None, seed: int = 1, device: int = 0) -> dict:
    """Renders `frames` frames with the cache (no ground truth); for profiling."""
    with CudaTracer(device) as t:
        t.initializeBuffers(scene, seed=seed)
        t.initializeImageBuffers(scene.width, scene.height)
        st = TracerState(scene=scene, filmWidth=scene.width, filmHeight=scene.height,
                         pixelCount=scene.width * scene.height)
        cache = RadianceCache(t, **(cache_config or {}))
        for _ in range(frames):
            t.run(st)
        return cache.stats()


def main(argv=None) -> int:
    import argparse
    import json
    import sys

    from . import scenes

    ap = argparse.ArgumentParser(description="radiance-cache frames on the heightfield + blobs scene")
    ap.add_argument("--scale", type=float, default=0.5, help="film scale (1 = 1920x1080)")
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--instances", type=int, default=200)
    ap.add_argument("--lookup-kernel", type=int, default=1, help="0: mma.sync, 1: tcgen05 with TMEM")
    args = ap.parse_args(argv)
    w, h = int(round(1920 * args.scale)), int(round(1080 * args.scale))
    sc = scenes.heightfield_blobs_scene(instances=args.instances, width=w, height=h)
    print(json.dumps(render_frames(sc, args.frames, cache_config=dict(lookup_kernel=args.lookup_kernel))))
    sys.stdout.flush()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
