"""Throughput benchmark of the GB300 path tracer (one JSON line on stdout).

Workload: the large single-scene configuration - a 1024x1024-quad value-noise
terrain (2,097,152 triangles) plus 300 instances of a subdivision-4 icosphere
(1,536,000 triangles), 4 Lambert + 4 Phong shaders, 8 quad lights, 1024x1024
pixels at 64 samples, max depth 8 with Russian roulette from depth 3, ray batches
of 2^20, power heuristic.  The scene is generated from a fixed seed (no public
scene exists for the reference); see msc-project_gb300/csrc/scenegen.cpp.

One step = one Pathtracer::process() pass (every pixel x sample, through the
sorted batch loop, filtered into the image).  Metric: Mrays/s = (closest-hit +
occlusion queries) / time.  `value` uses the device time of process() with the
scene resident on the GPU; `e2e` times the C-ABI call msc_process() that also
copies the image to host memory each step, by wall clock.

--impl reference times the reference algorithm on the host cores instead: the
reference renderer itself cannot be built here (Embree 2.6.1, TBB, Boost,
yaml-cpp, Eigen, OpenImageIO and OpenEXR are absent), so its CPU restatement
in oracle/ runs with every host thread on a bounded sample of the same paths.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(REPO, "msc-project_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "end-to-end Mrays/s on 1 GB300, batched/served vs plain; p50/p99 job latency"
SEED = 20261203
ALG_BYTES_TRACE = 52  # per closest-hit query: read ray 32 B (org, dir), write hit 20 B


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_scene(config, scale):
    import mscgpu
    d = os.path.join(tempfile.gettempdir(), "msc_bench_scenes", "c%d_s%d_%g" % (config, SEED + config, scale))
    y = os.path.join(d, "scene.yaml")
    if not os.path.exists(y):
        t = time.time()
        y = mscgpu.generate_scene(config, SEED + config, d, scale=scale)
        log("generated scene %s in %.1f s" % (y, time.time() - t))
    return y


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", "0", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                           "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(yaml, seconds=15.0, threads=0):
    """The CPU restatement on a bounded sample of the same paths (middle image columns)."""
    from oracle import oracle as O
    t = time.time()
    s = O.Scene(yaml)
    log("oracle scene load + SAH build %.1f s" % (time.time() - t))
    cores = threads or os.cpu_count() or 1
    first = (s.width // 2) * s.height * s.spp
    n = 1 << 15
    while True:
        t = time.time()
        c = s.render_range(first, n, 0, cores)
        dt = time.time() - t
        if dt > seconds / 4 or n >= s.paths // 2:
            break
        n = min(int(n * max(2.0, seconds / 4 / max(dt, 1e-3))), s.paths // 2)
    n = min(int(n * seconds / max(dt, 1e-3)), s.paths - first)
    t = time.time()
    c = s.render_range(first, n, 0, cores)
    dt = time.time() - t
    rays = int(c[0]) + int(c[1])
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
            "sample": "%d paths (sampleIDs %d..%d, the middle image columns), %d ray queries, %.1f s"
                      % (n, first, first + n - 1, rays, dt)}


def scene_set(n, lo_tris, hi_tris, seed):
    """n scenes by the terrain rules with triangle counts log-uniform in [lo, hi]."""
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        target = math.exp(rng.uniform(math.log(lo_tris), math.log(hi_tris)))
        # tris(s) ~ 2 (1024 s)^2 + 300 s * 5120
        a, b = 2.0 * 1024 * 1024, 300 * 5120.0
        s = (-b + math.sqrt(b * b + 4 * a * target)) / (2 * a)
        s = min(1.0, max(0.01, s))
        out.append(make_scene_scaled(1, seed + 17 * i, round(s, 4)))
    return out


def make_scene_scaled(config, seed, scale):
    import mscgpu
    d = os.path.join(tempfile.gettempdir(), "msc_bench_scenes", "c%d_s%d_%g" % (config, seed, scale))
    y = os.path.join(d, "scene.yaml")
    if not os.path.exists(y):
        y = mscgpu.generate_scene(config, seed, d, scale=scale)
    return y


def sphere_camera(rng, bbox, fov_lo=30.0, fov_hi=70.0):
    """A pinhole on the scene's bounding sphere looking at its centre (PinHoleCamera fields)."""
    import math
    import numpy as np
    lo, hi = bbox
    c = 0.5 * (lo + hi)
    r = 0.6 * float(np.linalg.norm(hi - lo))
    v = rng.normal(size=3)
    v[1] = abs(v[1]) + 0.3  # from above the horizon
    v /= np.linalg.norm(v)
    eye = c + r * v
    fwd = (c - eye) / np.linalg.norm(c - eye)
    fov = rng.uniform(fov_lo, fov_hi)
    focal = 36.0 / math.tan(math.radians(fov) / 2)
    rz = math.degrees(math.asin(max(-1.0, min(1.0, fwd[1]))))
    ry = math.degrees(math.atan2(-fwd[2], fwd[0]))
    t = eye - fwd * focal  # the pinhole sits at translation + normal * focal length
    return (tuple(float(x) for x in t), (0.0, ry, rz), focal)


def random_jobs(rng, scenes_bboxes, n, res_choices, spp_lo, spp_hi, depth_lo, depth_hi):
    jobs = []
    for _ in range(n):
        s = int(rng.integers(0, len(scenes_bboxes)))
        res = int(rng.choice(res_choices))
        jobs.append(dict(scene=s, width=res, height=res, spp=int(rng.integers(spp_lo, spp_hi + 1)),
                         min_depth=3, max_depth=int(rng.integers(depth_lo, depth_hi + 1)),
                         camera=sphere_camera(rng, scenes_bboxes[s]), seed=int(rng.integers(1, 1 << 30))))
    return jobs


def bench_forms(args):
    """Batched and served forms against the one-job-at-a-time loop on the same jobs."""
    import mscgpu
    import numpy as np
    t = time.time()
    scenes = scene_set(16, 1e4, 1e6, SEED + 300)
    bboxes = []
    for y in scenes:
        _, tv, _ = mscgpu.scene_load_host(y)
        p = tv.reshape(-1, 3)
        bboxes.append((p.min(0), p.max(0)))
    log("batched/served scene set ready in %.1f s" % (time.time() - t))
    rng = np.random.default_rng(SEED + 301)
    jobs = random_jobs(rng, bboxes, 48, [128, 256, 512], 4, 32, 4, 10)
    film = int(sum(j["width"] * j["height"] * j["spp"] for j in jobs)) + 1

    def new_batch(max_active=0, film_samples=film):
        b = mscgpu.Batch(batch_exponent=20, film_samples=film_samples)
        for y in scenes:
            b.add_scene(y)
        if max_active:
            b.set_max_active(max_active)
        return b

    out = {}
    # batched: every job in one wavefront
    b = new_batch()
    for j in jobs:
        b.submit(**j)
    t = time.time()
    b.run()
    wall = time.time() - t
    st = b.stats()
    rays = st["closest_queries"] + st["shadow_queries"]
    b.close()
    # the plain per-job loop on the same jobs: one job in flight at a time
    p = new_batch(max_active=1)
    res, pst = p.serve([(0.0, j) for j in jobs])
    p.close()
    plain_rate = (pst["closest_queries"] + pst["shadow_queries"]) / pst["wall_s"] / 1e6
    out["batched"] = {"workload": "%d jobs on 16 resident terrain scenes (1e4-1e6 tris, log-uniform), "
                                  "128^2-512^2, 4-32 spp, depth 4-10, cameras on the bounding sphere" % len(jobs),
                      "mrays_per_s": rays / wall / 1e6, "wall_s": wall,
                      "per_job_loop_mrays_per_s": plain_rate, "per_job_loop_wall_s": pst["wall_s"],
                      "speedup_vs_per_job_loop": (rays / wall / 1e6) / plain_rate if plain_rate else None}
    # served: Poisson arrivals, admission by film memory
    rate, dur = args.serve_rate, args.serve_seconds
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * dur * 1.5)))
    arrivals = arrivals[arrivals < dur]
    reqs = [(float(a), j) for a, j in zip(arrivals, random_jobs(rng, bboxes, len(arrivals), [128, 256], 4, 16, 4,
                                                                    10))]
    budget = 1 << 25
    for label, max_active in (("served", 0), ("served_per_job_loop", 1)):
        s = new_batch(max_active=max_active, film_samples=budget)
        res, sst = s.serve(reqs)
        s.close()
        out[label] = {"requests": len(reqs), "rate_per_s": rate, "seconds": dur,
                      "film_budget_samples": budget, "completed": sst["completed"],
                      "mrays_per_s": sst["mrays_per_s"], "p50_ms": 1e3 * sst["p50_s"], "p99_ms": 1e3 * sst["p99_s"],
                      "p999_ms": 1e3 * sst["p999_s"], "wall_s": sst["wall_s"]}
    out["served"]["workload"] = ("Poisson %g req/s for %g s on the 16 resident scenes, 128^2-256^2, 4-16 spp, "
                                 "depth 4-10, cameras on the bounding sphere, film budget %d samples"
                                 % (rate, dur, budget))
    return out


def run_reference(args, yaml, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    s = O.Scene(yaml)
    cores = os.cpu_count() or 1
    first = (s.width // 2) * s.height * s.spp
    n = 1 << 16
    t = time.time()
    s.render_range(first, n, 0, cores)
    dt = time.time() - t
    n = max(1 << 14, min(int(n * 8.0 / max(dt, 1e-3)), s.paths - first))  # ~8 s per step
    for w in range(args.warmup):
        s.render_range(first, n, 1000 + w, cores)
    times, rays = [], 0
    for k in range(args.steps):
        t = time.time()
        c = s.render_range(first, n, k, cores)
        times.append(time.time() - t)
        rays += int(c[0]) + int(c[1])
    total = sum(times)
    value = rays / total / 1e6
    out = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                            "sample": "%d paths per step (the middle image columns); the reference renderer "
                                      "cannot be built here (Embree/TBB/Boost/Eigen/yaml-cpp/OIIO absent), "
                                      "so its CPU restatement runs" % n},
           "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, help="scene config (1: large terrain scene, 0: box)")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (tests only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    import __graft_entry__ as g
    g.build()
    import mscgpu

    yaml = make_scene(args.config, args.scale)
    info, _, _ = mscgpu.scene_load_host(yaml)
    names = {1: "terrain 1024^2 quads + 300 icospheres, 8 quad lights, 4 Lambert + 4 Phong",
             0: "Cornell-style box, 1316 tris, 1 quad light"}
    cfg = {"workload": names.get(args.config, "config %d" % args.config), "scene_config": args.config,
           "scale": args.scale, "width": info["width"], "height": info["height"], "spp": info["spp"],
           "triangles": info["triangles"], "lights": info["lights"],
           "batch": 1 << (20 if args.config == 1 else 16), "seed": SEED + args.config,
           "l2": "inputs larger than L2: BVH + triangles ~0.4 GB, sample film 1.6 GB, ray pools 1.2 GB per step"}
    if args.impl == "reference":
        run_reference(args, yaml, cfg)
        return
    if int(os.environ.get("RANK", "0")) != 0:
        return  # one GPU per run: only rank 0 renders

    t = time.time()
    pt = mscgpu.Pathtracer(yaml)
    log("scene load + device BVH build %.1f s" % (time.time() - t))
    for _ in range(args.warmup):
        pt.process_device()
    clocks = ClockSampler()
    clocks.start()
    dev_ms, wall, rays, launches = [], [], 0, 0
    for _ in range(args.steps):
        t = time.time()
        pt.process_device()
        wall.append(time.time() - t)
        st = pt.stats()
        dev_ms.append(st["process_ms"])
        rays += st["closest_queries"] + st["shadow_queries"]
        launches += st["kernel_launches"]
    # end to end through the C ABI with the image copied to host memory every step
    e2e_wall, e2e_rays, batches = [], 0, 0
    for _ in range(args.steps):
        t = time.time()
        pt.process()
        img = pt.image()
        e2e_wall.append(time.time() - t)
        st = pt.stats()
        e2e_rays += st["closest_queries"] + st["shadow_queries"]
        batches += st["batches"]
    clocks.stop()
    # one profiled pass for the per-stage split (not part of the timed numbers)
    pt.set_profiling(True)
    pt.process_device()
    prof = pt.stats()
    pt.set_profiling(False)
    pt.close()

    total_ms = sum(dev_ms)
    value = rays / (total_ms / 1e3) / 1e6
    stage_ms = prof["stage_ms"]
    top = max(stage_ms, key=lambda k: stage_ms[k])
    peak, peak_kind = measured_peaks()
    trace_launches = max(1, prof["stage_launches"]["trace"])
    per_launch_ms = stage_ms["trace"] / trace_launches
    per_launch_bytes = ALG_BYTES_TRACE * prof["closest_queries"] / trace_launches
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    roofline = {"kernel": "k_trace_closest (closest-hit traversal)", "bound": "hbm", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": None,
                "alg_bytes": "52 B per closest-hit query (ray 32 B read, hit 20 B written; BVH bytes excluded)",
                "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()}, "top_stage": top}
    lat = sorted(dev_ms)
    out = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
           "latency_ms": {"p50": statistics.median(lat), "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
           "e2e": {"value": e2e_rays / sum(e2e_wall) / 1e6, "unit": "Mrays/s",
                   "h2d_bytes_per_step": int(24 * batches / args.steps),
                   "d2h_bytes_per_step": int(img.nbytes + 32 * batches / args.steps)},
           "gpu_launches": int(launches), "roofline": roofline, "clocks": clocks.summary(),
           "wall_ms_per_step": 1e3 * sum(wall) / args.steps}
    out["batches_per_step"] = batches / args.steps
    if not args.no_forms:
        out["forms"] = bench_forms(args)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(yaml)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
