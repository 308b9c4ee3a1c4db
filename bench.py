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
# DRAM bytes per closest-hit query of k_trace_closest, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the half-scale terrain:
# 76.5 MB and 75.1 MB for two launches of 1,048,576 rays (camera rays, first
# bounces), i.e. ~72 B per ray: the ray and hit records plus node and
# triangle misses.
DRAM_BYTES_PER_CLOSEST = (76.48e6 + 75.08e6) / (2 * 1048576)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def scene_generator():
    """The host-only scene generator executable (msc-scenegen): it writes the
    seeded YAML + OBJ files without loading the CUDA library, so that the CPU
    reference arm never loads the renderer's shared library."""
    from mscgpu import build as B  # the build script only; the package loads no library on import
    if not os.path.exists(B.SCENEGEN):
        B.build_scenegen()
    return B.SCENEGEN


def make_scene(config, scale, seed=None):
    seed = SEED + config if seed is None else seed
    d = os.path.join(tempfile.gettempdir(), "msc_bench_scenes", "c%d_s%d_%g" % (config, seed, scale))
    y = os.path.join(d, "scene.yaml")
    if not os.path.exists(y):
        t = time.time()
        os.makedirs(d, exist_ok=True)
        out = subprocess.run([scene_generator(), str(config), str(seed), repr(float(scale)), d], check=True,
                             stdout=subprocess.PIPE, text=True).stdout.strip()
        y = out or y
        log("generated scene %s in %.1f s" % (y, time.time() - t))
    return y


NAMES = {1: "terrain 1024^2 quads + 300 icospheres, 8 quad lights, 4 Lambert + 4 Phong",
         0: "Cornell-style box, 1316 tris, 1 quad light"}


def workload_config(args, width, height, spp, triangles, lights):
    """The workload's identity, printed alike by both arms."""
    return {"workload": NAMES.get(args.config, "config %d" % args.config), "scene_config": args.config,
            "scale": args.scale, "width": width, "height": height, "spp": spp, "triangles": triangles,
            "lights": lights, "batch": 1 << (20 if args.config == 1 else 16), "seed": SEED + args.config,
            "l2": "inputs larger than L2 (129 MB): BVH + triangles ~0.25 GB, sample film 1.6 GB, ray pool up to "
                  "1.6 GB, batch buffers ~1.3 GB, all read or written every step"}


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
                self.samples.append((time.time(), parts))

    def wait_first(self, timeout=10.0):
        """Waits (bounded) until nvidia-smi delivers its first sample, so that its
        start-up does not fall inside a timed region."""
        end = time.time() + timeout
        while self._proc and not self.samples and time.time() < end:
            time.sleep(0.05)

    def stop(self):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self, t0=None, t1=None):
        """Samples taken in [t0, t1] (the timed region; the next sample after it
        covers its end), else all of them."""
        picked = [p for (t, p) in self.samples if t0 is not None and t0 <= t <= t1 + 0.25]
        samples = picked if picked else [p for (_, p) in self.samples]
        if not samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(samples)}


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
    return make_scene(config, scale, seed)


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


def log_uniform_int(rng, lo, hi):
    import math
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def random_job(rng, scene, bbox, res_choices, spp_lo, spp_hi, depth_lo=4, depth_hi=10):
    res = int(rng.choice(res_choices))
    return dict(scene=scene, width=res, height=res, spp=log_uniform_int(rng, spp_lo, spp_hi), min_depth=3,
                max_depth=int(rng.integers(depth_lo, depth_hi + 1)),
                camera=sphere_camera(rng, bbox) if bbox is not None else None,
                seed=int(rng.integers(1, 1 << 30)))


def job_paths(j):
    return j["width"] * j["height"] * j["spp"]


def job_yaml(scene_yaml, job, out_path):
    """One job as the reference's engine takes it: a copy of the scene file with
    the job's image size, sample count, depth limits, pinhole camera and seed
    (msc::Pathtracer reads them from the file and has no setter for them).  The
    plain engine's autotuner is switched off: a one-pass job renders with the
    engine's default choice (batches of 8x the scene's `bin exponent`)."""
    import re
    text = open(scene_yaml).read()
    setup, rest = text.split("---", 1)
    t, r, f = job["camera"]
    subs = [(r"width: \d+", "width: %d" % job["width"]), (r"height: \d+", "height: %d" % job["height"]),
            (r"sample base: \d+", "sample base: 1"), (r"min depth: \d+", "min depth: %d" % job["min_depth"]),
            (r"max depth: \d+", "max depth: %d" % job["max_depth"]),
            (r"type: ThinLens", "type: PinHole"),
            (r"translation: \[[^\]]*\]", "translation: [%r, %r, %r]" % tuple(float(x) for x in t)),
            (r"rotation: \[[^\]]*\]", "rotation: [%r, %r, %r]" % tuple(float(x) for x in r)),
            (r"focal length: [^\n]*", "focal length: %r" % float(f))]
    for pat, rep in subs:
        setup = re.sub(pat, rep, setup, count=1)
    setup = re.sub(r"\n  focal distance: [^\n]*|\n  aperture: [^\n]*", "", setup)
    scene_doc, ext = rest.rsplit("---", 1)
    ext = re.sub(r"\n  seed: \d+", "", ext).rstrip("\n")
    ext += "\n  seed: %d\n  samples per pixel: %d\n  autotune: 0\n" % (job["seed"], job["spp"])
    with open(out_path, "w") as fo:
        fo.write(setup + "---" + scene_doc + "---" + ext)
    # the scene's OBJ files sit next to its YAML: link them beside the copy
    src_dir, dst_dir = os.path.dirname(scene_yaml), os.path.dirname(out_path)
    if os.path.abspath(src_dir) != os.path.abspath(dst_dir):
        for fn in os.listdir(src_dir):
            if fn.endswith(".obj") and not os.path.exists(os.path.join(dst_dir, fn)):
                os.symlink(os.path.join(src_dir, fn), os.path.join(dst_dir, fn))
    return out_path


def plain_api_jobs(scenes, jobs, max_jobs, limit_s):
    """The jobs rendered one by one through the reference's engine interface:
    msc_create from the job's scene file (scene parse + BVH build), one
    msc_process, msc_image, msc_destroy - as the reference's batch mode drives
    msc::Pathtracer (src/main.cpp:137-215).  Wall-clock per job."""
    import mscgpu
    rows, t_all = [], time.time()
    for i, j in enumerate(jobs[:max_jobs]):
        d = os.path.join(tempfile.gettempdir(), "msc_bench_jobs", "job%d" % i)
        os.makedirs(d, exist_ok=True)
        y = job_yaml(scenes[j["scene"]], j, os.path.join(d, "scene.yaml"))
        t = time.time()
        pt = mscgpu.Pathtracer(y)
        t_create = time.time() - t
        pt.process()
        pt.image()
        st = pt.stats()
        pt.close()
        rows.append({"create_s": t_create, "wall_s": time.time() - t,
                     "rays": st["closest_queries"] + st["shadow_queries"], "busy_ms": st["gpu_busy_ms"]})
        if time.time() - t_all > limit_s:
            break
    wall = sum(r["wall_s"] for r in rows)
    rays = sum(r["rays"] for r in rows)
    render = sum(r["wall_s"] - r["create_s"] for r in rows)
    return {"jobs": len(rows), "mrays_per_s": rays / wall / 1e6 if wall else None,
            "render_only_mrays_per_s": rays / render / 1e6 if render else None,
            "create_s_total": sum(r["create_s"] for r in rows), "wall_s": wall}


def rel_mse_against_fp64(b, scenes, jobs, ids, picks):
    """Relative MSE of batched job images against the FP64 oracle rendering the
    same jobs (same cameras, sample counts and per-path random sequences), and
    the same figure for the plain engine rendering each job from its own scene
    file: matched error means the two forms' images are the same."""
    import numpy as np
    import mscgpu
    from oracle import oracle as O
    out = []
    for k in picks:
        j = jobs[k]
        s = O.Scene(scenes[j["scene"]])
        t, r, f = j["camera"]
        s.set_job(width=j["width"], height=j["height"], spp=j["spp"], min_depth=j["min_depth"],
                  max_depth=j["max_depth"], cam_t=t, cam_r=r, focal=f, seed=j["seed"])
        ref, _, _, _ = s.render(0, double=True)
        img = b.image(ids[k]).astype(np.float32)
        d = os.path.join(tempfile.gettempdir(), "msc_bench_jobs", "mse%d" % k)
        os.makedirs(d, exist_ok=True)
        with mscgpu.Pathtracer(job_yaml(scenes[j["scene"]], j, os.path.join(d, "scene.yaml"))) as pt:
            pt.process()
            plain = pt.image()
        den = max(float(np.mean(ref ** 2)), 1e-30)
        out.append({"job": k, "paths": job_paths(j), "triangles": s.triangles,
                    "rel_mse": float(np.mean((img.astype(np.float64) - ref) ** 2) / den),
                    "plain_rel_mse": float(np.mean((plain.astype(np.float64) - ref) ** 2) / den),
                    "plain_image_bit_equal": bool(np.array_equal(img.view(np.uint32), plain.view(np.uint32)))})
    return out


def bench_forms(args):
    """Batched and served forms against the one-job-at-a-time loop on the same jobs.

    Batched: one job per scene over 64 terrain scenes with log-uniform triangle
    counts, resolutions {128^2 .. 1024^2}, 4-256 spp (log-uniform), depth 4-10,
    all submitted at once.  Served: Poisson arrivals on the first 16 scenes.
    The per-job loop is the same engine admitting one job at a time (the plain
    single-scene wavefront, scenes kept resident)."""
    import mscgpu
    import numpy as np
    t = time.time()
    scenes = scene_set(args.forms_scenes, 1e4, 3e6, SEED + 300)
    gen_s = time.time() - t
    film_cap = 1_800_000_000  # the film pool indexes samples with 31 bits
    t = time.time()
    b = mscgpu.Batch(batch_exponent=23, film_samples=film_cap)
    bboxes, tris = [], []
    for y in scenes:
        k = b.add_scene(y)
        lo, hi, n = b.scene_info(k)
        bboxes.append((lo, hi))
        tris.append(n)
    load_s = time.time() - t
    rng = np.random.default_rng(SEED + 301)
    while True:  # one job per scene
        jobs = [random_job(rng, i, bboxes[i], [128, 256, 512, 1024], 4, 256) for i in range(len(scenes))]
        if sum(job_paths(j) for j in jobs) < film_cap:
            break
    film = film_cap
    log("forms: %d scenes (%d..%d tris, %d total) generated in %.1f s, loaded + BVHs in %.1f s"
        % (len(scenes), min(tris), max(tris), sum(tris), gen_s, load_s))

    def rays_of(st):
        return st["closest_queries"] + st["shadow_queries"]

    out = {}
    # autotune on a sample of the same workload (untimed): the first 16 jobs at
    # up to 16 spp, one run per candidate until the tuner has booked them all
    b.autotune(windows=1)
    sample = [dict(j, spp=min(j["spp"], 16)) for j in jobs[:16]]
    for _ in range(24):
        ids = [b.submit(**j) for j in sample]
        b.run()
        for i in ids:
            b.release(i)
        if not b.tuning()["tuning"]:
            break
    tuned = b.tuning()
    tune_log = b.tune_log()
    # batched: every job in one wavefront, tuned choice
    s0 = b.stats()
    ids = [b.submit(**j) for j in jobs]
    t = time.time()
    b.run()
    wall = time.time() - t
    st1 = b.stats()
    rays = rays_of(st1) - rays_of(s0)
    busy = st1["gpu_busy_ms"] / 1e3
    # matched error: the smallest jobs' images against the FP64 oracle
    picks = sorted(range(len(jobs)), key=lambda k: (tris[jobs[k]["scene"]], job_paths(jobs[k])))[:3]
    try:
        mse = rel_mse_against_fp64(b, scenes, jobs, ids, picks)
    except Exception as e:  # the checker is optional on a box without the oracle
        mse = "unavailable: %s" % e
    for i in ids:
        b.release(i)
    # the per-job loop on the same jobs: one job in flight at a time, with the
    # same tuned settings, so the difference is only the merging of jobs
    tuned_kw = {k: tuned[k] for k in TUNE_KEYS}
    b.set_tuning(**tuned_kw)
    b.set_max_active(1)
    _, pst = b.serve([(0.0, j) for j in jobs])
    plain_rate = rays_of(pst) / pst["wall_s"] / 1e6
    rate = rays / wall / 1e6
    api = plain_api_jobs(scenes, jobs, len(jobs), args.plain_api_seconds)
    out["batched"] = {
        "workload": "%d jobs, one per terrain scene (%d-%d tris, log-uniform; %d total), resolutions "
                    "128^2-1024^2, 4-256 spp log-uniform, depth 4-10, RR from 3, cameras on the bounding sphere "
                    "(fov 30-70)" % (len(jobs), min(tris), max(tris), sum(tris)),
        "paths": sum(job_paths(j) for j in jobs), "mrays_per_s": rate, "wall_s": wall,
        "per_job_loop_mrays_per_s": plain_rate, "per_job_loop_wall_s": pst["wall_s"],
        "speedup_vs_per_job_loop": rate / plain_rate if plain_rate else None,
        "gpu_busy_fraction": busy / wall if wall else None,
        "per_job_loop_gpu_busy_fraction": pst["gpu_busy_s"] / pst["wall_s"] if pst["wall_s"] else None,
        "scene_load_s": load_s,
        "plain_api": dict(api, comparator="msc_create + msc_process + msc_image + msc_destroy per job, scene parse "
                                          "and BVH build included, as src/main.cpp drives msc::Pathtracer"),
        "e2e_incl_scene_load_mrays_per_s": rays / (wall + load_s) / 1e6,
        "speedup_e2e_vs_plain_api": ((rays / (wall + load_s) / 1e6) / api["mrays_per_s"]
                                     if api["mrays_per_s"] else None),
        "rel_mse_vs_fp64_oracle": mse,
        "tuned": {k: tuned[k] for k in TUNE_KEYS},
        "tune_samples_fields": "batch_exponent, bins, trace_block, persistent, digit_bits, ray_sort, hit_sort, "
                               "ray_key_bits, Mrays/s",
        "tune_samples": [[t["batch_exponent"], t["bins"], t["trace_block"], t["persistent"], t["digit_bits"],
                          t["ray_sort"], t["hit_sort"], t["ray_key_bits"], round(t["mrays_per_s"], 1)]
                         for t in tune_log]}
    # served: Poisson arrivals on the first 16 resident scenes, at each rate
    nres = min(16, len(scenes))
    out["served"] = {"workload": "Poisson arrivals on %d resident scenes, 128^2-512^2, 4-64 spp log-uniform, "
                                 "depth 4-10, cameras on the bounding sphere; admission by a film-memory budget of "
                                 "%d samples (%.1f GB); per rate: the served form, then the per-job loop on the "
                                 "same requests" % (nres, film, film * 24 / 1e9),
                     "rates": []}
    for spec in args.serve_rates.split(","):
        rrate, dur = (float(x) for x in spec.split(":")) if ":" in spec else (float(spec), args.serve_seconds)
        arrivals = np.cumsum(rng.exponential(1.0 / rrate, size=int(rrate * dur * 2) + 16))
        arrivals = arrivals[arrivals < dur]
        reqs = []
        for a in arrivals:
            k = int(rng.integers(0, nres))
            reqs.append((float(a), random_job(rng, k, bboxes[k], [128, 256, 512], 4, 64)))
        row = {"rate_per_s": rrate, "seconds": dur, "requests": len(reqs)}
        for label, max_active in (("served", 0), ("per_job_loop", 1)):
            b.set_max_active(max_active)
            b.set_tuning(**tuned_kw)
            _, sst = b.serve(reqs)
            row[label] = {"completed": sst["completed"], "mrays_per_s": sst["mrays_per_s"],
                          "p50_ms": 1e3 * sst["p50_s"], "p99_ms": 1e3 * sst["p99_s"],
                          "p999_ms": 1e3 * sst["p999_s"], "wall_s": sst["wall_s"],
                          "peak_film_samples": sst["peak_film_samples"],
                          "gpu_busy_fraction": sst["gpu_busy_s"] / sst["wall_s"] if sst["wall_s"] else None}
        row["speedup_vs_per_job_loop"] = (row["served"]["mrays_per_s"] / row["per_job_loop"]["mrays_per_s"]
                                          if row["per_job_loop"]["mrays_per_s"] else None)
        out["served"]["rates"].append(row)
        log("served at %g req/s: %s" % (rrate, json.dumps(row)))
    b.close()
    return out


def bench_c4(args):
    """The served form at its stated configuration: 16 resident scenes (terrain
    rules, triangle counts log-uniform in 10K-3M), Poisson requests at each rate
    for a window of 60 s, each a seeded camera on its scene's bounding sphere
    (fov 30-70) at 256^2-2048^2 pixels and 4-256 spp (log-uniform), depth
    4-10.  Admission follows the film-memory budget; at these rates the offered
    work exceeds what any single GPU renders, so admission closes at the end of
    the window and the requests still waiting are counted, not served.  Each
    rate runs the served form, then the one-job-at-a-time loop on the same
    requests; a sample of requests also goes through the plain engine interface
    (msc_create per request, since a request's camera and image size live in
    its scene file)."""
    import mscgpu
    import numpy as np
    scenes = scene_set(16, 1e4, 3e6, SEED + 400)
    film_cap = 2_000_000_000  # 48 GB of film samples (31-bit sample index)
    b = mscgpu.Batch(batch_exponent=23, film_samples=film_cap)
    b.set_memory_budget(120_000_000_000)  # the stated 120 GB: fixed buffers, scenes and job images
    bboxes, tris = [], []
    t = time.time()
    for y in scenes:
        k = b.add_scene(y)
        lo, hi, n = b.scene_info(k)
        bboxes.append((lo, hi))
        tris.append(n)
    load_s = time.time() - t
    rng = np.random.default_rng(SEED + 401)
    # tune on a sample of the request mix (untimed)
    b.autotune(windows=1)
    sample = [random_job(rng, k % 16, bboxes[k % 16], [256, 512], 4, 16) for k in range(16)]
    for _ in range(32):
        ids = [b.submit(**j) for j in sample]
        b.run()
        for i in ids:
            b.release(i)
        if not b.tuning()["tuning"]:
            break
    tuned = b.tuning()
    tuned_kw = {k: tuned[k] for k in TUNE_KEYS}
    out = {"workload": "16 resident terrain scenes (%d-%d tris, %d total; loaded in %.1f s), Poisson requests, "
                       "256^2-2048^2 (uniform over the four sizes), 4-256 spp log-uniform, depth 4-10, cameras on "
                       "the bounding sphere (fov 30-70); film budget %d samples (%.0f GB); admission closes after "
                       "the window" % (min(tris), max(tris), sum(tris), load_s, film_cap, film_cap * 24 / 1e9),
           "tuned": tuned_kw, "rates": []}
    used, fixed, _ = b.memory()
    out["device_memory"] = {"budget_gb": 120.0, "fixed_and_scenes_gb": round(fixed / 1e9, 2)}
    for spec in args.c4_rates.split(","):
        rrate, dur = (float(x) for x in spec.split(":"))
        arrivals = np.cumsum(rng.exponential(1.0 / rrate, size=int(rrate * dur * 2) + 16))
        arrivals = arrivals[arrivals < dur]
        reqs = []
        for a in arrivals:
            k = int(rng.integers(0, 16))
            reqs.append((float(a), random_job(rng, k, bboxes[k], [256, 512, 1024, 2048], 4, 256)))
        offered = sum(job_paths(j) for _, j in reqs)
        row = {"rate_per_s": rrate, "window_s": dur, "requests": len(reqs), "offered_paths": offered}
        for label, max_active in (("served", 0), ("per_job_loop", 1)):
            b.set_max_active(max_active)
            b.set_tuning(**tuned_kw)
            _, sst = b.serve(reqs, window_s=dur)
            row[label] = {"completed": sst["completed"], "not_admitted": sst["not_admitted"],
                          "mrays_per_s": sst["mrays_per_s"], "p50_s": sst["p50_s"], "p99_s": sst["p99_s"],
                          "p999_s": sst["p999_s"], "wall_s": sst["wall_s"],
                          "peak_film_samples": sst["peak_film_samples"],
                          "gpu_busy_fraction": sst["gpu_busy_s"] / sst["wall_s"] if sst["wall_s"] else None}
            log("c4 %g req/s %s: %s" % (rrate, label, json.dumps(row[label])))
        row["speedup_vs_per_job_loop"] = (row["served"]["mrays_per_s"] / row["per_job_loop"]["mrays_per_s"]
                                          if row["per_job_loop"]["mrays_per_s"] else None)
        out["rates"].append(row)
    b.close()
    # the plain engine interface on a sample of the same request mix
    sample = [random_job(rng, int(rng.integers(0, 16)), None, [256, 512, 1024, 2048], 4, 256) for _ in range(64)]
    for j in sample:
        j["camera"] = sphere_camera(rng, bboxes[j["scene"]])
    api = plain_api_jobs(scenes, sample, len(sample), args.plain_api_seconds)
    out["plain_api"] = dict(api, comparator="msc_create + msc_process + msc_image + msc_destroy per request")
    for row in out["rates"]:
        row["speedup_vs_plain_api"] = (row["served"]["mrays_per_s"] / api["mrays_per_s"]
                                       if api["mrays_per_s"] else None)
    return out


def bench_stress(args):
    """Hit-sort stress scene: sorted (64-bit hit key) against unsorted shading."""
    import mscgpu
    t = time.time()
    y = make_scene_scaled(2, SEED + 2, args.stress_scale)
    gen_s = time.time() - t
    t = time.time()
    pt = mscgpu.Pathtracer(y)
    load_s = time.time() - t
    out = {"workload": "2000 subdivided tori x 4000 tris (8 M) + floor, 4096 shader ids (Lambert/Phong) with "
                       "per-face 16x16 FP16 RGB texels (12.3 GB), 64 sphere lights of log-uniform power; "
                       "1024^2, 32 spp, depth 6" if args.stress_scale == 1.0 else
                       "hit-sort stress scene at scale %g" % args.stress_scale,
           "generate_s": gen_s, "load_s": load_s}
    modes = {}
    for label, hit_sort in (("sorted_64bit_key", True), ("unsorted", False)):
        pt.set_tuning(batch_exponent=22, trace_block=64, ray_sort=False, hit_sort=hit_sort)
        pt.process_device()  # warm-up (captures this choice's graph)
        ms, rays = 0.0, 0
        for _ in range(2):
            pt.process_device()
            st = pt.stats()
            ms += st["process_ms"]
            rays += st["closest_queries"] + st["shadow_queries"]
        pt.set_profiling(True)
        pt.process_device()
        prof = pt.stats()
        pt.set_profiling(False)
        sm = prof["stage_ms"]
        hits = prof["closest_queries"]
        modes[label] = {"mrays_per_s": rays / ms / 1e3, "ms_per_pass": ms / 2,
                        "shade_ms": round(sm["shade"], 3), "hit_sort_ms": round(sm["hit_sort"], 3),
                        "shading_mhits_per_s": hits / sm["shade"] / 1e3 if sm["shade"] > 0 else None,
                        "shading_incl_sort_mhits_per_s": hits / (sm["shade"] + sm["hit_sort"]) / 1e3}
    pt.close()
    out.update(modes)
    log("stress: %s" % json.dumps(out))
    return out


def scene_for(args):
    """The workload's scene file; --sample-base writes a copy with another sample base."""
    y = make_scene(args.config, args.scale)
    if args.sample_base > 0:
        import re
        text = open(y).read()
        text = re.sub(r"sample base: \d+", "sample base: %d" % args.sample_base, text, count=1)
        y2 = os.path.join(os.path.dirname(y), "scene_base%d.yaml" % args.sample_base)
        with open(y2, "w") as f:
            f.write(text)
        y = y2
    return y


def run_reference(args):
    """The CPU arm: the reference algorithm (its CPU restatement in oracle/) on
    the host cores, on the same scene files.  It loads neither the CUDA
    renderer's library nor anything built from its sources but the host-only
    scene generator, which runs as a separate executable."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import build as oracle_build
    oracle_build.build()
    from oracle import oracle as O
    yaml = scene_for(args)
    t = time.time()
    s = O.Scene(yaml)
    log("oracle scene load + SAH build %.1f s" % (time.time() - t))
    cfg = workload_config(args, s.width, s.height, s.spp, s.triangles, s.lights)
    cores = os.cpu_count() or 1
    first = (s.width // 2) * s.height * s.spp
    n = min(1 << 16, s.paths - first)
    t = time.time()
    s.render_range(first, n, 0, cores)
    dt = time.time() - t
    n = max(min(1 << 14, s.paths - first), min(int(n * 8.0 / max(dt, 1e-3)), s.paths - first))  # ~8 s per step
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


def timed_passes(pt, passes, warmup=2):
    """Device-timed passes of the plain engine: (Mrays/s, ms per pass, rays per pass)."""
    for _ in range(warmup):
        pt.process_device()
    ms, rays = 0.0, 0
    for _ in range(passes):
        pt.process_device()
        st = pt.stats()
        ms += st["process_ms"]
        rays += st["closest_queries"] + st["shadow_queries"]
    return rays / ms / 1e3, ms / passes, rays // passes


def profiled_pass(pt):
    pt.set_profiling(True)
    pt.process_device()
    prof = pt.stats()
    pt.set_profiling(False)
    return prof


TUNE_KEYS = ("batch_exponent", "trace_block", "ray_sort", "hit_sort", "bins", "persistent", "digit_bits",
             "ray_key_bits")


def hbm_stages(prof, peak, spp, batch_exponent, digit_bits=8):
    """Achieved HBM bandwidth of the bandwidth-bound stages from one profiled
    pass: algorithmic bytes per ray (or per sample) / the stage's event time."""
    sm = prof["stage_ms"]
    closest = prof["closest_queries"]
    paths = prof["width"] * prof["height"] * spp
    out = {}
    # the camera rays are made straight into their bins (film sample 24 B and
    # the ray with its key 52 B written, its bin byte written and read); batches
    # of 2^13 rays and more bin directly: the shading writes each continuing
    # ray (48 B) and its sort key (4 B) into its bin, and the bins stage is one
    # small commit per batch; smaller batches partition the continuing rays
    # through staging (read 48 B, written 48 B with its 4 B key, plus the
    # count, scan and commit passes)
    stages = [("raygen", sm["raygen"], 78.0 * paths, "78 B per camera ray: film sample 24 B, ray and key 52 B "
                                                     "into its bin, its bin byte 2 B")]
    if batch_exponent >= 13:
        shade_bytes, shade_what = 164.0 * closest, ("164 B per closest hit: ray 48 B and hit 16 B read, continuation "
                                                     "ray 48 B with its 4 B key into its bin and shadow ray 48 B "
                                                     "written")
    else:
        stages.append(("bins", sm["bins"], 112.0 * max(0, closest - paths), "112 B per continuing ray partitioned"))
        shade_bytes, shade_what = 160.0 * closest, ("160 B per closest hit: ray 48 B and hit 16 B read, "
                                                     "continuation ray 48 B and shadow ray 48 B written")
    for name, ms, nbytes, what in stages + [
            ("ray_sort", sm["ray_sort"], (32.0 if digit_bits == 8 else 36.0) * closest,
             "32 B per key: two 16 B passes (the ray-key kernel counts the digits)" if digit_bits == 8 else
             "36 B per key: histogram read + two 16 B passes"),
            ("filter", sm["filter"], 24.0 * paths, "24 B per film sample (radiance 16 B + position 8 B)"),
            ("shade", sm["shade"], shade_bytes, shade_what)]:
        if ms > 0:
            gbs = nbytes / (ms / 1e3) / 1e9
            out[name] = {"ms": round(ms, 3), "gbs": round(gbs, 1), "frac": round(gbs / peak, 4), "alg_bytes": what}
    return out


def bench_plain_extra(args, tuned):
    """C1 at its stated settings (batches of 2^20 rays, 32-bit ray keys, hit
    sort on, 6 direction bins) beside the tuned point, and the box scene."""
    import mscgpu
    out = {}
    yaml = make_scene(1, args.scale)
    pt = mscgpu.Pathtracer(yaml)
    pinned = dict(batch_exponent=20, trace_block=tuned["trace_block"], ray_sort=True, hit_sort=True, bins=6,
                  persistent=False, digit_bits=8, ray_key_bits=32)
    pt.set_tuning(**pinned)
    rate, ms, rays = timed_passes(pt, 3)
    prof = profiled_pass(pt)
    out["pinned"] = {"settings": "batches of 2^20 rays, 32-bit ray sort keys (4 x 8-bit digit passes), hit sort "
                                 "on, 6 direction bins, %d-thread traversal" % tuned["trace_block"],
                     "mrays_per_s": rate, "ms_per_pass": ms, "rays_per_pass": rays,
                     "stage_ms": {k: round(v, 3) for k, v in prof["stage_ms"].items()}}
    pt.close()
    y0 = make_scene(0, 1.0)
    pt = mscgpu.Pathtracer(y0)
    passes = 0
    while pt.tuning()["tuning"] and passes < 32:
        pt.process_device()
        passes += 1
    t0 = pt.tuning()
    rate, ms, rays = timed_passes(pt, 20)
    pt.set_tuning(batch_exponent=16, trace_block=t0["trace_block"], ray_sort=True, hit_sort=True, bins=6,
                  persistent=False, digit_bits=8, ray_key_bits=32)
    prate, pms, _ = timed_passes(pt, 20)
    st = pt.stats()
    pt.close()
    out["c0"] = {"workload": "Cornell-style box, 256^2 x 16 spp, depth 4, %d tris" % st["triangles"],
                 "tuned_mrays_per_s": rate, "tuned_ms_per_pass": ms, "rays_per_pass": rays,
                 "tuned": {k: t0[k] for k in TUNE_KEYS},
                 "pinned_mrays_per_s": prate, "pinned_ms_per_pass": pms,
                 "pinned": "batches of 2^16 rays, 32-bit ray keys, hit sort on, 6 bins"}
    return out


def run_gpu(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return  # one GPU per run: only rank 0 renders
    import __graft_entry__ as g
    g.build()
    import mscgpu

    yaml = scene_for(args)
    t = time.time()
    info, _, _ = mscgpu.scene_load_host(yaml)
    host_parse_s = time.time() - t
    cfg = workload_config(args, info["width"], info["height"], info["spp"], info["triangles"], info["lights"])

    t = time.time()
    pt = mscgpu.Pathtracer(yaml)
    create_s = time.time() - t
    st0 = pt.stats()
    scene_input = {"msc_create_s": round(create_s, 3), "load_s": round(st0["load_ms"] / 1e3, 3),
                   "bvh_build_s": round(st0["bvh_ms"] / 1e3, 3), "host_parse_only_s": round(host_parse_s, 3),
                   "triangles": info["triangles"]}
    log("scene input: %s" % json.dumps(scene_input))
    tuning_passes = 0
    if args.tuning != "auto":
        v = [int(x) for x in args.tuning.split(",")]
        v += [0, 8][len(v) - 5:]
        pt.set_tuning(batch_exponent=v[0], bins=v[1], trace_block=v[2], ray_sort=bool(v[3]), hit_sort=bool(v[4]),
                      persistent=bool(v[5]), digit_bits=v[6])
    else:
        # the engine tunes itself during its first passes: let it finish before the warm-up
        while pt.tuning()["tuning"] and tuning_passes < 32:
            pt.process_device()
            tuning_passes += 1
        log("autotuner settled after %d passes: %s" % (tuning_passes, pt.tuning()))
    # the clock sampler starts before the warm-up, so that nvidia-smi's own
    # start-up stays out of the timed region
    clocks = ClockSampler()
    clocks.start()
    for _ in range(args.warmup):
        pt.process_device()
    clocks.wait_first()
    t_timed = time.time()
    dev_ms, wall, rays, launches, busy_ms = [], [], 0, 0, 0.0
    for _ in range(args.steps):
        t = time.time()
        pt.process_device()
        wall.append(time.time() - t)
        st = pt.stats()
        dev_ms.append(st["process_ms"])
        busy_ms += st["gpu_busy_ms"]
        rays += st["closest_queries"] + st["shadow_queries"]
        launches += st["kernel_launches"]
    # end to end through the C ABI with the image copied to host memory every step
    e2e_wall, e2e_rays, batches = [], 0, 0
    for _ in range(args.steps):
        t = time.time()
        pt.process()
        img = pt.image(copy=False)  # msc_image: the host image the pass copied back
        e2e_wall.append(time.time() - t)
        st = pt.stats()
        e2e_rays += st["closest_queries"] + st["shadow_queries"]
        batches += st["batches"]
    t_timed_end = time.time()
    clocks.stop()
    # one profiled pass for the per-stage split (not part of the timed numbers)
    prof = profiled_pass(pt)
    tuned = pt.tuning()
    tuned_d = {k: tuned[k] for k in TUNE_KEYS}
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
                "traffic": DRAM_BYTES_PER_CLOSEST * prof["closest_queries"] / trace_launches,
                "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of an ncu capture of the half-scale "
                                "terrain (1,048,576 rays per launch: 76.5 MB and 75.1 MB), scaled by the rays of an "
                                "average full-size launch",
                "alg_bytes": "52 B per closest-hit query (ray 32 B read, hit 20 B written; BVH bytes excluded)",
                "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()}, "top_stage": top,
                "hbm_stages": hbm_stages(prof, peak, info["spp"], tuned_d["batch_exponent"], tuned_d["digit_bits"])}
    lat = sorted(dev_ms)
    out = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
           "latency_ms": {"p50": statistics.median(lat), "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
           "step_ms": [round(x, 3) for x in dev_ms],
           "e2e": {"value": e2e_rays / sum(e2e_wall) / 1e6, "unit": "Mrays/s",
                   "h2d_bytes_per_step": int(24 * batches / args.steps),
                   "d2h_bytes_per_step": int(img.nbytes + 32 * batches / args.steps)},
           "gpu_launches": int(launches), "roofline": roofline, "clocks": clocks.summary(t_timed, t_timed_end),
           "wall_ms_per_step": 1e3 * sum(wall) / args.steps}
    out["batches_per_step"] = batches / args.steps
    # device time of the work queued between the engine's host waits, over the
    # timed passes' device time: the rest is the GPU waiting for the host
    out["gpu_busy_fraction"] = busy_ms / total_ms if total_ms > 0 else None
    out["scene_input"] = scene_input
    extra = {}
    if not args.no_extra and args.config == 1:
        extra = bench_plain_extra(args, tuned_d)
        out["c0"] = extra["c0"]
    if not args.no_forms:
        out["forms"] = bench_forms(args)
    if not args.no_stress:
        out["hit_sort_stress"] = bench_stress(args)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(yaml)
    # last, so that a reader of the line's end sees them
    out["tuned"] = dict(tuned_d, tuning_passes=tuning_passes, mrays_per_s=round(value, 1))
    if "pinned" in extra:
        out["pinned"] = extra["pinned"]
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, help="scene config (1: large terrain scene, 0: box)")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (tests and profiling cases)")
    ap.add_argument("--sample-base", type=int, default=0,
                    help="override the scene's sample base (spp = base^2): small profiling cases at full spp")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--no-stress", action="store_true", help="skip the hit-sort stress scene")
    ap.add_argument("--no-extra", action="store_true", help="skip the stated-settings and box-scene measurements")
    ap.add_argument("--tuning", default="auto",
                    help="'auto' (the engine tunes itself) or batch_exp,bins,trace_block,ray_sort,hit_sort"
                         "[,persistent[,digit_bits]]")
    ap.add_argument("--stress-scale", type=float, default=1.0)
    ap.add_argument("--serve-rates", default="100:6,600:3",
                    help="Poisson request rates as rate:seconds (req/s, window), comma-separated")
    ap.add_argument("--forms-scenes", type=int, default=64)
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--c4", action="store_true",
                    help="only the served form at its stated configuration (Poisson 50/200/400 req/s, 60 s "
                         "windows); prints one JSON line of its own")
    ap.add_argument("--c4-rates", default="50:60,200:60,400:60")
    ap.add_argument("--plain-api-seconds", type=float, default=20.0,
                    help="time limit of the plain-API comparator (jobs rendered one by one through msc_create)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    elif args.c4:
        import __graft_entry__ as g
        g.build()
        print(json.dumps({"served_c4": bench_c4(args)}), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
