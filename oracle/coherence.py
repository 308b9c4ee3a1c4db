"""Ray-order coherence comparison - TEST INFRASTRUCTURE (a measurement, not product code).

Builds one batch of secondary rays as the render loop meets it (first-bounce
rays of the terrain scene: origins on surfaces, cosine-distributed directions,
the fullest cardinal direction bin, at most 2^20 rays), orders it three ways
and traces each order through the renderer's closest-hit entry point
(msc_trace_closest, kernel k_trace_closest):

  arrival   the order the rays leave shading (pixel order of their paths)
  morton    the project's ray key (msc_stage_ray_keys: origin and direction
            interleaved in the batch's origin box), stably sorted on its top
            16 bits as the render loop sorts a batch
  median    the reference's order: RaySort.cpp:7-118 restated by the oracle
            (oracle_median_split_order)

Run it under ncu to compare the three k_trace_closest launches (duration,
warp instructions, active lanes per instruction); its own JSON line reports
the closest-hit agreement of the three orders and each order's wall time
(which includes host copies, so only ncu's kernel figures compare coherence).

  python oracle/coherence.py [--scale 0.5]
"""
import argparse
import json
import math
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (os.path.join(REPO, "msc-project_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def secondary_batch(pt, tv, scene_lo, scene_hi, n_camera, rng, cap):
    """First-bounce rays of camera rays shot from above the scene."""
    c = 0.5 * (scene_lo + scene_hi)
    ext = float(np.max(scene_hi - scene_lo))
    eye = c + np.array([0.1 * ext, 0.45 * ext, 0.55 * ext], np.float32)
    # camera rays toward a grid of points on the scene's lower half
    side = int(math.sqrt(n_camera))
    u, v = np.meshgrid((np.arange(side) + 0.5) / side, (np.arange(side) + 0.5) / side, indexing="ij")
    tgt = np.stack([scene_lo[0] + u.ravel() * (scene_hi[0] - scene_lo[0]),
                    np.full(u.size, scene_lo[1] + 0.3 * (scene_hi[1] - scene_lo[1])),
                    scene_lo[2] + v.ravel() * (scene_hi[2] - scene_lo[2])], axis=1).astype(np.float32)
    d = tgt - eye[None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(eye, d.shape).astype(np.float32).copy()
    t, _, _, g, p = pt.trace_closest(o, d)
    hit = g >= 0
    # the scene triangle of (geomID, primID): triangles are numbered geomID-major
    geom = tv["geom"]
    first = np.searchsorted(geom, np.arange(int(geom.max()) + 1))
    tri = first[g[hit]] + p[hit]
    pos = o[hit] + d[hit] * t[hit, None]
    v0, v1, v2 = tv["v"][tri, 0:3], tv["v"][tri, 3:6], tv["v"][tri, 6:9]
    n = np.cross(v1 - v0, v2 - v0)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    n *= np.where((n * d[hit]).sum(axis=1) > 0, -1.0, 1.0)[:, None]  # the visible side
    # cosine-distributed directions about the normal
    m = n.shape[0]
    r1, r2 = rng.random(m), rng.random(m)
    phi, st, ct = 2 * math.pi * r1, np.sqrt(1 - r2), np.sqrt(r2)
    a = np.where(np.abs(n[:, 0:1]) > 0.9, [[0.0, 1.0, 0.0]], [[1.0, 0.0, 0.0]])
    s = np.cross(a, n)
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    w = np.cross(n, s)
    dirs = (s * (np.cos(phi) * st)[:, None] + w * (np.sin(phi) * st)[:, None] + n * ct[:, None]).astype(np.float32)
    org = (pos + n * 1e-3).astype(np.float32)
    from oracle import oracle as O
    bins = O.cardinal(dirs)
    fullest = int(np.bincount(bins, minlength=6).argmax())
    sel = np.nonzero(bins == fullest)[0][:cap]
    return org[sel], dirs[sel]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=float, default=0.5)
    ap.add_argument("--camera-rays", type=int, default=2048 * 2048)
    ap.add_argument("--batch", type=int, default=1 << 20)
    args = ap.parse_args()
    import __graft_entry__ as g
    g.build()
    import mscgpu
    from oracle import oracle as O
    d = os.path.join(tempfile.gettempdir(), "msc_coherence", "terrain_%g" % args.scale)
    y = os.path.join(d, "scene.yaml")
    if not os.path.exists(y):
        y = mscgpu.generate_scene(1, 20261204, d, scale=args.scale)
    info, tv, tg = mscgpu.scene_load_host(y)
    lo = tv.reshape(-1, 3).min(axis=0)
    hi = tv.reshape(-1, 3).max(axis=0)
    rng = np.random.default_rng(7)
    out = {"scene": "terrain at scale %g (%d triangles)" % (args.scale, info["triangles"])}
    with mscgpu.Pathtracer(y) as pt:
        org, dirs = secondary_batch(pt, {"v": tv, "geom": tg}, lo, hi, args.camera_rays, rng, args.batch)
        out["rays"] = int(org.shape[0])
        keys = mscgpu.ray_keys(org, dirs) >> np.uint32(16)
        orders = {"arrival": np.arange(org.shape[0]),
                  "morton": np.argsort(keys, kind="stable"),
                  "median": O.median_split_order(org, dirs).astype(np.int64)}
        ref = None
        for name in ("arrival", "morton", "median"):
            o = orders[name]
            t0 = time.time()
            t, _, _, gg, pp = pt.trace_closest(org[o], dirs[o])
            wall = time.time() - t0
            back = np.empty_like(gg)
            back[o] = gg * 10000000 + pp  # (geomID, primID) per ray in arrival order
            if ref is None:
                ref = back
            out[name] = {"wall_s_incl_copies": round(wall, 4), "same_hits_as_arrival": float((back == ref).mean())}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
