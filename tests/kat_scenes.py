"""Analytic known-answer scenes: scenes whose expected radiance has a closed form.

These pin the integrator (emitter hits, next-event estimation with multiple
importance sampling, Lambert BSDF sampling, Russian roulette, light picking)
of both the CUDA renderer and the CPU oracle against mathematics rather than
against each other.  The restated reference code is src/core/Integrator.cpp:20-246,
src/core/QuadLight.cpp:41-84, src/core/LambertShader.cpp:27-73 and
include/core/Common.h:35-48 of joshbainbridge/msc-project.

quad_over_plane / sphere_over_plane
    A Lambert plane y = 0 (reflectance rho, colour c) lit by two lights of
    different size and radiance, both facing the plane.  The camera's pinhole
    sits between the plane and the lights and looks straight down, so every
    camera ray meets the plane.  A sample whose camera ray meets the plane at p
    has the expected radiance  rho c / pi * E(p),  where E is the irradiance:
      * polygonal emitter of radiance Le (Lambert's contour integral,
        e.g. Arvo, "Applications of irradiance tensors to the simulation of
        non-Lambertian phenomena", SIGGRAPH 1995, eq. 9):
            E(p) = Le / 2 * | sum_i theta_i (g_i . n) |,
        theta_i the angle subtended at p by edge i, g_i the unit normal of the
        plane through p and that edge;
      * sphere of radius r, centre C, radiance Le, wholly above the horizon:
            E(p) = pi Le (r / d)^2 cos(theta),  d = |C - p|.
    The paths continue (depth >= 1), so the BSDF-sampled half of the MIS pair
    reaches the lights; with Russian roulette switched on at depth 0 the
    estimator stays unbiased.

phong_over_plane
    The same set-up with a modified-Phong plane (exponent 20) under one quad
    light: f = rho c (n + 2) / (2 pi) max(0, r . wi)^n has no closed-form
    integral over a polygon, so the expected radiance of each sample is the
    direct-lighting integral evaluated by a 16 x 16 Gauss-Legendre rule over
    the light (converged to ~1e-13 relative; the Monte Carlo tolerance is
    ~1e-3).

furnace
    A convex Lambert icosphere inside a closed cube of six inward-facing quad
    lights of radiance Le.  Every direction leaving the sphere meets an
    emitter, so a sample that hits the sphere has expected radiance
    rho c Le; a sample that sees a wall has radiance Le exactly.

`check_unbiased` compares per-sample radiance with its expectation: the mean
residual must lie within z standard errors (the estimators are unbiased, so
only Monte Carlo noise remains).
"""
import math
import os

import numpy as np

FILM_HALF = 36.0  # Camera.cpp:34-35 maps the film to [-36, 36] scene units across the width


def _setup(width, height, base, min_depth, max_depth, threshold, cam_t, cam_r, focal, spp=0, mis="balance",
           seed=4242):
    head = ("image:\n  width: %d\n  height: %d\n  sample base: %d\n"
            "settings:\n  min depth: %d\n  max depth: %d\n  threshold: %r\n  bucket size: 16\n"
            "  shading size: 4096\n  bin exponent: 12\n"
            "camera:\n  type: PinHole\n  translation: [%r, %r, %r]\n  rotation: [%r, %r, %r]\n"
            "  focal length: %r\nfilter:\n  type: Tent\nsampler:\n  type: Stratified\n"
            % (width, height, base, min_depth, max_depth, float(threshold), *map(float, cam_t),
               *map(float, cam_r), float(focal)))
    ext = "extensions:\n  mis: %s\n  seed: %d\n" % (mis, seed)
    if spp:
        ext += "  samples per pixel: %d\n" % spp
    return head, ext


def _shader(colour, refl):
    return ("shader:\n  type: Lambert\n  texture:\n    type: Constant\n    colour: [%r, %r, %r]\n"
            "  reflectance: %r\n" % (*map(float, colour), float(refl)))


def _object(filename, shader):
    return ("object:\n  type: Polygon\n  filename: %s\n  translation: [0.0, 0.0, 0.0]\n"
            "  rotation: [0.0, 0.0, 0.0]\n  scale: [1.0, 1.0, 1.0]\n  shader: %d\n" % (filename, shader))


def _quad_light(t, r, sx, sy, le):
    return ("light:\n  type: Quad\n  translation: [%r, %r, %r]\n  rotation: [%r, %r, %r]\n"
            "  scale: [%r, %r]\n  intensity: %r\n" % (*map(float, t), *map(float, r), float(sx), float(sy), float(le)))


def _sphere_light(c, radius, le):
    return ("light:\n  type: Sphere\n  translation: [%r, %r, %r]\n  radius: %r\n  intensity: %r\n"
            % (*map(float, c), float(radius), float(le)))


def _write(out_dir, head, scene, ext):
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "scene.yaml")
    with open(path, "w") as f:
        f.write(head + "---\n" + scene + "---\n" + ext)
    return path


def _write_plane_obj(path, half):
    # counter-clockwise seen from +y, so e1 x e2 (the renderer's shading normal) points up
    with open(path, "w") as f:
        f.write("v %r 0.0 %r\nv %r 0.0 %r\nv %r 0.0 %r\nv %r 0.0 %r\nf 1 2 3 4\n"
                % (-half, -half, -half, half, half, half, half, -half))


class PlaneScene:
    """Parameters of a plane scene, kept for the closed form."""

    def __init__(self, path, width, height, spp, focal, nodal, rho, colour, lights):
        self.path, self.width, self.height, self.spp = path, width, height, spp
        self.focal, self.nodal = focal, np.asarray(nodal, np.float64)
        self.rho, self.colour = rho, np.asarray(colour, np.float64)
        self.lights = lights  # ("quad", vertices (4,3), Le) or ("sphere", centre, radius, Le)

    def hit_points(self, xy):
        """Where each sample's camera ray meets the plane y = 0.

        The camera looks down -y (rotation z = -90 degrees): a film position
        (px, py) sits at film = nodal + (fy, focal, fx) and the ray leaves the
        pinhole towards nodal - film (PinHoleCamera.cpp:18-30)."""
        xy = np.asarray(xy, np.float64)
        fx = ((xy[:, 0] * 2.0 - self.width) / self.width) * FILM_HALF
        fy = ((xy[:, 1] * 2.0 - self.height) / self.width) * FILM_HALF
        s = self.nodal[1] / self.focal
        return np.stack([self.nodal[0] - fy * s, np.zeros_like(fx), self.nodal[2] - fx * s], axis=1)

    def irradiance(self, p):
        n = np.array([0.0, 1.0, 0.0])
        e = np.zeros(p.shape[0])
        for light in self.lights:
            if light[0] == "quad":
                e += polygon_irradiance(p, n, light[1], light[2])
            else:
                e += sphere_irradiance(p, n, light[1], light[2], light[3])
        return e

    def expected(self, xy):
        """Expected radiance (P, 3) of each sample from its film position."""
        e = self.irradiance(self.hit_points(xy))
        return (self.rho / math.pi) * e[:, None] * self.colour[None, :]


def polygon_irradiance(p, n, verts, le):
    """Irradiance at points p (N,3) with normal n from a uniform polygonal emitter
    of radiance le (Lambert's contour integral)."""
    a = np.asarray(verts, np.float64)[None, :, :] - p[:, None, :]
    a /= np.linalg.norm(a, axis=2, keepdims=True)
    b = np.roll(a, -1, axis=1)
    theta = np.arccos(np.clip((a * b).sum(axis=2), -1.0, 1.0))
    g = np.cross(a, b)
    g /= np.linalg.norm(g, axis=2, keepdims=True)
    return le * 0.5 * np.abs((theta * (g @ n)).sum(axis=1))


def sphere_irradiance(p, n, centre, radius, le):
    """Irradiance at points p (N,3) with normal n from a sphere of radiance le
    wholly above their horizon: pi le (r/d)^2 cos(theta)."""
    w = np.asarray(centre, np.float64)[None, :] - p
    d = np.linalg.norm(w, axis=1)
    cos = (w @ n) / d
    return math.pi * le * (radius / d) ** 2 * cos


def quad_over_plane(out_dir, width=64, height=64, base=4, rr=False, mis="balance", seed=4242, max_depth=2):
    """Two quad lights (1.0 x 0.6 at height 1.0, radiance 12; 0.4 x 0.4 at height 1.3,
    radiance 30) over a Lambert plane; the pinhole at height 0.5 looks down."""
    focal, nodal = 100.0, (0.05, 0.5, -0.03)
    rho, colour = 0.8, (0.9, 0.55, 0.3)
    os.makedirs(out_dir, exist_ok=True)
    _write_plane_obj(os.path.join(out_dir, "plane.obj"), 50.0)
    # Rotation z = -90 degrees turns the light's local x axis (its normal) to -y;
    # local (0, y, z) lands on (y, 0, z), so a light spans x +- sx/2, z +- sy/2.
    specs = [((0.1, 1.0, 0.0), 1.0, 0.6, 12.0), ((-0.6, 1.3, 0.5), 0.4, 0.4, 30.0)]
    lights, text = [], _shader(colour, rho) + _object("plane.obj", 0)
    for (c, sx, sy, le) in specs:
        text += _quad_light(c, (0.0, 0.0, -90.0), sx, sy, le)
        cx, cy, cz = c
        verts = [(cx - sx / 2, cy, cz - sy / 2), (cx + sx / 2, cy, cz - sy / 2), (cx + sx / 2, cy, cz + sy / 2),
                 (cx - sx / 2, cy, cz + sy / 2)]
        lights.append(("quad", np.array(verts), le))
    min_depth, threshold = (0, 2.0) if rr else (8, 0.01)
    head, ext = _setup(width, height, base, min_depth, max_depth, threshold,
                       (nodal[0], nodal[1] + focal, nodal[2]), (0.0, 0.0, -90.0), focal, mis=mis, seed=seed)
    path = _write(out_dir, head, text, ext)
    return PlaneScene(path, width, height, base * base, focal, nodal, rho, colour, lights)


def sphere_over_plane(out_dir, width=64, height=64, base=4, rr=False, mis="balance", seed=4343, max_depth=2):
    """Two sphere lights (radius 0.25 at height 1.0, radiance 10; radius 0.1 at
    height 0.8, radiance 40) over a Lambert plane; the pinhole at height 0.4 looks down."""
    focal, nodal = 100.0, (0.0, 0.4, 0.0)
    rho, colour = 0.7, (0.35, 0.8, 0.6)
    os.makedirs(out_dir, exist_ok=True)
    _write_plane_obj(os.path.join(out_dir, "plane.obj"), 50.0)
    specs = [((0.2, 1.0, -0.1), 0.25, 10.0), ((-0.5, 0.8, 0.3), 0.1, 40.0)]
    text = _shader(colour, rho) + _object("plane.obj", 0)
    lights = []
    for (c, r, le) in specs:
        text += _sphere_light(c, r, le)
        lights.append(("sphere", np.array(c, np.float64), r, le))
    min_depth, threshold = (0, 2.0) if rr else (8, 0.01)
    head, ext = _setup(width, height, base, min_depth, max_depth, threshold,
                       (nodal[0], nodal[1] + focal, nodal[2]), (0.0, 0.0, -90.0), focal, mis=mis, seed=seed)
    path = _write(out_dir, head, text, ext)
    return PlaneScene(path, width, height, base * base, focal, nodal, rho, colour, lights)


def icosphere(level):
    """Unit icosphere: (vertices (V,3), faces (F,3)) wound so that e1 x e2 points outward."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache, nf = {}, []

        def mid(i, j):
            k = (min(i, j), max(i, j))
            if k not in cache:
                m = verts[i] + verts[j]
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts)
    F = np.array(faces)
    e1, e2 = V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]
    out = (np.cross(e1, e2) * V[F].mean(axis=1)).sum(axis=1) > 0
    F[~out] = F[~out][:, [0, 2, 1]]
    return V, F


class FurnaceScene:
    def __init__(self, path, spp, rho, colour, le):
        self.path, self.spp, self.rho, self.colour, self.le = path, spp, rho, np.asarray(colour, np.float64), le

    def sphere_expected(self):
        return self.rho * self.colour * self.le


def furnace(out_dir, width=64, height=64, base=4, rr=False, mis="balance", max_depth=3, seed=4444):
    """A Lambert icosphere (radius 0.8, 1280 faces) in a cube of six inward-facing
    quad lights (side 4, radiance 2.5); the camera sits inside the cube."""
    os.makedirs(out_dir, exist_ok=True)
    rho, colour, le, half = 0.8, (0.9, 0.6, 0.3), 2.5, 2.0
    V, F = icosphere(3)
    V = V * 0.8
    with open(os.path.join(out_dir, "sphere.obj"), "w") as f:
        for p in V:
            f.write("v %r %r %r\n" % tuple(float(x) for x in p))
        for (a, b, c) in F:
            f.write("f %d %d %d\n" % (a + 1, b + 1, c + 1))
    text = _shader(colour, rho) + _object("sphere.obj", 0)
    # each light's local x axis is its normal; these rotations turn it inward
    walls = [((0, -half, 0), (0, 0, 90)), ((0, half, 0), (0, 0, -90)), ((-half, 0, 0), (0, 0, 0)),
             ((half, 0, 0), (0, 180, 0)), ((0, 0, -half), (0, -90, 0)), ((0, 0, half), (0, 90, 0))]
    for (t, r) in walls:
        text += _quad_light(t, r, 2 * half, 2 * half, le)
    focal = 60.0
    min_depth, threshold = (0, 2.0) if rr else (max_depth, 0.01)
    head, ext = _setup(width, height, base, min_depth, max_depth, threshold, (0.0, 0.0, 1.8 + focal),
                       (0.0, 90.0, 0.0), focal, mis=mis, seed=seed)
    path = _write(out_dir, head, text, ext)
    return FurnaceScene(path, base * base, rho, colour, le)


def check_unbiased(rad, expected, z=5.0, what=""):
    """Per channel: |mean(rad - expected)| <= z * standard error (+ a float32
    floor of 2e-5 relative).  Returns the relative error and relative standard
    error of the mean, so that callers can also require a discriminating test."""
    rad = np.asarray(rad, np.float64)
    expected = np.asarray(expected, np.float64)
    r = rad - expected
    n = r.shape[0]
    mean = r.mean(axis=0)
    se = r.std(axis=0, ddof=1) / math.sqrt(n)
    scale = np.abs(expected.mean(axis=0))
    ok = np.abs(mean) <= z * se + 2e-5 * scale
    assert ok.all(), "%s: mean residual %s exceeds %g standard errors %s (expected mean %s)" % (
        what, mean, z, se, expected.mean(axis=0))
    return mean / scale, se / scale


def _phong_shader(colour, refl, exponent):
    return ("shader:\n  type: Phong\n  texture:\n    type: Constant\n    colour: [%r, %r, %r]\n"
            "  reflectance: %r\n  exponent: %r\n" % (*map(float, colour), float(refl), float(exponent)))


class PhongPlaneScene(PlaneScene):
    """A glossy plane under one quad light.  The modified Phong lobe has no
    closed-form irradiance integral, so the expected radiance of a sample is
    the direct-lighting integral over the light's area evaluated by a
    Gauss-Legendre product rule (its error is far below the Monte Carlo noise
    the check allows):
        L(p, wo) = Le * int_A f(wi, wo) cos(theta_i) cos(theta_l) / d^2 dA,
        f = rho c (n + 2) / (2 pi) * max(0, r . wi)^n,  r = 2 (N . wo) N - wo."""

    def __init__(self, *a, exponent=20.0, nodes=16, **k):
        super().__init__(*a, **k)
        self.exponent = exponent
        self.gl = np.polynomial.legendre.leggauss(nodes)

    def expected(self, xy):
        p = self.hit_points(xy)
        wo = self.nodal[None, :] - p
        wo /= np.linalg.norm(wo, axis=1, keepdims=True)
        n = np.array([0.0, 1.0, 0.0])
        r = 2.0 * (wo @ n)[:, None] * n[None, :] - wo
        _, verts, le = self.lights[0]
        lo, hi = verts.min(axis=0), verts.max(axis=0)
        x, w = self.gl
        cx, hx = 0.5 * (lo[0] + hi[0]), 0.5 * (hi[0] - lo[0])
        cz, hz = 0.5 * (lo[2] + hi[2]), 0.5 * (hi[2] - lo[2])
        gx, gz = np.meshgrid(cx + hx * x, cz + hz * x, indexing="ij")
        gw = (np.outer(w, w) * hx * hz).ravel()
        pts = np.stack([gx.ravel(), np.full(gx.size, lo[1]), gz.ravel()], axis=1)
        out = np.empty(p.shape[0])
        for s0 in range(0, p.shape[0], 2048):
            wv = pts[None, :, :] - p[s0:s0 + 2048, None, :]
            d2 = (wv * wv).sum(axis=2)
            wi = wv / np.sqrt(d2)[:, :, None]
            cos_i = wi[:, :, 1]  # receiver normal +y; the light faces -y, so cos_l = cos_i
            lobe = np.maximum(0.0, (wi * r[s0:s0 + 2048, None, :]).sum(axis=2)) ** self.exponent
            out[s0:s0 + 2048] = ((lobe * cos_i * cos_i / d2) * gw[None, :]).sum(axis=1)
        f = self.rho * (self.exponent + 2.0) / (2.0 * math.pi) * le
        return f * out[:, None] * self.colour[None, :]


def phong_over_plane(out_dir, width=64, height=64, base=4, rr=False, mis="balance", seed=4545, exponent=20.0):
    """One quad light (1.0 x 0.6 at height 1.0, radiance 12) over a modified-Phong
    plane (exponent 20); the pinhole at height 0.5 looks down."""
    focal, nodal = 100.0, (0.05, 0.5, -0.03)
    rho, colour = 0.8, (0.9, 0.55, 0.3)
    os.makedirs(out_dir, exist_ok=True)
    _write_plane_obj(os.path.join(out_dir, "plane.obj"), 50.0)
    c, sx, sy, le = (0.1, 1.0, 0.0), 1.0, 0.6, 12.0
    text = _phong_shader(colour, rho, exponent) + _object("plane.obj", 0) + _quad_light(c, (0.0, 0.0, -90.0), sx, sy, le)
    verts = np.array([(c[0] - sx / 2, c[1], c[2] - sy / 2), (c[0] + sx / 2, c[1], c[2] - sy / 2),
                      (c[0] + sx / 2, c[1], c[2] + sy / 2), (c[0] - sx / 2, c[1], c[2] + sy / 2)])
    min_depth, threshold = (0, 2.0) if rr else (8, 0.01)
    head, ext = _setup(width, height, base, min_depth, 2, threshold,
                       (nodal[0], nodal[1] + focal, nodal[2]), (0.0, 0.0, -90.0), focal, mis=mis, seed=seed)
    path = _write(out_dir, head, text, ext)
    return PhongPlaneScene(path, width, height, base * base, focal, nodal, rho, colour, [("quad", verts, le)],
                           exponent=exponent)
