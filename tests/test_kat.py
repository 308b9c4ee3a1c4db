"""Analytic known-answer tests of the CPU oracle (no GPU).

The oracle's FP32 and FP64 integrators are checked against closed-form
radiance (tests/kat_scenes.py): direct lighting of a Lambert plane by quad and
sphere lights, and a Lambert sphere inside a cube of emitters (a furnace).
Each estimator is unbiased, so the mean per-sample residual must stay within
5 standard errors; the relative standard error is held below 0.5 % so that a
missing cosine, pdf or MIS term (errors of 10 % and more) cannot pass.  A
negative control shows that the check rejects a biased estimator: paths cut
at depth 0 lose the BSDF-sampled half of the MIS pair."""
import math

import numpy as np
import pytest

import kat_scenes as K  # noqa: E402


@pytest.mark.parametrize("light", ["quad", "sphere"])
@pytest.mark.parametrize("rr", [False, True])
@pytest.mark.parametrize("mis", ["balance", "power"])
def test_oracle_direct_lighting_matches_closed_form(built, tmp_path, light, rr, mis):
    _, oracle = built
    make = K.quad_over_plane if light == "quad" else K.sphere_over_plane
    sc = make(str(tmp_path), width=128, height=128, rr=rr, mis=mis)
    s = oracle.Scene(sc.path)
    for double in (False, True):
        _, rgb, xy, _ = s.render(0, double=double)
        rel, se = K.check_unbiased(rgb, sc.expected(xy), what="%s %s rr=%s fp64=%s" % (light, mis, rr, double))
        assert (se < 5e-3).all(), se


@pytest.mark.parametrize("rr", [False, True])
def test_oracle_phong_direct_lighting_matches_quadrature(built, tmp_path, rr):
    """The modified Phong lobe (an extension of the reference's shaders) against
    the direct-lighting integral by Gauss-Legendre quadrature."""
    _, oracle = built
    sc = K.phong_over_plane(str(tmp_path), width=64, height=64, rr=rr)
    s = oracle.Scene(sc.path)
    for double in (False, True):
        _, rgb, xy, _ = s.render(0, double=double)
        rel, se = K.check_unbiased(rgb, sc.expected(xy), what="phong rr=%s fp64=%s" % (rr, double))
        assert (se < 6e-3).all(), se


@pytest.mark.parametrize("rr", [False, True])
def test_oracle_furnace_matches_closed_form(built, tmp_path, rr):
    _, oracle = built
    sc = K.furnace(str(tmp_path), width=128, height=128, rr=rr)
    s = oracle.Scene(sc.path)
    for double in (False, True):
        _, rgb, _, _ = s.render(0, double=double)
        wall = (rgb == sc.le).all(axis=1)  # camera rays that see a wall return Le exactly
        assert 0.3 < wall.mean() < 0.7
        sphere = rgb[~wall]
        K.check_unbiased(sphere, np.broadcast_to(sc.sphere_expected(), sphere.shape),
                         what="furnace rr=%s fp64=%s" % (rr, double))


def test_closed_form_check_rejects_a_biased_estimator(built, tmp_path):
    """Paths cut at depth 0 keep only the light-sampled half of the MIS pair
    (Integrator.cpp:184-185 stops them before BSDF sampling): about 20 % low."""
    _, oracle = built
    sc = K.quad_over_plane(str(tmp_path), width=128, height=128, max_depth=0)
    _, rgb, xy, _ = oracle.Scene(sc.path).render(0)
    exp = sc.expected(xy)
    with pytest.raises(AssertionError):
        K.check_unbiased(rgb, exp, what="depth 0")
    assert (rgb.mean(axis=0) / exp.mean(axis=0) < 0.9).all()


def test_closed_forms_agree_with_monte_carlo():
    """The two irradiance formulas against plain Monte Carlo integration."""
    rng = np.random.default_rng(5)
    p = np.array([[0.05, 0.0, -0.03], [0.3, 0.0, 0.2]])
    n = np.array([0.0, 1.0, 0.0])
    verts = np.array([(-0.4, 1.0, -0.3), (0.6, 1.0, -0.3), (0.6, 1.0, 0.3), (-0.4, 1.0, 0.3)])
    e = K.polygon_irradiance(p, n, verts, 12.0)
    N = 400000
    u = rng.uniform(size=(N, 2))
    q = np.stack([-0.4 + u[:, 0], np.ones(N), -0.3 + 0.6 * u[:, 1]], axis=1)
    for i in range(2):
        w = q - p[i]
        d2 = (w * w).sum(axis=1)
        mc = 12.0 * 0.6 * (w[:, 1] ** 2 / d2 ** 2).mean()  # Le * area * cos cos / d^2
        assert abs(mc - e[i]) < 2e-3 * e[i]
    c, r = np.array([0.2, 1.0, -0.1]), 0.25
    es = K.sphere_irradiance(p, n, c, r, 10.0)
    for i in range(2):
        w = c - p[i]
        d = np.linalg.norm(w)
        ctm = math.sqrt(1 - (r / d) ** 2)
        ct = 1 - u[:, 0] * (1 - ctm)
        phi = 2 * math.pi * u[:, 1]
        st = np.sqrt(1 - ct * ct)
        a = w / d
        b1 = np.cross([1.0, 0.0, 0.0], a)
        b1 /= np.linalg.norm(b1)
        b2 = np.cross(a, b1)
        dirs = b1 * (np.cos(phi) * st)[:, None] + b2 * (np.sin(phi) * st)[:, None] + a * ct[:, None]
        mc = 10.0 * np.maximum(dirs[:, 1], 0).mean() * 2 * math.pi * (1 - ctm)
        assert abs(mc - es[i]) < 2e-3 * es[i]
