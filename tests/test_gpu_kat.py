"""Analytic known-answer tests of the CUDA renderer, through the C ABI.

The GPU's per-sample radiance (msc_get_samples) on the closed-form scenes of
tests/kat_scenes.py: direct lighting of a Lambert plane by quad and sphere
lights, and a Lambert sphere inside a cube of emitters.  The mean residual must
stay within 5 standard errors of Monte Carlo noise; with 4 M samples the
relative standard error is below 0.1 %.  The same scenes are then rendered by
the FP32 oracle at a small size and compared per sample (the same per-path
random sequence on both sides)."""
import numpy as np
import pytest

import kat_scenes as K  # noqa: E402

pytestmark = pytest.mark.gpu


def _render(mscgpu, path):
    with mscgpu.Pathtracer(path) as pt:
        assert pt.process() == 1
        rgb, xy = pt.samples()
    return rgb, xy


@pytest.mark.parametrize("light", ["quad", "sphere"])
@pytest.mark.parametrize("rr", [False, True])
@pytest.mark.parametrize("mis", ["balance", "power"])
def test_direct_lighting_matches_closed_form(built, tmp_path, light, rr, mis):
    mscgpu, _ = built
    make = K.quad_over_plane if light == "quad" else K.sphere_over_plane
    sc = make(str(tmp_path), width=256, height=256, base=8, rr=rr, mis=mis)
    rgb, xy = _render(mscgpu, sc.path)
    rel, se = K.check_unbiased(rgb, sc.expected(xy), what="GPU %s %s rr=%s" % (light, mis, rr))
    assert (se < 1e-3).all(), se


@pytest.mark.parametrize("rr,mis", [(False, "balance"), (True, "balance"), (False, "power")])
def test_phong_direct_lighting_matches_quadrature(built, tmp_path, rr, mis):
    mscgpu, _ = built
    sc = K.phong_over_plane(str(tmp_path), width=128, height=128, base=4, rr=rr, mis=mis)
    rgb, xy = _render(mscgpu, sc.path)
    rel, se = K.check_unbiased(rgb, sc.expected(xy), what="GPU phong %s rr=%s" % (mis, rr))
    assert (se < 4e-3).all(), se


@pytest.mark.parametrize("rr", [False, True])
def test_furnace_matches_closed_form(built, tmp_path, rr):
    mscgpu, _ = built
    sc = K.furnace(str(tmp_path), width=256, height=256, base=8, rr=rr)
    rgb, _ = _render(mscgpu, sc.path)
    wall = (rgb == sc.le).all(axis=1)
    assert 0.3 < wall.mean() < 0.7
    sphere = rgb[~wall]
    K.check_unbiased(sphere, np.broadcast_to(sc.sphere_expected(), sphere.shape), what="GPU furnace rr=%s" % rr)


@pytest.mark.parametrize("which", ["quad", "sphere", "phong", "furnace"])
def test_known_answer_scenes_match_the_oracle_per_sample(built, tmp_path, which):
    mscgpu, oracle = built
    make = {"quad": K.quad_over_plane, "sphere": K.sphere_over_plane, "phong": K.phong_over_plane,
            "furnace": K.furnace}[which]
    sc = make(str(tmp_path), width=64, height=64, rr=True)
    rgb, xy = _render(mscgpu, sc.path)
    _, wrgb, wxy, _ = oracle.Scene(sc.path).render(0)
    assert np.array_equal(xy.view(np.uint32), wxy.view(np.uint32))
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() > 0.995, same.mean()
    rel = np.abs(rgb - wrgb) / np.maximum(np.abs(wrgb), 1e-3)
    assert (rel <= 1e-4).all(axis=1).mean() > 0.995
