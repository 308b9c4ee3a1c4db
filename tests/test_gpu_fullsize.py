"""GPU against the FP32 oracle at the full sizes of the two plain workloads.

* The Cornell-style box as the benchmark generates it: 256 x 256 pixels,
  16 spp, max depth 4, 1,316 triangles, batches of 2^16 rays (`bin exponent:
  16`), every one of its 1,048,576 samples compared.
* The large terrain scene as the benchmark generates it: 1024 x 1024 pixels,
  64 spp, 3,633,168 triangles, 8 lights, Phong and Lambert, power heuristic,
  Russian roulette; one GPU pass, and the oracle renders three ranges of 2^18
  paths (the first image columns, the middle columns that the CPU baseline
  times, the last columns) that are compared per sample.

Tolerances (the same per-path random sequence on both sides): film positions
bit-exact; >= 99.5 % (box) / 99 % (terrain) of samples bit-equal, the rest
meeting closest-hit near-ties; per-sample radiance within 1e-4 relative on the
same fractions; closest-hit and occlusion query counts equal (box) or within
0.1 % (occlusion: a near-tie can end a path one bounce earlier or later)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20261203  # the benchmark's seed; config k uses SEED + k


def _per_sample(rgb, wrgb, frac):
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() >= frac, same.mean()
    rel = np.abs(rgb - wrgb) / np.maximum(np.abs(wrgb), 1e-3)
    assert (rel <= 1e-4).all(axis=1).mean() >= frac
    return same.mean()


def test_full_size_box_scene_matches_oracle_per_sample(built, scene_dir):
    mscgpu, oracle = built
    y = mscgpu.generate_scene(0, SEED, str(scene_dir / "box_full"))
    assert "bin exponent: 16" in open(y).read()
    with mscgpu.Pathtracer(y) as pt:
        assert pt.process() == 1
        img = pt.image()
        rgb, xy = pt.samples()
        st = pt.stats()
    assert (st["width"], st["height"], st["spp"]) == (256, 256, 16)
    s = oracle.Scene(y)
    assert st["triangles"] == s.triangles == 1316
    ref, wrgb, wxy, counts = s.render(0)
    assert np.array_equal(xy.view(np.uint32), wxy.view(np.uint32))
    _per_sample(rgb, wrgb, 0.995)
    assert st["closest_queries"] == int(counts[0])
    assert abs(st["shadow_queries"] - int(counts[1])) <= 1e-3 * int(counts[1])
    r = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert (r <= 1e-4).all(axis=-1).mean() >= 0.99


def test_full_size_terrain_scene_sampled_ranges_match_oracle(built, scene_dir):
    mscgpu, oracle = built
    y = mscgpu.generate_scene(1, SEED + 1, str(scene_dir / "terrain_full"))
    with mscgpu.Pathtracer(y) as pt:
        assert pt.process() == 1
        rgb, xy = pt.samples()
        st = pt.stats()
    assert (st["width"], st["height"], st["spp"]) == (1024, 1024, 64)
    s = oracle.Scene(y)
    assert st["triangles"] == s.triangles == 3633168
    P = s.paths
    n = 1 << 18
    for first in (0, (s.width // 2) * s.height * s.spp, P - n):
        wrgb, wxy, _ = s.render_range_rgb(first, n, 0)
        assert np.array_equal(xy[first:first + n].view(np.uint32), wxy.view(np.uint32))
        _per_sample(rgb[first:first + n], wrgb, 0.99)
