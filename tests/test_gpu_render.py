"""End-to-end renders on the GPU against the CPU oracle.

Levels (tolerances stated in each test):
  close     - the same per-path random sequence on both sides: per-sample FP32
              radiance agrees to the bit except for paths that meet a closest-hit
              near-tie; per-pixel radiance within 1e-4 relative for >= 99% of pixels.
  converged - the GPU image against the FP64 oracle: relative MSE stated.
plus the reference engine's API semantics (iteration count, clear, terminate)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(img, ref, rel=1e-4, frac=0.99):
    r = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    ok = (r <= rel).all(axis=-1).mean()
    assert ok >= frac, "only %.4f of pixels within %g relative" % (ok, rel)
    return ok


def test_box_scene_close_to_fp32_oracle(built, box_scene):
    mscgpu, oracle = built
    s = oracle.Scene(box_scene)
    with mscgpu.Pathtracer(box_scene) as pt:
        assert pt.process() == 1
        img = pt.image()
        rgb, xy = pt.samples()
        st = pt.stats()
    ref, wrgb, wxy, counts = s.render(0)
    assert np.array_equal(xy.view(np.uint32), wxy.view(np.uint32))  # film positions are bit-exact
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() > 0.995, same.mean()
    assert st["closest_queries"] == int(counts[0])
    assert abs(st["shadow_queries"] - int(counts[1])) <= 1e-3 * int(counts[1])
    _close(img, ref)
    assert img.mean() > 0.01


def test_tiny_scene_iterations_accumulate_like_the_oracle(built, tiny_scene):
    mscgpu, oracle = built
    s = oracle.Scene(tiny_scene)
    ref = None
    with mscgpu.Pathtracer(tiny_scene) as pt:
        for it in range(3):
            assert pt.process() == it + 1
            ref, _, _, _ = s.render(it, pixels=ref)
        _close(pt.image(), ref)
        pt.clear()
        assert np.all(pt.image() == 0)
        assert pt.process() == 1


def test_power_heuristic_and_box_filter_match_oracle(built, tmp_path, tiny_scene):
    mscgpu, oracle = built
    text = open(tiny_scene).read()
    text = text.replace("mis: balance", "mis: power").replace("type: Tent", "type: Box")
    text = text.replace("type: Stratified", "type: Independent")
    y = tmp_path / "scene.yaml"
    y.write_text(text)
    import os
    import shutil
    for f in os.listdir(os.path.dirname(tiny_scene)):
        if f.endswith(".obj"):
            shutil.copy(os.path.join(os.path.dirname(tiny_scene), f), tmp_path / f)
    with mscgpu.Pathtracer(str(y)) as pt:
        pt.process()
        img = pt.image()
    ref, _, _, _ = oracle.Scene(str(y)).render(0)
    _close(img, ref)


def test_thin_lens_grid_and_nonsquare_spp_match_oracle(built, tmp_path, tiny_scene):
    mscgpu, oracle = built
    import os
    import shutil
    d = os.path.dirname(tiny_scene)
    for f in os.listdir(d):
        if f.endswith(".obj"):
            shutil.copy(os.path.join(d, f), tmp_path / f)
    text = open(tiny_scene).read()
    cam_start = text.index("camera:")
    cam_end = text.index("filter:")
    text = text[:cam_start] + ("camera:\n  type: ThinLens\n  translation: [0, 1, 30]\n  rotation: [0, 90, 0]\n"
                               "  focal length: 24\n  focal distance: 31\n  aperture: 8\n") + text[cam_end:]
    text = text.replace("type: Stratified", "type: Grid").replace("mis: balance", "samples per pixel: 6")
    y = tmp_path / "scene.yaml"
    y.write_text(text)
    with mscgpu.Pathtracer(str(y)) as pt:
        pt.process()
        img = pt.image()
        assert pt.stats()["spp"] == 6
    ref, _, _, _ = oracle.Scene(str(y)).render(0)
    _close(img, ref)


def test_terrain_with_phong_matches_oracle(built, scene_dir):
    """Scaled-down terrain scene: Phong lobes, 8 lights, power heuristic, Russian roulette."""
    mscgpu, oracle = built
    y = mscgpu.generate_scene(1, 77, str(scene_dir / "terrain_small"), scale=0.05)
    with mscgpu.Pathtracer(y) as pt:
        pt.process()
        img = pt.image()
        rgb, _ = pt.samples()
    ref, wrgb, _, _ = oracle.Scene(y).render(0)
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() > 0.99, same.mean()
    _close(img, ref, frac=0.98)


def test_converged_against_fp64_oracle(built, tiny_scene):
    """Relative MSE of the GPU image against the FP64 oracle, same samples: < 1e-8."""
    mscgpu, oracle = built
    with mscgpu.Pathtracer(tiny_scene) as pt:
        pt.process()
        img = pt.image().astype(np.float64)
    ref64, _, _, _ = oracle.Scene(tiny_scene).render(0, double=True)
    rel_mse = float(np.mean((img - ref64) ** 2) / np.mean(ref64 ** 2))
    assert rel_mse < 1e-8, rel_mse


def test_terminate_stops_process_and_returns_zero(built, box_scene):
    mscgpu, _ = built
    with mscgpu.Pathtracer(box_scene) as pt:
        assert pt.active()
        pt.process()
        before = pt.image()
        pt.terminate()
        assert not pt.active()
        assert pt.process() == 0          # Pathtracer.cpp:486-487
        assert np.array_equal(pt.image(), before)


def test_terminate_from_another_thread(built, box_scene):
    mscgpu, _ = built
    with mscgpu.Pathtracer(box_scene) as pt:
        t = threading.Timer(0.001, pt.terminate)
        t.start()
        results = [pt.process() for _ in range(50)]
        t.join()
        assert results[-1] == 0 and not pt.active()


def test_device_process_then_image(built, tiny_scene):
    mscgpu, oracle = built
    with mscgpu.Pathtracer(tiny_scene) as pt:
        assert pt.process_device() == 1
        img = pt.image()
    ref, _, _, _ = oracle.Scene(tiny_scene).render(0)
    _close(img, ref)


def _with_extensions(yaml_path, out_path, **ext):
    """A copy of the scene next to its OBJ files with extension keys replaced or added."""
    import re
    text = open(yaml_path).read()
    head, tail = text.rsplit("extensions:", 1)
    lines = [ln for ln in tail.splitlines() if ln.strip()]
    keys = {ln.split(":", 1)[0].strip(): ln for ln in lines}
    for k, v in ext.items():
        keys[k.replace("_", " ")] = "  %s: %s" % (k.replace("_", " "), v)
    open(out_path, "w").write(head + "extensions:\n" + "\n".join(keys.values()) + "\n")
    return out_path


@pytest.fixture(scope="module")
def stress_scene(built, scene_dir):
    mscgpu, _ = built
    return mscgpu.generate_scene(2, 4242, str(scene_dir / "stress_small"), scale=0.03)


def test_stress_scene_sphere_lights_and_face_texels_match_oracle(built, stress_scene):
    """Sphere lights (hits, cone NEE, MIS), per-face FP16 texels, 4096 shaders, 64-bit hit key."""
    mscgpu, oracle = built
    with mscgpu.Pathtracer(stress_scene) as pt:
        pt.process()
        img = pt.image()
        rgb, _ = pt.samples()
    s = oracle.Scene(stress_scene)
    assert s.lights >= 2
    ref, wrgb, _, _ = s.render(0)
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() > 0.99, same.mean()
    assert float(ref.max()) > 0.0
    _close(img, ref, frac=0.98)


def test_hit_key_width_and_sorting_do_not_change_the_image(built, stress_scene, tmp_path):
    mscgpu, _ = built
    d = stress_scene.rsplit("/", 1)[0]
    images = []
    for name, ext in (("k64", dict(hit_key_bits=64)), ("k32", dict(hit_key_bits=32)), ("off", dict(hit_sort=0))):
        y = _with_extensions(stress_scene, "%s/%s.yaml" % (d, name), autotune=0, **ext)
        with mscgpu.Pathtracer(y) as pt:
            pt.process()
            images.append(pt.image())
    for im in images[1:]:
        assert np.array_equal(im.view(np.uint32), images[0].view(np.uint32))


def test_ray_and_hit_sorts_do_not_change_the_image(built, box_scene):
    """Sorted or not, a batch is traced and shaded in place in the bin pool;
    the order of rays within a batch must not change any path's result."""
    mscgpu, _ = built
    imgs = []
    for rs, hs, e in ((False, False, 12), (True, False, 12), (False, True, 10), (True, True, 14)):
        with mscgpu.Pathtracer(box_scene) as pt:
            pt.set_tuning(batch_exponent=e, ray_sort=rs, hit_sort=hs)
            pt.process()
            imgs.append(pt.image())
    for im in imgs[1:]:
        assert np.array_equal(im.view(np.uint32), imgs[0].view(np.uint32))


@pytest.mark.parametrize("nbins", [26, 98])
def test_direction_bin_count_does_not_change_the_image(built, box_scene, nbins):
    mscgpu, _ = built
    imgs = []
    for nb in (6, nbins):
        with mscgpu.Pathtracer(box_scene) as pt:
            pt.set_tuning(batch_exponent=12, trace_block=128, ray_sort=True, hit_sort=True, bins=nb)
            assert pt.tuning()["bins"] == nb
            pt.process()
            imgs.append(pt.image())
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))


def test_image_textures_match_oracle(built, tmp_path):
    """Standard and (nested) Layered textures from PFM / PPM images."""
    from texture_scene import make_texture_scene
    mscgpu, oracle = built
    y = make_texture_scene(mscgpu, str(tmp_path))
    with mscgpu.Pathtracer(y) as pt:
        pt.process()
        img = pt.image()
        rgb, _ = pt.samples()
    ref, wrgb, _, _ = oracle.Scene(y).render(0)
    same = (rgb.view(np.uint32) == wrgb.view(np.uint32)).all(axis=1)
    assert same.mean() > 0.99, same.mean()
    _close(img, ref)


@pytest.mark.parametrize("which", ["box", "terrain"])
def test_persistent_traversal_gives_the_same_image(built, box_scene, scene_dir, which):
    """Per-lane ray refill changes only the scheduling: every ray's steps and hit are the same."""
    mscgpu, _ = built
    y = box_scene if which == "box" else mscgpu.generate_scene(1, 77, str(scene_dir / "terrain_small"), scale=0.05)
    imgs = []
    for pers in (False, True):
        with mscgpu.Pathtracer(y) as pt:
            e = pt.tuning()["batch_exponent"]
            pt.set_tuning(batch_exponent=e, trace_block=128, ray_sort=True, hit_sort=False, bins=6, persistent=pers)
            assert pt.tuning()["persistent"] == int(pers)
            pt.process()
            imgs.append(pt.image())
            st = pt.stats()
            assert st["closest_queries"] > 0
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))


def test_ray_key_width_does_not_change_the_image(built, box_scene):
    """8-, 16-, 24- and 32-bit ray sort keys order the batches differently;
    every path's result, and so the image, stays the same."""
    mscgpu, _ = built
    imgs = []
    for kb in (8, 16, 24, 32):
        with mscgpu.Pathtracer(box_scene) as pt:
            pt.set_tuning(batch_exponent=12, ray_sort=True, hit_sort=False, ray_key_bits=kb)
            assert pt.tuning()["ray_key_bits"] == kb
            pt.process()
            imgs.append(pt.image())
    for im in imgs[1:]:
        assert np.array_equal(im.view(np.uint32), imgs[0].view(np.uint32))
