"""Batched and served forms on the GPU.

Every job's image must be the same alone and in the mix (bit for bit: each
path draws the same per-path random sequence and adds to its own samples in
the same order whatever batch it rides in), the batched single-job case must
equal the plain engine, and a job with its own camera and resolution must
match the CPU oracle rendering that job (per-pixel 1e-4 relative on >= 99%)."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(img, ref, rel=1e-4, frac=0.99):
    r = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    ok = (r <= rel).all(axis=-1).mean()
    assert ok >= frac, "only %.4f of pixels within %g relative" % (ok, rel)


@pytest.fixture(scope="module")
def scenes(built, scene_dir):
    mscgpu, _ = built
    return [mscgpu.generate_scene(100, 1234, str(scene_dir / "tiny")),
            mscgpu.generate_scene(0, 20261203, str(scene_dir / "box64"), scale=0.25),
            mscgpu.generate_scene(1, 77, str(scene_dir / "terrain_small"), scale=0.05)]


JOBS = [dict(scene=0), dict(scene=1, spp=3), dict(scene=2, max_depth=3),
        dict(scene=1, width=40, height=24, camera=((0.0, 1.0, 60.0), (0.0, 90.0, -2.0), 55.0)),
        dict(scene=0, width=17, height=9, spp=5, seed=99), dict(scene=2, width=32, height=32, spp=2)]


def _batch(mscgpu, scenes, jobs, exp=14):
    b = mscgpu.Batch(batch_exponent=exp, film_samples=1 << 22)
    for s in scenes:
        b.add_scene(s)
    ids = [b.submit(**j) for j in jobs]
    b.run()
    return b, ids


def test_single_job_batch_equals_plain(built, scenes):
    mscgpu, _ = built
    with mscgpu.Pathtracer(scenes[1]) as pt:
        pt.process()
        plain = pt.image()
    b, ids = _batch(mscgpu, [scenes[1]], [dict(scene=0)], exp=16)
    assert np.array_equal(b.image(ids[0]).view(np.uint32), plain.view(np.uint32))
    b.close()


def test_each_job_is_the_same_alone_and_in_the_mix(built, scenes):
    mscgpu, _ = built
    mixed, ids = _batch(mscgpu, scenes, JOBS)
    st = mixed.stats()
    assert st["closest_queries"] > 0 and st["batches"] > 0
    for k, job in enumerate(JOBS):
        alone, aid = _batch(mscgpu, scenes, [job])
        a = alone.image(aid[0])
        m = mixed.image(ids[k])
        assert a.shape == m.shape
        assert np.array_equal(a.view(np.uint32), m.view(np.uint32)), "job %d differs in the mix" % k
        alone.close()
    mixed.close()


def _with_camera(yaml_path, out_dir, width, height, camera):
    """The same scene with its image size and camera block replaced (a PinHole camera)."""
    import os
    import shutil
    t, r, f = camera
    src = os.path.dirname(yaml_path)
    shutil.copytree(src, out_dir, dirs_exist_ok=True)
    text = open(yaml_path).read()
    head, rest = text.split("---", 1)
    head = re.sub(r"width: \d+", "width: %d" % width, head)
    head = re.sub(r"height: \d+", "height: %d" % height, head)
    cam = ("camera:\n  type: PinHole\n  translation: [%r, %r, %r]\n  rotation: [%r, %r, %r]\n"
           "  focal length: %r\n" % (*t, *r, f))
    head = re.sub(r"camera:\n(  .*\n)+", cam, head)
    out = os.path.join(out_dir, "scene.yaml")
    open(out, "w").write(head + "---" + rest)
    return out


def test_job_camera_equals_the_same_camera_in_the_scene(built, scenes, tmp_path):
    mscgpu, _ = built
    job = JOBS[3]
    b, ids = _batch(mscgpu, scenes, [job])
    img = b.image(ids[0])
    b.close()
    y = _with_camera(scenes[1], str(tmp_path / "cam"), job["width"], job["height"], job["camera"])
    with mscgpu.Pathtracer(y) as pt:
        pt.process()
        plain = pt.image()
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))


def test_job_with_its_own_camera_matches_oracle(built, scenes):
    mscgpu, oracle = built
    # an oblique camera: no pixel ray runs exactly along a wall or through a shared edge
    job = dict(scene=1, width=40, height=24, camera=((0.37, 1.21, 59.3), (3.7, 87.3, -2.2), 55.0))
    b, ids = _batch(mscgpu, scenes, [job])
    img = b.image(ids[0])
    s = oracle.Scene(scenes[1])
    t, r, f = job["camera"]
    s.set_job(width=job["width"], height=job["height"], cam_t=t, cam_r=r, focal=f, seed=20261203)
    ref, _, _, _ = s.render(0)
    assert img.shape == ref.shape
    _close(img, ref)
    b.close()


def test_served_requests_complete_and_match_alone(built, scenes):
    mscgpu, _ = built
    rng = np.random.default_rng(4)
    t = np.cumsum(rng.exponential(0.01, size=12))
    reqs = [(float(t[i]), JOBS[i % len(JOBS)]) for i in range(12)]
    # a film pool for only a few jobs at a time: later requests wait for memory
    b = mscgpu.Batch(batch_exponent=14, film_samples=300000)
    for s in scenes:
        b.add_scene(s)
    results, st = b.serve(reqs)
    assert st["completed"] == 12
    assert all(r["status"] == 0 for r in results)
    assert all(r["latency_s"] > 0 and r["done_s"] >= r["admit_s"] for r in results)
    assert 0 < st["p50_s"] <= st["p99_s"] <= st["p999_s"]
    assert st["peak_film_samples"] <= 300000
    for i, r in enumerate(results[:6]):
        alone, aid = _batch(mscgpu, scenes, [JOBS[i % len(JOBS)]])
        assert np.array_equal(b.image(r["job_id"]).view(np.uint32), alone.image(aid[0]).view(np.uint32))
        alone.close()
    b.close()


def test_serve_refuses_a_job_larger_than_the_film_pool(built, scenes):
    mscgpu, _ = built
    b = mscgpu.Batch(batch_exponent=12, film_samples=4000)  # the tiny scene's own job needs 4096
    b.add_scene(scenes[0])
    results, st = b.serve([(0.0, dict(scene=0)), (0.0, dict(scene=0, width=8, height=8, spp=1))])
    assert results[0]["status"] < 0 and results[1]["status"] == 0
    assert st["completed"] == 1
    b.close()


def test_scene_info_is_the_triangle_box(built, scenes):
    mscgpu, _ = built
    b = mscgpu.Batch(batch_exponent=12, film_samples=1 << 12)
    for k, y in enumerate(scenes):
        assert b.add_scene(y) == k
        lo, hi, n = b.scene_info(k)
        info, tv, _ = mscgpu.scene_load_host(y)
        p = tv.reshape(-1, 3)
        assert n == info["triangles"]
        assert np.array_equal(lo, p.min(0)) and np.array_equal(hi, p.max(0))
    with pytest.raises(mscgpu.MscError):
        b.scene_info(len(scenes))
    b.close()


def test_results_do_not_depend_on_the_tuning_choice(built, scenes):
    """Every tuning gives the same images bit for bit: batch sizes below 2^13
    partition the continuing rays through staging, larger ones append them
    straight into their bins from the shading kernel."""
    mscgpu, _ = built
    ref, rids = _batch(mscgpu, scenes, JOBS)
    want = [ref.image(i) for i in rids]
    ref.close()
    for cfg in (dict(batch_exponent=10, trace_block=64, ray_sort=False, hit_sort=True),
                dict(batch_exponent=12, trace_block=256, ray_sort=True, hit_sort=False),
                dict(batch_exponent=14, trace_block=128, ray_sort=False, hit_sort=False),
                dict(batch_exponent=13, trace_block=128, ray_sort=True, hit_sort=False, persistent=True, bins=26),
                dict(batch_exponent=12, trace_block=64, ray_sort=True, hit_sort=True, bins=98, digit_bits=11),
                dict(batch_exponent=14, trace_block=256, ray_sort=True, hit_sort=True, digit_bits=4),
                # direct binning (batches of 2^13 rays and more) into 98 bins, and with 24-bit ray keys
                dict(batch_exponent=13, trace_block=64, ray_sort=True, hit_sort=False, bins=98),
                dict(batch_exponent=14, trace_block=128, ray_sort=True, hit_sort=False, bins=26, ray_key_bits=24)):
        b = mscgpu.Batch(batch_exponent=14, film_samples=1 << 22)
        for s in scenes:
            b.add_scene(s)
        b.set_tuning(**cfg)
        t = b.tuning()
        assert (t["batch_exponent"], t["trace_block"]) == (cfg["batch_exponent"], cfg["trace_block"])
        ids = [b.submit(**j) for j in JOBS]
        b.run()
        for k, i in enumerate(ids):
            assert np.array_equal(b.image(i).view(np.uint32), want[k].view(np.uint32)), (cfg, k)
        b.close()


def test_autotuner_books_samples_and_keeps_results(built, scenes):
    mscgpu, _ = built
    ref, rids = _batch(mscgpu, scenes, JOBS)
    want = [ref.image(i) for i in rids]
    ref.close()
    b = mscgpu.Batch(batch_exponent=19, film_samples=1 << 22)
    for s in scenes:
        b.add_scene(s)
    b.autotune(windows=1)
    for _ in range(6):  # the tuner spends one run per candidate; keep feeding work
        ids = [b.submit(**j) for j in JOBS]
        b.run()
        for k, i in enumerate(ids):
            assert np.array_equal(b.image(i).view(np.uint32), want[k].view(np.uint32))
            b.release(i)
        if not b.tuning()["tuning"]:
            break
    log = b.tune_log()
    assert len(log) >= 2 and all(s["mrays_per_s"] >= 0 for s in log)
    t = b.tuning()
    assert t["trace_block"] in (64, 128, 256) and 6 <= t["batch_exponent"] <= 19
    with pytest.raises(mscgpu.MscError):
        b.set_tuning(batch_exponent=20)  # above the capacity given at create
    b.close()


def test_memory_budget_counts_scenes_and_job_images(built, scenes):
    """Admission by device memory: fixed buffers and resident scenes count, a job
    whose image would not fit waits (MSC_ERR_BUSY), a scene that would not fit
    is refused, and a released job's image returns its bytes."""
    mscgpu, _ = built
    b = mscgpu.Batch(batch_exponent=12, film_samples=1 << 22)
    used0, fixed0, jobs0 = b.memory()
    assert fixed0 > 0 and jobs0 == 0 and used0 == fixed0
    b.add_scene(scenes[0])
    used1, fixed1, _ = b.memory()
    assert fixed1 > fixed0  # the scene's BVH, triangles and tables
    small = 3 * 4 * 16 * 16
    b.set_memory_budget(used1 + small + 1024)
    with pytest.raises(mscgpu.MscError) as e:
        b.submit(0, width=64, height=64, spp=1)  # a 49 KB image
    assert e.value.code == -5 and "budget" in str(e.value)
    jid = b.submit(0, width=16, height=16, spp=1)
    assert b.memory()[2] == small
    with pytest.raises(mscgpu.MscError) as e:
        b.add_scene(scenes[2])
    assert e.value.code == -5
    b.run()
    b.release(jid)
    assert b.memory()[2] == 0
    b.set_memory_budget(0)
    b.add_scene(scenes[2])
    b.close()


def test_serve_window_closes_admission_and_reports_busy_time(built, scenes):
    """msc_serve_window: requests that arrive after the window are not served
    (MSC_ERR_BUSY, counted); the admitted ones complete and match the same job
    rendered alone; the GPU busy time is positive and below the wall time."""
    mscgpu, _ = built
    reqs = [(0.0, JOBS[0]), (0.0, JOBS[1]), (0.0, JOBS[4]), (5.0, JOBS[0]), (6.0, JOBS[1])]
    b = mscgpu.Batch(batch_exponent=14, film_samples=1 << 20)
    for s in scenes:
        b.add_scene(s)
    results, st = b.serve(reqs, window_s=0.5)
    assert st["completed"] == 3 and st["not_admitted"] == 2
    assert [r["status"] for r in results] == [0, 0, 0, -5, -5]
    assert 0.0 < st["gpu_busy_s"] <= st["wall_s"]
    assert st["wall_s"] < 5.0  # the late requests were not waited for
    alone, aid = _batch(mscgpu, scenes, [JOBS[1]])
    assert np.array_equal(b.image(results[1]["job_id"]).view(np.uint32), alone.image(aid[0]).view(np.uint32))
    alone.close()
    b.close()
