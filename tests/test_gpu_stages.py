"""Stage parity on the GPU through the C ABI: cardinal bins, the stable bin
partition, ray sort keys and the radix sort are bit-exact against the CPU
oracle; closest-hit and occlusion queries match it except at stated near-ties."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dirs(rng, n):
    n0, n = n, max(n, 16)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # exact ties between components and signed zeros exercise the tie rules
    d[: n // 16, 1] = d[: n // 16, 0]
    d[n // 16: n // 8, 2] = -d[n // 16: n // 8, 0]
    d[n // 8: n // 8 + 8] = np.array([[0, 0, 0], [-0.0, 0, 0], [1, 1, 1], [-1, -1, -1], [0, -0.0, 1], [0, 0, -0.0],
                                      [1, -1, 0], [-1, 1, 0]], np.float32)
    return d[:n0]


@pytest.mark.parametrize("n", [1, 7, 1000, 200003])
def test_cardinal_bins_bit_exact(built, n):
    mscgpu, oracle = built
    d = _dirs(np.random.default_rng(n), max(n, 16))[:n]
    assert np.array_equal(mscgpu.cardinal(d), oracle.cardinal(d))


def _rays(rng, n, dead_frac=0.2):
    r = np.zeros((n, 12), np.float32)
    r[:, 0:3] = rng.uniform(-5, 5, size=(n, 3))
    r[:, 3] = rng.uniform(0.1, 1, size=n)
    r[:, 4:7] = _dirs(rng, n)
    depth = rng.integers(0, 8, size=n).astype(np.int32)
    depth[rng.random(n) < dead_frac] = -1
    r[:, 7] = depth.view(np.float32)
    r[:, 8:11] = rng.uniform(0, 1, size=(n, 3))
    r[:, 11] = np.arange(n, dtype=np.int32).view(np.float32)
    return r


@pytest.mark.parametrize("n", [0, 1, 5, 2047, 2048, 2049, 100000])
def test_bin_partition_stable_and_bit_exact(built, n):
    mscgpu, oracle = built
    rays = _rays(np.random.default_rng(n + 1), n)
    cap = max(n, 1)
    got, gc = mscgpu.bin_partition(rays, cap)
    want, wc = oracle.bin_partition(rays, cap)
    assert np.array_equal(gc, wc)
    for b in range(6):
        g = got[b * cap: b * cap + gc[b]]
        w = want[b * cap: b * cap + wc[b]]
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


@pytest.mark.parametrize("n", [1, 3, 4097, 65536, 300001])
def test_ray_keys_bit_exact(built, n):
    mscgpu, oracle = built
    rng = np.random.default_rng(n + 2)
    org = rng.uniform(-3, 7, size=(n, 3)).astype(np.float32)
    org[: n // 3, 1] = 2.5  # a flat extent on part of the batch
    d = _dirs(rng, max(n, 16))[:n]
    d[np.abs(d).max(axis=1) == 0] = [0, 0, 1]
    assert np.array_equal(mscgpu.ray_keys(org, d), oracle.ray_keys(org, d))


@pytest.mark.parametrize("n,bits", [(1, 32), (2, 8), (4095, 32), (4096, 16), (4097, 22), (100000, 30),
                                    (1 << 20, 32), (777777, 11)])
def test_radix_sort_is_the_stable_order(built, n, bits):
    mscgpu, oracle = built
    rng = np.random.default_rng(n * 31 + bits)
    keys = rng.integers(0, 1 << min(bits, 20), size=n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 4] = keys[0]  # long runs of equal keys test stability
    if bits < 32:
        keys |= rng.integers(0, 2, size=n, dtype=np.uint32) << np.uint32(31)  # bits above `bits` are ignored
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = mscgpu.sort_pairs(keys, vals, bits)
    wk, wv = oracle.stable_sort_pairs(keys, vals, bits)
    assert np.array_equal(gv, wv)
    assert np.array_equal(gk, wk)


def test_radix_sort_full_size_properties(built):
    """2^24 keys: output sorted, a permutation of the input, stable."""
    mscgpu, _ = built
    n = 1 << 24
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    keys[::3] = 12345
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = mscgpu.sort_pairs(keys, vals, 32)
    assert np.all(gk[1:] >= gk[:-1])
    assert np.array_equal(np.sort(gv), vals)
    assert np.array_equal(keys[gv], gk)
    eq = gk[1:] == gk[:-1]
    assert np.all(gv[1:][eq] > gv[:-1][eq])


def _scene_rays(oracle_scene, rng, n):
    tv, _ = oracle_scene.triangles_array()
    lo, hi = tv.reshape(-1, 3).min(0), tv.reshape(-1, 3).max(0)
    org = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = _dirs(rng, n)
    d[np.abs(d).max(axis=1) == 0] = [0, 1, 0]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return org, d.astype(np.float32)


def _with_bvh(path, form, tmp_path):
    """A copy of the scene YAML whose extension document selects the BVH form."""
    import os
    import shutil
    d = os.path.dirname(path)
    for f in os.listdir(d):
        if f.endswith(".obj"):
            shutil.copy(os.path.join(d, f), tmp_path / f)
    text = open(path).read().replace("extensions:\n", "extensions:\n  bvh: %s\n" % form)
    y = tmp_path / "scene.yaml"
    y.write_text(text)
    return str(y)


@pytest.mark.parametrize("form", ["wide", "binary"])
def test_closest_hit_matches_oracle(built, box_scene, form, tmp_path):
    mscgpu, oracle = built
    s = oracle.Scene(box_scene)
    org, d = _scene_rays(s, np.random.default_rng(11), 200000)
    with mscgpu.Pathtracer(_with_bvh(box_scene, form, tmp_path)) as pt:
        t, u, v, g, p = pt.trace_closest(org, d)
    wt, wu, wv, wg, wp = s.trace(org, d)
    same = (g == wg) & (p == wp)
    # primitive ids agree except at near-ties: two hits within 1e-5 relative distance
    tie = ~same & (np.abs(t - wt) <= 1e-5 * np.maximum(np.abs(wt), 1e-3))
    assert np.all(same | tie), np.flatnonzero(~(same | tie))[:10]
    assert tie.mean() < 1e-3
    hit = same & (wg >= 0)
    assert hit.sum() > 1000
    for a, b in ((t, wt), (u, wu), (v, wv)):
        assert np.all(np.abs(a[hit] - b[hit]) <= 1e-5 * np.maximum(np.abs(b[hit]), 1e-3))
    # the same arithmetic on both sides: most hits agree to the bit
    assert (t[hit].view(np.uint32) == wt[hit].view(np.uint32)).mean() > 0.999


def _duplicated_scene(mscgpu, out_dir):
    """The tiny scene with every box face listed twice in its OBJ and the
    icosphere object placed twice: coincident triangles, so many rays meet two
    candidates at exactly the same distance."""
    import os
    import re
    y = mscgpu.generate_scene(100, 1234, str(out_dir))
    box = os.path.join(str(out_dir), "box.obj")
    lines = open(box).read().splitlines()
    open(box, "w").write("\n".join(lines + [l for l in lines if l.startswith("f ")]) + "\n")
    text = open(y).read()
    obj = re.search(r"object:\n  type: Polygon\n  filename: icosphere.obj\n(?:  .*\n)*", text).group(0)
    head, scene, ext = text.split("---")
    open(y, "w").write(head + "---" + scene + obj + "---" + ext)
    return y


@pytest.mark.parametrize("form", ["wide", "binary"])
def test_exact_ties_go_to_the_smaller_triangle_index(built, tmp_path, form):
    """Equal distances are settled by the scene triangle index (geomID, then
    primID) on both sides, whatever order the two BVHs present the candidates in."""
    mscgpu, oracle = built
    y = _duplicated_scene(mscgpu, tmp_path / "dup")
    s = oracle.Scene(y)
    org, d = _scene_rays(s, np.random.default_rng(21), 100000)
    with mscgpu.Pathtracer(_with_bvh(y, form, tmp_path)) as pt:
        t, u, v, g, p = pt.trace_closest(org, d)
    wt, wu, wv, wg, wp = s.trace(org, d)
    assert np.array_equal(g, wg) and np.array_equal(p, wp)
    hit = wg >= 0
    assert (t[hit].view(np.uint32) == wt[hit].view(np.uint32)).mean() > 0.999
    # triangles of one copy of the box faces (fan triangulation of each face)
    ntri = sum(len(l.split()) - 3 for l in open(str(tmp_path / "dup" / "box.obj")) if l.startswith("f ")) // 2
    geoms = open(y).read().split("---")[1].split("object:")[1:]
    box_g = [i for i, m in enumerate(geoms) if "box.obj" in m]
    ico_g = [i for i, m in enumerate(geoms) if "icosphere.obj" in m]
    # the first copy always wins, and both coincident sets are hit
    on_box = np.isin(g, box_g)
    assert np.all(p[on_box] < ntri) and on_box.sum() > 100
    assert len(ico_g) == 2 and not np.any(g == ico_g[1]) and (g == ico_g[0]).sum() > 100


@pytest.mark.parametrize("form", ["wide", "binary"])
def test_occlusion_matches_oracle(built, box_scene, form, tmp_path):
    mscgpu, oracle = built
    s = oracle.Scene(box_scene)
    rng = np.random.default_rng(12)
    org, d = _scene_rays(s, rng, 100000)
    tmax = rng.uniform(0.01, 3.0, size=org.shape[0]).astype(np.float32)
    with mscgpu.Pathtracer(_with_bvh(box_scene, form, tmp_path)) as pt:
        got = pt.trace_occluded(org, d, tmax)
    want = s.occluded(org, d, tmax)
    assert (got != want).mean() < 1e-3
    assert 0.05 < want.mean() < 0.95


def test_sort_keys64_is_the_stable_order(built):
    """The 64-bit hit key order (low word, then high word) = a stable sort on the whole key."""
    mscgpu, _ = built
    rng = np.random.default_rng(64)
    for n in (1, 1000, 70001):
        hi = rng.integers(0, 1 << 12, n, dtype=np.uint64) << np.uint64(52)
        mid = rng.integers(0, 1 << 23, n, dtype=np.uint64) << np.uint64(29)
        lo = rng.integers(0, 1 << 29, n, dtype=np.uint64)
        keys = hi | (mid if n < 5000 else (mid & np.uint64(0xF << 29))) | (lo & np.uint64(0xFF))  # many ties
        perm = mscgpu.sort_keys64(keys)
        assert np.array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


@pytest.mark.parametrize("nbins", [6, 26, 98])
def test_ray_bins_bit_exact(built, nbins):
    mscgpu, oracle = built
    d = _dirs(np.random.default_rng(nbins), 50000)
    got = mscgpu.ray_bins(d, nbins)
    assert np.array_equal(got, oracle.ray_bins(d, nbins))
    assert got.min() >= 0 and got.max() < nbins
    assert len(np.unique(got)) == nbins  # every cell is reached


@pytest.mark.parametrize("nbins,n", [(26, 1), (26, 9000), (98, 2049), (98, 150000)])
def test_bin_partition_n_bins_stable_and_bit_exact(built, nbins, n):
    """The chunked bin pool: every bin's rays in arrival order, across chunk boundaries."""
    mscgpu, oracle = built
    rays = _rays(np.random.default_rng(n + nbins), n)
    cap = max(n, 1)
    got, gc = mscgpu.bin_partition(rays, cap, nbins)
    want, wc = oracle.bin_partition_n(rays, nbins, cap)
    assert np.array_equal(gc, wc)
    for b in range(nbins):
        assert np.array_equal(got[b * cap: b * cap + gc[b]].view(np.uint32), want[b * cap: b * cap + wc[b]].view(np.uint32))


@pytest.mark.parametrize("digit_bits", [4, 8, 11])
@pytest.mark.parametrize("n,bits", [(1, 32), (2047, 32), (2049, 22), (100000, 32), (300001, 13), (1 << 20, 30)])
def test_radix_digit_widths_are_the_stable_order(built, digit_bits, n, bits):
    """4-, 8- and 11-bit digits (the autotuner's widths) give CPU std::stable_sort's order."""
    mscgpu, oracle = built
    rng = np.random.default_rng(n + bits + digit_bits)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[: n // 3] & np.uint32(0xF0F)  # many equal digits
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = mscgpu.sort_pairs_digits(keys, vals, bits, digit_bits)
    wk, wv = oracle.stable_sort_pairs(keys, vals, bits)
    assert np.array_equal(gv, wv)
    assert np.array_equal(gk, wk)


def test_lookback_wait_that_runs_out_is_reported(built):
    """The sort's look-back spins are bounded: with a first tile that never posts
    its counts, every later tile gives up after the cap, the call returns, and the
    host reads MSC_ERR_DEVICE; the same sort with nothing withheld is the stable order."""
    mscgpu, _ = built
    rng = np.random.default_rng(9)
    n = 50000
    keys = rng.integers(0, 1 << 16, size=n, dtype=np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    rc, _, _ = mscgpu.sort_lookback_check(keys, vals, 16, 512, True)
    assert rc == -4  # MSC_ERR_DEVICE
    assert b"look-back" in mscgpu.load_library().msc_last_error(None)
    rc, k, v = mscgpu.sort_lookback_check(keys, vals, 16, 512, False)
    assert rc == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v, order.astype(np.uint32)) and np.array_equal(k, keys[order])
