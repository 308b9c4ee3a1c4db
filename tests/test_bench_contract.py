"""The benchmark's reference arm runs on the host alone (the CPU restatement of
the reference's render loop): its JSON line keeps the bench contract."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(built):
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--scale", "0.25"], cwd=REPO, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["unit"] == "Mrays/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] >= 3
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["config"]["workload"].startswith("terrain")


def test_reference_arm_loads_no_library_of_the_renderer(built):
    """The CPU arm may load the oracle only: neither libmscgpu.so nor the CUDA
    runtime appear among the process's mapped files after a run."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', "
            "'--scale', '0.25']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED', 'libmscgpu' in maps, 'liboracle' in maps, 'libcuda.so' in maps, file=sys.stderr)")
    p = subprocess.run([sys.executable, "-c", code], cwd=REPO, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = [l for l in p.stderr.splitlines() if l.startswith("MAPPED")][-1]
    assert line == "MAPPED False True False", line


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_stage_bandwidths_follow_the_binning_form():
    """roofline.hbm_stages charges each stage the bytes its kernels move: camera
    rays to raygen, the continuing rays to shading when batches bin directly
    (2^13 rays and more), to the bins stage otherwise; the sort reads no
    histogram pass with 8-bit digits (the key kernel counts them)."""
    b = _bench_module()
    prof = {"stage_ms": {"raygen": 1.5, "bins": 0.15, "ray_sort": 1.7, "filter": 0.7, "shade": 7.0},
            "closest_queries": 125_000_000, "width": 1024, "height": 1024}
    paths = 1024 * 1024 * 64
    direct = b.hbm_stages(prof, 6760.9, 64, 24, 8)
    assert "bins" not in direct
    assert abs(direct["raygen"]["gbs"] - 78.0 * paths / 1.5e-3 / 1e9) < 0.1
    assert abs(direct["shade"]["gbs"] - 164.0 * 125e6 / 7.0e-3 / 1e9) < 0.1
    assert abs(direct["ray_sort"]["gbs"] - 32.0 * 125e6 / 1.7e-3 / 1e9) < 0.1
    staged = b.hbm_stages(prof, 6760.9, 64, 12, 4)
    assert abs(staged["bins"]["gbs"] - 112.0 * (125e6 - paths) / 0.15e-3 / 1e9) < 0.1
    assert abs(staged["shade"]["gbs"] - 160.0 * 125e6 / 7.0e-3 / 1e9) < 0.1
    assert abs(staged["ray_sort"]["gbs"] - 36.0 * 125e6 / 1.7e-3 / 1e9) < 0.1
    for v in list(direct.values()) + list(staged.values()):
        assert abs(v["frac"] - v["gbs"] / 6760.9) < 1e-3
