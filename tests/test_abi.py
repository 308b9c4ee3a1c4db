"""The C ABI on the CPU: the library loads, exports every function that
include/msc_gpu.h declares, rejects bad arguments without touching a GPU, and
the C++ drop-in header compiles against it."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(REPO, "include", "msc_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(msc_\w+)\(", text, re.M)))


def test_every_declared_symbol_is_exported(built):
    mscgpu, _ = built
    lib = C.CDLL(mscgpu.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bad_arguments_are_rejected_without_a_device(built):
    mscgpu, _ = built
    lib = mscgpu.load_library()
    it = C.c_int(5)
    assert lib.msc_process(None, C.byref(it)) == -1
    assert lib.msc_destroy(None) == -1
    assert lib.msc_clear(None) == -1
    assert lib.msc_terminate(None) == -1
    assert lib.msc_stage_cardinal(None, -1, None) == -1
    assert lib.msc_sort_pairs(None, None, 4, 8) == -1
    assert lib.msc_sort_pairs(None, None, 4, 40) == -1
    out = C.c_void_p()
    assert lib.msc_create(None, C.byref(out)) == -1
    assert lib.msc_generate_scene(7, 1, 1.0, b"/tmp/x", C.create_string_buffer(64), 64) == -2


def test_empty_inputs_are_no_ops(built):
    mscgpu, _ = built
    assert mscgpu.cardinal(np.zeros((0, 3), np.float32)).shape == (0,)
    assert mscgpu.ray_keys(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32)).shape == (0,)
    k, v = mscgpu.sort_pairs(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    assert k.shape == (0,) and v.shape == (0,)


def test_cpp_dropin_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text("""
#include <msc_pathtracer.hpp>
int render(const char* yaml) {
  msc::Pathtracer pt(yaml);          // the reference's constructor signature
  int it = pt.process();
  float* px; int w, h;
  pt.image(&px, &w, &h);
  if (!pt.active()) return -1;
  pt.clear();
  pt.terminate();
  return it + w * h;
}
""")
    r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I" + os.path.join(REPO, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
