"""Builds the CPU oracle (test infrastructure) and, where the reference
sources are present, the reference's own OBJ reader into oracle/_ref/.

  oracle/_build/liboracle.so  - the C++ restatement (oracle.cpp)
  oracle/_ref/libreftinyobj.so - thirdparty/tinyobjloader/tiny_obj_loader.cpp of
                                 the reference, compiled from where it lies,
                                 plus the C shim ref_tinyobj_shim.cpp

The rest of the reference (Embree 2.6.1, TBB, Boost, yaml-cpp, Eigen, OIIO,
OpenEXR) is not available here, so nothing else of it is compiled.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(REF_OUT, "libreftinyobj.so")
# where the reference's sources lie (read only); MSC_REFERENCE_DIR overrides it
REFERENCE = os.environ.get("MSC_REFERENCE_DIR", "/root/reference")

FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread"]


def _stale(out, srcs):
    return not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), p.stdout[-4000:]))


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle.h")]
    if force or _stale(LIB, srcs):
        _run(["g++"] + FLAGS + [srcs[0], "-o", LIB])
    ref_src = os.path.join(REFERENCE, "thirdparty", "tinyobjloader", "tiny_obj_loader.cpp")
    if os.path.exists(ref_src):
        os.makedirs(REF_OUT, exist_ok=True)
        shim = os.path.join(HERE, "ref_tinyobj_shim.cpp")
        if force or _stale(REF_LIB, [shim, ref_src]):
            _run(["g++", "-O2", "-std=c++11", "-fPIC", "-shared", "-ffp-contract=off",
                  "-I" + os.path.join(REFERENCE, "thirdparty"), shim, ref_src, "-o", REF_LIB])
    return LIB


if __name__ == "__main__":
    build(force="-f" in sys.argv)
    print(LIB)
