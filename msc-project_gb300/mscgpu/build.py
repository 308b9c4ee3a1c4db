"""Builds libmscgpu.so (the CUDA renderer behind include/msc_gpu.h) in-tree.

Every translation unit is compiled in parallel for sm_103a only.  The flags
that pin the arithmetic matter for parity: implicit contraction is off on the
device (-fmad=false) and on the host (-ffp-contract=off), division and square
root are IEEE (-prec-div/-prec-sqrt) and denormals are kept (-ftz=false).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libmscgpu.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["sort.cu", "bvh.cu", "render.cu", "core.cu", "engine.cu", "noalloc.cu"]
CPP_SOURCES = ["scene.cpp", "scenegen.cpp", "imageio.cpp"]
CLI = os.path.join(HERE, "msc-gpu")
SCENEGEN = os.path.join(HERE, "msc-scenegen")

NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-ftz=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-v", "--expt-relaxed-constexpr",
    "-I" + CSRC, "-I" + os.path.join(REPO, "include"),
]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
             "-I" + os.path.join(CUDA_HOME, "include"), "-I" + os.path.join(REPO, "include")]


def _run(cmd, log):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError("build step failed (%s):\n%s" % (" ".join(cmd), p.stdout[-6000:]))
    return p.stdout


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_scenegen(force=False):
    """The scene generator as a host-only executable (no CUDA library loaded):
    the benchmark's CPU arm writes its scene files with it."""
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, "scenegen.cpp"), os.path.join(CSRC, "scenegen_main.cpp"), os.path.join(CSRC, "scene.h"),
            os.path.join(CSRC, "dmath.h")]
    if force or _stale(SCENEGEN, srcs):
        _run(["g++"] + CXX_FLAGS + srcs[:2] + ["-o", SCENEGEN], os.path.join(OUT_DIR, "scenegen.log"))
    return SCENEGEN


def build(verbose=False, force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "msc_gpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            if src.endswith(".cu"):
                cmd = [NVCC] + NVCC_FLAGS + ["-c", s, "-o", o]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-c", s, "-o", o]
            jobs.append((cmd, o + ".log"))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(lambda j: _run(*j), jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"],
             os.path.join(OUT_DIR, "link.log"))
    cli_src = os.path.join(CSRC, "cli.cpp")
    if force or _stale(CLI, [cli_src, LIB]):
        _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include"), cli_src, "-o", CLI, "-L" + HERE,
              "-lmscgpu", "-Wl,-rpath,$ORIGIN"], os.path.join(OUT_DIR, "cli.log"))
    build_scenegen(force)
    return LIB


def ptxas_report():
    """Register / spill / shared-memory report of the last device build."""
    out = []
    for src in CU_SOURCES:
        log = os.path.join(OUT_DIR, src + ".o.log")
        if os.path.exists(log):
            out.append(open(log).read())
    return "\n".join(out)


def clean():
    shutil.rmtree(OUT_DIR, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
