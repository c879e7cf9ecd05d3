"""Builds libhdog.so (CUDA, sm_103a), libhdog_synth.so and the hdog_main executable
in-tree under _build/.  Run as a script or call build(); rebuilds only what changed."""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CU_SOURCES = ["norm.cu", "dog.cu", "sweep.cu", "ccl.cu", "regions.cu", "records.cu", "soft.cu", "capi.cu", "noalloc.cu", "graph.cu"]
HEADERS = ["common.cuh", "kernels.cuh", "json_min.hpp", os.path.join(INCLUDE, "hdog.h")]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]

LIB = os.path.join(OUT, "libhdog.so")
SYNTH = os.path.join(OUT, "libhdog_synth.so")
MAIN = os.path.join(OUT, "hdog_main")
STAGE = os.path.join(OUT, "hdog_stage_test")
STAGE_DIR = os.path.join(OUT, "test")
STAGE_NAMES = ["Normalize_test", "DoG_test", "Hessian_test", "CCL_test", "Regional_test"]


def _mtime(p):
    return os.path.getmtime(p) if os.path.exists(p) else -1.0


def _stale(target, deps):
    t = _mtime(target)
    return t < 0 or any(_mtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _arch_guard():
    """Drops build products made on another host architecture (the tree is shared
    between an x86-64 build host and aarch64 GPU hosts)."""
    stamp = os.path.join(OUT, "ARCH")
    here = platform.machine()
    if os.path.exists(stamp) and open(stamp).read().strip() == here:
        return
    for f in os.listdir(OUT):
        path = os.path.join(OUT, f)
        if os.path.isdir(path) and not os.path.islink(path):
            shutil.rmtree(path)
        else:
            os.remove(path)
    with open(stamp, "w") as fh:
        fh.write(here + "\n")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    _arch_guard()
    hdrs = [h if os.path.isabs(h) else os.path.join(CSRC, h) for h in HEADERS]
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([NVCC] + NVFLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    synth_src = os.path.join(CSRC, "synth.c")
    if _stale(SYNTH, [synth_src, os.path.join(CSRC, "synth.h")]):
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
              "-o", SYNTH, synth_src, "-lm"])
    main_src = os.path.join(CSRC, "hdog_main.cpp")
    if _stale(MAIN, [main_src, LIB]):
        _run(["g++", "-O2", "-std=c++17", "-o", MAIN, main_src, "-L" + OUT, "-lhdog", "-Wl,-rpath,$ORIGIN"])
    # the reference's stage programs (test/*_test): one binary, linked under their names
    stage_src = os.path.join(CSRC, "hdog_stage_test.cpp")
    if _stale(STAGE, [stage_src, os.path.join(CSRC, "json_min.hpp"), LIB]):
        _run(["g++", "-O2", "-std=c++17", "-o", STAGE, stage_src, "-L" + OUT, "-lhdog", "-Wl,-rpath,$ORIGIN:$ORIGIN/.."])
    os.makedirs(STAGE_DIR, exist_ok=True)
    for name in STAGE_NAMES:
        link = os.path.join(STAGE_DIR, name)
        if not os.path.lexists(link):
            os.symlink(os.path.join("..", os.path.basename(STAGE)), link)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
