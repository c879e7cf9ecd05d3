"""TEST INFRASTRUCTURE: builds the checker, never the product.

1. oracle/_build/liboracle.so from hdog_oracle.c (the CPU restatement), with
   -ffp-contract=off so no host compiler adds contractions of its own.
2. oracle/_ref/*.cubin: the reference's own CUDA kernels (CUBIC-informatics src/3D),
   compiled unmodified for sm_103a straight from where they lie under the read-only
   reference checkout, when that checkout is present.  Only device code is built; the
   launcher in oracle/ref_cubin.py restates the reference's host-side launch geometry
   and drives the kernels through the CUDA driver API on a GPU host.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
# the reference checkout: HDOG_REFERENCE, else its location in the build container
REFERENCE = os.environ.get("HDOG_REFERENCE", "/root/reference")
REF_KERNEL_FILES = ["NormalizeFilter", "DoG3DFilter", "Hessian3DFilter_element", "CCL3D", "Eigenvalues",
                    "Erosion3DFilter"]


def _stale(t, deps):
    return not os.path.exists(t) or any(os.path.getmtime(d) > os.path.getmtime(t) for d in deps)


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "ARCH")
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        for f in (LIB, os.path.join(BUILD, "libref_features.so")):
            if os.path.exists(f):
                os.remove(f)
        with open(stamp, "w") as fh:
            fh.write(platform.machine() + "\n")
    src = os.path.join(HERE, "hdog_oracle.c")
    hdr = os.path.join(HERE, "hdog_oracle.h")
    if _stale(LIB, [src, hdr]):
        flags = ["-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared"]
        if platform.machine() in ("x86_64", "AMD64"):
            flags.append("-mfma")   # hardware fmaf; results are IEEE fma either way
        subprocess.run(["gcc"] + flags + ["-o", LIB, src, "-lm"], check=True)
    return LIB


def build_ref_features():
    """oracle/_build/libref_features.so: the reference's region reductions restated with CUB
    (ref_features.cu), for oracle/ref_records.py on a GPU host."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libref_features.so")
    src = os.path.join(HERE, "ref_features.cu")
    if _stale(out, [src]) or not _same_arch():
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler",
                        "-fPIC", "-shared", "-o", out, src], check=True)
    return out


def _same_arch():
    stamp = os.path.join(BUILD, "ARCH")
    return os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()


def build_reference_cubins():
    """Returns the list of cubins built, [] when the reference checkout is absent."""
    src_dir = os.path.join(REFERENCE, "src", "3D")
    if not os.path.isdir(src_dir):
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    inc = ["-I" + os.path.join(REFERENCE, "deps", "cuda-samples", "Common"), "-I" + src_dir]
    out = []
    procs = []
    for name in REF_KERNEL_FILES:
        src = os.path.join(src_dir, name + ".cu")
        dst = os.path.join(REF_OUT, name + ".cubin")
        out.append(dst)
        if _stale(dst, [src]):
            procs.append(subprocess.Popen(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                                           "-w"] + inc + [src, "-o", dst]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference cubin build failed")
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref_features())
    print(build_reference_cubins())
