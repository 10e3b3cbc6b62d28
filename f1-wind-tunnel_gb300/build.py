"""Build libwt.so (the sm_103a kernels and the C ABI of include/wt.h).

    python f1-wind-tunnel_gb300/build.py [--verbose]

Each .cu file in csrc/ is compiled by its own nvcc process (in parallel) for
sm_103a only, then linked into f1-wind-tunnel_gb300/_build/libwt.so.  No
floating-point contraction (-fmad=false on the device, -ffp-contract=off on the
host side): the voxelizer, the collide-stream step and the heat pass then give
the same bits as the reference's arithmetic.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwt.so")
ROOT = os.path.dirname(HERE)

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    "-std=c++17", "--expt-relaxed-constexpr", "-O3", "-lineinfo", ARCH, "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "wt.h"), __file__]
    return max(os.path.getmtime(f) for f in files)


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime()


def build(verbose=False, force=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
        cmd = [cc, *NVCC_FLAGS, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, "-shared", ARCH, "-cudart", "shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
