"""Build the engine's shared library in-tree with nvcc for sm_103a.

Output: lbm_gb300/liblbm_gb300.so (git-ignored).  Each CUDA translation unit
is compiled in parallel to an object, then linked.  Flags: -fmad=false keeps
f32 arithmetic in source order (no FMA contraction), which the bit-exact
parity with the reference's shader arithmetic relies on.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbm_gb300.so")
SOURCES = ["lbm_capi.cu", "lbm_noalloc.cu", "lbm_batch.cu", "lbm_cnn.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                     "-Xptxas", "-v", "--expt-relaxed-constexpr"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    log = os.path.join(BUILD, os.path.splitext(src)[0] + ".ptxas.txt")
    cmd = [nvcc()] + NVCC_FLAGS + ["-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(CSRC, src),
                                    "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
    return obj


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    inc = os.path.join(HERE, "..", "include")
    deps = ([os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(inc, f) for f in os.listdir(inc)]
            + [os.path.abspath(__file__)])
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
    os.replace(tmp, LIB)
    if verbose:
        for src in SOURCES:
            with open(os.path.join(BUILD, os.path.splitext(src)[0] + ".ptxas.txt")) as f:
                sys.stdout.write(f.read())
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
