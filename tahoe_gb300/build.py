"""In-tree build of the tahoe_gb300 CUDA library.

Compiles every translation unit under tahoe_gb300/csrc for sm_103a with nvcc
(in parallel, one object per unit) and links tahoe_gb300/_build/libtahoe_gb300.so.
No cmake, no architecture-specific host flags: the same recipe builds on the
x86_64 development host and on the aarch64 GPU hosts.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtahoe_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", SRC]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _sources():
    return sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cpp")))


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = (_sources() + glob.glob(os.path.join(SRC, "*.h")) + glob.glob(os.path.join(SRC, "*.cuh")) +
            glob.glob(os.path.join(INCLUDE, "*.h")))
    return any(os.path.getmtime(p) > t for p in deps)


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        for src, obj, rc, log in ex.map(lambda s: _compile(s, extra), _sources()):
            if rc != 0 or verbose or ptxas_info:
                sys.stderr.write(log)
            if rc != 0:
                raise RuntimeError("nvcc failed on %s" % os.path.basename(src))
            objs.append(obj)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
