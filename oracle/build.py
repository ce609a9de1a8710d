"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/oracle.cpp with g++ into oracle/_build/liboracle.so.  Plain
portable C++17: no architecture flags, so the same recipe builds on x86_64 and
on aarch64 hosts.

Where the reference source tree is present (TAHOE_REFERENCE_DIR, default
/root/reference), it also compiles the one reference path that builds from
its own few source files: the MSR structure builder (MSRBuilderT and the
toolbox classes it uses, twelve files, compiled directly with g++ -- the
reference's own build system is not run) with the driver oracle/ref_msr.cpp,
into oracle/_ref/ref_msr.  The element path does not build that way (its
factories need the whole library, see the design notes).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", src, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


REF_DIR = os.path.join(HERE, "_ref")
REF_MSR = os.path.join(REF_DIR, "ref_msr")
# the reference's own sources of its MSR structure builder, relative to the
# toolbox source directory
REF_MSR_SOURCES = (
    "graph/MSRBuilderT.cpp", "graph/GraphT.cpp", "graph/GraphBaseT.cpp", "graph/PartitionT.cpp",
    "graph/RootedLevelT.cpp", "common/ExceptionT.cpp", "abc/array/iArray2DT.cpp", "abc/array/iArrayT.cpp",
    "abc/array/ArraySettings.cpp", "abc/other/StringT.cpp", "fstreamT/ifstreamT.cpp", "fstreamT/fstreamT.cpp",
)


def reference_dir():
    d = os.environ.get("TAHOE_REFERENCE_DIR", "/root/reference")
    return d if os.path.isdir(os.path.join(d, "toolbox", "src")) else None


def build_ref(force=False):
    """oracle/_ref/ref_msr from the reference's sources, or None when the
    reference tree is absent (the GPU host: the tests that need it skip)."""
    ref = reference_dir()
    if ref is None:
        return REF_MSR if os.path.exists(REF_MSR) else None
    tb = os.path.join(ref, "toolbox", "src")
    srcs = [os.path.join(tb, s) for s in REF_MSR_SOURCES] + [os.path.join(HERE, "ref_msr.cpp")]
    if (not force and os.path.exists(REF_MSR)
            and os.path.getmtime(REF_MSR) >= max(os.path.getmtime(s) for s in srcs)):
        return REF_MSR
    incs = []
    for d, _, _ in os.walk(tb):
        incs.append("-I" + d)
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_MSR + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++11", "-w"] + incs + srcs + ["-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, REF_MSR)
    return REF_MSR


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
