"""Build recipe of libgvx.so (the CUDA library) for sm_103a.

Compiles every csrc/*.cu translation unit in parallel with nvcc and links them
into gvdb-voxels_gb300/libgvx.so.  No cmake, no torch extension machinery: the
library is a plain C-ABI shared object (include/gvx.h).  The nvdb::VolumeGVDB
drop-in class (cpp/, include/gvx_volume_gvdb.h) is compiled with g++ into
libgvx_volume.so, linked against libgvx.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgvx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                     "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_volume()
    return LIB


VOLUME_SRC = os.path.join(HERE, "cpp", "gvx_volume_gvdb.cpp")
VOLUME_LIB = os.path.join(HERE, "libgvx_volume.so")


def build_volume():
    """libgvx_volume.so: the nvdb::VolumeGVDB drop-in class (include/gvx_volume_gvdb.h)
    over libgvx, found next to it at run time"""
    tmp = VOLUME_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I", os.path.join(ROOT, "include"),
           VOLUME_SRC, "-o", tmp, "-L", HERE, "-lgvx", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for the VolumeGVDB class:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, VOLUME_LIB)
    return VOLUME_LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
