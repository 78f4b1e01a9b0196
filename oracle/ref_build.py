"""Recipe: compile the reference's own CUDA kernels to PTX for parity pinning.

TEST INFRASTRUCTURE ONLY.  Compiles, from the sources where they lie in the
reference checkout (dunyazad/gvdb-voxels, GVDB Voxels 1.1.1), the two kernel
translation units its library JIT-loads at run time:

  source/gvdb_library/kernels/cuda_gvdb_module.cu    (particles, nodes, apron kernels)
  source/gvdb_library/kernels/cuda_gvdb_copydata.cu  (fill / copy kernels)

from the checkout named by $GVDB_REFERENCE or found beside the repository,
with the reference's own flags (--use_fast_math, PTX output, see
source/gvdb_library/CMakeLists.txt:37-60), targeting sm_103a, into
oracle/_ref/*.ptx.  The PTX is text: it is loaded as is by the harness
(oracle/ref_harness.cu) on the GPU machine and is never read or edited here.
Only the reference's sources are used; nothing is copied into this repository
(oracle/_ref/ is git-ignored).
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: $GVDB_REFERENCE, else a directory named "reference"
# beside the repository (absent on machines that only run the prebuilt PTX)
REF = os.environ.get("GVDB_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
KDIR = os.path.join(REF, "source", "gvdb_library", "kernels")
UNITS = ("cuda_gvdb_module.cu", "cuda_gvdb_copydata.cu")


def available():
    return all(os.path.exists(os.path.join(KDIR, u)) for u in UNITS)


def build():
    if not available():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT, exist_ok=True)
    outs = []
    for u in UNITS:
        dst = os.path.join(OUT, u.replace(".cu", ".ptx"))
        cmd = [nvcc, "-ptx", "-arch=sm_103a", "--use_fast_math", "-std=c++11", "-w", "-I", KDIR,
               os.path.join(KDIR, u), "-o", dst + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference kernel build failed for %s:\n%s" % (u, r.stderr[-2000:]))
        os.replace(dst + ".tmp", dst)
        outs.append(dst)
    return outs


if __name__ == "__main__":
    print(build())
    sys.exit(0)
