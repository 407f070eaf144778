"""Build libnlmgpu.so (the CUDA library) in-tree with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then linked
into nlmech_gb300/libnlmgpu.so.  The FP64 "plain" kernels and the neighbour
builder are compiled with --fmad=false so that their arithmetic is the
separately rounded sequence of the reference expressions.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnlmgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
# translation unit -> extra flags
UNITS = {
    "fd_host.cu": [],
    "host_common.cu": [],
    "fd_kernels.cu": [],
    "host_io.cu": [],
    "batch_host.cu": [],
    "qs_host.cu": [],
    "esqs_host.cu": [],
    "neighbor.cu": ["--fmad=false"],
    "fd_fp64.cu": ["--fmad=false"],
    "fd_fp32.cu": [],
    "es_fp64.cu": ["--fmad=false"],
    "es_fp32.cu": [],
    "qs.cu": [],
    "noalloc.cu": ["--fmad=false"],
    "mlp.cu": [],
    "esqs.cu": ["--fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def _deps():
    out = []
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    out.append(os.path.join(HERE, "..", "include", "nlmgpu.h"))
    out.append(os.path.abspath(__file__))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, extra=None):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def one(unit):
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[unit], *(extra or []), "-c",
               os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(UNITS))) as ex:
        objs = list(ex.map(one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if v else None
    print(build(force=True, verbose=v, extra=extra))
