"""In-tree build of the CUDA library (libtrans_gb300.so) for sm_103a with nvcc.

Translation units are compiled in parallel; the FP64 unit is compiled without fused
multiply-add (-fmad=false) so that its arithmetic rounds as the reference's does.  The mixed
unit (k_mixed.cu) contracts to fused multiply-add and evaluates FP32 division and square root
with the hardware approximations (-prec-div=false -prec-sqrt=false: at most 2 ulp, against a
~10-instruction correctly rounded sequence); its FP64 arithmetic is unaffected.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtrans_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
UNITS = {
    "api.cu": ["-fmad=false"],
    "engine.cu": ["-fmad=false"],
    "worklist.cu": ["-fmad=false"],
    "stages.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "batch.cu": ["-fmad=false"],
    "k_fp64.cu": ["-fmad=false"],
    "k_integrals.cu": ["-fmad=false"],
    "k_geometry.cu": ["-fmad=false"],
    "k_mixed.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "trans_gpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_unit(item):
        src, flags = item
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
