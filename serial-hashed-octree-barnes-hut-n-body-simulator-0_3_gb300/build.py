"""Builds libbhgpu.so in place with nvcc for sm_103a (no cmake, no torch extension).

Each translation unit is compiled in parallel to an object file under _build/, then linked
into libbhgpu.so next to this file with the CUDA runtime linked statically.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libbhgpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["bh_api.cu", "bh_sort.cu", "bh_tree.cu", "bh_walk.cu", "bh_adjoint.cu", "bh_diag.cu", "bh_aux.cu", "bh_ic.cpp",
           "bh_io.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: libbhgpu needs the CUDA toolkit to build")
    return cand


# Per-file flags. The walk flushes FP32 denormals to zero: every quantity it handles (positions,
# masses, softened distances, multipoles) is many orders of magnitude above the denormal range,
# and without denormal support rsqrtf and the FP32 arithmetic need fewer instructions. The
# initial-condition generators keep every FP64 product and sum separately rounded, as the host
# code they restate does (no contraction into fused multiply-adds).
FILE_FLAGS = {"bh_walk.cu": ["-ftz=true"], "bh_aux.cu": ["-fmad=false"]}


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
           "-I" + os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj] + FILE_FLAGS.get(src, []) + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra_flags=()):
    """Compiles every source and links libbhgpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra_flags)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = OUT + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, extra_flags=["-Xptxas", "-v"] if "-v" in sys.argv else []))
