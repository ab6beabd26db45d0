"""Build the sm_103a engine library in-tree: femtech_gb300/libftgpu.so.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked with the CUDA runtime.  ``python -m femtech_gb300.build`` or
``build()`` from Python; the output path is returned.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libftgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ft_elem_f32.cu", "ft_elem_f64.cu", "ft_api.cu", "ft_patches.cpp", "ft_noalloc.cu",
           "ft_mlp.cu", "ft_meshio.cpp", "ft_vtu.cpp", "ft_probe.cu"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libftgpu.so")
    return path


# The FP32 element kernels use approximate division / square root (their
# results are checked against the FP64 oracle at the mixed-mode tolerance);
# every other translation unit keeps IEEE arithmetic.
EXTRA = {"ft_elem_f32.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]}


def _compile(src, verbose):
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           *EXTRA.get(src, []),
           "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-c",
           os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, out.stdout, out.stderr))
    return obj, out.stderr


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    newest = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
    newest = max(newest, os.path.getmtime(os.path.join(ROOT, "include", "ftgpu.h")))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, log in res:
            sys.stderr.write(log)
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *[o for o, _ in res], "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n" + out.stdout + out.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
