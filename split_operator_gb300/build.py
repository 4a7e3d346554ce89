"""Compile the CUDA/C++ sources of the library into an in-tree shared object.

``python -m split_operator_gb300.build`` (or ``build()``) runs nvcc on every
translation unit in parallel for sm_103a and links
``split_operator_gb300/_build/libsplit_operator_gb300.so``.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsplit_operator_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         # host-side warnings (misleading indentation, dangling else, unused values) are errors
         "-Xcompiler", "-Wall", "-Xcompiler", "-Werror=misleading-indentation",
         "-Xcompiler", "-Werror=dangling-else"] + ARCH


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src):
    obj = os.path.join(OUT, src + ".o")
    cmd = [NVCC, *FLAGS, "-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"] if os.environ.get("SO_PTXAS_VERBOSE") else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    objs = []
    for src, obj, r in results:
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        objs.append(obj)
    tmp = LIB + ".tmp"
    cmd = [NVCC, "-shared", *ARCH, "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
