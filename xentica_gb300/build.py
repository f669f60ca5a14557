"""Build ``libxk.so`` (the C-ABI in ``include/xk.h``) in-tree with nvcc.

Every ``csrc/*.cu`` is compiled for sm_103a in parallel, then linked into
``xentica_gb300/libxk.so``.  Run ``python -m xentica_gb300.build``.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libxk.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-O2",
         "-Xptxas", "-O3"]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else "nvcc"


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cuh")]
    deps.append(os.path.join(HERE, "..", "include", "xk.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    if verbose:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose=False):
    """Compile and link; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cu"))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(sources)) as pool:
        objs = list(pool.map(lambda s: _compile(s, verbose), sources))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
