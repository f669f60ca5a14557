"""Run the reference's own generated kernels on the CPU (test infrastructure).

This is oracle tooling, never product code.  It imports the reference
package from a source checkout (``--ref``), with two missing third-party
modules replaced by stubs:

* ``pycuda.{autoinit,compiler,gpuarray}`` -- ``SourceModule`` only keeps the
  source text, ``gpuarray`` wraps NumPy arrays (reference
  ``xentica/core/base.py:94-96``, ``:527-569``);
* ``cached_property`` -- mapped to ``functools.cached_property``.

The reference translator (``Translator.build_source``,
``xentica/core/base.py:440-446``) then produces exactly the CUDA C it would
hand to nvcc.  That source is compiled with g++ through ``ref_shim.h`` into a
shared object, and the model's ``gpu.kernels.{emit,absorb,render}`` are
swapped for ctypes calls into it, so the reference's own ``step()`` /
``render()`` (``base.py:703-753``) drive the reference's own kernels.

It must run in a separate interpreter because the reference package is also
called ``xentica``.  Usage (one JSON job on argv, results to an ``.npz``)::

    python oracle/ref_harness.py --ref <reference checkout> --job '<json>'

Job keys: ``model`` ("pkg.mod:Class" or "path/file.py:Class"), ``experiment``
(same form), ``exp_overrides`` (dict of attributes for a derived experiment
class), ``model_kwargs``, ``checkpoints`` (sorted step counts at which the main
plane and colours are recorded), ``render`` (optional ``{"viewport": [w, h]}``
rendered at every checkpoint), ``set_params`` (``{step: {name: value}}``),
``threads``, ``out`` (npz path), ``workdir`` (build dir for the .so),
``time_steps`` (if set, only time that many steps and report the rate).
"""
import argparse
import ctypes
import functools
import hashlib
import importlib
import importlib.util
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_STUBS = {
    "pycuda/__init__.py": "",
    "pycuda/autoinit.py": "context = None\n",
    "pycuda/compiler.py": (
        "class SourceModule:\n"
        "    def __init__(self, source, options=None):\n"
        "        self.source = source\n"
        "    def get_function(self, name):\n"
        "        def _unbound(*a, **k):\n"
        "            raise RuntimeError('kernel %s not bound' % name)\n"
        "        return _unbound\n"),
    "pycuda/gpuarray.py": (
        "import numpy as np\n"
        "class GPUArray:\n"
        "    def __init__(self, arr):\n"
        "        self.arr = np.ascontiguousarray(arr)\n"
        "        self._block = (1, 1, 1)\n"
        "        self._grid = (1, 1)\n"
        "    def get(self):\n"
        "        return self.arr.copy()\n"
        "def to_gpu(arr):\n"
        "    return GPUArray(np.array(arr))\n"
        "def zeros(shape, dtype=np.float64):\n"
        "    return GPUArray(np.zeros(shape, dtype=dtype))\n"),
    "cached_property.py": "from functools import cached_property\n",
}

_CTYPES = {
    "int": ctypes.c_int32, "int32": ctypes.c_int32, "float": ctypes.c_float,
    "bool": ctypes.c_bool,
}


def _install_stubs():
    root = tempfile.mkdtemp(prefix="xk_refstubs_")
    for rel, text in _STUBS.items():
        path = os.path.join(root, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            fh.write(text)
    sys.path.insert(0, root)


def _load_obj(spec):
    mod_name, attr = spec.rsplit(":", 1)
    if mod_name.endswith(".py"):
        if not os.path.isabs(mod_name):   # relative to the repository root
            mod_name = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    mod_name)
        name = "xk_refjob_" + hashlib.md5(mod_name.encode()).hexdigest()[:8]
        sp = importlib.util.spec_from_file_location(name, mod_name)
        mod = importlib.util.module_from_spec(sp)
        sys.modules[name] = mod
        sp.loader.exec_module(mod)
    else:
        mod = importlib.import_module(mod_name)
    return getattr(mod, attr)


def _kernel_wrappers(model):
    """C++ wrappers that run each generated kernel over T OpenMP threads."""
    def sig(params):
        return [(p.ctype if p.ctype != "int32" else "int", "p%d" % k)
                for k, p in enumerate(params)]
    ctype = model.main.ctype
    out = ["#include <omp.h>",
           "thread_local xk_dim3 threadIdx = {0, 0, 0};",
           "thread_local xk_dim3 blockIdx = {0, 0, 0};",
           "xk_dim3 blockDim = {1, 1, 1};",
           "xk_dim3 gridDim = {1, 1, 1};"]
    kernels = {
        "emit": [(ctype, "*fld")] + sig(model._emit_params),
        "absorb": [(ctype, "*fld"), ("int3", "*col")] + sig(model._absorb_params),
        "render": list(model.renderer.args) + sig(model._render_params),
    }
    for name, args in kernels.items():
        decl = ", ".join("%s %s" % a for a in args) + ", int n"
        call = ", ".join(a[1].lstrip("*") for a in args) + ", n"
        out.append(
            'extern "C" void xkref_%s(int threads, %s) {\n'
            "  gridDim.x = threads;\n"
            "  #pragma omp parallel num_threads(threads)\n"
            "  { blockIdx.x = omp_get_thread_num(); %s(%s); }\n"
            "}" % (name, decl, name, call))
    return "\n".join(out) + "\n"


def compile_cpp(cpp, so):
    """g++ recipe for one dumped reference kernel source."""
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-fopenmp", "-shared", "-fPIC",
           "-include", os.path.join(HERE, "ref_shim.h"), cpp, "-o", so]
    subprocess.run(cmd, check=True)


def compile_model(model, workdir, name=None):
    """Compile the model's generated source; return the loaded CDLL."""
    src = model.cuda_source + "\n" + _kernel_wrappers(model)
    key = name or hashlib.sha1(src.encode()).hexdigest()[:16]
    os.makedirs(workdir, exist_ok=True)
    cpp = os.path.join(workdir, "ref_%s.cpp" % key)
    so = os.path.join(workdir, "ref_%s.so" % key)
    if not os.path.exists(so) or name:
        with open(cpp, "w") as fh:
            fh.write(src)
        compile_cpp(cpp, so)
    return ctypes.CDLL(so), cpp


def bind_kernels(model, lib, threads):
    """Replace the stub kernels with ctypes calls into the compiled source."""
    def arg(v):
        if hasattr(v, "arr"):
            return v.arr.ctypes.data_as(ctypes.c_void_p)
        if isinstance(v, (np.integer, int, np.bool_, bool)):
            return ctypes.c_int32(int(v))
        if isinstance(v, (np.floating, float)):
            return ctypes.c_float(float(v))
        raise TypeError(type(v))

    def make(name):
        fn = getattr(lib, "xkref_" + name)

        def call(*args, block=None, grid=None):
            fn(ctypes.c_int(threads), *[arg(a) for a in args])
        return call
    model.gpu.kernels.emit = make("emit")
    model.gpu.kernels.absorb = make("absorb")
    model.gpu.kernels.render = make("render")


def run_job(job):
    if job.get("py_random_seed") is not None:
        # some example experiments draw from Python's global random stream when
        # their module is imported; seed it so two processes build the same
        import random
        random.seed(job["py_random_seed"])
    model_cls = _load_obj(job["model"])
    exp_cls = _load_obj(job["experiment"])
    overrides = dict(job.get("exp_overrides", {}))
    for key, val in list(overrides.items()):
        if isinstance(val, list) and key == "size":
            overrides[key] = tuple(val)
    if overrides:
        exp_cls = type("XkJobExperiment", (exp_cls,), overrides)
    model = model_cls(exp_cls, **job.get("model_kwargs", {}))
    threads = int(job.get("threads", 1))
    lib, cpp = compile_model(model, job.get("workdir") or tempfile.mkdtemp(), job.get("name"))
    bind_kernels(model, lib, threads)
    n = model.cells_num
    res = {"cells_num": np.int64(n), "size": np.array(model.size),
           "dtype": np.array(str(model.main.dtype.__name__
                                 if hasattr(model.main.dtype, "__name__")
                                 else model.main.dtype)),
           "init_cells": model.gpu.arrays.cells.get()[:n],
           "cpp": np.array(cpp)}
    if job.get("time_steps"):
        k = int(job["time_steps"])
        model.step()
        t0 = time.perf_counter()
        for _ in range(k):
            model.step()
        dt = time.perf_counter() - t0
        res["seconds"] = np.float64(dt)
        res["steps"] = np.int64(k)
        np.savez(job["out"], **res)
        return
    if job.get("load_pickle"):
        model.load(job["load_pickle"])
        res["loaded_cells"] = model.gpu.arrays.cells.get()[:n]
        res["loaded_colors"] = model.gpu.arrays.colors.get()
    viewport = (job.get("render") or {}).get("viewport")
    if viewport:
        model.set_viewport(tuple(viewport))
    set_params = {int(k): v for k, v in job.get("set_params", {}).items()}
    done = 0
    for cp in job.get("checkpoints", []):
        while done < cp:
            for name, val in set_params.get(done, {}).items():
                setattr(model, name, val)
            model.step()
            done += 1
        res["cells_%d" % cp] = model.gpu.arrays.cells.get()[:n]
        res["colors_%d" % cp] = model.gpu.arrays.colors.get()
        if viewport:
            res["img_%d" % cp] = model.render()
    if job.get("save_pickle"):
        model.save(job["save_pickle"])
    if job.get("load_pickle") or job.get("save_pickle"):
        # the random streams after the load / save: the next draws
        res["rng_standard"] = np.int64(model.random.standard.getrandbits(32))
        res["rng_numpy"] = model.random.numpy.randint(0, 2 ** 31 - 1, 4)
    np.savez(job["out"], **res)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True)
    ap.add_argument("--job", required=True)
    args = ap.parse_args()
    sys.dont_write_bytecode = True
    _install_stubs()
    sys.path.insert(1, args.ref)
    job = json.loads(args.job)
    for extra in job.get("sys_path", []):
        sys.path.insert(1, extra)
    run_job(job)


def run_reference(job, ref_root, timeout=3600):
    """Run ``job`` in a fresh interpreter; return the loaded npz dict."""
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    out = job.get("out")
    if not out:
        fd, out = tempfile.mkstemp(suffix=".npz", prefix="xk_ref_")
        os.close(fd)
        job = dict(job, out=out)
    subprocess.run([sys.executable, os.path.abspath(__file__), "--ref", ref_root,
                    "--job", json.dumps(job)], check=True, env=env,
                   timeout=timeout, cwd=tempfile.gettempdir())
    with np.load(out) as data:
        return {k: data[k] for k in data.files}


if __name__ == "__main__":
    main()
