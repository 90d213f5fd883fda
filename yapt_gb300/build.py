"""Build recipe for the native parts of yapt_gb300 (in-tree, no cmake).

Outputs (git-ignored, next to this file):
  libyaptgpu.so        CUDA kernels for sm_103a + the C ABI of include/yapt_gpu.h
  py_yapt*.so          pybind11 module mirroring YAPT's Python surface

Device code is compiled with -fmad=false -prec-div=true -prec-sqrt=true
-ftz=false so that its floating-point results are reproducible operation by
operation; host code that must agree with it is compiled with -ffp-contract=off.
"""
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(CUDA_HOME, "include"),
             "-Wall", "-Wno-unused-function"]

# extra nvcc flags for experiments on variants (e.g. YG_NVCC_EXTRA="-DYG_EVAL_OUTLINE"); empty normally
NVCC_FLAGS += os.environ.get("YG_NVCC_EXTRA", "").split()

CUDA_SOURCES = ["yg_integrator.cu", "yg_bdpt.cu", "yg_serve_kernels.cu", "yg_nn.cu", "yg_bvh_build.cu", "yg_atrous.cu", "yg_display.cu", "yg_capi.cu"]
CXX_SOURCES = ["yg_tables.cpp", "yg_server.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hs


def build_lib(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append([NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    lib = os.path.join(HERE, "libyaptgpu.so")
    if jobs or not os.path.exists(lib):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lpthread"])
    return lib


def build_pybind(verbose=False):
    """py_yapt: pybind11 bindings (headers bundled with torch) over libyaptgpu.so."""
    import torch  # noqa: F401  (only for the bundled pybind11 headers)
    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    py_inc = sysconfig.get_paths()["include"]
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    src = os.path.join(CSRC, "py_yapt.cpp")
    out = os.path.join(HERE, "py_yapt" + ext)
    if _newer(out, [src, os.path.join(HERE, "libyaptgpu.so")] + _headers()):
        return out
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + torch_inc, "-I" + py_inc,
          "-I" + os.path.join(ROOT, "include"), src, "-o", out, "-L" + HERE, "-lyaptgpu",
          "-Wl,-rpath,$ORIGIN"])
    return out


def build_all(verbose=False):
    lib = build_lib(verbose)
    mods = [lib]
    if os.path.exists(os.path.join(sysconfig.get_paths()["include"], "Python.h")):
        mods.append(build_pybind(verbose))
    else:
        print("py_yapt not built: no Python development headers (Python.h) on this machine", file=sys.stderr)
    return mods


if __name__ == "__main__":
    for p in build_all(verbose=True):
        print(p)
