r"""In-tree build of the native parts of pyci_gb300.

* ``pyci_gb300/lib/libpyci_gb300.so`` -- the sm_103a kernels and the C ABI of
  ``include/pyci_gb300.h`` (nvcc, ``-gencode arch=compute_103a,code=sm_103a``);
* ``pyci_gb300/_pyci*.so`` -- the C++ host module mirroring the reference's
  ``pyci._pyci`` classes, linked against the library (g++, pybind11 headers as
  shipped inside torch, no other dependency).

Translation units compile in parallel; nothing is rebuilt when its outputs are
newer than every source.
"""

import concurrent.futures
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
INCLUDE = os.path.join(ROOT, "include")
LIBNAME = "libpyci_gb300.so"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["build.cu", "spmv.cu", "ops.cu", "davidson.cu", "batch.cu", "capi.cu", "noalloc.cu", "gram_tc.cu", "hci.cu", "rdm.cu", "fcix.cu", "docx.cu"]
CPP_SOURCES = ["dense.cpp"]
HEADERS = ["internal.h", "detops.cuh", "dense.h", "split_bits.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _pybind_include():
    try:
        import torch.utils.cpp_extension as ce  # torch ships pybind11 headers
        for p in ce.include_paths():
            if os.path.exists(os.path.join(p, "pybind11", "pybind11.h")):
                return p
    except Exception:
        pass
    try:
        import pybind11
        return pybind11.get_include()
    except Exception:
        raise RuntimeError("pybind11 headers not found (neither torch's copy nor the pybind11 package)")


def build_library(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "pyci_gb300.h")]
    common = ["-O3", "-std=c++17", "-I" + INCLUDE, "-I" + CSRC]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers + [__file__]):
            jobs.append([NVCC] + ARCH + common + ["-lineinfo", "-Xcompiler", "-fPIC",
                                                  "--expt-relaxed-constexpr", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers + [__file__]):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(LIBDIR, LIBNAME)
    if _newer(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lpthread"])
    return lib


def build_host_module(verbose=False):
    src = os.path.join(CSRC, "host", "pyci_module.cpp")
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    out = os.path.join(HERE, "_pyci" + suffix)
    lib = os.path.join(LIBDIR, LIBNAME)
    if not _newer(out, [src, lib, os.path.join(INCLUDE, "pyci_gb300.h"), __file__]):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
           "-I" + INCLUDE, "-I" + _pybind_include(),
           "-I" + sysconfig.get_paths()["include"], src, "-o", out,
           "-L" + LIBDIR, "-lpyci_gb300", "-Wl,-rpath,$ORIGIN/lib"]
    text = _run(cmd)
    if verbose and text.strip():
        print(text)
    return out


def build(verbose=False):
    lib = build_library(verbose)
    mod = build_host_module(verbose)
    return lib, mod


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
