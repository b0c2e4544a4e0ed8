"""In-tree build of the native libraries (no setuptools, no cmake).

- ``liblue_gb300.so``: the CUDA kernels and the C-ABI of include/lue_gb300.h, compiled by nvcc for
  sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), one object per translation unit, compiled
  in parallel, linked with ``nvcc -shared``.
- ``liblue_synth.so``: the synthetic-terrain generator (gcc, ``-ffp-contract=off`` so that x86-64 and
  aarch64 produce identical bytes).

Outputs go to ``lue_gb300/_build/``; a library is rebuilt when any of its sources is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-lineinfo", GENCODE, "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def gpu_library(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    target = os.path.join(BUILD, "liblue_gb300.so")
    srcs = cuda_sources()
    hdrs = headers()
    if not force and not _stale(target, srcs + hdrs + [__file__]):
        return target
    objs = []
    cmds = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs + [__file__]):
            cmds.append([nvcc(), *NVCC_FLAGS, "-Xptxas", "-v" if verbose else "-O3", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(len(cmds) or 1, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        for log in logs:
            print(log)
    tmp = target + f".tmp{os.getpid()}"
    _run([nvcc(), GENCODE, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, target)
    return target


def synth_library(force=False):
    os.makedirs(BUILD, exist_ok=True)
    target = os.path.join(BUILD, "liblue_synth.so")
    src = os.path.join(CSRC, "synthetic.c")
    if force or _stale(target, [src, __file__]):
        tmp = target + f".tmp{os.getpid()}"
        _run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", tmp, src, "-lm"])
        os.replace(tmp, target)
    return target


def cpp_example(force=False):
    """The C++ mirror's example program (examples/accu_example.cpp), linked against liblue_gb300.so."""
    lib = gpu_library()
    target = os.path.join(BUILD, "accu_example")
    src = os.path.join(PKG, "examples", "accu_example.cpp")
    hpp = os.path.join(CSRC, "lue_gb300.hpp")
    if force or _stale(target, [src, hpp, lib, __file__]):
        cuda = os.path.dirname(os.path.dirname(nvcc()))
        tmp = target + f".tmp{os.getpid()}"
        _run(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include"), src,
              "-o", tmp, "-L" + BUILD, "-llue_gb300", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
              "-Wl,-rpath," + BUILD])
        os.replace(tmp, target)
    return target


def build_all(force=False, verbose=False):
    return {"gpu": gpu_library(force, verbose), "synth": synth_library(force), "cpp_example": cpp_example(force)}
