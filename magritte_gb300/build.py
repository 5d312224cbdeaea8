"""Builds the in-tree native libraries of magritte_gb300.

  * ``_build/libmgr_gpu.so``  -- the CUDA formal-solve library (C ABI in
    include/magritte_gb300.h), compiled for sm_103a only.
  * ``_build/core*.so``       -- the host-side Model (C++) with pybind11 bindings,
    linked against libmgr_gpu.so.

Translation units compile in parallel.  Host code is compiled with
-ffp-contract=off so that a*b+c rounds as on the reference's x86-64 build on every
architecture (the GPU machine is aarch64, where GCC would otherwise contract).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
GPU_LIB = os.path.join(BUILD, "libmgr_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["mgr_abi.cu", "mgr_fo2.cu", "mgr_noalloc.cu", "mgr_ali.cu", "mgr_sc0.cu", "mgr_image.cu", "mgr_batch.cu", "mgr_adjoint.cu", "mgr_adjoint_fo2.cu", "mgr_peaks.cu"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_gpu(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "magritte_gb300.h"))
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    if not force and _newer(GPU_LIB, srcs + headers + [__file__]):
        return GPU_LIB
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include")]
    if verbose:
        common += ["-Xptxas", "-v"]
    objs = []
    cmds = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        cmds.append([nvcc] + common + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        results = list(ex.map(_run, cmds))
    if verbose:
        for r in results:
            sys.stderr.write(r.stdout + r.stderr)
    tmp = GPU_LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


EMU_LIB = os.path.join(BUILD, "libmgr_emu.so")


def build_emu(force=False):
    """CPU emulation of the kernel's per-lane code, for the test-suite only."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "emu", "mgr_emu.cu")
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    if not force and _newer(EMU_LIB, [src] + headers + [__file__]):
        return EMU_LIB
    tmp = EMU_LIB + ".tmp"
    _run([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp",
                             "-I", os.path.join(ROOT, "include"), src, "-o", tmp, "-lgomp"])
    os.replace(tmp, EMU_LIB)
    return EMU_LIB


def build(verbose=False, force=False):
    build_gpu(verbose=verbose, force=force)
    try:
        from . import _corebuild
    except ImportError:
        _corebuild = None
    if _corebuild is not None:
        _corebuild.build_core(verbose=verbose, force=force)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(GPU_LIB)
