"""Builds the host-side Model module ``core`` (C++ with pybind11) into _build/.

pybind11's headers come from the PyTorch installation (torch/include), which
ships them on every machine this package runs on; Python's own headers come from
sysconfig.  The module links libmgr_gpu.so with an $ORIGIN rpath.
"""
import concurrent.futures as cf
import os
import subprocess
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
HOST = os.path.join(PKG, "csrc", "host")
BUILD = os.path.join(PKG, "_build")
SOURCES = ["model.cpp", "bindings.cpp"]


def core_path():
    return os.path.join(BUILD, "core" + sysconfig.get_config_var("EXT_SUFFIX"))


def _pybind11_include():
    import torch  # only for the location of its bundled pybind11 headers
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    if not os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
        raise RuntimeError("pybind11 headers not found under " + inc)
    return inc


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_core(verbose=False, force=False):
    from .build import GPU_LIB, _newer
    out = core_path()
    srcs = [os.path.join(HOST, s) for s in SOURCES]
    deps = srcs + [os.path.join(HOST, "model.hpp"), os.path.join(ROOT, "include", "magritte_gb300.h"), GPU_LIB,
                   __file__]
    if not force and _newer(out, deps):
        return out
    cxx = os.environ.get("CXX", "g++")
    flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
             "-I", _pybind11_include(), "-I", sysconfig.get_paths()["include"]]
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(_run, [[cxx] + flags + ["-c", s, "-o", o] for s, o in zip(srcs, objs)]))
    tmp = out + ".tmp"
    _run([cxx, "-shared", "-o", tmp] + objs + ["-L", BUILD, "-l:libmgr_gpu.so", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, out)
    return out
