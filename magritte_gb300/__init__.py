"""magritte_gb300: the formal-solve hot path of Magritte on GB300 (sm_103a).

``magritte_gb300.core`` is the host Model (C++, pybind11) with the reference's
Python API; it runs the formal solve through libmgr_gpu.so (include/magritte_gb300.h).
Both are built in-tree by ``magritte_gb300.build``.
"""
import importlib.machinery
import importlib.util
import os
import sys

__version__ = "0.1.0"

_HERE = os.path.dirname(os.path.abspath(__file__))


def _load_core():
    from ._corebuild import core_path
    path = core_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run `python -m magritte_gb300.build` first")
    loader = importlib.machinery.ExtensionFileLoader("magritte_gb300.core", path)
    spec = importlib.util.spec_from_file_location("magritte_gb300.core", path, loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    sys.modules["magritte_gb300.core"] = mod
    return mod


def __getattr__(name):
    if name == "core":
        mod = _load_core()
        globals()["core"] = mod
        return mod
    raise AttributeError(name)
