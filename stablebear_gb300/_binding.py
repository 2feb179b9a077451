"""The compiled binding ``_sb_gb300`` (pybind11, ``pymodule/sb_module.cpp``).

It exposes the reference's pybind classes (``Distance_f32_f32``,
``Distance_f64_f64``, ``InnerProduct_f32_f32``, ``InnerProduct_f64_f64``,
``StoppableTask_void``) as compiled C++ over the C ABI, next to
``libsbgpu.so``.  ``compiled()`` loads it once; where it was not built (no
pybind11 headers or no Python.h on the machine) it returns None and the
ctypes classes in ``distance.py`` serve the same API.  Both bindings call the
same CUDA library; neither has a CPU path.
"""
from __future__ import annotations

import importlib.util
import os
import sysconfig
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(_HERE, "_lib", "_sb_gb300" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

_mod = None
_tried = False
_lock = threading.Lock()


def compiled():
    global _mod, _tried
    if _tried:
        return _mod
    with _lock:
        if not _tried:
            if os.environ.get("SBG_BINDING", "") != "ctypes" and os.path.exists(PATH):
                spec = importlib.util.spec_from_file_location("_sb_gb300", PATH)
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
                _mod = mod
            _tried = True
    return _mod


def name() -> str:
    """Which binding the package's classes use: "pybind11" or "ctypes"."""
    return "pybind11" if compiled() is not None else "ctypes"
