"""Build recipe for the native library ``stablebear_gb300/_lib/libsbgpu.so``.

Every translation unit under ``csrc/`` is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
one shared library with the CUDA runtime linked statically.  The library is
built in-tree (git-ignored) so the Python package loads it from its own
directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libsbgpu.so")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fvisibility=hidden"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build stablebear_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(nvcc: str, src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    extra = list(extra or [])
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    hdrs = _headers() + [__file__]
    objs = [os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s, *hdrs])]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 1)) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, extra) for s, o in todo]
            for f in futs:
                f.result()
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-cudart", "static", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    build_pymodule(force=force, verbose=verbose)
    return LIB


# ---- the compiled Python binding (pybind11) ----------------------------------

PYMODULE_SRC = os.path.join(HERE, "pymodule", "sb_module.cpp")


def pymodule_path() -> str:
    import sysconfig
    return os.path.join(OUT_DIR, "_sb_gb300" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def pybind11_include() -> str | None:
    """pybind11's headers: the pybind11 package where installed, else the
    copy PyTorch ships in its include directory (found without importing
    torch)."""
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    import importlib.util
    spec = importlib.util.find_spec("torch")
    for loc in (spec.submodule_search_locations or []) if spec else []:
        inc = os.path.join(loc, "include")
        if os.path.isfile(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    return None


def build_pymodule(force: bool = False, verbose: bool = False) -> str | None:
    """Compiles ``_sb_gb300`` (host C++ over the C ABI, linked to
    libsbgpu.so).  Returns its path, or None where pybind11's headers or
    Python.h are missing (the ctypes binding then serves the same API)."""
    import sysconfig
    pyinc = sysconfig.get_paths()["include"]
    inc = pybind11_include()
    if inc is None or not os.path.isfile(os.path.join(pyinc, "Python.h")):
        if verbose:
            print(f"_sb_gb300 not built: {'no pybind11 headers' if inc is None else 'no Python.h in ' + pyinc}")
        return None
    out = pymodule_path()
    if force or _stale(out, [PYMODULE_SRC, LIB, os.path.join(INCLUDE, "sbgpu.h"), __file__]):
        cxx = shutil.which("g++") or shutil.which("c++")
        if cxx is None:
            raise RuntimeError("no C++ compiler for the _sb_gb300 binding")
        cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I", pyinc, "-I", inc,
               "-I", INCLUDE, PYMODULE_SRC, "-L", OUT_DIR, "-lsbgpu", "-Wl,-rpath,$ORIGIN", "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"_sb_gb300 build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(out + ".tmp", out)
    if verbose:
        print(out)
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
