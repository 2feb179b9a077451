"""Build recipe for the oracle (test infrastructure only).

* ``oracle/liboracle.so`` — the C restatement in ``pcf_oracle.c``; built on
  every machine (gcc, ``-ffp-contract=off`` so x86-64 and aarch64 round the
  same way).
* ``oracle/liboracle_o3_off.so`` / ``liboracle_o3_fast.so`` — the same source
  built ``-O3`` for the host CPU without and with FMA contraction; only the
  CPU-baseline timings use them.
* ``oracle/_ref/libsbref.so`` — ``ref_harness.cpp`` compiled against the
  stablebear reference's own headers.  Built only when the reference tree is
  present: ``SBREF_ROOT`` when set, else a stablebear checkout named
  ``reference`` beside this repository's directory.  The reference is never
  copied into this repository.
* ``oracle/_ref/ref_kernels.cubin`` + ``ref_kernels.json`` — the reference's
  own CUDA block kernel (``ref_gpu_kernel.cu`` instantiating
  ``include/sbear/cuda/cuda_pcf_kernel.cuh``), device code only, for sm_103a,
  with its entry names as ptxas prints them.  Built only where the reference
  tree is present; a cubin carries no host code, so it also loads on hosts of
  another CPU architecture.
* ``oracle/_ref/libsbrefgpu.so`` — ``ref_gpu.cpp``, the host harness that
  loads that cubin through the CUDA driver API; built wherever the CUDA
  toolkit is (it holds no reference code).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libsbref.so")
REF_ROOT = os.environ.get("SBREF_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "pcf_oracle.c")
    if force or _stale(ORACLE_SO, [src, __file__]):
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", ORACLE_SO, src, "-lpthread", "-lm"]
        subprocess.run(cmd, check=True)
    return ORACLE_SO


# Timed CPU-baseline builds of the same source: optimised for the host CPU,
# once without and once with FMA contraction (the reference's own builds use
# gcc defaults, which contract `val += (r - l) * op` into an FMA where the
# target has one).  The bitwise parity tests keep the -O2 -ffp-contract=off
# build above; these two only time the CPU path.
TIMED_SO = {"off": os.path.join(HERE, "liboracle_o3_off.so"), "fast": os.path.join(HERE, "liboracle_o3_fast.so")}


def native_cpu_flag() -> str:
    import platform
    # gcc spells "tune and select instructions for this CPU" -mcpu on Arm, -march on x86
    return "-mcpu=native" if platform.machine().lower() in ("aarch64", "arm64") else "-march=native"


def build_oracle_timed(contract: str = "fast", force: bool = False) -> str:
    if contract not in TIMED_SO:
        raise ValueError("contract must be 'off' or 'fast'")
    src = os.path.join(HERE, "pcf_oracle.c")
    out = TIMED_SO[contract]
    if force or _stale(out, [src, __file__]):
        cmd = ["gcc", "-O3", native_cpu_flag(), "-std=c11", f"-ffp-contract={contract}", "-fPIC", "-shared",
               "-o", out, src, "-lpthread", "-lm"]
        subprocess.run(cmd, check=True)
    return out


def build_ref(force: bool = False) -> str | None:
    inc = os.path.join(REF_ROOT, "include")
    if not os.path.isdir(os.path.join(inc, "sbear")):
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    os.makedirs(REF_DIR, exist_ok=True)
    if force or _stale(REF_SO, [src, __file__]):
        cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared",
               "-I", inc, "-o", REF_SO, src]
        subprocess.run(cmd, check=True)
    return REF_SO


REF_CUBIN = os.path.join(REF_DIR, "ref_kernels.cubin")
REF_ENTRIES = os.path.join(REF_DIR, "ref_kernels.json")
REF_GPU_SO = os.path.join(REF_DIR, "libsbrefgpu.so")


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isdir(os.path.join(cand, "include")):
            return cand
    raise RuntimeError("CUDA toolkit not found")


def build_ref_gpu_kernel(force: bool = False) -> str | None:
    """The reference's block kernel as a cubin, plus its entry names."""
    import json
    import re
    inc = os.path.join(REF_ROOT, "include")
    if not os.path.isdir(os.path.join(inc, "sbear")):
        return None
    src = os.path.join(HERE, "ref_gpu_kernel.cu")
    os.makedirs(REF_DIR, exist_ok=True)
    if force or _stale(REF_CUBIN, [src, __file__]) or not os.path.exists(REF_ENTRIES):
        nvcc = os.path.join(_cuda_home(), "bin", "nvcc")
        # the reference's CUDA options (CMakeLists.txt: --expt-relaxed-constexpr,
        # BUILD_WITH_CUDA=1, release optimisation); whole-program device code
        cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
               "--expt-relaxed-constexpr", "-DBUILD_WITH_CUDA=1", "-Xptxas", "-v", "-I", inc,
               "-o", REF_CUBIN, src]
        r = subprocess.run(cmd, capture_output=True, text=True, check=True)
        names = re.findall(r"Compiling entry function '([^']+)'", r.stdout + r.stderr)
        entries = {}
        for nm in names:
            # the template arguments <float, float, ...> / <double, double, ...> mangle as "Iff" / "Idd"
            suffix = "_f32" if "integrateIff" in nm else ("_f64" if "integrateIdd" in nm else None)
            if suffix is None:
                continue
            for key, tag in (("l1", "OperationL1Dist"), ("lp", "OperationLpDist"), ("inner", "OperationL2InnerProduct")):
                if tag in nm:
                    entries[key + suffix] = nm
        with open(REF_ENTRIES, "w") as f:
            json.dump(entries, f, indent=1)
    return REF_CUBIN


def build_ref_gpu_harness(force: bool = False) -> str:
    src = os.path.join(HERE, "ref_gpu.cpp")
    os.makedirs(REF_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "sbgpu", "compat.hpp")
    if force or _stale(REF_GPU_SO, [src, hdr, __file__]):
        cuda = _cuda_home()
        libdirs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib64", "stubs"),
                               os.path.join(cuda, "targets", "sbsa-linux", "lib", "stubs")) if os.path.isdir(d)]
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(cuda, "include"),
               "-o", REF_GPU_SO, src] + [f"-L{d}" for d in libdirs] + ["-lcuda"]
        subprocess.run(cmd, check=True)
    return REF_GPU_SO


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_oracle_timed("off", force))
    print(build_oracle_timed("fast", force))
    print(build_ref(force))
    print(build_ref_gpu_kernel(force))
    print(build_ref_gpu_harness(force))
