"""Build recipe for the oracle (test infrastructure only).

* ``oracle/liboracle.so`` — the C restatement in ``pcf_oracle.c``; built on
  every machine (gcc, ``-ffp-contract=off`` so x86-64 and aarch64 round the
  same way).
* ``oracle/_ref/libsbref.so`` — ``ref_harness.cpp`` compiled against the
  stablebear reference's own headers.  Built only when the reference tree is
  present (``SBREF_ROOT``, default ``/root/reference``); the reference is
  never copied into this repository.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libsbref.so")
REF_ROOT = os.environ.get("SBREF_ROOT", "/root/reference")


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


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
