"""The reference's block pipeline (scheduler -> PcfBlockOp::exec_block ->
BlockResultWriter) driven over include/sbgpu/block_op.hpp gives the
factories' results bit for bit (tests/cpp/test_block_op.cpp)."""
import os
import subprocess

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def test_block_pipeline_matches_factories(tmp_path):
    from stablebear_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "test_block_op")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_block_op.cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lsbgpu", "-Wl,-rpath," + os.path.dirname(lib),
                    "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
