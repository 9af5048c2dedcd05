"""The tile partitions of the two-stream launches, checked on the host: the
near / far parts of a block step's panel tiles and of a front's
tensor-core Schur tiles (spk_kernels.cuh) cover the one-launch form's
tiles exactly once, and a Schur tile lands in the near part exactly when
one of its entries targets a front of the next level.  Compiled with nvcc
(the device code of the header needs it), run on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tile_partitions(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "tile_parts"
    subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "sparspak.jl_gb300", "csrc"),
                    "-o", str(exe), os.path.join(ROOT, "tests", "native", "tile_parts.cu")],
                   check=True, capture_output=True, timeout=600)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0 and out.stdout.strip().endswith("bad 0"), out.stdout + out.stderr
