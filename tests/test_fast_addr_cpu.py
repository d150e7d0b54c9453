"""Host check of the fast kernels' shared-memory address arithmetic (no GPU).

``tests/cpu/fast_addr_check.cu`` includes ``gbs_fast.cuh`` and is built by
nvcc as a host program: the bank swizzle is a permutation inside every
128-byte group, ``swz_join`` agrees with the swizzle on disjoint operands,
the register order of ``run()`` is a permutation that ``inv_outm``
inverts, and the per-pair shared memory of ``kf3_xr`` keeps its buffers
aligned.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_fast_address_arithmetic(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "fast_addr_check"
    cmd = [nvcc, "-std=c++17", "-O1", "-I", str(HERE.parent / "include"),
           str(HERE / "cpu" / "fast_addr_check.cu"), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and run.stdout.strip() == "ok", run.stdout + run.stderr
