"""The integer-pipe FP64 compares and conversions (openmc_gb300/csrc/
fp64_int.cuh) give the hardware operations' results bit for bit: a small
CUDA program checks each function on 2^26 seeded bit patterns and special
values (signed zeros, infinities, NaNs, subnormals, rounding ties)."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def test_fp64_int_helpers_match_hardware(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "fp64_int_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", str(exe),
                    str(ROOT / "tests" / "native" / "fp64_int_check.cu")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    counts = dict(line.split() for line in r.stdout.strip().splitlines())
    assert int(counts.pop("samples")) == 1 << 26
    assert all(int(v) == 0 for v in counts.values()), counts
    assert r.returncode == 0
