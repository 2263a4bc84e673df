"""The rollouts' branch-free division and angle wrap (FastArith, mppi_generic_vendor_gb300/csrc/mg_math.cuh) against
their IEEE definitions on the GPU: compiles tests/cuda/fast_arith_check.cu with the library's device flags and runs
it on every 64th significand of the dividend (every divisor significand; 2^40 pairs), every float for the wrap.  Run
the program with stride 1 for all 2^46 significand pairs (about 40 s on a GB300)."""
import subprocess
from pathlib import Path

import pytest

from mppi_generic_vendor_gb300 import build as B

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_fast_arith_matches_ieee(tmp_path):
    exe = tmp_path / "fast_arith_check"
    subprocess.run([B.nvcc_path(), *B.ARCH_FLAGS, "-O3", "-std=c++17", "--fmad=false",
                    str(ROOT / "tests" / "cuda" / "fast_arith_check.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "64"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 not correctly rounded, 0 reported invalid" in r.stdout, r.stdout
    assert "0 mismatches" in r.stdout, r.stdout
