"""The integer FP32 <-> FP64 conversions of the contraction epilogue and the
injection planes (csrc/fp_bits.cuh) against the C conversions, on the CPU."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_the_hardware_rounding(tmp_path):
    exe = str(tmp_path / "fp_bits_check")
    src = os.path.join(HERE, "fp_bits_check.cpp")
    inc = os.path.join(HERE, "..", "fd2d_noise_gb300", "csrc")
    try:
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", inc, src, "-o", exe], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError) as e:
        pytest.skip(f"no host compiler: {e}")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
