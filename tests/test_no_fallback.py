"""The product path has no CPU fallback: without the built library, or
without a CUDA device, every solve raises instead of returning results.

Both checks run on a machine without a GPU; on a GPU machine the second one
is skipped (the GPU tests cover the working path there).
"""
import os
import subprocess
import sys

import pytest

from tests.problems import media, small_cfg, stations

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_missing_library_raises_on_load():
    code = ("from fd2d_noise_gb300 import _lib\n"
            "try:\n"
            "    _lib.load('/nonexistent/libfd2d.so')\n"
            "except ImportError as e:\n"
            "    print('raised:', e)\n"
            "else:\n"
            "    raise SystemExit('loaded a library that does not exist')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "raised:" in r.stdout and "no CPU fallback" in r.stdout


def _has_gpu() -> bool:
    import torch
    return torch.cuda.is_available()


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a CUDA device")
def test_solve_without_device_raises(fd2d_lib):
    from fd2d_noise_gb300 import _lib, solvers
    cfg = small_cfg(nx=24, nz=20, nt=8, order=4, K=4, fs=5, fw=1)
    mu, rho = media(cfg)
    src, rec = stations(cfg, 1, seed=3), stations(cfg, 2, seed=4)
    for prec in ("fp32", "fp64"):
        with pytest.raises(_lib.FD2DError) as e:
            solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision=prec)
        assert e.value.status == 8 and "no CUDA device" in str(e.value)
