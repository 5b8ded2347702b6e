"""The FP32-pipe FP64-accurate arithmetic the streaming kernels use (dfloat.cuh): exact
split and join, sums and products, against FP64 on the device."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "2d_dvm_microflows_gb300", "csrc")


def test_dfloat_accuracy(gpulib, tmp_path):
    exe = tmp_path / "dfl_selftest"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", CSRC, os.path.join(HERE, "csrc", "dfl_selftest.cu"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout.split()
    assert out[0] == "ok", out
    split, add, mul, fma, total = (float(v) for v in out[1:])
    assert split <= 2.0 ** -47  # the split keeps 48 significant bits, rounded
    assert add <= 2.0 ** -44
    assert mul <= 2.0 ** -44
    assert fma <= 2.0 ** -44
    assert total <= 1e-13  # 256 terms, each rounding at most about 2^-48 of the sum


def test_pair_power_accuracy(tmp_path):
    """dfl_pow, the pair x^q the collide kernel uses for g^(2 - 2 omega) on grids without a
    speed table and for the VSS polar angle, against the FP64 pow: within 2e-14 relative for
    arguments from 1e-20 to 1e5 and the exponents of the molecular models ((2 - 2 omega)/2
    for VHS omega 0.55 to 0.95, 1/alpha for VSS alpha 1.01 and 1.4)."""
    exe = tmp_path / "dfl_pow_selftest"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", CSRC, os.path.join(HERE, "csrc", "dfl_pow_selftest.cu"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout.split()
    assert out[0] == "ok", out
    errs = [float(v) for v in out[1:]]
    assert len(errs) == 7
    assert max(errs) <= 2e-14, errs
