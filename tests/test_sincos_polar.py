"""The mixed tracer's polar sin/cos (nullpath_gb300/csrc/tracer_mixed.cuh)
compiled for the host by nvcc and measured against libm: at most 2 ulps
for sin and cos over (0, pi), including near the poles and the equator
where one of them is small."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_sincos_polar_accuracy(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "probe"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "nullpath_gb300", "csrc"),
                    os.path.join(HERE, "probes", "sincos_polar_probe.cu"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=300).stdout.split()
    n, es, ec = int(out[0]), float(out[1]), float(out[2])
    assert n > 100_000_000 // 7
    assert es <= 2.0 and ec <= 2.0, (es, ec)
