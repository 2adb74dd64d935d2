"""Double-float arithmetic of the mixed path's FP64-class islands
(nullpath_gb300/csrc/dfloat.cuh), compiled for the host by nvcc with FP
contraction off (the device code uses round-to-nearest intrinsics that never
contract), against exact rational arithmetic and mpmath:
  + and -   relative error <= 4 u^2      (u = 2^-24; the bounds of the
  *         relative error <= 6 u^2       algorithms are 3, 5 and 15 u^2)
  /         relative error <= 16 u^2
  sin, cos  absolute error <= 8e-15 on (-0.1, pi + 0.1)."""
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
U2 = Fraction(1, 2 ** 48)


def _df(rng, n, lo_exp=-30, hi_exp=30):
    """n random normalised DF values (hi, lo) as float32 pairs."""
    hi = (rng.uniform(1, 2, n) * np.exp2(rng.integers(lo_exp, hi_exp, n)) * rng.choice([-1, 1], n)).astype(np.float32)
    ulp = np.spacing(np.abs(hi)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, n) * ulp).astype(np.float32)
    return hi, lo


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path_factory.mktemp("df") / "probe"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "nullpath_gb300", "csrc"),
                    os.path.join(HERE, "probes", "dfloat_probe.cu"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)

    def run(lines):
        out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", check=True, capture_output=True,
                             text=True, timeout=300).stdout.split("\n")
        return [[float.fromhex(v) for v in l.split()] for l in out if l.strip()]
    return run


def _hex(x):
    return float(x).hex()


@pytest.mark.parametrize("op,bound", [("+", 4), ("-", 4), ("*", 6), ("/", 16)])
def test_df_arithmetic(probe, op, bound):
    rng = np.random.default_rng(7)
    n = 4000
    ah, al = _df(rng, n)
    bh, bl = _df(rng, n)
    if op in "+-":
        # heavy cancellation: b close to -a (for +) or a (for -)
        k = n // 4
        bh[:k] = -ah[:k] if op == "+" else ah[:k]
        bl[:k] = (rng.uniform(-1, 1, k) * np.spacing(np.abs(ah[:k]))).astype(np.float32)
    lines = ["%s %s %s %s %s" % (op, _hex(a), _hex(b), _hex(c), _hex(d)) for a, b, c, d in zip(ah, al, bh, bl)]
    res = probe(lines)
    worst = Fraction(0)
    for i, r in enumerate(res):
        x = Fraction(float(ah[i])) + Fraction(float(al[i]))
        y = Fraction(float(bh[i])) + Fraction(float(bl[i]))
        exact = {"+": x + y, "-": x - y, "*": x * y, "/": x / y if y != 0 else None}[op]
        got = Fraction(r[0]) + Fraction(r[1])
        if exact is None or exact == 0:
            assert got == 0
            continue
        worst = max(worst, abs(got - exact) / abs(exact))
    assert worst <= bound * U2, float(worst / U2)


def test_df_sincos(probe):
    import mpmath
    mpmath.mp.prec = 160
    rng = np.random.default_rng(11)
    th = np.concatenate([rng.uniform(-0.1, np.pi + 0.1, 3000), np.pi / 2 + rng.uniform(-1e-6, 1e-6, 500),
                         rng.uniform(0, 1e-6, 200), np.pi - rng.uniform(0, 1e-6, 200)])
    hi = th.astype(np.float32)
    lo = (th - hi.astype(np.float64)).astype(np.float32)
    res = probe(["s %s %s 0x0p+0 0x0p+0" % (_hex(a), _hex(b)) for a, b in zip(hi, lo)])
    es = ec = 0.0
    for i, r in enumerate(res):
        x = mpmath.mpf(float(hi[i])) + mpmath.mpf(float(lo[i]))
        es = max(es, float(abs(mpmath.mpf(r[0]) + mpmath.mpf(r[1]) - mpmath.sin(x))))
        ec = max(ec, float(abs(mpmath.mpf(r[2]) + mpmath.mpf(r[3]) - mpmath.cos(x))))
    assert es <= 8e-15 and ec <= 8e-15, (es, ec)
