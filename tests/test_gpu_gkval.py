"""The GEOKERR validation harness with the library's GPU solver as the port
(geokerr_complete_stream_cuda through the C ABI) and the CPU restatement as
the reference, as the reference's `gkval validate` runs its CUDA port against
the Fortran GEOKERR."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import geokerr_golden as gg  # noqa: E402
import oracle  # noqa: E402
from nullpath_gb300 import geokerr as gk  # noqa: E402

pytestmark = pytest.mark.gpu

# u0 mu0 uf a lam q2: the reference CLI's built-in case, then outgoing rays
# with polar turning points, an equatorial ray and a near-extremal spin.
CASES = [
    (0.1, 0.8, 0.01, 0.5, 2.0, 4.0),
    (0.05, 0.3, 0.001, 0.9, -3.0, 12.0),
    (0.02, 0.0, 0.001, 0.7, 3.0, 0.0),
    (0.2, -0.4, 0.002, 0.998, 1.5, 20.0),
    (0.01, 0.5, 0.001, 0.3, 0.5, 8.0),
    (0.08, -0.1, 0.004, 0.95, -1.0, 25.0),
]


def _run(args, cwd, ok=(0,)):
    p = subprocess.run([oracle.GKVAL_BIN] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert p.returncode in ok, (args, p.returncode, p.stdout, p.stderr)
    return p


def _ledger(run):
    return [json.loads(l) for l in (run / "ledger.ndjson").read_text().splitlines() if l.strip()]


@pytest.fixture()
def cases_file(tmp_path):
    (tmp_path / "cases.txt").write_text("".join("%r %r %r %r %r %r 0\n" % c for c in CASES))
    return tmp_path


def test_gkval_gpu_port_passes_fp64_profile(cuda, cases_file):
    """Every case passes |gpu - cpu| <= 1e-10 (1 + |x|) on u, mu, t, phi and
    affine over the adaptive 4096-sample grid, and the run audits clean."""
    tmp = cases_file
    _run(["init", "--run-id", "GPU", "--atol", "1e-10", "--rtol", "1e-10", "--max-ulps", str(10 ** 15)], tmp)
    p = _run(["validate", "GPU", "--cases", "cases.txt", "--port", "gpu"], tmp)
    print(p.stdout)
    led = _ledger(tmp / "runs" / "GPU")
    assert len(led) == len(CASES) and all(l["success"] for l in led), p.stdout
    assert all(max(l["max_abs"]) < 1e-9 for l in led)
    assert "%d verified, 0 mismatched" % len(CASES) in _run(["audit", "GPU"], tmp).stdout


def test_gkval_gpu_port_bitexact_windows(cuda, cases_file):
    """Under the bit-exact profile every failing case's window holds the CPU
    reference and the GPU port samples at the reported index, and the
    first-failure index is the first sample whose bits differ."""
    tmp = cases_file
    _run(["init", "--run-id", "BX", "--profile", "bitexact"], tmp)
    p = _run(["validate", "BX", "--cases", "cases.txt", "--port", "gpu"], tmp, ok=(0, 2))
    print(p.stdout)
    run = tmp / "runs" / "BX"
    led = _ledger(run)
    assert len(led) == len(CASES)
    assert "%d verified, 0 mismatched" % len(CASES) in _run(["audit", "BX"], tmp).stdout
    names = ["u", "mu", "t", "phi", "affine"]
    lib = oracle.gkval()
    for l, c in zip(led, CASES):
        if l["success"]:
            continue
        f = names.index(l["first_fail"]["field"])
        idx = l["first_fail"]["index"]
        dlam = np.frombuffer(np.uint64(l["grid"]["dlam_bits"]).tobytes(), np.float64)[0]
        rc, port = gk.stream(c[0], c[2], c[1], c[3], c[4], c[5], 0.0, dlam, 4096, complete=True)
        assert rc == 0
        ref = oracle.geokerr_eval_lambda(c[0], c[1], c[2], c[3], c[4], c[5], 0.0, 0.0, dlam, 4096)
        for k in range(f):   # earlier fields agree bit for bit
            assert np.array_equal(ref[names[k]].view(np.uint64), port[names[k]].view(np.uint64))
        seg = idx - idx % 1024
        a, b = ref[names[f]][seg:seg + 1024].copy(), port[names[f]][seg:seg + 1024].copy()
        if f == 3:
            for x in (a, b):
                lib.gkv_unwrap(x.ctypes.data, x.size)
        diff = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
        assert diff.size and seg + diff[0] == idx
        wins = list((run / "fail_windows" / str(l["case_id"])).iterdir())
        assert len(wins) == 1
        w = gg.read_fail_window(str(wins[0]))
        assert w["field"] == f and w["start"] <= idx < w["end"]
        assert np.array_equal(w["ref"], a[w["start"] - seg:w["end"] - seg])
        assert np.array_equal(w["port"], b[w["start"] - seg:w["end"] - seg])
