"""GEOKERR validation harness (oracle/gkval_core.cpp, oracle/gkval): its
primitives against independent restatements (hashlib SHA-256, numpy), the
reference's fixtures (fail windows, manifests, the cached GEOKERR grid of
geokerr_port/validation/cache/geokerr), and the CLI end to end with the oracle
as both solvers, including a difference planted in the port data."""
import ctypes as C
import hashlib
import json
import math
import os
import shutil
import struct
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import geokerr_golden as gg  # noqa: E402
import oracle  # noqa: E402

MAX64 = 2 ** 64 - 1
CASES = """# u0 mu0 uf a lam q2 [t0]
0.1 0.8 0.01 0.5 2.0 4.0 0
0.05 0.3 0.001 0.9 -3 12
0.02 0 0.001 0.7 3 0
0.2 -0.4 0.002 0.998 1.5 20 0
"""


@pytest.fixture(scope="module")
def gk(built):
    return oracle.gkval()


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _f(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def test_sha256_matches_hashlib(gk):
    rng = np.random.default_rng(1)
    for n in (0, 1, 3, 55, 56, 63, 64, 65, 119, 120, 1000, 4099):
        m = rng.integers(0, 256, n, dtype=np.uint8)
        out = np.zeros(32, np.uint8)
        gk.gkv_sha256(_vp(m) if n else None, n, _vp(out))
        assert out.tobytes() == hashlib.sha256(m.tobytes()).digest(), n


def test_placeholder_hash(gk):
    """The reference's stand-in hash: 64-bit state spread over 32 bytes."""
    m = np.frombuffer(b"leafRUN\x01", np.uint8).copy()
    out = np.zeros(32, np.uint8)
    gk.gkv_placeholder_hash(_vp(m), m.size, _vp(out))
    s = 0x1234567890ABCDEF
    for byte in m.tobytes():
        s = ((s ^ byte) * 0x100000001B3) & MAX64
    assert out.tobytes() == bytes((s >> (8 * (i % 8))) & 0xFF for i in range(32))


def test_ulp_distance(gk):
    d = gk.gkv_ulp_distance
    assert d(1.0, np.nextafter(1.0, 2.0)) == 1
    assert d(1.0, 1.0) == 0 and d(-0.0, 0.0) == 0
    tiny = 5e-324
    # the ordered map keeps -0 and +0 in two slots (gkval_core.c:236-245), so
    # crossing zero costs one ULP more than the count of doubles in between
    assert d(tiny, -tiny) == 3 and d(0.0, tiny) == 1 and d(-tiny, 0.0) == 2 and d(-tiny, -0.0) == 1
    assert d(float("nan"), 1.0) == MAX64 and d(1.0, float("nan")) == MAX64
    assert d(float("inf"), float("inf")) == 0 and d(float("inf"), -float("inf")) == MAX64
    assert d(float("inf"), 1.0) == MAX64
    assert d(1.0, 2.0) == 2 ** 52
    assert d(-1.0, 1.0) == 2 * _bits(1.0) + 1
    rng = np.random.default_rng(2)
    for x in rng.normal(size=200) * 10.0 ** rng.integers(-30, 30, 200):
        k = int(rng.integers(0, 1000))
        y = x
        for _ in range(k):
            y = np.nextafter(y, np.inf)
        assert d(x, y) == k


def test_acceptance_predicate(gk):
    """|a-b| <= atol + rtol max(|a|,|b|) AND ulp <= max_ulps (gkval_core.c:264-299)."""
    rng = np.random.default_rng(3)
    a = rng.normal(size=4000)
    b = a + rng.normal(size=4000) * 10.0 ** rng.integers(-18, -8, 4000)
    b[::97] = a[::97]
    for atol, rtol, mu in ((0.0, 0.0, 0), (1e-12, 1e-12, 2), (1e-3, 1e-3, 100), (1e-10, 0.0, 10 ** 9)):
        want = [(abs(x - y) <= atol + rtol * max(abs(x), abs(y))) and gk.gkv_ulp_distance(x, y) <= mu
                for x, y in zip(a, b)]
        got = [bool(gk.gkv_accept_sample(x, y, atol, rtol, mu)) for x, y in zip(a, b)]
        assert got == want
        first = gk.gkv_first_fail(_vp(a), _vp(b), a.size, atol, rtol, mu)
        assert first == (want.index(False) if False in want else -1)
    assert not gk.gkv_accept_sample(float("nan"), float("nan"), 1.0, 1.0, MAX64)


def test_unwrap(gk):
    x = np.array([0.0, 3.0, -3.0, 3.2, -2.9, 0.1])
    ref = x.copy()
    for i in range(1, ref.size):
        dd = ref[i] - ref[i - 1]
        ref[i] += -2 * math.pi if dd > math.pi else (2 * math.pi if dd < -math.pi else 0.0)
    gk.gkv_unwrap(_vp(x), x.size)
    assert np.array_equal(x, ref)
    assert np.all(np.abs(np.diff(x)) <= math.pi)


def _quant_py(x, lsb):
    """Round-to-nearest-even of the fraction at bit lsb, carry into the exponent."""
    b = _bits(x)
    e = (b >> 52) & 0x7FF
    if e == 0x7FF:
        return None
    if lsb == 0:
        return b
    sign, frac = b & (1 << 63), b & ((1 << 52) - 1)
    unit = 1 << lsb
    tail, kept = frac & (unit - 1), frac & ~(unit - 1)
    if tail > unit // 2 or (tail == unit // 2 and kept & unit):
        kept += unit
        if kept >> 52:
            kept, e = 0, e + 1
            if e >= 0x7FF:
                return None
    return sign | (e << 52) | kept


def test_quantize(gk):
    q = C.c_uint64()
    cases = [1.0, -1.0, 0.1, 1 / 3, 2.5e-310, 1e300, _f(0x3FFFFFFFFFFFFFFF), _f(0x3FF0000000000080),
             _f(0x3FF0000000000180), _f(0x3FF0000000000081), _f(0x7FEFFFFFFFFFFFFF)]
    rng = np.random.default_rng(4)
    cases += list(rng.normal(size=300) * 10.0 ** rng.integers(-300, 300, 300))
    for x in cases:
        for lsb in (0, 1, 8, 20, 52):
            rc = gk.gkv_quantize(float(x), lsb, C.byref(q))
            want = _quant_py(float(x), lsb)
            if want is None:
                assert rc == -4, (x, lsb)
            else:
                assert rc == 0 and q.value == want, (x, lsb)
    # ties: 0x...080 rounds to even (down), 0x...180 rounds up; carry into the next binade
    gk.gkv_quantize(_f(0x3FF0000000000080), 8, C.byref(q))
    assert q.value == 0x3FF0000000000000
    gk.gkv_quantize(_f(0x3FF0000000000180), 8, C.byref(q))
    assert q.value == 0x3FF0000000000200
    gk.gkv_quantize(_f(0x3FFFFFFFFFFFFFFF), 8, C.byref(q))
    assert _f(q.value) == 2.0
    assert gk.gkv_quantize(float("nan"), 8, C.byref(q)) == -4
    assert gk.gkv_quantize(float("inf"), 0, C.byref(q)) == -4
    assert gk.gkv_quantize(_f(0x7FEFFFFFFFFFFFFF), 8, C.byref(q)) == -4   # rounds to infinity
    assert gk.gkv_quantize(1.0, 53, C.byref(q)) == -1


def _leaf_py(run_id, case_id, field, start, end, q):
    return (b"leaf" + run_id.encode() + struct.pack("<QIQQ", case_id, field, start, end) +
            np.asarray(q, "<u8").tobytes())


def test_leaf_node_merkle_sha256(gk):
    q = np.arange(7, dtype=np.uint64) * 0x0123456789
    out = np.zeros(32, np.uint8)
    gk.gkv_hash_leaf(0, b"RUN", 5, 3, 1024, 1031, _vp(q), q.size, _vp(out))
    assert out.tobytes() == hashlib.sha256(_leaf_py("RUN", 5, 3, 1024, 1031, q)).digest()
    node = lambda l, r: hashlib.sha256(b"node" + l + r).digest()
    rng = np.random.default_rng(5)
    for n in (0, 1, 2, 3, 5, 8, 11):
        hs = rng.integers(0, 256, (n, 32), dtype=np.uint8)
        got = np.zeros(32, np.uint8)
        gk.gkv_merkle(0, _vp(hs) if n else None, n, _vp(got))
        lvl = [bytes(h) for h in hs]
        if not lvl:
            want = bytes(32)
        else:
            while len(lvl) > 1:
                lvl = [node(lvl[i], lvl[i + 1]) if i + 1 < len(lvl) else lvl[i] for i in range(0, len(lvl), 2)]
            want = lvl[0]
        assert got.tobytes() == want, n


def test_fail_window_format_and_reference_files(gk, tmp_path):
    """The reference's own fail windows load through the C reader and are
    rewritten byte for byte (gkval_io.c:140-225)."""
    for path in gg.fail_windows():
        w = gg.read_fail_window(path)
        run = tmp_path / os.path.basename(path)
        (run / "fail_windows" / "7").mkdir(parents=True)
        name = "%s_%d_%d.bin" % ("u", w["start"], w["end"])
        shutil.copy(path, run / "fail_windows" / "7" / name)
        ref = np.zeros(w["size"])
        port = np.zeros(w["size"])
        assert gk.gkv_load_fail_window(str(run).encode(), 7, w["field"], w["start"], w["end"], _vp(ref),
                                       _vp(port)) == 0
        assert np.array_equal(ref, w["ref"]) and np.array_equal(port, w["port"], equal_nan=True)
        assert gk.gkv_load_fail_window(str(run).encode(), 7, 1, w["start"], w["end"], _vp(ref), _vp(port)) != 0
        out = tmp_path / ("re_" + os.path.basename(path))
        out.mkdir()
        assert gk.gkv_save_fail_window(str(out).encode(), 7, w["field"], w["start"], w["end"], _vp(ref),
                                       _vp(port)) == 0
        assert (out / "fail_windows" / "7" / name).read_bytes() == open(path, "rb").read()


def test_fail_window_bounds(gk):
    s, e = C.c_uint64(), C.c_uint64()
    for seg, fail, n, want in ((0, 5, 1024, (0, 32)), (0, 137, 1024, (121, 153)), (1024, 1020, 1024, (2016, 2048)),
                               (4096, 3, 10, (4096, 4106)), (0, 202, 1024, (186, 218))):
        gk.gkv_fail_window_bounds(seg, fail, n, 32, C.byref(s), C.byref(e))
        assert (s.value, e.value) == want


def test_adaptive_grid_matches_reference_cache(gk):
    """The per-case lambda grid of the reference's cached GEOKERR run
    (adaptive_lambda, K = 6, S = 4096) is reproduced bit for bit."""
    g = gg.read_cache()
    lam0, dlam = C.c_double(), C.c_double()
    assert gk.gkv_adaptive_grid(g["u0"], g["mu0"], g["uf"], g["a"], g["Lz"], g["Q2"], g["S"], 6.0, C.byref(lam0),
                                C.byref(dlam)) == 0
    assert lam0.value == g["lam0"] and _bits(dlam.value) == _bits(g["dlam"])
    assert gk.gkv_check_fp_env(0) == 0


def _run(args, cwd, ok=(0,)):
    p = subprocess.run([oracle.GKVAL_BIN] + args, cwd=cwd, capture_output=True, text=True, timeout=300)
    assert p.returncode in ok, (args, p.returncode, p.stdout, p.stderr)
    return p


def _ledger(run):
    return [json.loads(l) for l in (run / "ledger.ndjson").read_text().splitlines() if l.strip()]


@pytest.mark.parametrize("name", ["BITEXACT_BASELINE", "CARLSON_TEST_RELAXED", "CARLSON_TEST_MORE_RELAXED"])
def test_manifest_matches_reference_runs(built, tmp_path, name):
    """`gkval init` writes the reference's manifests (plus the hash key)."""
    want = json.load(open(os.path.join(HERE, "golden", "gkval_manifests", name + ".json")))
    tol = want["tolerances"]
    args = ["init", "--run-id", name, "--runs-dir", "runs"]
    if tol["max_ulps"] == 0:
        args += ["--profile", "bitexact"]
    else:
        args += ["--atol", repr(tol["atol"]), "--rtol", repr(tol["rtol"]), "--max-ulps", str(tol["max_ulps"]),
                 "--quant-lsb", str(want["quant_lsb"])]
    _run(args, tmp_path)
    got = json.loads((tmp_path / "runs" / name / "manifest.json").read_text())
    assert got.pop("hash") == "sha256"
    assert got == want


def test_cli_self_check_audit_and_tamper(built, tmp_path):
    (tmp_path / "cases.txt").write_text(CASES)
    _run(["init", "--run-id", "BX", "--profile", "bitexact"], tmp_path)
    p = _run(["validate", "BX", "--cases", "cases.txt", "--port", "oracle"], tmp_path)
    assert "4 passed, 0 failed" in p.stdout
    run = tmp_path / "runs" / "BX"
    led = _ledger(run)
    assert [l["case_id"] for l in led] == [0, 1, 2, 3] and all(l["success"] for l in led)
    assert all(l["max_ulp"] == [0] * 5 for l in led)
    assert len({l["case_root"] for l in led}) == 4 and all(l["case_root"] != "0" * 64 for l in led)
    assert "4 verified, 0 mismatched" in _run(["audit", "BX"], tmp_path).stdout
    # resume after completion adds nothing
    _run(["validate", "BX", "--cases", "cases.txt", "--port", "oracle", "--resume"], tmp_path)
    assert len(_ledger(run)) == 4
    # a changed root is caught
    text = (run / "ledger.ndjson").read_text()
    r0 = led[1]["case_root"]
    (run / "ledger.ndjson").write_text(text.replace(r0, r0[:-1] + ("0" if r0[-1] != "0" else "1")))
    p = _run(["audit", "BX"], tmp_path, ok=(2,))
    assert "case 1: MISMATCH" in p.stdout and "3 verified, 1 mismatched" in p.stdout


def test_cli_planted_difference(built, tmp_path):
    """A difference planted in the port data (on the CPU) is reported at its
    index with the reference's window rule, and audited."""
    (tmp_path / "cases.txt").write_text(CASES)
    _run(["init", "--run-id", "PL", "--profile", "relaxed", "--hash", "placeholder"], tmp_path)
    p = _run(["validate", "PL", "--cases", "cases.txt", "--port", "oracle", "--plant", "t:2000:50"], tmp_path)
    assert "4 passed" in p.stdout                   # 50 ULPs is within the relaxed profile's 100
    p = _run(["validate", "PL", "--cases", "cases.txt", "--port", "oracle", "--plant", "mu:1037:101"], tmp_path,
             ok=(2,))
    assert "0 passed, 4 failed" in p.stdout
    run = tmp_path / "runs" / "PL"
    led = _ledger(run)
    fails = [l for l in led if not l["success"]]
    assert len(fails) == 4
    for l in fails:
        assert l["first_fail"] == {"field": "mu", "index": 1037} and l["case_root"] == "0" * 64
        assert l["max_ulp"][1] == 101
        wpath = run / "fail_windows" / str(l["case_id"]) / "mu_1024_1056.bin"
        w = gg.read_fail_window(str(wpath))
        assert (w["field"], w["start"], w["end"]) == (1, 1024, 1056)
        diff = [gk_ulp(a, b) for a, b in zip(w["ref"], w["port"])]
        assert diff[1037 - 1024] == 101 and sum(d != 0 for d in diff) == 1
    assert "8 verified, 0 mismatched" in _run(["audit", "PL"], tmp_path).stdout
    p = _run(["diff", "PL", "2", "mu"], tmp_path)
    assert "samples [1024, 1056)" in p.stdout and p.stdout.count("\n") >= 34
    assert "no fail windows" in _run(["diff", "PL", "2", "phi"], tmp_path).stdout
    # the placeholder hash gives other roots than SHA-256 for the same data
    _run(["init", "--run-id", "SH", "--profile", "relaxed"], tmp_path)
    _run(["validate", "SH", "--cases", "cases.txt", "--port", "oracle"], tmp_path)
    roots_sha = [l["case_root"] for l in _ledger(tmp_path / "runs" / "SH")]
    roots_ph = [l["case_root"] for l in led[:4]]
    assert all(a != b for a, b in zip(roots_sha, roots_ph))


def gk_ulp(a, b):
    return oracle.gkval().gkv_ulp_distance(float(a), float(b))


def test_cli_rejects_bad_arguments(built, tmp_path):
    _run(["init"], tmp_path, ok=(1,))
    _run(["init", "--run-id", "X", "--profile", "nope"], tmp_path, ok=(1,))
    _run(["init", "--run-id", "X", "--quant-lsb", "53"], tmp_path, ok=(1,))
    _run(["validate", "MISSING", "--port", "oracle"], tmp_path, ok=(1,))
    _run(["init", "--run-id", "X"], tmp_path)
    _run(["validate", "X", "--port", "oracle", "--plant", "bogus:1:1"], tmp_path, ok=(1,))
    _run(["validate", "X", "--port", "oracle", "--cases", "absent.txt"], tmp_path, ok=(1,))
    p = _run(["validate", "X", "--port", "oracle"], tmp_path)   # the built-in case
    assert "1 passed" in p.stdout
