"""The `render` tool on the GPU: progressive passes, device tone mapping and
the PPM / raw outputs against the library's own render of the same scene."""
import json
import os
import subprocess

import numpy as np
import pytest

import nullpath_gb300 as npx

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "nullpath_gb300", "lib", "render")


def _read_ppm(path):
    data = open(path, "rb").read()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6" and parts[2] == b"255"
    w, h = map(int, parts[1].split())
    return np.frombuffer(parts[3], dtype=np.uint8).reshape(h, w, 3)


def _read_raw(path):
    b = open(path, "rb").read()
    magic, ver, w, h, spp = np.frombuffer(b[:20], dtype=np.uint32)
    assert magic == 0x5752504E and ver == 1
    f = np.frombuffer(b[20:], dtype=np.float32)
    return f[:3 * w * h].reshape(3, h, w), f[3 * w * h:].reshape(h, w), int(spp)


def _tonemap(mean, ev=0.0, gamma=2.2, reinhard=False):
    v = mean.astype(np.float32) * np.float32(2.0 ** ev)
    if reinhard:
        v = v / (np.float32(1) + v)
    if abs(gamma - 1.0) > 1e-6:
        v = np.power(np.maximum(v, 0).astype(np.float32), np.float32(1.0 / gamma))
    v = np.clip(v, 0, 1)
    return (np.float32(255) * v).astype(np.uint8).transpose(1, 2, 0)


def test_cli_passes_match_library_render(cuda, tmp_path):
    out = str(tmp_path / "a.ppm")
    raw = str(tmp_path / "a.raw")
    side = str(tmp_path / "a.json")
    p = subprocess.run([CLI, "--w", "48", "--h", "32", "--samples", "2", "--spp-total", "6", "--checkpoint-every", "2",
                        "--spin", "0.6", "--theta", "75", "--tonemap", "reinhard", "--exposure", "1",
                        "--out", out, "--out-raw", raw, "--json", side], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.strip().splitlines()
    assert lines[-1] == "Wrote %s" % out
    # checkpoints after every 2nd pass and after the last (render.cu:570)
    assert [l.split("@")[1].strip() for l in lines[:-1]] == ["4 spp", "6 spp"]
    mean, rc, spp = _read_raw(raw)
    assert spp == 6
    sc = npx.reference_defaults().replace(width=48, height=32, spp=6, spin=0.6, theta_deg=75.0)
    rgb, rcross = npx.render(sc, "fp64")
    ref = rgb.cpu().numpy() / 6.0
    assert np.allclose(mean, ref, rtol=1e-6, atol=1e-7)
    ppm = _read_ppm(out)
    want = _tonemap(mean, ev=1.0, reinhard=True)
    diff = np.abs(ppm.astype(int) - want.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.999
    meta = json.load(open(side))
    assert meta["spp"] == 6 and meta["passes"] == 3 and meta["precision"] == "fp64"


def test_cli_frames_and_pattern(cuda, tmp_path):
    pat = str(tmp_path / "f_%03d.ppm")
    side = str(tmp_path / "f.json")
    p = subprocess.run([CLI, "--w", "24", "--h", "16", "--frames", "3", "--turns", "0.5", "--phi0", "20",
                        "--outpat", pat, "--bg", "point", "--json", side,
                        "--precision", "mixed", "--benchmark", "--w", "24", "--h", "16"],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    files = [pat % i for i in range(3)]
    assert all(os.path.exists(f) for f in files)
    imgs = [_read_ppm(f) for f in files]
    # the spacetime, disk and both skies depend on no azimuth (render.cu:74-86,
    # 312-359): every frame gives the same image, so the orbit is checked
    # through the azimuth each frame was rendered at (render.cu:630-635)
    assert imgs[0].shape == (16, 24, 3) and np.array_equal(imgs[0], imgs[1]) and np.array_equal(imgs[0], imgs[2])
    phis = json.load(open(side))["frame_phi_deg"]
    want = [20.0 + 360.0 * 0.5 * float(np.float32(i) / np.float32(3)) for i in range(3)]
    assert np.allclose(phis, want, rtol=0, atol=1e-9), phis
    bad = subprocess.run([CLI, "--w", "8", "--h", "8", "--frames", "2", "--outpat", str(tmp_path / "x_%d_%d.ppm")],
                         capture_output=True, text=True, timeout=120)
    assert bad.returncode == 1 and "Invalid --outpat" in bad.stderr


def test_camera_azimuth_rotates_crossings(cuda):
    """phi_deg enters the ray start: every equatorial crossing's azimuth moves
    by exactly the camera's azimuth, and nothing else changes."""
    sc = npx.benchmark_scene(width=32, height=18, spp=1)
    rng = np.random.default_rng(4)
    px, py = rng.uniform(0, 32, 400), rng.uniform(0, 18, 400)
    a = {k: v.cpu().numpy() for k, v in npx.trace_rays(sc, px, py, precision="fp64").items()}
    b = {k: v.cpu().numpy() for k, v in npx.trace_rays(sc.replace(phi_deg=37.0), px, py, precision="fp64").items()}
    ca, cb = a["cross"], b["cross"]
    assert np.array_equal(a["status"], b["status"]) and np.array_equal(ca[..., 0], cb[..., 0])
    hit = ca[..., 0] > 0
    assert hit.sum() > 100
    d = np.angle(np.exp(1j * (cb[..., 1][hit] - ca[..., 1][hit] - np.radians(37.0))))
    assert np.abs(d).max() < 1e-9


def test_resume_is_bit_identical(cuda, tmp_path):
    """An interrupted render resumed from its accumulator file ends
    bit-identical to the uninterrupted one (same --samples per pass)."""
    common = ["--w", "40", "--h", "24", "--samples", "2", "--spin", "0.7", "--theta", "70", "--precision", "mixed"]
    full_raw, full_ppm = str(tmp_path / "full.raw"), str(tmp_path / "full.ppm")
    p = subprocess.run([CLI] + common + ["--spp-total", "8", "--out", full_ppm, "--out-raw", full_raw],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    acc = str(tmp_path / "half.npac")
    p = subprocess.run([CLI] + common + ["--spp-total", "4", "--out", str(tmp_path / "half.ppm"),
                                         "--accum-out", acc], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    res_raw, res_ppm = str(tmp_path / "res.raw"), str(tmp_path / "res.ppm")
    p = subprocess.run([CLI] + common + ["--spp-total", "8", "--resume", acc, "--out", res_ppm, "--out-raw", res_raw],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip().splitlines()[-2].split("@")[1].strip() == "8 spp"
    m1, r1, s1 = _read_raw(full_raw)
    m2, r2, s2 = _read_raw(res_raw)
    assert s1 == s2 == 8
    assert np.array_equal(m1, m2) and np.array_equal(r1, r2)
    assert np.array_equal(_read_ppm(full_ppm), _read_ppm(res_ppm))
    # the file carries a hash of the scene: another spin, precision or
    # --samples refuses to resume it
    for change in (["--spin", "0.5"], ["--precision", "fp64"], ["--samples", "1"]):
        args = list(common)
        i = args.index(change[0])
        args[i + 1] = change[1]
        p = subprocess.run([CLI] + args + ["--spp-total", "8", "--resume", acc, "--out", res_ppm],
                           capture_output=True, text=True, timeout=300)
        assert p.returncode == 1 and "different scene" in p.stderr, (change, p.stderr)
    # a truncated leftover of an interrupted write (acc + ".tmp") is ignored
    with open(acc + ".tmp", "wb") as f:
        f.write(b"NPAC")
    p = subprocess.run([CLI] + common + ["--spp-total", "8", "--resume", acc, "--out", res_ppm],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
