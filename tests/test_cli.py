"""The `render` command-line tool (csrc/render_cli.cpp): the reference's
validation messages and exit codes (render.cu:431-465) without a GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "nullpath_gb300", "lib", "render")


def _run(*args):
    p = subprocess.run([CLI] + list(args), capture_output=True, text=True, timeout=60)
    return p.returncode, p.stdout, p.stderr


@pytest.mark.parametrize("args,msg", [
    (["--w", "0"], "Invalid image dimensions."),
    (["-h", "-3"], "Invalid image dimensions."),
    (["--tile", "0"], "Invalid tile height."),
    (["--samples", "0"], "Invalid samples per pixel."),
    (["--spp-total", "-1"], "Invalid total spp."),
    (["--frames", "0"], "Invalid frame count."),
    (["--mass", "0"], "Invalid mass or camera radius."),
    (["--rcam", "-2"], "Invalid mass or camera radius."),
    (["--spin", "1.0"], "Spin must satisfy |a/M| < 1."),
    (["--fov", "179"], "Invalid FOV; expected (0, 179) degrees."),
])
def test_invalid_arguments_exit_1(built, args, msg):
    rc, out, err = _run(*args)
    assert rc == 1 and err.strip() == msg


def test_no_device_reported(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    rc, out, err = _run("--w", "8", "--h", "8")
    assert rc == 1 and "No CUDA devices found." in err


@pytest.mark.parametrize("args,msg", [
    (["--precision", "mixed", "--crossing", "root"], "Root crossings on --precision mixed need --integrator rkf78."),
    (["--mode", "research", "--precision", "mixed"], "Research mode needs --precision fp64."),
    (["--precision", "mixed", "--integrator", "rkf78", "--inv-gate", "1e-12"],
     "The invariant gate needs --precision fp64."),
])
def test_research_settings_need_fp64(built, args, msg):
    """Research mode and the invariant gate run on the FP64 path only, and
    root crossings on the mixed path are Henon steps of its 7(8) integrator;
    the CLI refuses the other combinations before touching a device."""
    rc, out, err = _run("--w", "8", "--h", "8", *args)
    assert rc == 1 and err.strip() == msg


@pytest.mark.parametrize("args,msg", [
    (["--inv-gate", "-1"], "Invalid invariant gate."),
    (["--inv-gate", "2"], "Invalid invariant gate."),
])
def test_invalid_research_arguments(built, args, msg):
    rc, out, err = _run("--w", "8", "--h", "8", *args)
    assert rc == 1 and err.strip() == msg


def test_resume_file_checks(built, tmp_path):
    """--resume reads and checks the accumulator file before any device work."""
    import struct
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(tmp_path / "absent.npac"))
    assert rc == 1 and err.strip() == "Cannot read %s." % (tmp_path / "absent.npac")
    bad = tmp_path / "bad.npac"
    bad.write_bytes(b"not an accumulator")
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(bad))
    assert rc == 1 and err.strip() == "%s is not an accumulator file." % bad
    old = tmp_path / "old.npac"
    old.write_bytes(struct.pack("<5I", 0x4341504E, 1, 8, 8, 2) + b"\0" * 4 * (3 * 64 + 64 + 3))
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(old))
    assert rc == 1 and err.strip() == "%s is an accumulator of another version (no scene hash); render it again." % old
    other = tmp_path / "other.npac"
    other.write_bytes(struct.pack("<7I", 0x4341504E, 2, 4, 4, 2, 0, 0) + b"\0" * 4 * (3 * 16 + 16 + 3))
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(other))
    assert rc == 1 and err.strip() == "%s holds a different image size." % other
    scene = tmp_path / "scene.npac"
    scene.write_bytes(struct.pack("<7I", 0x4341504E, 2, 8, 8, 2, 123, 456) + b"\0" * 4 * (3 * 64 + 64 + 3))
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(scene))
    assert rc == 1 and err.strip() == ("%s was rendered from a different scene, precision or --samples; "
                                       "it cannot be resumed." % scene)
    short = tmp_path / "short.npac"
    short.write_bytes(struct.pack("<3I", 0x4341504E, 2, 8))
    rc, out, err = _run("--w", "8", "--h", "8", "--resume", str(short))
    assert rc == 1 and err.strip() == "%s is truncated." % short
    rc, out, err = _run("--w", "8", "--h", "8", "--frames", "3", "--accum-out", str(tmp_path / "a.npac"))
    assert rc == 1 and err.strip() == "--resume and --accum-out need a single frame."
