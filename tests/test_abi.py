"""The C ABI library loads without a GPU, exports every function declared in
include/*.h, and its structs have the layout the Python mirror assumes."""
import ctypes as C
import os
import re
import subprocess

import pytest

import nullpath_gb300 as npx
from nullpath_gb300._abi import Scene, RenderStats

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _declared_functions():
    names = set()
    for f in os.listdir(INC):
        # np_kerr.h is a header-only C++ API (inline functions), not a C ABI
        if not f.endswith(".h") or f == "np_kerr.h":
            continue
        src = open(os.path.join(INC, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_functions():
    names = _declared_functions()
    assert "np_render_device" in names and "np_render_host" in names


@pytest.mark.parametrize("name", _declared_functions())
def test_library_exports_declared_symbol(built, name):
    lib = C.CDLL(npx.lib_path())
    assert hasattr(lib, name), name


def test_struct_layout_matches_c(built, tmp_path):
    fields = [f for f, _ in Scene._fields_]
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "np_render.h"', 'int main(void){',
            'printf("%zu %zu\\n", sizeof(np_scene_t), sizeof(np_render_stats_t));']
    for f in fields:
        prog.append('printf("%%zu\\n", offsetof(np_scene_t, %s));' % f)
    prog.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(prog))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I" + INC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == C.sizeof(Scene)
    assert int(out[1]) == C.sizeof(RenderStats)
    for f, off in zip(fields, out[2:]):
        assert getattr(Scene, f).offset == int(off), f


def test_scene_helpers_and_validation(built):
    lib = npx.load()
    s = Scene()
    lib.np_scene_defaults(C.byref(s))
    assert (s.width, s.height, s.mass, s.r_cam, s.max_steps) == (1280, 720, 10.0, 50.0, 10000)
    assert lib.np_scene_validate(C.byref(s)) == 0
    b = Scene()
    lib.np_scene_benchmark(C.byref(b))
    ref = npx.benchmark_scene()
    for f, _ in Scene._fields_:
        assert getattr(b, f) == getattr(ref, f), f
    assert abs(lib.np_isco_radius(1.0, 0.0) - 6.0) < 1e-12
    assert abs(lib.np_isco_radius(1.0, 0.9) - 2.3208830417618866) < 1e-12
    # render.cu:431-465 rejections
    for bad in (dict(width=0), dict(spp=0), dict(mass=-1.0), dict(spin=1.0), dict(fov_y_deg=179.0)):
        t = s.replace(**bad)
        assert lib.np_scene_validate(C.byref(t)) == npx._abi.NP_ERR_INVALID
        assert lib.np_last_error()


def test_render_host_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(npx.NullPathError):
        npx.render_host(npx.benchmark_scene(width=8, height=8, spp=1))


def test_batch_struct_layouts(built, tmp_path):
    from nullpath_gb300.batch import BatchStats, BatchTune
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "np_render.h"', 'int main(void){',
            'printf("%zu %zu\\n", sizeof(np_batch_stats_t), sizeof(np_batch_tune_t));']
    for f, _ in BatchStats._fields_:
        prog.append('printf("%%zu\\n", offsetof(np_batch_stats_t, %s));' % f)
    for f, _ in BatchTune._fields_:
        prog.append('printf("%%zu\\n", offsetof(np_batch_tune_t, %s));' % f)
    prog.append("return 0;}")
    src = tmp_path / "blayout.c"
    src.write_text("\n".join(prog))
    exe = tmp_path / "blayout"
    subprocess.run(["gcc", "-I" + INC, str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == C.sizeof(BatchStats) and out[1] == C.sizeof(BatchTune)
    offs = out[2:]
    for (f, _), off in zip(BatchStats._fields_, offs[:len(BatchStats._fields_)]):
        assert getattr(BatchStats, f).offset == off, f
    for (f, _), off in zip(BatchTune._fields_, offs[len(BatchStats._fields_):]):
        assert getattr(BatchTune, f).offset == off, f


def test_uneven_scene_draws():
    from nullpath_gb300.batch import uneven_scenes, RESOLUTIONS
    a = uneven_scenes(256, seed=1)
    b = uneven_scenes(256, seed=1)
    assert [(s.width, s.spp, s.spin, s.theta_deg, s.disk_max_orders) for s in a] == \
           [(s.width, s.spp, s.spin, s.theta_deg, s.disk_max_orders) for s in b]
    assert all(s.width == s.height and s.width in RESOLUTIONS for s in a)
    assert all(1 <= s.spp <= 8 and 1 <= s.disk_max_orders <= 3 for s in a)
    assert all(0.0 <= s.spin <= 0.998 and 5.0 <= s.theta_deg <= 85.0 for s in a)
    assert {s.width for s in a} == set(RESOLUTIONS)


def test_non_finite_fields_are_rejected(built):
    """Fault injection on the host: NaN or infinite values in any floating
    field of the scene are refused with NP_ERR_INVALID and a message, before
    any device work."""
    lib = npx.load()
    base = npx.benchmark_scene(width=8, height=8, spp=1)
    assert lib.np_scene_validate(C.byref(base)) == 0
    nan, inf = float("nan"), float("inf")
    for f, typ in Scene._fields_:
        if typ is not C.c_double:
            continue
        for v in (nan, inf, -inf):
            t = base.replace(**{f: v})
            assert lib.np_scene_validate(C.byref(t)) == npx._abi.NP_ERR_INVALID, (f, v)
            assert lib.np_last_error(), f
    # tolerances must be positive (rtol) and non-negative (atol)
    assert lib.np_scene_validate(C.byref(base.replace(rtol=0.0))) == npx._abi.NP_ERR_INVALID
    assert lib.np_scene_validate(C.byref(base.replace(atol=-1.0))) == npx._abi.NP_ERR_INVALID
