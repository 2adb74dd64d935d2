"""Build recipes: the CUDA library (sm_103a), the render CLI and the CPU oracle.

Everything is compiled in-tree with explicit nvcc / g++ command lines (no
cmake, no setuptools), so the same recipe runs on x86 and on the Arm GPU host.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "nullpath_gb300")
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
LIBNAME = "libnullpath_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "-Xcompiler", "-ffp-contract=off",
           "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["np_render.cu", "geokerr.cu", "adjoint.cu", "kerr_api.cu", "carlson.cu", "schwarzschild.cu"]
# The GEOKERR solver (geokerr.cu) is compiled without implicit multiply-add
# contraction, and its source spells out the operation order of its CPU
# restatement (oracle/geokerr_oracle.cpp, -ffp-contract=off): for rays that
# pass near a pole the sampled phi has a condition number of ~3e4 in the
# potential's coefficients, so the two agree to 1e-12 only with the same
# rounding.  The same holds between its device code and its host build
# (np_geokerr_points_host): both evaluate the closed forms of geokerr_cf.cuh
# with +, -, *, / and sqrt only, so they give the same bits.
PER_FILE_NVFLAGS = {"geokerr.cu": ["-fmad=false"]}


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd, cwd=None):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _deps():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def build_library(force=False, verbose=False):
    """Compiles csrc/*.cu into nullpath_gb300/lib/libnullpath_gb300.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    target = os.path.join(LIBDIR, LIBNAME)
    if not force and not _stale(target, _deps()):
        return target
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
        out = _run([nvcc] + ARCH + NVFLAGS + PER_FILE_NVFLAGS.get(src, []) +
                   ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", obj])
        if verbose:
            print(out)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(CU_SOURCES))) as ex:
        objs = list(ex.map(compile_one, CU_SOURCES))
    tmp = target + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, target)
    return target


def build_cli(force=False):
    """Links the `render` command-line tool (csrc/render_cli.cpp) against the library."""
    src = os.path.join(CSRC, "render_cli.cpp")
    if not os.path.exists(src):
        return None
    target = os.path.join(LIBDIR, "render")
    lib = os.path.join(LIBDIR, LIBNAME)
    if not force and not _stale(target, [src, lib, os.path.join(INCLUDE, "np_render.h")]):
        return target
    cxx = shutil.which("g++") or "g++"
    _run([cxx, "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, src, "-o", target,
          "-L" + LIBDIR, "-lnullpath_gb300", "-Wl,-rpath,$ORIGIN"])
    return target


def build_oracle(force=False):
    """Builds oracle/liboracle.so, and oracle/_ref from the reference checkout
    named by NP_REFERENCE_DIR (default /root/reference) when it exists."""
    args = ["make", "-s", "-C", ORACLE]
    ref = os.environ.get("NP_REFERENCE_DIR", "/root/reference")
    if os.path.isfile(os.path.join(ref, "include", "bh_kerr.h")):
        args.append("REF_DIR=" + ref)
    if force:
        args.append("-B")
    _run(args)
    return os.path.join(ORACLE, "liboracle.so")


def build_all(force=False, verbose=False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_library, force, verbose)
        f_orc = ex.submit(build_oracle, force)
        lib = f_lib.result()
        orc = f_orc.result()
    cli = build_cli(force)
    return lib, orc, cli
