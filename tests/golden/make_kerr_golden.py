"""Generates tests/golden/kerr_api_golden.txt: the output of
kerr_api_probe.cpp built against the reference's own physics headers
(include/bh_common.h, bh_types.h, bh_kerr.h, bh_schwarzschild.h of the
reference checkout), with the flags the tests use for the np_kerr.h build.

    python tests/golden/make_kerr_golden.py <reference checkout>
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math"]


def main(ref):
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "probe_ref")
        subprocess.run(["g++"] + FLAGS + ["-DPROBE_REF", "-D__device__=", "-D__host__=", "-D__global__=",
                                          "-I" + os.path.join(ref, "include"), "-I/usr/local/cuda/include",
                                          os.path.join(HERE, "kerr_api_probe.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    with open(os.path.join(HERE, "kerr_api_golden.txt"), "w") as f:
        f.write(out)
    print("wrote %d values" % len(out.splitlines()))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: %s <reference checkout>" % sys.argv[0])
    main(sys.argv[1])
