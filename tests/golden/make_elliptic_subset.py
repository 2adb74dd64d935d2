"""Writes elliptic_subset.txt: every 8th R_F / R_C / R_D row of the
reference's elliptic fixtures (geokerr_port/validation/test_data/
elliptic_inputs.dat and elliptic_reference.dat, the Fortran Carlson values to
12 significant digits), as `kind x y z p value` lines.  R_J rows of those
files are not valid references and are left out.

    python tests/golden/make_elliptic_subset.py <reference checkout>
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    d = os.path.join(ref_root, "geokerr_port", "validation", "test_data")
    inp = [l.split() for l in open(os.path.join(d, "elliptic_inputs.dat")) if l.strip() and not l.strip().isdigit()]
    ref = [l.split() for l in open(os.path.join(d, "elliptic_reference.dat")) if l.strip() and not l.strip().isdigit()]
    assert len(inp) == len(ref)
    rows = []
    for i, (a, b) in enumerate(zip(inp, ref)):
        if a[0].upper() not in ("RF", "RC", "RD") or i % 8:
            continue
        assert a[0] == b[0]
        rows.append(" ".join([a[0].upper()] + a[1:5] + [b[-1]]))
    with open(os.path.join(HERE, "elliptic_subset.txt"), "w") as f:
        f.write("# kind x y z p value   (every 8th R_F/R_C/R_D row of the reference's elliptic fixtures)\n")
        f.write("\n".join(rows) + "\n")
    print(len(rows), "rows")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: %s <reference checkout>" % sys.argv[0])
    main(sys.argv[1])
