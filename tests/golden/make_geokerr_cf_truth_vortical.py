"""Writes tests/golden/geokerr_cf_truth_vortical.npz: GEOKERR points of the
q2 < 0 (vortical) rays of the 128 x 128 standard grid (r_o = 1e6 M,
i = 60 deg, [-12, 12]^2, 32 points) at a = 0.9 and 0.998, computed at 40
digits by quadrature (oracle/geokerr_cf_mp.py, points_vortical): the truth
for the library's closed forms of these rays (two real radial roots below
the motion, or two complex pairs).

    python tests/golden/make_geokerr_cf_truth_vortical.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import geokerr_cf_mp as cfmp  # noqa: E402


def main():
    rows = []
    for a in (0.9, 0.998):
        g = oracle.geokerr_camera_grid(a, 0.5, 128, 128)
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        sel = np.flatnonzero(g["q2"] < 0)
        # every other vortical ray keeps the file small and spans both cases
        for i in sel[::3]:
            out = cfmp.points_vortical(1e-6, uplus, 0.5, a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i], 1, 32, 0.5)
            if out is None or len(out["u"]) != 32:
                continue
            rows.append((a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i],
                         [[float(x) for x in out[k]] for k in ("u", "mu", "dt", "dphi", "lam")],
                         out["tpm"], out["tpr"]))
            print(a, i, flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "geokerr_cf_truth_vortical.npz"),
                        a=np.array([r[0] for r in rows]), l=np.array([r[1] for r in rows]),
                        q2=np.array([r[2] for r in rows]), su=np.array([r[3] for r in rows]),
                        sm=np.array([r[4] for r in rows]), pts=np.array([r[5] for r in rows]),
                        tpm=np.array([r[6] for r in rows], dtype=np.int32),
                        tpr=np.array([r[7] for r in rows], dtype=np.int32))


if __name__ == "__main__":
    main()
