"""Writes tests/golden/geokerr_cf_truth.npz: GEOKERR points of camera-grid
rays computed in closed form at 40 digits (oracle/geokerr_cf_mp.py), the
truth against which the library's closed form and the Taylor oracle are
both measured.  Rays: per spin, the 128 x 128 standard grid (r_o = 1e6 M,
i = 60 deg, [-12, 12]^2, 32 points) cells of smallest |l| (near-polar
orbits), closest to the shadow edge on both sides (near-double radial
roots), and a seeded random sample.

    python tests/golden/make_geokerr_cf_truth.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import geokerr_cf_mp as cfmp  # noqa: E402


def pick(a, g, rng):
    l, q2 = g["l"], g["q2"]
    ok = q2 > 0
    idx = list(np.argsort(np.where(ok, np.abs(l), np.inf))[:4])
    # distance from the shadow edge: smallest |sigma| or |u3 - u2| of U's roots
    gap = np.full(l.size, np.inf)
    for i in np.flatnonzero(ok):
        r = np.roots([-a * a * q2[i], 2 * ((l[i] - a) ** 2 + q2[i]), a * a - l[i] ** 2 - q2[i], 0.0, 1.0])
        c = r[np.abs(r.imag) > 1e-12]
        rr = np.sort(r[np.abs(r.imag) <= 1e-12].real)
        gap[i] = np.min(np.abs(c.imag)) if c.size else (rr[2] - rr[1] if rr.size == 4 else np.inf)
    idx += list(np.argsort(gap)[:4])
    idx += list(rng.choice(np.flatnonzero(ok), 6, replace=False))
    return sorted(set(int(i) for i in idx))


def main():
    rng = np.random.default_rng(11)
    rows = []
    for a in (0.9, 0.5, 0.998, 0.1):
        g = oracle.geokerr_camera_grid(a, 0.5, 128, 128)
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        for i in pick(a, g, rng):
            out = cfmp.points(1e-6, uplus, 0.5, a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i], 1, 32, 0.5)
            if out is None or len(out["u"]) != 32:
                continue
            rows.append((a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i],
                         [[float(x) for x in out[k]] for k in ("u", "mu", "dt", "dphi", "lam")],
                         out["tpm"], out["tpr"]))
            print(a, i, flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "geokerr_cf_truth.npz"),
                        a=np.array([r[0] for r in rows]), l=np.array([r[1] for r in rows]),
                        q2=np.array([r[2] for r in rows]), su=np.array([r[3] for r in rows]),
                        sm=np.array([r[4] for r in rows]), pts=np.array([r[5] for r in rows]),
                        tpm=np.array([r[6] for r in rows], dtype=np.int32),
                        tpr=np.array([r[7] for r in rows], dtype=np.int32))


if __name__ == "__main__":
    main()
